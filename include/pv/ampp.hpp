// C++ drop-in for pelican-lofar's beam-processing modules over the libpv C ABI.
//
// The classes keep the names, constructor (from the module's XML
// ConfigNode), run() signatures and data-set layouts of the reference
// modules, so pipeline code written against them compiles against this
// header instead:
//
//   AdapterTimeSeriesDataSet::config(), deserialise()                         lib/AdapterTimeSeriesDataSet.h
//   PPFChanneliser::run(const TimeSeriesDataSetC32*, SpectrumDataSetC32*)      lib/PPFChanneliser.h:68-69
//   StokesGenerator::run(const SpectrumDataSetC32*, SpectrumDataSetStokes*)   lib/StokesGenerator.h:42-43
//   StokesIntegrator::run(const SpectrumDataSetStokes*, SpectrumDataSetStokes*) lib/StokesIntegrator.h:46
//   RFI_Clipper::run(WeightedSpectrumDataSet*), bandPass()                    lib/RFI_Clipper.h:37-38
//   DedispersionModule::dedisperse(WeightedSpectrumDataSet*), connect(),
//       unlockCallback(), onChainCompletion(), waitForJobCompletion(),
//       lockNumber(), maxshift(), numberOfSamples()                            lib/DedispersionModule.h:76-104,
//                                                                              lib/AsyncronousModule.h:40-53
//   LockingPtrContainer::next(), unlock()                                     lib/LockingPtrContainer.hpp
//   DedispersionAnalyser::analyse(DedispersionSpectra*, DedispersionDataAnalysis*) lib/DedispersionAnalyser.h:31
//   SigprocStokesWriter::sendStream(), DedispersionDataAnalysisOutput::sendStream()
//                                                                              lib/SigprocStokesWriter.h,
//                                                                              lib/DedispersionDataAnalysisOutput.h
//
// XML options are read with the reference's element and attribute names
// and defaults.  Errors the reference throws as QString (or reports with
// exit()) are thrown here as std::runtime_error with the same text.  Data
// sets live in host memory as in the reference; each run() moves its data
// through device memory.  The DedispersionModule is asynchronous as the
// reference's: dedisperse() returns once the samples are in the device
// ring, a worker thread calls the connected functors, and input blobs stay
// locked (lockNumber) until the buffers holding their samples are
// exported.  DedispersionPipeline keeps a chunk on the device from the
// voltages to the dedispersion when it computes Stokes I only.
//
// Qt and the pelican core are absent: ConfigNode here is a small XML reader
// of one module element, and blobs are plain classes.
#pragma once

#include <pv.h>

#include <arpa/inet.h>
#include <netinet/in.h>
#include <sys/socket.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cctype>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <ctime>
#include <iostream>
#include <complex>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace pelican {

// ---------------------------------------------------------------------------
// ConfigNode: one XML element with attributes and child elements.
// ---------------------------------------------------------------------------
class ConfigNode {
  public:
    ConfigNode() = default;

    // The first element named `tag` in an XML document (any depth).
    static ConfigNode fromString(const std::string& xml, const std::string& tag) {
        std::vector<ConfigNode> roots;
        size_t pos = 0;
        parse_children(xml, pos, roots, "");
        const ConfigNode* n = find(roots, tag);
        if (!n) throw std::runtime_error("ConfigNode: no element <" + tag + ">");
        return *n;
    }
    static ConfigNode fromFile(const std::string& path, const std::string& tag) {
        std::ifstream f(path);
        if (!f) throw std::runtime_error("ConfigNode: cannot open " + path);
        std::stringstream ss;
        ss << f.rdbuf();
        ConfigNode n = fromString(ss.str(), tag);
        const size_t slash = path.find_last_of('/');
        n.set_search_path(slash == std::string::npos ? "." : path.substr(0, slash));
        return n;
    }

    const std::string& name() const { return name_; }
    bool hasAttribute(const std::string& a) const { return attrs_.count(a) != 0; }
    std::string getAttribute(const std::string& a) const {
        auto it = attrs_.find(a);
        return it == attrs_.end() ? std::string() : it->second;
    }
    // The attribute of the first child element `tag` (ConfigNode::getOption).
    std::string getOption(const std::string& tag, const std::string& attribute,
                          const std::string& def = "") const {
        for (const auto& c : children_)
            if (c.name_ == tag && c.hasAttribute(attribute)) return c.getAttribute(attribute);
        return def;
    }
    // Resolves a file name against the configuration's directory.
    std::string searchFile(const std::string& file) const {
        if (file.empty()) throw std::runtime_error("file name empty");
        if (file[0] == '/' || std::ifstream(file).good()) return file;
        const std::string p = search_path_ + "/" + file;
        if (std::ifstream(p).good()) return p;
        throw std::runtime_error("file \"" + file + "\" not found");
    }
    void set_search_path(const std::string& p) {
        search_path_ = p;
        for (auto& c : children_) c.set_search_path(p);
    }
    const std::vector<ConfigNode>& children() const { return children_; }

  private:
    std::string name_;
    std::map<std::string, std::string> attrs_;
    std::vector<ConfigNode> children_;
    std::string search_path_ = ".";

    static const ConfigNode* find(const std::vector<ConfigNode>& nodes, const std::string& tag) {
        for (const auto& n : nodes) {
            if (n.name_ == tag) return &n;
            if (const ConfigNode* c = find(n.children_, tag)) return c;
        }
        return nullptr;
    }
    static void skip_ws(const std::string& s, size_t& p) {
        while (p < s.size() && std::isspace((unsigned char)s[p])) ++p;
    }
    // Parses elements until the closing tag `close` (or the end of the text).
    static void parse_children(const std::string& s, size_t& p, std::vector<ConfigNode>& out,
                               const std::string& close) {
        while (p < s.size()) {
            const size_t lt = s.find('<', p);
            if (lt == std::string::npos) { p = s.size(); return; }
            p = lt;
            if (s.compare(p, 4, "<!--") == 0) {
                const size_t e = s.find("-->", p);
                p = e == std::string::npos ? s.size() : e + 3;
                continue;
            }
            if (s.compare(p, 2, "<?") == 0 || s.compare(p, 2, "<!") == 0) {
                const size_t e = s.find('>', p);
                p = e == std::string::npos ? s.size() : e + 1;
                continue;
            }
            if (s.compare(p, 2, "</") == 0) {
                const size_t e = s.find('>', p);
                const std::string tag = trim(s.substr(p + 2, e - p - 2));
                p = e == std::string::npos ? s.size() : e + 1;
                if (tag != close)
                    throw std::runtime_error("ConfigNode: </" + tag + "> closes <" + close + ">");
                return;
            }
            ConfigNode n;
            ++p;
            const size_t ns = p;
            while (p < s.size() && !std::isspace((unsigned char)s[p]) && s[p] != '>' && s[p] != '/') ++p;
            n.name_ = s.substr(ns, p - ns);
            bool self_closing = false;
            for (;;) {
                skip_ws(s, p);
                if (p >= s.size()) throw std::runtime_error("ConfigNode: unterminated <" + n.name_ + ">");
                if (s[p] == '/') { self_closing = true; p = s.find('>', p) + 1; break; }
                if (s[p] == '>') { ++p; break; }
                const size_t as = p;
                while (p < s.size() && s[p] != '=' && !std::isspace((unsigned char)s[p])) ++p;
                const std::string key = s.substr(as, p - as);
                skip_ws(s, p);
                if (p >= s.size() || s[p] != '=') throw std::runtime_error("ConfigNode: attribute " + key);
                ++p;
                skip_ws(s, p);
                const char q = s[p];
                if (q != '"' && q != '\'') throw std::runtime_error("ConfigNode: unquoted " + key);
                const size_t ve = s.find(q, p + 1);
                n.attrs_[key] = s.substr(p + 1, ve - p - 1);
                p = ve + 1;
            }
            if (!self_closing) parse_children(s, p, n.children_, n.name_);
            out.push_back(std::move(n));
        }
        if (!close.empty()) throw std::runtime_error("ConfigNode: <" + close + "> not closed");
    }
    static std::string trim(const std::string& x) {
        size_t a = 0, b = x.size();
        while (a < b && std::isspace((unsigned char)x[a])) ++a;
        while (b > a && std::isspace((unsigned char)x[b - 1])) --b;
        return x.substr(a, b - a);
    }
};

namespace ampp {

// Throws the library's last error text for a failed call.
inline void pv_check(int rc) {
    if (rc != PV_OK) throw std::runtime_error(pv_last_error());
}
inline std::string lower(std::string s) {
    for (auto& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}
inline unsigned to_uint(const std::string& s) { return s.empty() ? 0u : (unsigned)std::stoul(s); }
inline float to_float(const std::string& s) { return s.empty() ? 0.0f : std::stof(s); }

// A device buffer owned by a module.
class DeviceBuffer {
  public:
    ~DeviceBuffer() { pv_device_free(p_); }
    void* get(size_t bytes) {
        if (bytes > n_) {
            pv_device_free(p_);
            p_ = nullptr;
            n_ = 0;
            pv_check(pv_device_alloc(&p_, (long long)bytes));
            n_ = bytes;
        }
        return p_;
    }
    template <typename T>
    T* as(size_t count) { return static_cast<T*>(get(count * sizeof(T))); }

  private:
    void* p_ = nullptr;
    size_t n_ = 0;
};

// ---------------------------------------------------------------------------
// Data sets (lib/TimeSeriesDataSet.h, lib/SpectrumDataSet.h)
// ---------------------------------------------------------------------------
class DataBlob {
  public:
    virtual ~DataBlob() = default;
    void setBlockRate(double r) { block_rate_ = r; }
    double getBlockRate() const { return block_rate_; }
    void setLofarTimestamp(double t) { timestamp_ = t; }
    double getLofarTimestamp() const { return timestamp_; }
    double getTime(unsigned sample) const { return timestamp_ + sample * block_rate_; }

  protected:
    double block_rate_ = 0.0, timestamp_ = 0.0;
};

// complex<float> [subband][polarisation][block][channel] (TimeSeriesDataSet.h:145-151)
class TimeSeriesDataSetC32 : public DataBlob {
  public:
    void resize(unsigned nBlocks, unsigned nSubbands, unsigned nPols, unsigned nTimesPerBlock) {
        nb_ = nBlocks; ns_ = nSubbands; np_ = nPols; nt_ = nTimesPerBlock;
        d_.assign((size_t)nb_ * ns_ * np_ * nt_, {0.0f, 0.0f});
    }
    unsigned nTimeBlocks() const { return nb_; }
    unsigned nSubbands() const { return ns_; }
    unsigned nPolarisations() const { return np_; }
    unsigned nTimesPerBlock() const { return nt_; }
    std::complex<float>* data() { return d_.data(); }
    const std::complex<float>* data() const { return d_.data(); }
    std::complex<float>* timeSeriesData(unsigned b, unsigned s, unsigned p) {
        return d_.data() + ((size_t)nb_ * (s * np_ + p) + b) * nt_;
    }

  private:
    unsigned nb_ = 0, ns_ = 0, np_ = 0, nt_ = 0;
    std::vector<std::complex<float>> d_;
};

// T [block][subband][polarisation][channel] (SpectrumDataSet.h:229-235)
template <typename T>
class SpectrumDataSet : public DataBlob {
  public:
    void resize(unsigned nBlocks, unsigned nSubbands, unsigned nPols, unsigned nChannels) {
        nb_ = nBlocks; ns_ = nSubbands; np_ = nPols; nc_ = nChannels;
        d_.assign((size_t)nb_ * ns_ * np_ * nc_, T());
    }
    // The shape without clearing the data (kept where the size does not change).
    void reshape(unsigned nBlocks, unsigned nSubbands, unsigned nPols, unsigned nChannels) {
        nb_ = nBlocks; ns_ = nSubbands; np_ = nPols; nc_ = nChannels;
        d_.resize((size_t)nb_ * ns_ * np_ * nc_);
    }
    unsigned nTimeBlocks() const { return nb_; }
    unsigned nSubbands() const { return ns_; }
    unsigned nPolarisations() const { return np_; }
    unsigned nChannels() const { return nc_; }
    size_t size() const { return d_.size(); }
    T* data() { return d_.data(); }
    const T* data() const { return d_.data(); }
    long index(unsigned s, unsigned nSub, unsigned p, unsigned nPol, unsigned b, unsigned nChan) const {
        return (long)nChan * (nPol * ((long)nSub * b + s) + p);
    }
    T* spectrumData(unsigned b, unsigned s, unsigned p) {
        return d_.data() + (size_t)nc_ * (np_ * ((size_t)ns_ * b + s) + p);
    }

  private:
    unsigned nb_ = 0, ns_ = 0, np_ = 0, nc_ = 0;
    std::vector<T> d_;
};
using SpectrumDataSetC32 = SpectrumDataSet<std::complex<float>>;
// float [time][subband][stokes][channel]
using SpectrumDataSetStokes = SpectrumDataSet<float>;

// The Stokes data and its weights, 1 everywhere (WeightedSpectrumDataSet.h:26-47).
class WeightedSpectrumDataSet : public DataBlob {
  public:
    explicit WeightedSpectrumDataSet(SpectrumDataSetStokes* d = nullptr) { reset(d); }
    void reset(SpectrumDataSetStokes* d) {
        data_ = d;
        if (d) {
            const size_t before = w_.size();
            w_.reshape(d->nTimeBlocks(), d->nSubbands(), d->nPolarisations(), d->nChannels());
            if (w_.size() > before) std::fill(w_.data() + before, w_.data() + w_.size(), 1.0f);
        }
    }
    SpectrumDataSetStokes* stats() const { return data_; }
    SpectrumDataSetStokes* dataSet() const { return data_; }
    SpectrumDataSet<float>* weights() { return &w_; }

  private:
    SpectrumDataSetStokes* data_ = nullptr;
    SpectrumDataSet<float> w_;
};

// ---------------------------------------------------------------------------
// Dedispersion results (lib/DedispersionSpectra.h, DedispersionDataAnalysis.h,
// DedispersionEvent.h)
// ---------------------------------------------------------------------------
class DedispersionSpectra : public DataBlob {
  public:
    void resize(unsigned timebins, unsigned dedispersionBins, float start, float width) {
        t_ = timebins; n_ = dedispersionBins; lower_ = start; width_ = width;
        d_.assign((size_t)t_ * n_, 0.0f);
    }
    std::vector<float>& data() { return d_; }
    const std::vector<float>& data() const { return d_; }
    // BinMap::binIndex / binAssignmentNumber (lib/src/BinMap.cpp)
    int dmIndex(float dm) const { return (int)(0.5 + ((double)dm - lower_) / width_); }
    float dm(unsigned i) const { return (float)(lower_ + width_ * i); }
    float dmAmplitude(unsigned t, int dm) const { return d_[t + (size_t)t_ * dm]; }
    float dmAmplitude(unsigned t, float dm) const { return dmAmplitude(t, dmIndex(dm)); }
    int dmBins() const { return (int)n_; }
    int timeSamples() const { return (int)t_; }
    float dmMax() const { return dm(n_ - 1); }
    double dmLow() const { return lower_; }
    double dmStep() const { return width_; }
    void setFirstSample(unsigned s) { first_ = s; }
    unsigned firstSample() const { return first_; }
    // the channel count the analyser's RMS is taken from (inputDataBlobs()[0])
    void setInputShape(unsigned nChannels, unsigned nSubbands) { nch_ = nChannels; nsub_ = nSubbands; }
    unsigned inputChannels() const { return nch_; }
    unsigned inputSubbands() const { return nsub_; }
    float getRMS() const { return rms_; }
    void setRMS(float r) { rms_ = r; }
    // The Stokes blobs whose samples the buffer holds, oldest first
    // (DedispersionSpectra::inputDataBlobs, filled by DedispersionBuffer::copy
    // and addSamples); valid while the functors run.
    const std::vector<const SpectrumDataSetStokes*>& inputDataBlobs() const { return inputs_; }
    void setInputDataBlobs(const std::vector<const SpectrumDataSetStokes*>& b) { inputs_ = b; }

  private:
    unsigned t_ = 0, n_ = 0, first_ = 0, nch_ = 0, nsub_ = 0;
    double lower_ = 0.0, width_ = 1.0;
    float rms_ = 0.0f;
    std::vector<float> d_;
    std::vector<const SpectrumDataSetStokes*> inputs_;
};

class DedispersionEvent {
  public:
    DedispersionEvent(int dmIndex, unsigned timeIndex, const DedispersionSpectra* d, float factor,
                      float value)
        : dm_(dmIndex), t_(timeIndex), d_(d), f_(factor), v_(value) {}
    unsigned timeBin() const { return t_; }
    float dm() const { return d_->dm(dm_); }
    int dmIndex() const { return dm_; }
    float amplitude() const { return d_->dmAmplitude(t_, dm_); }
    float mfValue() const { return v_; }
    float mfBinning() const { return f_; }
    double getTime() const { return d_->getTime(t_ + d_->firstSample()); }

  private:
    int dm_;
    unsigned t_;
    const DedispersionSpectra* d_;
    float f_, v_;
};

class DedispersionDataAnalysis : public DataBlob {
  public:
    void reset(const DedispersionSpectra* d) { data_ = d; ev_.clear(); }
    void addEvent(unsigned dm, unsigned timeBin, float factor, float value) {
        ev_.emplace_back((int)dm, timeBin, data_, factor, value);
    }
    int eventsFound() const { return (int)ev_.size(); }
    const std::vector<DedispersionEvent>& events() const { return ev_; }
    const DedispersionSpectra* data() const { return data_; }
    float getRMS() const { return rms_; }
    void setRMS(float r) { rms_ = r; }

  private:
    const DedispersionSpectra* data_ = nullptr;
    std::vector<DedispersionEvent> ev_;
    float rms_ = 0.0f;
};

// ---------------------------------------------------------------------------
// Modules
// ---------------------------------------------------------------------------

// lib/src/AdapterTimeSeriesDataSet.cpp:35-293.  The reference reads one
// chunk of UDP packets from a QIODevice; deserialise() takes the same bytes
// from host memory, unpacks them on the GPU and fills the blob given to
// config(), with the first packet's time stamp and block rate.
class AdapterTimeSeriesDataSet {
  public:
    explicit AdapterTimeSeriesDataSet(const ConfigNode& config) {
        c_.fixed_size_packets = lower(config.getOption("fixedSizePackets", "value", "true")).rfind("true", 0) == 0;
        c_.sample_bits = (int)to_uint(config.getOption("dataBitSize", "value", "0"));
        c_.packets_per_chunk = (int)to_uint(config.getOption("udpPacketsPerIteration", "value", "0"));
        c_.samples_per_packet = (int)to_uint(config.getOption("samplesPerPacket", "value", "0"));
        c_.nchan = (int)to_uint(config.getOption("outputChannelsPerSubband", "value", "0"));
        c_.nsub = (int)to_uint(config.getOption("subbandsPerPacket", "value", "0"));
        c_.npol = (int)to_uint(config.getOption("nRawPolarisations", "value", "0"));
        c_.clock_mhz = (int)to_uint(config.getOption("clock", "value", "200"));
    }
    // AbstractStreamAdapter::config: the blob to fill and the chunk's bytes.
    void config(TimeSeriesDataSetC32* data, size_t chunkSize) {
        data_ = data;
        chunk_ = chunkSize;
    }
    void deserialise(const void* chunk) {
        long long psize = 0;
        int nblocks = 0;
        pv_check(pv_udp_check(&c_, (long long)chunk_, &psize, &nblocks));
        if (!data_) throw std::runtime_error("AdapterTimeSeriesDataSet: Cannot deserialise into an unallocated blob!.");
        data_->resize((unsigned)nblocks, (unsigned)c_.nsub, (unsigned)c_.npol, (unsigned)c_.nchan);
        const size_t n = (size_t)nblocks * c_.nsub * c_.npol * c_.nchan;
        void* d_in = din_.get(chunk_);
        void* d_out = dout_.get(8 * n);
        pv_check(pv_device_copy(d_in, chunk, (long long)chunk_, nullptr));
        pv_check(pv_udp_unpack(&c_, d_in, (long long)chunk_, d_out, PV_UDP_OUT_C32, nullptr));
        pv_check(pv_device_copy(data_->data(), d_out, (long long)(8 * n), nullptr));
        pv_check(pv_synchronize(nullptr));
        double ts = 0.0, rate = 0.0;
        pv_check(pv_udp_time(&c_, chunk, &ts, &rate));
        data_->setLofarTimestamp(ts);
        data_->setBlockRate(rate);
        if (ts - last_ > rate) std::cout << "Adapter: data out of sequence -- " << ts - last_ << std::endl;
        last_ = ts + (double)nblocks * c_.nchan * rate;  // TimeSeriesDataSet::getEndLofarTimestamp
    }

  private:
    pv_udp_config c_{};
    TimeSeriesDataSetC32* data_ = nullptr;
    size_t chunk_ = 0;
    double last_ = 0.0;
    DeviceBuffer din_, dout_;
};

// lib/src/ABDataAdapter.cpp:14-173: options <spectrum packets>, <packet
// channels>, <packet samples>, <samplingTime seconds>.  deserialise() takes
// the chunk's bytes from host memory: the headers are read on the host
// (pv_ab_headers) and the Stokes-I spectra are assembled on the GPU
// (pv_ab_unpack) into the one-subband, one-polarisation blob given to
// config(), with the chunk's last packet's time and the sampling time.
class ABDataAdapter {
  public:
    explicit ABDataAdapter(const ConfigNode& config) {
        c_.packets_per_spectrum = (int)to_uint(config.getOption("spectrum", "packets"));
        c_.channels = (int)to_uint(config.getOption("packet", "channels"));
        c_.samples_per_packet = (int)to_uint(config.getOption("packet", "samples"));
        c_.tsamp = to_float(config.getOption("samplingTime", "seconds"));
    }
    // AbstractStreamAdapter::config: the blob to fill and the chunk's bytes.
    void config(SpectrumDataSetStokes* data, size_t chunkSize) {
        data_ = data;
        chunk_ = chunkSize;
    }
    void deserialise(const void* chunk) {
        if (!data_) throw std::runtime_error("ABDataAdapter: Cannot deserialise into an unallocated blob!.");
        const long long npk = c_.channels > 0 ? (long long)chunk_ / (8 + 8LL * c_.channels) : 0;
        std::vector<int> index((size_t)std::max<long long>(1, npk));
        long long nsp = 0, nbl = 0, gaps = 0;
        double ts = 0.0;
        pv_check(pv_ab_headers(&c_, &st_, chunk, (long long)chunk_, index.data(), (long long)index.size(), &nsp,
                               &nbl, &ts, &gaps));
        if (gaps) std::cerr << "FATAL! " << gaps << " packet(s) more than one sample after the previous" << std::endl;
        gaps_ += gaps;
        data_->resize((unsigned)nbl, 1, 1, (unsigned)c_.channels);
        void* d_in = din_.get(chunk_);
        int* d_index = dindex_.as<int>(index.size());
        float* d_out = dout_.as<float>(std::max<size_t>(1, data_->size()));
        pv_check(pv_device_copy(d_in, chunk, (long long)chunk_, nullptr));
        if (nsp) pv_check(pv_device_copy(d_index, index.data(), 4 * nsp, nullptr));
        pv_check(pv_ab_unpack(&c_, d_in, (long long)chunk_, d_index, nsp, nbl, d_out, nullptr));
        if (data_->size()) pv_check(pv_device_copy(data_->data(), d_out, (long long)(4 * data_->size()), nullptr));
        pv_check(pv_synchronize(nullptr));
        data_->setLofarTimestamp(ts);
        data_->setBlockRate(c_.tsamp);
    }
    long long gaps() const { return gaps_; }

  private:
    pv_ab_config c_{};
    pv_ab_state st_{};
    SpectrumDataSetStokes* data_ = nullptr;
    size_t chunk_ = 0;
    long long gaps_ = 0;
    DeviceBuffer din_, dindex_, dout_;
};

// lib/src/PPFChanneliser.cpp:29-290
class PPFChanneliser {
  public:
    explicit PPFChanneliser(const ConfigNode& config) {
        nchan_ = to_uint(config.getOption("outputChannelsPerSubband", "value", "512"));
        const unsigned taps = to_uint(config.getOption("filter", "nTaps", "8"));
        const std::string window = lower(config.getOption("filter", "filterWindow", "kaiser"));
        const int w = pv_window_from_name(window.c_str());
        if (w < 0) throw std::runtime_error(pv_last_error());
        pv_check(pv_ppf_create(&h_, (int)nchan_, (int)taps, w, nullptr));
    }
    ~PPFChanneliser() { pv_ppf_destroy(h_); }
    PPFChanneliser(const PPFChanneliser&) = delete;
    PPFChanneliser& operator=(const PPFChanneliser&) = delete;

    // run() followed by StokesGenerator's Stokes I, fused in one device pass
    // into d_stokes [block][subband][1][channel] (the fused pipeline); the
    // values equal run() then StokesGenerator::run with numberOfStokes 1.
    void runStokesIDevice(const TimeSeriesDataSetC32* in, float* d_stokes, void* stream) {
        if (!in || in->nTimeBlocks() == 0 || in->nSubbands() == 0)
            throw std::runtime_error("PPFChanneliser: Empty time data blob");
        if (in->nTimesPerBlock() != nchan_)
            throw std::runtime_error("PPFChanneliser: Data blob has incorrect number of channels");
        if (in->nPolarisations() != 2) throw std::runtime_error("StokesGenerator: needs 2 polarisations");
        const unsigned ns = in->nSubbands(), nb = in->nTimeBlocks();
        const size_t n = (size_t)ns * 2 * nb * nchan_;
        float* d_in = din_.as<float>(2 * n);
        pv_check(pv_device_copy(d_in, in->data(), (long long)(8 * n), stream));
        int nu = 0;
        pv_check(pv_channelise(h_, d_in, 0, (int)ns, (int)nb, 1, 1, 1, d_stokes, &nu, stream));
    }

    void run(const TimeSeriesDataSetC32* in, SpectrumDataSetC32* out) {
        if (!in || in->nTimeBlocks() == 0 || in->nSubbands() == 0)
            throw std::runtime_error("PPFChanneliser: Empty time data blob");
        if (in->nTimesPerBlock() != nchan_)
            throw std::runtime_error("PPFChanneliser: Data blob has incorrect number of channels");
        const unsigned ns = in->nSubbands(), np = in->nPolarisations(), nb = in->nTimeBlocks();
        const size_t n = (size_t)ns * np * nb * nchan_;
        float* d_in = din_.as<float>(2 * n);
        float* d_out = dout_.as<float>(2 * n);
        pv_check(pv_device_copy(d_in, in->data(), (long long)(8 * n), nullptr));
        pv_check(pv_ppf_run(h_, d_in, (int)ns, (int)np, (int)nb, d_out, nullptr));
        out->resize(nb, ns, np, nchan_);
        pv_check(pv_device_copy(out->data(), d_out, (long long)(8 * n), nullptr));
        pv_check(pv_synchronize(nullptr));
        out->setBlockRate(in->getBlockRate() * nchan_);  // PPFChanneliser.cpp:99
        out->setLofarTimestamp(in->getLofarTimestamp());
    }

    unsigned channels() const { return nchan_; }

  private:
    pv_ppf* h_ = nullptr;
    unsigned nchan_ = 0;
    DeviceBuffer din_, dout_;
};

// lib/src/StokesGenerator.cpp:40-108
class StokesGenerator {
  public:
    explicit StokesGenerator(const ConfigNode& config)
        : nstokes_(to_uint(config.getOption("numberOfStokes", "value", "4"))) {
        if (nstokes_ != 1 && nstokes_ != 4)
            throw std::runtime_error("StokesGenerator: You can either generate 1 or 4 Stokes parameters.");
    }
    unsigned numberOfStokes() const { return nstokes_; }
    void run(const SpectrumDataSetC32* in, SpectrumDataSetStokes* out) {
        const unsigned nt = in->nTimeBlocks(), ns = in->nSubbands(), nc = in->nChannels();
        if (in->nPolarisations() != 2) throw std::runtime_error("StokesGenerator: needs 2 polarisations");
        const size_t n = (size_t)nt * ns * 2 * nc;
        float* d_in = din_.as<float>(2 * n);
        float* d_out = dout_.as<float>((size_t)nt * ns * nstokes_ * nc);
        pv_check(pv_device_copy(d_in, in->data(), (long long)(8 * n), nullptr));
        pv_check(pv_stokes(d_in, (int)nt, (int)ns, (int)nc, (int)nstokes_, d_out, nullptr));
        out->resize(nt, ns, nstokes_, nc);
        pv_check(pv_device_copy(out->data(), d_out, (long long)(4 * out->size()), nullptr));
        pv_check(pv_synchronize(nullptr));
        out->setBlockRate(in->getBlockRate());
        out->setLofarTimestamp(in->getLofarTimestamp());
    }

  private:
    unsigned nstokes_;
    DeviceBuffer din_, dout_;
};

// lib/src/StokesIntegrator.cpp:32-119
class StokesIntegrator {
  public:
    explicit StokesIntegrator(const ConfigNode& config)
        : window_(to_uint(config.getOption("integrateTimeBins", "value", "1"))),
          bin_(to_uint(config.getOption("integrateFrequencyChannels", "value", "1"))) {}
    void run(const SpectrumDataSetStokes* in, SpectrumDataSetStokes* out) {
        const unsigned nt = in->nTimeBlocks(), ns = in->nSubbands(), np = in->nPolarisations(),
                       nc = in->nChannels();
        const size_t n = (size_t)nt * ns * np * nc;
        float* d_in = din_.as<float>(n);
        float* d_out = dout_.as<float>(n);
        pv_check(pv_device_copy(d_in, in->data(), (long long)(4 * n), nullptr));
        int nu = 0;
        pv_check(pv_integrate(d_in, (int)nt, (int)ns, (int)np, (int)nc, (int)window_, (int)bin_, d_out,
                              &nu, nullptr));
        out->resize((unsigned)nu, ns, np, nc / bin_);
        pv_check(pv_device_copy(out->data(), d_out, (long long)(4 * out->size()), nullptr));
        pv_check(pv_synchronize(nullptr));
        const unsigned w = nt < window_ ? (nt ? nt : 1) : window_;
        out->setBlockRate(in->getBlockRate() * w);  // StokesIntegrator.cpp:53-59
        out->setLofarTimestamp(in->getLofarTimestamp());
    }

  private:
    unsigned window_, bin_;
    DeviceBuffer din_, dout_;
};

// The clipper's bandpass model as RFI_Clipper::bandPass() returns it
// (lib/BandPass.h:34-80): the rebinned model the next spectrum is compared
// with, its mean and RMS (setMean/setRMS after every spectrum,
// RFI_Clipper.cpp:562-563), the median and the polynomial.  A snapshot,
// refreshed by each bandPass() call.
class BandPass {
  public:
    const std::vector<float>& currentSet() const { return set_; }
    float intensityOfBin(unsigned i) const { return set_[i]; }
    float mean() const { return mean_; }
    float rms() const { return rms_; }
    float median() const { return median_; }
    // the polynomial's constant term as setMean leaves it (the other
    // coefficients are the file's, scaled by the rebinning)
    float params0() const { return params0_; }
    unsigned nBins() const { return (unsigned)set_.size(); }

  private:
    friend class RFI_Clipper;
    std::vector<float> set_;
    float mean_ = 0.0f, rms_ = 0.0f, median_ = 0.0f, params0_ = 0.0f;
};

// lib/src/RFI_Clipper.cpp:22-573 (the BandPassData file is read here and
// parsed by the library, BandPassAdapter.cpp:30-108)
class RFI_Clipper {
  public:
    explicit RFI_Clipper(const ConfigNode& config) {
        const bool active = !(config.hasAttribute("active") && lower(config.getAttribute("active")) == "false");
        std::string text;
        const std::string file = config.getOption("BandPassData", "file", "");
        if (!file.empty() && active) {
            std::string path;
            try {
                path = config.searchFile(file);
            } catch (const std::exception& e) {
                throw std::runtime_error(std::string("RFI_Clipper: ") + e.what());
            }
            std::ifstream f(path);
            if (!f) throw std::runtime_error("RFI_Clipper: Cannot open File \"" + file + "\"");
            std::stringstream ss;
            ss << f.rdbuf();
            text = ss.str();
        } else if (active) {
            throw std::runtime_error("RFI_Clipper: <BandPassData file=?> not defined");
        }
        const float cr = config.hasAttribute("channelRejectionRMS")
                             ? to_float(config.getAttribute("channelRejectionRMS")) : 10.0f;
        const float sr = config.hasAttribute("spectrumRejectionRMS")
                             ? to_float(config.getAttribute("spectrumRejectionRMS")) : 4.0f;
        const int history = std::stoi(config.getOption("History", "maximum", "10"));
        const int zero_dm = config.getOption("zeroDMing", "active") == "true";
        const int mor = config.getOption("computeRMSfromMean", "active", "true") == "true";
        const int matching = config.getOption("Band", "matching") == "true";
        pv_check(pv_rfi_create(&h_, text.c_str(), cr, sr, history, zero_dm, mor, matching, active ? 1 : 0));
    }
    ~RFI_Clipper() { pv_rfi_destroy(h_); }
    RFI_Clipper(const RFI_Clipper&) = delete;
    RFI_Clipper& operator=(const RFI_Clipper&) = delete;

    void run(WeightedSpectrumDataSet* weighted) {
        SpectrumDataSetStokes* d = weighted->stats();
        const size_t n = d->size();
        float* dd = dbuf_.as<float>(n);
        pv_check(pv_device_copy(dd, d->data(), (long long)(4 * n), nullptr));
        runDevice(dd, d->nTimeBlocks(), d->nSubbands(), d->nPolarisations(), d->nChannels(), nullptr);
        pv_check(pv_device_copy(d->data(), dd, (long long)(4 * n), nullptr));
        pv_check(pv_synchronize(nullptr));
    }
    // run() on Stokes data already in device memory, asynchronously on stream.
    void runDevice(float* d_stokes, unsigned nt, unsigned nsub, unsigned npol, unsigned nchan, void* stream) {
        pv_check(pv_rfi_run(h_, d_stokes, (int)nt, (int)nsub, (int)npol, (int)nchan, nullptr, stream));
        nbins_ = nsub * nchan;
    }
    // The bandpass in use (lib/RFI_Clipper.h:38); empty before the first run.
    const BandPass& bandPass() const {
        if (nbins_) {
            bp_.set_.resize(nbins_);
            float st[4];
            pv_check(pv_rfi_bandpass_current(h_, bp_.set_.data(), (int)nbins_, st));
            bp_.mean_ = st[0];
            bp_.rms_ = st[1];
            bp_.median_ = st[2];
            bp_.params0_ = st[3];
        }
        return bp_;
    }

  private:
    pv_rfi* h_ = nullptr;
    unsigned nbins_ = 0;
    DeviceBuffer dbuf_;
    mutable BandPass bp_;
};

// lib/LockingPtrContainer.hpp: a pool of blobs handed out by next() and
// given back by unlock() (a pipeline's ring of Stokes blobs that the
// DedispersionModule holds until their buffers are exported).
template <typename T>
class LockingPtrContainer {
  public:
    explicit LockingPtrContainer(std::vector<T*>* data = nullptr) {
        if (data) reset(data);
    }
    void reset(std::vector<T*>* data) {
        std::lock_guard<std::mutex> l(m_);
        data_ = data;
        available_.assign(data->begin(), data->end());
    }
    // The next free blob.  The reference waits without limit
    // (LockingPtrContainer.hpp:37-43); here a wait longer than wait_s seconds
    // throws, since only a history too small for the module's buffers can
    // make it.
    T* next(double wait_s = 60.0) {
        std::unique_lock<std::mutex> l(m_);
        if (!cv_.wait_for(l, std::chrono::duration<double>(wait_s), [&] { return !available_.empty(); }))
            throw std::runtime_error("LockingPtrContainer: no free data blob (the pipeline's <history> is "
                                     "smaller than the blobs its DedispersionModule buffers hold)");
        T* p = available_.front();
        available_.pop_front();
        return p;
    }
    void unlock(const T* d) {
        {
            std::lock_guard<std::mutex> l(m_);
            available_.push_back(const_cast<T*>(d));
        }
        cv_.notify_one();
    }
    int numberAvailable() const {
        std::lock_guard<std::mutex> l(m_);
        return (int)available_.size();
    }
    bool allAvailable() const {
        std::lock_guard<std::mutex> l(m_);
        return !data_ || available_.size() == data_->size();
    }

  private:
    std::vector<T*>* data_ = nullptr;
    std::deque<T*> available_;
    mutable std::mutex m_;
    std::condition_variable cv_;
};

// lib/src/DedispersionModule.cpp:45-325 with the reference's buffering and
// the asynchronous contract of lib/AsyncronousModule.h:40-53.  dedisperse()
// moves the blob's samples into the device ring and, when a buffer fills,
// launches its dedispersion, then returns.  A worker thread takes each
// filled buffer in order, copies its DedispersionSpectra back, calls the
// connect() functors, unlocks the buffer's input blobs (unlockCallback gets
// those whose lock count reaches 0) and then the onChainCompletion()
// callbacks.  A buffer whose GPU job fails is not delivered: its blobs are
// unlocked and the error is printed, as GPU_Job::Failed is
// (DedispersionModule.cpp:299-311).  Lock counts follow the reference
// (:216-246, AsyncronousModule.cpp:113-131): the blobs added since the last
// fill are locked once when a buffer fills, the blobs whose samples the
// next buffer's overlap holds once more, and the blob being added once more
// when it continues past the buffer outside that overlap; exporting a
// buffer unlocks each of its input blobs once.  Input blobs must stay alive
// and unchanged until unlocked.  The functors of one module run one after
// another on its worker thread.
class DedispersionModule {
  public:
    using Functor = std::function<void(DedispersionSpectra*)>;
    using UnlockCallback = std::function<void(const std::vector<DataBlob*>&)>;

    explicit DedispersionModule(const ConfigNode& config) {
        const float pow2 = to_float(config.getOption("timeBinsPerBufferPow2", "value", "15"));
        samples_ = 1u << (unsigned)pow2;
        tdms_ = to_uint(config.getOption("dedispersionSamples", "value", "1984"));
        dm_step_ = to_float(config.getOption("dedispersionStepSize", "value", "0.0"));
        dm_low_ = to_float(config.getOption("dedispersionMinimum", "value", "0.0"));
        fch1_ = std::stod(config.getOption("frequencyChannel1", "MHz", "0.0"));
        foff_ = std::stod(config.getOption("channelBandwidth", "MHz", "1.0"));
        pv_check(pv_ddmod_create(&h_, (int)samples_, (int)tdms_, dm_low_, dm_step_, fch1_, foff_));
    }
    ~DedispersionModule() {
        waitForJobCompletion();
        {
            std::lock_guard<std::mutex> l(q_mu_);
            stop_ = true;
        }
        q_cv_.notify_all();
        if (worker_.joinable()) worker_.join();
        pv_ddmod_destroy(h_);
    }
    DedispersionModule(const DedispersionModule&) = delete;
    DedispersionModule& operator=(const DedispersionModule&) = delete;

    void connect(const Functor& f) { functors_.push_back(f); }
    void unlockCallback(const UnlockCallback& f) { unlock_.push_back(f); }
    void onChainCompletion(const std::function<void()>& f) { chain_.push_back(f); }
    // Blocks until every filled buffer has been exported (AsyncronousModule.cpp:49-51).
    void waitForJobCompletion() const {
        std::unique_lock<std::mutex> l(q_mu_);
        idle_cv_.wait(l, [&] { return jobs_.empty() && !busy_; });
    }
    // Locks this module holds on a blob (AsyncronousModule.cpp:113-119).
    int lockNumber(const DataBlob* d) const {
        std::lock_guard<std::mutex> l(locks_mu_);
        auto it = locks_.find(d);
        return it == locks_.end() ? 0 : it->second;
    }
    unsigned numberOfSamples() const { return samples_; }
    int maxshift() const {
        int p[6] = {0};
        std::lock_guard<std::mutex> l(dd_mu_);
        pv_check(pv_ddmod_params(h_, p));
        return p[0];
    }

    void dedisperse(WeightedSpectrumDataSet* weighted) {
        add(weighted->dataSet(), weighted->dataSet()->data(), nullptr);
    }
    void dedisperse(DataBlob* blob) {
        auto* w = dynamic_cast<WeightedSpectrumDataSet*>(blob);
        if (!w) throw std::runtime_error("DedispersionModule: expecting a WeightedSpectrumDataSet");
        dedisperse(w);
    }
    // dedisperse() of a blob whose Stokes data (the blob's layout) are
    // already in device memory at d_stokes, ordered on stream: the fused
    // pipeline's path, with no host copy of the samples.
    void dedisperseDevice(WeightedSpectrumDataSet* weighted, const float* d_stokes, void* stream) {
        add(weighted->dataSet(), d_stokes, stream);
    }

  private:
    struct Span {
        const SpectrumDataSetStokes* blob;
        long long start, end;  // the blob's samples in the stream
    };
    struct Job {
        std::vector<const SpectrumDataSetStokes*> inputs;
        unsigned nch, nsub;
        double rate, t0;
    };

    void add(SpectrumDataSetStokes* d, const float* data, void* stream) {
        if (!have_t0_) {  // sample 0 of the stream: times are t0 + (t + firstSample) * rate
            t0_ = d->getLofarTimestamp();
            have_t0_ = true;
        }
        const long long nt = d->nTimeBlocks();
        spans_.push_back(Span{d, received_, received_ + nt});
        received_ += nt;
        pending_.push_back(d);
        int done = 0, p[6] = {0};
        {
            std::lock_guard<std::mutex> l(dd_mu_);
            pv_check(pv_ddmod_add(h_, data, (int)nt, (int)d->nSubbands(), (int)d->nPolarisations(),
                                  (int)d->nChannels(), d->getBlockRate(), &done, stream));
            pv_check(pv_ddmod_params(h_, p));
        }
        if (done == 0) return;
        const long long nout = p[2], B = samples_;
        std::vector<Job> jobs;
        {
            std::lock_guard<std::mutex> l(locks_mu_);
            for (int i = 0; i < done; ++i) {
                const long long first = filled_ * nout, end = first + B, next = first + nout;
                Job job{{}, d->nChannels(), d->nSubbands(), d->getBlockRate(), t0_};
                for (const Span& sp : spans_)
                    if (sp.start < end && sp.end > first) job.inputs.push_back(sp.blob);
                for (const DataBlob* b : pending_) ++locks_[b];  // lockAllUnprotected(_blobs)
                pending_.clear();
                bool in_next = false;
                for (const Span& sp : spans_)
                    if (sp.start < end && sp.end > next) {  // the overlap copied to the next buffer
                        ++locks_[sp.blob];
                        in_next = in_next || sp.blob == d;
                    }
                if (received_ > end && !in_next) ++locks_[d];
                ++filled_;
                jobs.push_back(std::move(job));
            }
            // blobs wholly before the next buffer are in no later buffer
            while (!spans_.empty() && spans_.front().end <= filled_ * nout) spans_.pop_front();
        }
        {
            std::lock_guard<std::mutex> l(q_mu_);
            for (Job& j : jobs) jobs_.push_back(std::move(j));
            if (!worker_.joinable()) worker_ = std::thread([this] { work(); });
        }
        q_cv_.notify_one();
    }

    void work() {
        for (;;) {
            Job job;
            {
                std::unique_lock<std::mutex> l(q_mu_);
                q_cv_.wait(l, [&] { return stop_ || !jobs_.empty(); });
                if (jobs_.empty()) return;
                job = std::move(jobs_.front());
                jobs_.pop_front();
                busy_ = true;
            }
            export_job(job);
            {
                std::lock_guard<std::mutex> l(q_mu_);
                busy_ = false;
            }
            idle_cv_.notify_all();
        }
    }

    void export_job(const Job& job) {
        DedispersionSpectra out;
        bool ok = true;
        try {
            std::lock_guard<std::mutex> l(dd_mu_);
            int p[6] = {0};
            pv_check(pv_ddmod_params(h_, p));
            out.resize((unsigned)p[2], tdms_, dm_low_ < 0.0f ? 0.0f : dm_low_, dm_step_);
            int nout = 0;
            long long first = 0;
            pv_check(pv_ddmod_pop(h_, out.data().data(), (long long)out.data().size(), &nout, &first, nullptr));
            out.setFirstSample((unsigned)first);
        } catch (const std::exception& e) {
            std::cerr << "DedispersionModule: " << e.what() << std::endl;
            ok = false;
        }
        if (ok) {
            out.setInputShape(job.nch, job.nsub);
            out.setBlockRate(job.rate);
            out.setLofarTimestamp(job.t0);
            out.setInputDataBlobs(job.inputs);
            for (auto& f : functors_) f(&out);
        }
        // exportComplete (DedispersionModule.cpp:317-325) and the unlock triggers
        std::vector<DataBlob*> freed;
        {
            std::lock_guard<std::mutex> l(locks_mu_);
            for (const SpectrumDataSetStokes* b : job.inputs) {
                auto it = locks_.find(b);
                if (it != locks_.end() && --it->second == 0) {
                    freed.push_back(const_cast<SpectrumDataSetStokes*>(b));
                    locks_.erase(it);
                }
            }
        }
        for (auto& f : unlock_) f(freed);
        if (ok)
            for (auto& f : chain_) f();
    }

    pv_ddmod* h_ = nullptr;
    double t0_ = 0.0;
    bool have_t0_ = false;
    unsigned samples_ = 0, tdms_ = 0;
    float dm_step_ = 0.0f, dm_low_ = 0.0f;
    double fch1_ = 0.0, foff_ = 0.0;
    std::vector<Functor> functors_;
    std::vector<std::function<void()>> chain_;
    std::vector<UnlockCallback> unlock_;
    // caller-thread bookkeeping
    std::deque<Span> spans_;
    std::vector<const DataBlob*> pending_;  // added since the last fill (the reference's _blobs)
    long long received_ = 0, filled_ = 0;
    // shared with the worker
    mutable std::mutex dd_mu_, locks_mu_, q_mu_;
    std::unordered_map<const DataBlob*, int> locks_;
    std::deque<Job> jobs_;
    bool busy_ = false, stop_ = false;
    mutable std::condition_variable idle_cv_;
    std::condition_variable q_cv_;
    std::thread worker_;
};

// lib/src/DedispersionAnalyser.cpp:30-203
class DedispersionAnalyser {
  public:
    explicit DedispersionAnalyser(const ConfigNode& config)
        : threshold_(to_float(config.getOption("detectionThreshold", "in_sigma", "6.0"))),
          bin_pow2_(to_uint(config.getOption("power2ForBinning", "value", "6"))) {}

    int analyse(DedispersionSpectra* data, DedispersionDataAnalysis* result) {
        result->reset(data);
        // sigma of the dedispersed sum: sqrt(nChannels * nSubbands) (DedispersionAnalyser.cpp:36-38)
        const float rms = std::sqrt((float)data->inputChannels() * (float)data->inputSubbands());
        result->setRMS(rms);
        const int tdms = data->dmBins(), nsamp = data->timeSamples();
        const size_t n = (size_t)tdms * nsamp;
        float* d = dbuf_.as<float>(n ? n : 1);
        if (n) pv_check(pv_device_copy(d, data->data().data(), (long long)(4 * n), nullptr));
        long long count = 0;
        const long long cap = 1 << 20;
        pv_event* ev = evbuf_.as<pv_event>((size_t)cap);
        pv_check(pv_analyse(d, nsamp, tdms, nsamp, threshold_, rms, (int)bin_pow2_, ev, cap, &count, nullptr));
        std::vector<pv_event> h((size_t)std::min(count, cap));
        if (!h.empty())
            pv_check(pv_device_copy(h.data(), ev, (long long)(sizeof(pv_event) * h.size()), nullptr));
        pv_check(pv_synchronize(nullptr));
        for (const auto& e : h) result->addEvent((unsigned)e.dm, (unsigned)e.t, e.bin_factor, e.value);
        return result->eventsFound();
    }

  private:
    float threshold_;
    unsigned bin_pow2_;
    DeviceBuffer dbuf_, evbuf_;
};

// ---------------------------------------------------------------------------
// Pipeline driver
// ---------------------------------------------------------------------------

// What both pipeline drivers do with a dedispersed buffer
// (DedispersionPipeline.cpp:111-150, ABPipeline.cpp:142-170): analyse it,
// send the result to the "TriggerInput" outputs, and to the
// "DedispersionDataAnalysis" outputs when the event count lies in
// <events min max> (at least min when min >= max), with each of the
// buffer's input blobs to the "SignalFoundSpectrum" outputs.  The analysis
// runs on the DedispersionModule's worker thread, beside the next run().
// The Stokes blobs the module reads come from a ring of <history> blobs
// (createBlobs + LockingPtrContainer, DedispersionPipeline.cpp:83-90) that
// the module's unlock callback refills (updateBufferLock, :209-217).
class PipelineAnalysis {
  public:
    using Output = std::function<void(const DedispersionDataAnalysis&)>;
    using SpectrumOutput = std::function<void(const SpectrumDataSetStokes&)>;
    virtual ~PipelineAnalysis() {
        if (dd_) dd_->waitForJobCompletion();
    }
    // AbstractPipeline::dataOutput: "TriggerInput" or "DedispersionDataAnalysis"
    void connectOutput(const std::string& stream, const Output& f) { outputs_.emplace_back(stream, f); }
    // "SignalFoundSpectrum": each input blob of a buffer that reaches the
    // "DedispersionDataAnalysis" outputs (for a SigprocStokesWriter)
    void connectSpectrumOutput(const std::string& stream, const SpectrumOutput& f) {
        spectrum_outputs_.emplace_back(stream, f);
    }
    // Buffers analysed so far (complete after waitForJobCompletion()).
    unsigned buffers() const { return buffers_.load(); }
    // Waits until every filled buffer has been analysed and sent.
    void waitForJobCompletion() const { dd_->waitForJobCompletion(); }
    const DedispersionModule& dedispersionModule() const { return *dd_; }
    unsigned history() const { return (unsigned)ring_.size(); }

  protected:
    // the modules after the first stages: RFI_Clipper, DedispersionModule, DedispersionAnalyser
    void setup(const std::string& config_file, unsigned history) {
        rfi_.reset(new RFI_Clipper(ConfigNode::fromFile(config_file, "RFI_Clipper")));
        dd_.reset(new DedispersionModule(ConfigNode::fromFile(config_file, "DedispersionModule")));
        an_.reset(new DedispersionAnalyser(ConfigNode::fromFile(config_file, "DedispersionAnalyser")));
        dd_->connect([this](DedispersionSpectra* d) { analysis(d); });
        dd_->unlockCallback([this](const std::vector<DataBlob*>& blobs) {
            for (DataBlob* b : blobs) stokes_buffer_.unlock(static_cast<SpectrumDataSetStokes*>(b));
        });
        history = std::max(history, 1u);
        for (unsigned k = 0; k < history; ++k) ring_.emplace_back(new SpectrumDataSetStokes);
        for (auto& b : ring_) ring_ptrs_.push_back(b.get());
        stokes_buffer_.reset(&ring_ptrs_);
    }
    void emit(const std::string& stream, const DedispersionDataAnalysis& r) {
        for (auto& o : outputs_)
            if (o.first == stream) o.second(r);
    }
    void analysis(DedispersionSpectra* d) {
        ++buffers_;
        DedispersionDataAnalysis result;
        if (!an_->analyse(d, &result)) return;
        emit("TriggerInput", result);
        const unsigned n = (unsigned)result.eventsFound();
        if (min_ >= max_ ? n >= min_ : (n >= min_ && n <= max_)) {
            emit("DedispersionDataAnalysis", result);
            for (const SpectrumDataSetStokes* b : d->inputDataBlobs())
                for (auto& o : spectrum_outputs_)
                    if (o.first == "SignalFoundSpectrum") o.second(*b);
        }
    }

    unsigned min_ = 5, max_ = 0;
    std::atomic<unsigned> buffers_{0};
    std::unique_ptr<RFI_Clipper> rfi_;
    std::unique_ptr<DedispersionModule> dd_;
    std::unique_ptr<DedispersionAnalyser> an_;
    std::vector<std::pair<std::string, Output>> outputs_;
    std::vector<std::pair<std::string, SpectrumOutput>> spectrum_outputs_;
    std::vector<std::unique_ptr<SpectrumDataSetStokes>> ring_;
    std::vector<SpectrumDataSetStokes*> ring_ptrs_;
    LockingPtrContainer<SpectrumDataSetStokes> stokes_buffer_;
};

// pipelines/udpstream/src/DedispersionPipeline.cpp:48-155: per chunk of
// voltages, PPFChanneliser -> StokesGenerator -> RFI_Clipper ->
// DedispersionModule (no StokesIntegrator in this pipeline: :101-104).
// Modules and limits come from one XML file with the reference's element
// names; outputs are callbacks in place of the pelican output manager.
// With numberOfStokes 1 (and <fused value="true"/>, the default) the chunk
// stays in device memory from the voltages to the dedispersion ring: one
// fused PPF + Stokes-I pass, the clipper on the device and the module
// reading the clipped spectra there, where the module chain copies each
// stage's data set to the host and back.  The results are identical; the
// Stokes blobs receive the clipped spectra only when a
// "SignalFoundSpectrum" output is connected.
class DedispersionPipeline : public PipelineAnalysis {
  public:
    explicit DedispersionPipeline(const std::string& config_file) {
        const ConfigNode c = ConfigNode::fromFile(config_file, "DedispersionPipeline");
        min_ = to_uint(c.getOption("events", "min", "5"));
        max_ = to_uint(c.getOption("events", "max", "0"));
        const unsigned history = to_uint(c.getOption("history", "value", "10"));
        ppf_.reset(new PPFChanneliser(ConfigNode::fromFile(config_file, "PPFChanneliser")));
        stokes_.reset(new StokesGenerator(ConfigNode::fromFile(config_file, "StokesGenerator")));
        fused_ = stokes_->numberOfStokes() == 1 && lower(c.getOption("fused", "value", "true")) == "true";
        setup(config_file, history);
    }
    bool fused() const { return fused_; }
    void run(TimeSeriesDataSetC32* timeSeries) {
        SpectrumDataSetStokes* stokes = stokes_buffer_.next();
        if (fused_) {
            const unsigned nb = timeSeries->nTimeBlocks(), ns = timeSeries->nSubbands(), nc = ppf_->channels();
            float* d = dstokes_.as<float>((size_t)nb * ns * nc);
            ppf_->runStokesIDevice(timeSeries, d, nullptr);
            stokes->reshape(nb, ns, 1, nc);
            stokes->setBlockRate(timeSeries->getBlockRate() * nc);  // PPFChanneliser.cpp:99
            stokes->setLofarTimestamp(timeSeries->getLofarTimestamp());
            WeightedSpectrumDataSet w(stokes);
            rfi_->runDevice(d, nb, ns, 1, nc, nullptr);
            if (!spectrum_outputs_.empty()) {
                pv_check(pv_device_copy(stokes->data(), d, (long long)(4 * stokes->size()), nullptr));
                pv_check(pv_synchronize(nullptr));
            }
            dd_->dedisperseDevice(&w, d, nullptr);
            return;
        }
        ppf_->run(timeSeries, &spectra_);
        stokes_->run(&spectra_, stokes);
        WeightedSpectrumDataSet w(stokes);
        rfi_->run(&w);
        dd_->dedisperse(&w);
    }

  private:
    std::unique_ptr<PPFChanneliser> ppf_;
    std::unique_ptr<StokesGenerator> stokes_;
    SpectrumDataSetC32 spectra_;
    DeviceBuffer dstokes_;
    bool fused_ = false;
};

// pipelines/udpstream/src/ABPipeline.cpp:56-140: the ALFABURST driver.  Each
// chunk's spectra (ABDataAdapter) go through the StokesIntegrator (its
// element is optional: 1 and 1 when absent, as createModule gives), are
// copied to the next blob of the ring (:83-87), then go through the
// RFI_Clipper, the DedispersionModule and the analyser; <events min max>
// default to 5 and 5.
class ABPipeline : public PipelineAnalysis {
  public:
    explicit ABPipeline(const std::string& config_file) {
        const ConfigNode c = ConfigNode::fromFile(config_file, "ABPipeline");
        const unsigned history = to_uint(c.getOption("history", "value", "10"));
        min_ = to_uint(c.getOption("events", "min", "5"));
        max_ = to_uint(c.getOption("events", "max", "5"));
        ConfigNode integ;
        try {
            integ = ConfigNode::fromFile(config_file, "StokesIntegrator");
        } catch (const std::runtime_error&) {
        }
        integrator_.reset(new StokesIntegrator(integ));
        setup(config_file, history);
    }
    void run(SpectrumDataSetStokes* stokes) {
        if (!stokes) throw std::runtime_error("No stokes!");
        SpectrumDataSetStokes* buf = stokes_buffer_.next();
        integrator_->run(stokes, &integrated_);
        *buf = integrated_;
        WeightedSpectrumDataSet w(buf);
        rfi_->run(&w);
        dd_->dedisperse(&w);
    }

  private:
    std::unique_ptr<StokesIntegrator> integrator_;
    SpectrumDataSetStokes integrated_;
};

// ---------------------------------------------------------------------------
// Output streams
// ---------------------------------------------------------------------------

// "<path>_D%Y%m%dT%H%M%S<ext>" in local time, as both reference writers name
// their files (SigprocStokesWriter.cpp:104-111, DedispersionDataAnalysisOutput.cpp:20-28).
inline std::string stamped_name(const std::string& path, const char* ext) {
    char ts[22];
    const time_t now = time(nullptr);
    struct tm tm_now;
    localtime_r(&now, &tm_now);
    strftime(ts, sizeof ts, "D%Y%m%dT%H%M%S", &tm_now);
    return path + "_" + ts + ext;
}

// lib/src/SigprocStokesWriter.cpp:15-293: the header values derive from the
// options with the reference's types (float members, unsigned options, a
// double 0.5 and 1e6); the data block is reordered and quantised on the GPU.
class SigprocStokesWriter {
  public:
    explicit SigprocStokesWriter(const ConfigNode& c) {
        nsub_ = to_uint(c.getOption("subbandsPerPacket", "value", "1"));
        const int n_total = (int)to_uint(c.getOption("totalComplexSubbands", "value", "1"));
        const float clock = to_float(c.getOption("clock", "value", "200"));
        const unsigned integ = to_uint(c.getOption("integrateTimeBins", "value", "1"));
        const unsigned integ_f = to_uint(c.getOption("integrateFrequencyChannels", "value", "1"));
        const unsigned nchan = to_uint(c.getOption("outputChannelsPerSubband", "value", "128")) / integ_f;
        const unsigned nraw = to_uint(c.getOption("nRawPolarisations", "value", "2"));
        nbits_ = to_uint(c.getOption("dataBits", "value", "32"));
        const float nrange = (float)((int)std::pow(2.0, (double)nbits_) - 1.0);
        crop_min_ = to_float(c.getOption("scale", "min", "0.0"));
        const std::string mx = c.getOption("scale", "max", "X");
        try {
            size_t used = 0;
            crop_max_ = std::stof(mx, &used);
            if (used != mx.size()) crop_max_ = nrange;
        } catch (const std::exception&) {
            crop_max_ = nrange;
        }
        const std::string path = c.getOption("file", "filepath");
        const unsigned top = (unsigned)to_float(c.getOption("topSubbandIndex", "value", "150"));
        const unsigned lbahba = (unsigned)to_float(c.getOption("LBA_0_or_HBA_1", "value", "1"));
        const float sbw = clock / (float)(nraw * (unsigned)n_total);
        const float cw = sbw / (float)nchan;
        float fch1 = 0.0f;
        if (c.getOption("fch1", "value").empty()) {
            const float base = sbw * (float)top;
            if (lbahba == 0)
                fch1 = (float)((double)base + 0.5 * sbw - 0.5 * cw);
            else if (clock == 200)
                fch1 = (float)((double)(100 + base) + 0.5 * sbw - 0.5 * cw);
            else if (clock == 160)
                fch1 = (float)((double)(160 + base) + 0.5 * sbw - 0.5 * cw);
        } else {
            fch1 = to_float(c.getOption("fch1", "value", "1400.0"));
        }
        const float foff = c.getOption("foff", "value").empty() ? -cw : to_float(c.getOption("foff", "value", "1.0"));
        float tsamp = 0.0f;
        if (c.getOption("tsamp", "value").empty())
            tsamp = (float)((float)(nraw * (unsigned)n_total * nchan * integ_f * integ) / clock / 1e6);
        else
            tsamp = to_float(c.getOption("tsamp", "value", "1.0"));
        npols_ = to_uint(c.getOption("params", "nPolsToWrite", "1"));
        write_header_ = c.hasAttribute("writeHeader") && lower(c.getAttribute("writeHeader")) == "true";
        const std::string ra = c.getOption("RAJ", "value", "000000.0"), dec = c.getOption("DecJ", "value", "000000.0");
        const float dec_v = to_float(dec);
        std::string name = ra.substr(0, 4) + (dec_v > 0.0f ? "+" + dec.substr(0, 4) : dec.substr(0, 5));
        p_.machine_id = (int)to_uint(c.getOption("MachineID", "value", "9"));
        p_.telescope_id = (int)to_uint(c.getOption("TelescopeID", "value", "0"));
        p_.nchans = (int)(nchan * nsub_);
        p_.nbits = (int)nbits_;
        p_.nifs = (int)npols_;
        p_.src_raj = to_float(ra);
        p_.src_dej = dec_v;
        p_.fch1 = fch1;
        p_.foff = foff;
        p_.tsamp = tsamp;
        std::snprintf(p_.source_name, sizeof p_.source_name, "%s", name.c_str());
        file_.open(stamped_name(path, ".fil"), std::ios::out | std::ios::binary);
    }
    const pv_sigproc_params& params() const { return p_; }

    void sendStream(const SpectrumDataSetStokes* stokes) {
        if (!stokes) {
            std::cerr << "SigprocStokesWriter::send(): Only SpectrumDataSetStokes data can be written by the "
                         "SigprocWriter" << std::endl;
            return;
        }
        if (write_header_) {
            write_header_ = false;
            p_.tstart = pv_sigproc_mjd(stokes->getLofarTimestamp());
            long long n = 0;
            pv_sigproc_header(&p_, nullptr, 0, &n);
            std::vector<char> h((size_t)n);
            pv_check(pv_sigproc_header(&p_, h.data(), n, &n));
            file_.write(h.data(), n);
        }
        const unsigned nt = stokes->nTimeBlocks(), ns = stokes->nSubbands(), np = stokes->nPolarisations(),
                       nc = stokes->nChannels();
        const size_t in_n = (size_t)nt * ns * np * nc;
        if (nbits_ != 8 && nbits_ != 32) pv_check(pv_sigproc_pack(nullptr, 0, 1, 1, 1, 1, (int)nbits_, 0, 0, nullptr, nullptr));
        const size_t out_n = (size_t)nt * npols_ * ns * nc * (nbits_ / 8);
        float* d_in = din_.as<float>(in_n);
        void* d_out = dout_.get(out_n);
        std::vector<char> h(out_n);
        pv_check(pv_device_copy(d_in, stokes->data(), (long long)(4 * in_n), nullptr));
        pv_check(pv_sigproc_pack(d_in, (int)nt, (int)ns, (int)np, (int)nc, (int)npols_, (int)nbits_, crop_min_,
                                 crop_max_, d_out, nullptr));
        pv_check(pv_device_copy(h.data(), d_out, (long long)out_n, nullptr));
        pv_check(pv_synchronize(nullptr));
        file_.write(h.data(), (std::streamsize)out_n);
        file_.flush();
    }

  private:
    pv_sigproc_params p_{};
    unsigned nsub_ = 1, nbits_ = 32, npols_ = 1;
    float crop_min_ = 0.0f, crop_max_ = 255.0f;
    bool write_header_ = false;
    std::ofstream file_;
    DeviceBuffer din_, dout_;
};

// lib/src/DedispersionDataAnalysisOutput.cpp:18-112
class DedispersionDataAnalysisOutput {
  public:
    explicit DedispersionDataAnalysisOutput(const ConfigNode& c) {
        file_.open(stamped_name(c.getOption("file", "name"), ".dat"), std::ios::out | std::ios::binary);
        if (!file_) {
            std::cerr << "DedispersionDataAnalysisOutput: unable to open file for writing" << std::endl;
            return;
        }
        file_ << PV_EVENTS_TEXT_HEADER;
        file_.flush();
    }
    void sendStream(const DedispersionDataAnalysis* data) {
        if (!data || !data->data() || !file_) return;
        const DedispersionSpectra* d = data->data();
        std::vector<pv_event> ev;
        ev.reserve(data->events().size());
        for (const auto& e : data->events())
            ev.push_back(pv_event{(int32_t)e.dmIndex(), (int32_t)e.timeBin(), e.mfBinning(), e.mfValue()});
        ++dump_;
        long long n = 0;
        auto call = [&](char* buf, long long cap) {
            return pv_events_text(ev.data(), (long long)ev.size(), d->getLofarTimestamp(), d->getBlockRate(),
                                  d->firstSample(), d->dmLow(), d->dmStep(), data->getRMS(), dump_, buf, cap, &n);
        };
        call(nullptr, 0);
        std::vector<char> text((size_t)n);
        pv_check(call(text.data(), n));
        file_.write(text.data(), n);
        file_.flush();
    }

  private:
    std::ofstream file_;
    int dump_ = 0;
};

// lib/src/TriggerOutput.cpp:33-204.  Options <Receiver host port/>, <Trigger
// format/>, <Logfile name/>, <Telescope stationID beamID/>, <RADec rajd
// decjd/>, <frequencyChannel1 MHz/>, <Threshold snr events/>.  Each buffer
// that raises a FRATS trigger (pv_trigger_message) goes as one UDP datagram to
// every receiver and as one line appended to the log file.  The receiver host
// is an IPv4 address, as QHostAddress(host) takes it; the identifier root is
// the construction time (yyyyMMddhhmm, local) and the beam id to two digits.
class TriggerOutput {
  public:
    explicit TriggerOutput(const ConfigNode& c) {
        const std::string host = c.getOption("Receiver", "host");
        const int port = std::atoi(c.getOption("Receiver", "port", "0").c_str());
        if (!host.empty() && port != 0) addReceiver(host, (uint16_t)port);
        format_ = c.getOption("Trigger", "format");
        const std::string log = c.getOption("Logfile", "name");
        if (!log.empty()) addFile(log);
        station_ = c.getOption("Telescope", "stationID");
        char ts[16];
        const time_t now = time(nullptr);
        struct tm tm_now;
        localtime_r(&now, &tm_now);
        strftime(ts, sizeof ts, "%Y%m%d%H%M", &tm_now);
        std::string beam = c.getOption("Telescope", "beamID");
        if (beam.size() < 2) beam.insert(0, 2 - beam.size(), '0');
        id_root_ = std::string(ts) + "-" + beam;
        ra_ = c.getOption("RADec", "rajd");
        dec_ = c.getOption("RADec", "decjd");
        cfreq_ = c.getOption("frequencyChannel1", "MHz");
        snr_ = to_float(c.getOption("Threshold", "snr"));
        min_events_ = std::atoi(c.getOption("Threshold", "events", "0").c_str());
    }
    ~TriggerOutput() {
        for (auto& r : receivers_) close(r.first);
    }
    TriggerOutput(const TriggerOutput&) = delete;
    TriggerOutput& operator=(const TriggerOutput&) = delete;

    void addReceiver(const std::string& host, uint16_t port) {
        sockaddr_in a{};
        a.sin_family = AF_INET;
        a.sin_port = htons(port);
        if (inet_pton(AF_INET, host.c_str(), &a.sin_addr) != 1) {
            std::cerr << "TriggerOutput: not an IPv4 address: " << host << std::endl;
            return;
        }
        const int s = socket(AF_INET, SOCK_DGRAM, 0);
        if (s < 0) {
            std::cerr << "TriggerOutput: no UDP socket" << std::endl;
            return;
        }
        receivers_.emplace_back(s, a);
    }
    void addFile(const std::string& name) {
        auto f = std::make_unique<std::ofstream>(name, std::ios::out | std::ios::app | std::ios::binary);
        if (!*f) {
            std::cerr << "unable to open file for writing: " << name << std::endl;
            return;
        }
        files_.push_back(std::move(f));
    }
    // The message sent for this buffer, or "" when it raised none.
    std::string sendStream(const DedispersionDataAnalysis* data) {
        if (format_ != "FRATS") {
            std::cerr << "Trigger format not recognized / implemented";
            return "";
        }
        if (!data || !data->data()) return "";
        const DedispersionSpectra* d = data->data();
        std::vector<pv_event> ev;
        ev.reserve(data->events().size());
        for (const auto& e : data->events())
            ev.push_back(pv_event{(int32_t)e.dmIndex(), (int32_t)e.timeBin(), e.mfBinning(), e.mfValue()});
        long long n = 0;
        auto call = [&](char* buf, long long cap) {
            return pv_trigger_message(ev.data(), (long long)ev.size(), d->getLofarTimestamp(), d->getBlockRate(),
                                      d->firstSample(), d->dmLow(), d->dmStep(), data->getRMS(), min_events_, snr_,
                                      station_.c_str(), id_root_.c_str(), counter_ + 1, cfreq_.c_str(), ra_.c_str(),
                                      dec_.c_str(), buf, cap, &n);
        };
        pv_check(call(nullptr, 0));
        if (n == 0) return "";
        std::string msg((size_t)n, '\0');
        pv_check(call(&msg[0], n));
        ++counter_;
        if (ra_.empty()) std::cerr << "No RA/Dec found, conversion not yet implemented";
        for (auto& r : receivers_)
            sendto(r.first, msg.data(), msg.size(), 0, reinterpret_cast<const sockaddr*>(&r.second), sizeof r.second);
        for (auto& f : files_) {
            *f << msg << '\n';
            f->flush();
        }
        return msg;
    }
    int messages() const { return counter_; }

  private:
    std::vector<std::pair<int, sockaddr_in>> receivers_;
    std::vector<std::unique_ptr<std::ofstream>> files_;
    std::string format_, station_, id_root_, ra_, dec_, cfreq_;
    float snr_ = 0.0f;
    int min_events_ = 0, counter_ = 0;
};

}  // namespace ampp
}  // namespace pelican
