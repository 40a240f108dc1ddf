// Drives the C++ module shim (include/pv/ampp.hpp) for tests/test_cpp_shim.py.
//
//   test_ampp config            XML option parsing (no GPU)
//   test_ampp chain DIR         PPF -> Stokes -> integrator -> RFI on DIR/volt.bin with
//                               DIR/config.xml; writes DIR/{ppf,stokes,integ,rfi}.bin
//   test_ampp ddmod DIR N       DedispersionModule + analyser on DIR/blob.bin (float32
//                               [nt][nsub][1][nchan], shape in DIR/shape.txt) with
//                               DIR/config.xml; prints "AMP <dmAmplitude(0, 10.0)>" and
//                               "EVENTS <count>" per completed buffer
//   test_ampp ddout DIR N       ddmod with a DedispersionDataAnalysisOutput from DIR/config.xml;
//                               writes DIR/events.bin (pv_event per event) and prints
//                               "META start rate first dmlow dmstep rms" per buffer; with a
//                               TriggerOutput element also "TRIGGER <message>" per trigger sent
//   test_ampp sigproc DIR       SigprocStokesWriter (DIR/config.xml) over DIR/stokes.bin
//                               (float [t][sub][pol][chan], shape and time stamp in DIR/shape.txt)
//   test_ampp pipeline DIR N    N chunks of DIR/chunks.bin through AdapterTimeSeriesDataSet and
//                               DedispersionPipeline into a DedispersionDataAnalysisOutput;
//                               prints "BUFFERS n"
//   test_ampp outputs DIR       (no GPU) DIR/events.bin and DIR/meta.txt (start rate first dmlow
//                               dmstep rms ntime ndm) as one analysed buffer, sent twice through a
//                               DedispersionDataAnalysisOutput and a TriggerOutput from
//                               DIR/config.xml; prints "TRIGGER <message>" per trigger sent
//   test_ampp ab DIR N          N chunks of DIR/chunks.bin through ABDataAdapter and ABPipeline into a
//                               DedispersionDataAnalysisOutput; writes DIR/spectra.bin (the adapter's
//                               blobs) and prints "BUFFERS n", "GAPS g", "TIME t rate" per chunk and
//                               "SIGNAL dump t blocks" per SignalFoundSpectrum blob
//   test_ampp udp DIR           AdapterTimeSeriesDataSet on DIR/chunk.bin with DIR/config.xml;
//                               writes DIR/ts.bin, prints "SHAPE nb ns np nt" and "TIME ts rate"
#include <pv/ampp.hpp>
#include <thread>
#include <mutex>
#include <chrono>
#include <atomic>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>

using namespace pelican;
using namespace pelican::ampp;

namespace {

int failures = 0;
void expect(bool ok, const char* what) {
    if (!ok) {
        std::fprintf(stderr, "FAILED: %s\n", what);
        ++failures;
    }
}

template <typename T>
std::vector<T> read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    std::vector<char> raw((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    std::vector<T> v(raw.size() / sizeof(T));
    std::memcpy(v.data(), raw.data(), v.size() * sizeof(T));
    return v;
}
template <typename T>
void write_file(const std::string& path, const T* p, size_t n) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(p), (std::streamsize)(n * sizeof(T)));
}

int config_mode() {
    const std::string xml = R"(<?xml version="1.0"?>
<!-- a pipeline configuration in the reference's layout -->
<configuration version="1.0">
  <pipeline>
    <modules>
      <PPFChanneliser>
        <outputChannelsPerSubband value="16"/>
        <filter nTaps="8" filterWindow="Kaiser" />
      </PPFChanneliser>
      <RFI_Clipper active="true" channelRejectionRMS="5.0" spectrumRejectionRMS="4.5">
        <zeroDMing active="true" />
        <BandPassData file="band.bp" />
        <Band matching="true" />
        <History maximum="10000" />
      </RFI_Clipper>
      <DedispersionModule>
        <timeBinsPerBufferPow2 value="14"/>
        <frequencyChannel1 MHz="150.0"/>
        <channelBandwidth MHz='-0.0029296875'/>
      </DedispersionModule>
    </modules>
  </pipeline>
</configuration>)";
    const ConfigNode ppf = ConfigNode::fromString(xml, "PPFChanneliser");
    expect(ppf.getOption("outputChannelsPerSubband", "value", "512") == "16", "option value");
    expect(ppf.getOption("filter", "nTaps", "4") == "8", "second attribute");
    expect(lower(ppf.getOption("filter", "filterWindow")) == "kaiser", "window");
    expect(ppf.getOption("processingThreads", "value", "2") == "2", "default");
    const ConfigNode rfi = ConfigNode::fromString(xml, "RFI_Clipper");
    expect(rfi.hasAttribute("channelRejectionRMS") && rfi.getAttribute("channelRejectionRMS") == "5.0",
           "element attribute");
    expect(!rfi.hasAttribute("nothing"), "missing attribute");
    expect(rfi.getOption("History", "maximum", "10") == "10000", "history");
    expect(rfi.getOption("zeroDMing", "active") == "true", "zeroDMing");
    const ConfigNode dd = ConfigNode::fromString(xml, "DedispersionModule");
    expect(dd.getOption("channelBandwidth", "MHz") == "-0.0029296875", "single quotes");
    expect(dd.getOption("dedispersionSamples", "value", "1984") == "1984", "dd default");
    bool threw = false;
    try {
        ConfigNode::fromString("<a><b></a>", "a");
    } catch (const std::runtime_error&) {
        threw = true;
    }
    expect(threw, "mismatched tags throw");
    threw = false;
    try {
        RFI_Clipper r(ConfigNode::fromString("<RFI_Clipper active=\"true\"/>", "RFI_Clipper"));
    } catch (const std::runtime_error& e) {
        threw = std::string(e.what()) == "RFI_Clipper: <BandPassData file=?> not defined";
    }
    expect(threw, "RFI_Clipper without a bandpass throws the reference message");
    if (!failures) std::printf("CONFIG OK\n");
    return failures ? 1 : 0;
}

int chain_mode(const std::string& dir) {
    const ConfigNode ppf_cfg = ConfigNode::fromFile(dir + "/config.xml", "PPFChanneliser");
    const ConfigNode st_cfg = ConfigNode::fromFile(dir + "/config.xml", "StokesGenerator");
    const ConfigNode in_cfg = ConfigNode::fromFile(dir + "/config.xml", "StokesIntegrator");
    const ConfigNode rfi_cfg = ConfigNode::fromFile(dir + "/config.xml", "RFI_Clipper");
    std::ifstream shape(dir + "/shape.txt");
    unsigned nsub, npol, nblk, nchan;
    shape >> nsub >> npol >> nblk >> nchan;
    const auto v = read_file<std::complex<float>>(dir + "/volt.bin");
    TimeSeriesDataSetC32 ts;
    ts.resize(nblk, nsub, npol, nchan);
    std::memcpy(ts.data(), v.data(), v.size() * sizeof(v[0]));
    ts.setBlockRate(5.12e-6);
    PPFChanneliser ppf(ppf_cfg);
    StokesGenerator stokes(st_cfg);
    StokesIntegrator integ(in_cfg);
    RFI_Clipper rfi(rfi_cfg);
    SpectrumDataSetC32 spectra;
    SpectrumDataSetStokes st, it;
    ppf.run(&ts, &spectra);
    stokes.run(&spectra, &st);
    integ.run(&st, &it);
    write_file(dir + "/ppf.bin", spectra.data(), spectra.size());
    write_file(dir + "/stokes.bin", st.data(), st.size());
    write_file(dir + "/integ.bin", it.data(), it.size());
    WeightedSpectrumDataSet w(&it);
    rfi.run(&w);
    write_file(dir + "/rfi.bin", it.data(), it.size());
    std::printf("SHAPES %u %u %u %u %g\n", it.nTimeBlocks(), it.nSubbands(), it.nPolarisations(),
                it.nChannels(), it.getBlockRate());
    return 0;
}

// DedispersionModuleTest (lib/test/src/DedispersionModuleTest.cpp:109-275):
// nblobs blobs go through the module; prints the lock count of every blob
// after each dedisperse() call, what the functor saw (the known answer, the
// events, whether dedisperse() had returned and on which thread it ran),
// and after waitForJobCompletion() the lock counts and the blobs the unlock
// callback released, in order.
int ddmod_mode(const std::string& dir, int nblobs) {
    const ConfigNode dd_cfg = ConfigNode::fromFile(dir + "/config.xml", "DedispersionModule");
    const ConfigNode an_cfg = ConfigNode::fromFile(dir + "/config.xml", "DedispersionAnalyser");
    std::ifstream shape(dir + "/shape.txt");
    unsigned nt, nsub, nchan;
    double tsamp;
    shape >> nt >> nsub >> nchan >> tsamp;
    const auto data = read_file<float>(dir + "/blob.bin");
    std::vector<std::unique_ptr<SpectrumDataSetStokes>> blobs;
    for (int b = 0; b < nblobs; ++b) {
        blobs.emplace_back(new SpectrumDataSetStokes);
        SpectrumDataSetStokes& st = *blobs.back();
        st.resize(nt, nsub, 1, nchan);
        std::memcpy(st.data(), data.data() + (size_t)b * st.size(), st.size() * sizeof(float));
        st.setBlockRate(tsamp);
    }
    auto index_of = [&](const DataBlob* d) {
        for (size_t k = 0; k < blobs.size(); ++k)
            if (blobs[k].get() == d) return (int)k;
        return -1;
    };
    DedispersionModule dd(dd_cfg);
    DedispersionAnalyser an(an_cfg);
    std::vector<int> unlocked;
    std::mutex mu;
    int completed = 0;
    std::atomic<int> started{0}, returned{0};
    std::atomic<int> async_ok{1}, other_thread{1};
    const std::thread::id main_id = std::this_thread::get_id();
    dd.unlockCallback([&](const std::vector<DataBlob*>& freed) {
        std::lock_guard<std::mutex> l(mu);
        for (const DataBlob* b : freed) unlocked.push_back(index_of(b));
    });
    dd.onChainCompletion([&]() { ++completed; });
    dd.connect([&](DedispersionSpectra* s) {
        if (std::this_thread::get_id() == main_id) other_thread = 0;
        // the dedisperse() call that filled this buffer returns first
        const auto t_end = std::chrono::steady_clock::now() + std::chrono::seconds(10);
        while (returned.load() < started.load() && std::chrono::steady_clock::now() < t_end)
            std::this_thread::sleep_for(std::chrono::milliseconds(1));
        if (returned.load() < started.load()) async_ok = 0;
        DedispersionDataAnalysis result;
        const int n = an.analyse(s, &result);
        std::printf("AMP %g\nEVENTS %d\nFIRST %u\nINPUTS %zu\n", s->dmAmplitude(0u, 10.0f), n, s->firstSample(),
                    s->inputDataBlobs().size());
    });
    for (int b = 0; b < nblobs; ++b) {
        WeightedSpectrumDataSet w(blobs[b].get());
        ++started;
        dd.dedisperse(&w);
        ++returned;
        std::printf("LOCKS_ADD%d", b);
        for (auto& x : blobs) std::printf(" %d", dd.lockNumber(x.get()));
        std::printf("\n");
    }
    dd.waitForJobCompletion();
    std::printf("LOCKS_END");
    for (auto& x : blobs) std::printf(" %d", dd.lockNumber(x.get()));
    std::printf("\nUNLOCKED");
    for (int k : unlocked) std::printf(" %d", k);
    std::printf("\nASYNC %d\nTHREAD %d\n", async_ok.load(), other_thread.load());
    std::printf("MAXSHIFT %d\nCOMPLETED %d\n", dd.maxshift(), completed);
    return 0;
}

int ddout_mode(const std::string& dir, int nblobs) {
    const ConfigNode dd_cfg = ConfigNode::fromFile(dir + "/config.xml", "DedispersionModule");
    const ConfigNode an_cfg = ConfigNode::fromFile(dir + "/config.xml", "DedispersionAnalyser");
    const ConfigNode out_cfg = ConfigNode::fromFile(dir + "/config.xml", "DedispersionDataAnalysisOutput");
    std::ifstream shape(dir + "/shape.txt");
    unsigned nt, nsub, nchan;
    double tsamp, t0;
    shape >> nt >> nsub >> nchan >> tsamp >> t0;
    const auto blob = read_file<float>(dir + "/blob.bin");
    DedispersionModule dd(dd_cfg);
    DedispersionAnalyser an(an_cfg);
    DedispersionDataAnalysisOutput out(out_cfg);
    std::unique_ptr<TriggerOutput> trigger;
    try {
        trigger.reset(new TriggerOutput(ConfigNode::fromFile(dir + "/config.xml", "TriggerOutput")));
    } catch (const std::runtime_error&) {
    }
    std::ofstream evf(dir + "/events.bin", std::ios::binary);
    dd.connect([&](DedispersionSpectra* s) {
        DedispersionDataAnalysis result;
        an.analyse(s, &result);
        out.sendStream(&result);
        if (trigger) {
            const std::string m = trigger->sendStream(&result);
            if (!m.empty()) std::printf("TRIGGER %s\n", m.c_str());
        }
        for (const auto& e : result.events()) {
            const pv_event pe{(int32_t)e.dmIndex(), (int32_t)e.timeBin(), e.mfBinning(), e.mfValue()};
            evf.write(reinterpret_cast<const char*>(&pe), sizeof pe);
        }
        std::printf("META %.17g %.17g %u %.17g %.17g %.9g %d\n", s->getLofarTimestamp(), s->getBlockRate(),
                    s->firstSample(), s->dmLow(), s->dmStep(), result.getRMS(), result.eventsFound());
    });
    std::vector<std::unique_ptr<SpectrumDataSetStokes>> held;  // locked until their buffers are exported
    for (int b = 0; b < nblobs; ++b) {
        held.emplace_back(new SpectrumDataSetStokes);
        SpectrumDataSetStokes& st = *held.back();
        st.resize(nt, nsub, 1, nchan);
        std::memcpy(st.data(), blob.data() + (size_t)b * st.size(), st.size() * sizeof(float));
        st.setBlockRate(tsamp);
        st.setLofarTimestamp(t0 + (double)b * nt * tsamp);
        WeightedSpectrumDataSet w(&st);
        dd.dedisperse(&w);
    }
    dd.waitForJobCompletion();
    return 0;
}

int sigproc_mode(const std::string& dir) {
    const ConfigNode cfg = ConfigNode::fromFile(dir + "/config.xml", "SigprocStokesWriter");
    std::ifstream shape(dir + "/shape.txt");
    unsigned nt, nsub, npol, nchan;
    double t0;
    shape >> nt >> nsub >> npol >> nchan >> t0;
    const auto data = read_file<float>(dir + "/stokes.bin");
    SigprocStokesWriter w(cfg);
    for (int half = 0; half < 2; ++half) {  // two blobs: the header precedes the first only
        SpectrumDataSetStokes st;
        st.resize(nt / 2, nsub, npol, nchan);
        std::memcpy(st.data(), data.data() + (size_t)half * st.size(), st.size() * sizeof(float));
        st.setLofarTimestamp(t0);
        w.sendStream(&st);
    }
    std::printf("NCHANS %d\n", w.params().nchans);
    return 0;
}

int pipeline_mode(const std::string& dir, int nchunks) {
    const std::string xml = dir + "/config.xml";
    const auto all = read_file<unsigned char>(dir + "/chunks.bin");
    const size_t chunk = all.size() / (size_t)nchunks;
    AdapterTimeSeriesDataSet adapter(ConfigNode::fromFile(xml, "AdapterTimeSeriesDataSet"));
    DedispersionPipeline pipeline(xml);
    DedispersionDataAnalysisOutput out(ConfigNode::fromFile(xml, "DedispersionDataAnalysisOutput"));
    pipeline.connectOutput("DedispersionDataAnalysis",
                           [&](const DedispersionDataAnalysis& r) { out.sendStream(&r); });
    TimeSeriesDataSetC32 ts;
    for (int k = 0; k < nchunks; ++k) {
        adapter.config(&ts, chunk);
        adapter.deserialise(all.data() + (size_t)k * chunk);
        pipeline.run(&ts);
    }
    pipeline.waitForJobCompletion();
    std::printf("BUFFERS %u\nFUSED %d\n", pipeline.buffers(), pipeline.fused() ? 1 : 0);
    return 0;
}

int outputs_mode(const std::string& dir) {
    const std::string xml = dir + "/config.xml";
    std::ifstream meta(dir + "/meta.txt");
    double start, rate, dmlow, dmstep;
    unsigned first, ntime, ndm;
    float rms;
    meta >> start >> rate >> first >> dmlow >> dmstep >> rms >> ntime >> ndm;
    const auto ev = read_file<pv_event>(dir + "/events.bin");
    DedispersionSpectra spectra;
    spectra.resize(ntime, ndm, (float)dmlow, (float)dmstep);
    spectra.setFirstSample(first);
    spectra.setLofarTimestamp(start);
    spectra.setBlockRate(rate);
    DedispersionDataAnalysis result;
    result.reset(&spectra);
    result.setRMS(rms);
    for (const pv_event& e : ev) result.addEvent((unsigned)e.dm, (unsigned)e.t, e.bin_factor, e.value);
    DedispersionDataAnalysisOutput out(ConfigNode::fromFile(xml, "DedispersionDataAnalysisOutput"));
    TriggerOutput trigger(ConfigNode::fromFile(xml, "TriggerOutput"));
    for (int k = 0; k < 2; ++k) {
        out.sendStream(&result);
        const std::string m = trigger.sendStream(&result);
        if (!m.empty()) std::printf("TRIGGER %s\n", m.c_str());
    }
    return 0;
}

int ab_mode(const std::string& dir, int nchunks) {
    const std::string xml = dir + "/config.xml";
    const auto all = read_file<unsigned char>(dir + "/chunks.bin");
    const size_t chunk = all.size() / (size_t)nchunks;
    ABDataAdapter adapter(ConfigNode::fromFile(xml, "ABDataAdapter"));
    ABPipeline pipeline(xml);
    DedispersionDataAnalysisOutput out(ConfigNode::fromFile(xml, "DedispersionDataAnalysisOutput"));
    int dumps = 0;
    pipeline.connectOutput("DedispersionDataAnalysis", [&](const DedispersionDataAnalysis& r) {
        out.sendStream(&r);
        ++dumps;
    });
    pipeline.connectSpectrumOutput("SignalFoundSpectrum", [&](const SpectrumDataSetStokes& s) {
        std::printf("SIGNAL %d %.17g %u\n", dumps, s.getLofarTimestamp(), s.nTimeBlocks());
    });
    std::ofstream sp(dir + "/spectra.bin", std::ios::binary);
    SpectrumDataSetStokes stokes;
    for (int k = 0; k < nchunks; ++k) {
        adapter.config(&stokes, chunk);
        adapter.deserialise(all.data() + (size_t)k * chunk);
        sp.write(reinterpret_cast<const char*>(stokes.data()), (std::streamsize)(stokes.size() * sizeof(float)));
        std::printf("TIME %.17g %.17g\n", stokes.getLofarTimestamp(), stokes.getBlockRate());
        pipeline.run(&stokes);
    }
    pipeline.waitForJobCompletion();
    std::printf("BUFFERS %u\nGAPS %lld\n", pipeline.buffers(), adapter.gaps());
    return 0;
}

int udp_mode(const std::string& dir) {
    const ConfigNode cfg = ConfigNode::fromFile(dir + "/config.xml", "AdapterTimeSeriesDataSet");
    const auto chunk = read_file<unsigned char>(dir + "/chunk.bin");
    AdapterTimeSeriesDataSet adapter(cfg);
    TimeSeriesDataSetC32 ts;
    adapter.config(&ts, chunk.size());
    adapter.deserialise(chunk.data());
    write_file(dir + "/ts.bin", ts.data(), (size_t)ts.nTimeBlocks() * ts.nSubbands() * ts.nPolarisations() *
                                               ts.nTimesPerBlock());
    std::printf("SHAPE %u %u %u %u\nTIME %.17g %.17g\n", ts.nTimeBlocks(), ts.nSubbands(), ts.nPolarisations(),
                ts.nTimesPerBlock(), ts.getLofarTimestamp(), ts.getBlockRate());
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string mode = argv[1];
    try {
        if (mode == "config") return config_mode();
        if (mode == "chain" && argc >= 3) return chain_mode(argv[2]);
        if (mode == "ddmod" && argc >= 4) return ddmod_mode(argv[2], std::atoi(argv[3]));
        if (mode == "udp" && argc >= 3) return udp_mode(argv[2]);
        if (mode == "ddout" && argc >= 4) return ddout_mode(argv[2], std::atoi(argv[3]));
        if (mode == "sigproc" && argc >= 3) return sigproc_mode(argv[2]);
        if (mode == "pipeline" && argc >= 4) return pipeline_mode(argv[2], std::atoi(argv[3]));
        if (mode == "ab" && argc >= 4) return ab_mode(argv[2], std::atoi(argv[3]));
        if (mode == "outputs" && argc >= 3) return outputs_mode(argv[2]);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "EXCEPTION %s\n", e.what());
        return 3;
    }
    return 2;
}
