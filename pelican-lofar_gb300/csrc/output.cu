// Outputs after the path: the sigproc filterbank writer and the event text
// stream.
//
// SigprocStokesWriter (lib/src/SigprocStokesWriter.cpp:15-293): a header of
// length-prefixed keywords with int32 / float64 values (:118-181), then per
// spectrum, for each written polarisation, the subbands and within them the
// channels in descending order (:207-234), as float32 or as one byte
// rint((min(x, max) - min) * 255 / (max - min)), 0 below min (:288-293).
// The reorder and quantisation run on the device over the filterbank that is
// already there, so 8-bit output leaves the GPU at a quarter of the bytes.
//
// DedispersionDataAnalysisOutput (lib/src/DedispersionDataAnalysisOutput.cpp:
// 58-112): one text line per event after the first (the time stamp
// carrier), "mjd,   dm, snr, binFactor", then a summary line per buffer.
// QTextStream prints reals as %g with 14 significant digits
// (setRealNumberPrecision(14), default SmartNotation); floats are widened to
// double first.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "pv_internal.cuh"

namespace {

template <bool U8>
__global__ void __launch_bounds__(256)
sigproc_pack_kernel(const float* __restrict__ in, int nt, int nsub, int npol, int nchan, int npw,
                    float cmin, float cmax, float nrange, float delta, void* __restrict__ out) {
    const long long per = (long long)npw * nsub * nchan;  // output values per spectrum
    const long long total = per * nt;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < total;
         j += (long long)gridDim.x * blockDim.x) {
        const long long t = j / per;
        const int r = (int)(j - t * per);
        const int p = r / (nsub * nchan);
        const int q = r - p * nsub * nchan;
        const int s = nsub - 1 - q / nchan;
        const int i = nchan - 1 - q % nchan;
        const float x = __ldg(in + (((t * nsub + s) * npol + p) * (long long)nchan + i));
        if (U8) {
            const float f = x > cmax ? cmax : x;
            const int ci = f < cmin ? 0 : __float2int_rn(__fdiv_rn(__fmul_rn(__fsub_rn(f, cmin), nrange), delta));
            reinterpret_cast<unsigned char*>(out)[j] = (unsigned char)(ci & 0xff);
        } else {
            reinterpret_cast<float*>(out)[j] = x;
        }
    }
}

// The same order, four outputs per thread when nchan % 4 == 0: outputs q..q+3
// of a row (spectrum t, written polarisation p) are channels i..i-3 of one
// subband, one aligned float4 read backwards.  blockIdx.y is the row group,
// blockIdx.x the position in the row.
template <bool U8>
__device__ __forceinline__ unsigned char quantise(float x, float cmin, float cmax, float nrange, float delta) {
    const float f = x > cmax ? cmax : x;
    const int ci = f < cmin ? 0 : __float2int_rn(__fdiv_rn(__fmul_rn(__fsub_rn(f, cmin), nrange), delta));
    return (unsigned char)(ci & 0xff);
}

template <bool U8>
__global__ void __launch_bounds__(256)
sigproc_pack4_kernel(const float* __restrict__ in, int nrows, int nsub, int npol, int nchan, int npw, float cmin,
                     float cmax, float nrange, float delta, void* __restrict__ out) {
    const int per = nsub * nchan;  // outputs per row
    const int q = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
    if (q >= per) return;
    for (long long row = blockIdx.y; row < nrows; row += gridDim.y) {
        const long long t = row / npw;
        const int p = (int)(row - t * npw);
        const int sr = q / nchan, ir = q - sr * nchan;
        const int s = nsub - 1 - sr, i = nchan - 1 - ir;  // channels i, i-1, i-2, i-3
        const float4 v =
            __ldg(reinterpret_cast<const float4*>(in + ((t * nsub + s) * npol + p) * (long long)nchan + i - 3));
        const long long o = row * per + q;
        if (U8) {
            uchar4 b;
            b.x = quantise<true>(v.w, cmin, cmax, nrange, delta);
            b.y = quantise<true>(v.z, cmin, cmax, nrange, delta);
            b.z = quantise<true>(v.y, cmin, cmax, nrange, delta);
            b.w = quantise<true>(v.x, cmin, cmax, nrange, delta);
            reinterpret_cast<uchar4*>(out)[o >> 2] = b;
        } else {
            reinterpret_cast<float4*>(out)[o >> 2] = make_float4(v.w, v.z, v.y, v.x);
        }
    }
}

struct Buf {
    char* p;
    long long cap, n;
    void put(const void* src, size_t k) {
        if (n + (long long)k <= cap && p) std::memcpy(p + n, src, k);
        n += (long long)k;
    }
    void str(const char* s) {
        const int len = (int)std::strlen(s);
        put(&len, 4);
        put(s, (size_t)len);
    }
    void i32(const char* name, int v) {
        str(name);
        put(&v, 4);
    }
    void f64(const char* name, double v) {
        str(name);
        put(&v, 8);
    }
};

}  // namespace

extern "C" int pv_sigproc_header(const pv_sigproc_params* h, char* h_buf, long long cap, long long* h_len) {
    if (!h || !h_len || cap < 0) {
        pv::set_error("pv_sigproc_header: invalid arguments");
        return PV_ERR_ARG;
    }
    char name[sizeof(h->source_name) + 1];
    std::memcpy(name, h->source_name, sizeof(h->source_name));
    name[sizeof(h->source_name)] = '\0';
    Buf b{h_buf, cap, 0};
    b.str("HEADER_START");
    b.i32("machine_id", h->machine_id);
    b.i32("telescope_id", h->telescope_id);
    b.i32("data_type", 1);
    b.str("source_name");
    b.str(name);
    b.f64("src_raj", h->src_raj);
    b.f64("src_dej", h->src_dej);
    b.f64("fch1", h->fch1);
    b.f64("foff", h->foff);
    b.i32("nchans", h->nchans);
    b.f64("tsamp", h->tsamp);
    b.i32("nbits", h->nbits);
    b.f64("tstart", h->tstart);
    b.i32("nifs", h->nifs);
    b.str("HEADER_END");
    *h_len = b.n;
    if (b.n > cap) {
        pv::set_error("pv_sigproc_header: %lld bytes needed", b.n);
        return PV_ERR_ARG;
    }
    return PV_OK;
}

extern "C" double pv_sigproc_mjd(double lofar_timestamp) {
    return (lofar_timestamp - 1293840000.0) / 86400 + 55562.0;  // 2011-01-01 00:00 UTC is MJD 55562
}

extern "C" int pv_sigproc_pack(const float* d_stokes, int nt, int nsub, int npol, int nchan, int npols_write,
                               int nbits, float crop_min, float crop_max, void* d_out, void* stream) {
    if (nbits != 8 && nbits != 32) {
        pv::set_error("SigprocStokesWriter: %d bit datafiles not yet supported", nbits);
        return PV_ERR_CONFIG;
    }
    if (!d_stokes || !d_out || nt < 0 || nsub <= 0 || npol <= 0 || nchan <= 0 || npols_write <= 0 ||
        npols_write > npol) {
        pv::set_error("pv_sigproc_pack: invalid arguments");
        return PV_ERR_ARG;
    }
    const long long total = (long long)nt * npols_write * nsub * nchan;
    if (total == 0) return PV_OK;
    const float nrange = 255.0f;  // (int)pow(2, 8) - 1.0 (SigprocStokesWriter.cpp:27)
    const float delta = crop_max - crop_min;
    cudaStream_t s = pv::as_stream(stream);
    const uintptr_t align = reinterpret_cast<uintptr_t>(d_stokes) | reinterpret_cast<uintptr_t>(d_out);
    if (nchan % 4 == 0 && align % 16 == 0) {
        const int per = nsub * nchan;
        const long long rows = (long long)nt * npols_write;
        const dim3 grid((unsigned)pv::ceil_div(per / 4, 256),
                        (unsigned)std::min<long long>(rows, std::max(1LL, pv::sm_count() * 64LL / pv::ceil_div(per / 4, 256))));
        if (nbits == 8)
            sigproc_pack4_kernel<true><<<grid, 256, 0, s>>>(d_stokes, (int)rows, nsub, npol, nchan, npols_write,
                                                            crop_min, crop_max, nrange, delta, d_out);
        else
            sigproc_pack4_kernel<false><<<grid, 256, 0, s>>>(d_stokes, (int)rows, nsub, npol, nchan, npols_write,
                                                             crop_min, crop_max, nrange, delta, d_out);
        return pv::check_launch("sigproc_pack4_kernel");
    }
    const int blocks = (int)std::min<long long>(pv::ceil_div<long long>(total, 256), pv::sm_count() * 16LL);
    if (nbits == 8)
        sigproc_pack_kernel<true><<<blocks, 256, 0, s>>>(d_stokes, nt, nsub, npol, nchan, npols_write, crop_min,
                                                         crop_max, nrange, delta, d_out);
    else
        sigproc_pack_kernel<false><<<blocks, 256, 0, s>>>(d_stokes, nt, nsub, npol, nchan, npols_write,
                                                          crop_min, crop_max, nrange, delta, d_out);
    return pv::check_launch("sigproc_pack_kernel");
}

extern "C" int pv_events_text(const pv_event* h_events, long long n, double start_timestamp, double block_rate,
                              long long first_sample, double dm_low, double dm_step, float rms, int dump_index,
                              char* h_buf, long long cap, long long* h_len) {
    if ((!h_events && n > 0) || !h_len || cap < 0) {
        pv::set_error("pv_events_text: invalid arguments");
        return PV_ERR_ARG;
    }
    std::string out;
    char line[256];
    auto time_of = [&](long long t) {  // DedispersionSpectra::getTime -> SpectrumDataSet::getTime
        return start_timestamp + (double)(unsigned)(t + first_sample) * block_rate;
    };
    float snr_max = 0.0f, dm_best = 0.0f;
    for (long long i = 1; i < n; ++i) {
        const pv_event& e = h_events[i];
        const double mjd = time_of(e.t) / 86400;
        const float dm = (float)(dm_low + dm_step * e.dm);  // BinMap::binAssignmentNumber
        const float snr = (float)(e.value / (rms * std::sqrt((double)e.bin_factor)));
        if (snr > snr_max) {
            dm_best = dm;
            snr_max = snr;
        }
        std::snprintf(line, sizeof line, "%.14g,   %.14g, %.14g, %d\n", mjd, (double)dm, (double)snr, (int)e.bin_factor);
        out += line;
    }
    const double mjd0 = (n > 0 ? time_of(h_events[0].t) : time_of(0)) / 86400;
    std::snprintf(line, sizeof line, "# Written buffer :%d | MJDstart: %.14g | Best DM: %.14g | Max SNR: %.14g  Done\n",
                  dump_index, mjd0, (double)dm_best, (double)snr_max);
    out += line;
    *h_len = (long long)out.size();
    if (h_buf && (long long)out.size() <= cap) std::memcpy(h_buf, out.data(), out.size());
    if ((long long)out.size() > cap) {
        pv::set_error("pv_events_text: %lld bytes needed", (long long)out.size());
        return PV_ERR_ARG;
    }
    return PV_OK;
}

namespace {
// QString::arg(a, width, '0'): right-aligned, padded on the left, never cut.
std::string zero_pad(const std::string& s, size_t width) {
    return s.size() >= width ? s : std::string(width - s.size(), '0') + s;
}
std::string fixed(double v, int digits) {  // QString::number(v, 'f', digits)
    char b[64];
    std::snprintf(b, sizeof b, "%.*f", digits, v);
    return b;
}
}  // namespace

extern "C" int pv_trigger_message(const pv_event* h_events, long long n, double start_timestamp, double block_rate,
                                  long long first_sample, double dm_low, double dm_step, float rms, int min_events,
                                  float snr_threshold, const char* station, const char* id_root, int message_number,
                                  const char* cfreq_mhz, const char* beam_ra, const char* beam_dec, char* h_buf,
                                  long long cap, long long* h_len) {
    if ((!h_events && n > 0) || !h_len || cap < 0 || !station || !id_root || !cfreq_mhz || !beam_ra || !beam_dec) {
        pv::set_error("pv_trigger_message: invalid arguments");
        return PV_ERR_ARG;
    }
    *h_len = 0;
    if (n < (long long)min_events) return PV_OK;  // eventsFound() counts the analyser's first event
    // The reference declares the running maximum and its event without a value; they start at
    // "no event" here, so only an SNR above 0 can win.  The first of equal SNRs is kept.
    long long best = -1;
    float snr_max = 0.0f;
    for (long long i = 0; i < n; ++i) {
        const float snr = h_events[i].value / (rms * std::sqrt(h_events[i].bin_factor));
        if (snr > snr_max) {
            snr_max = snr;
            best = i;
        }
    }
    if (best < 0 || !(snr_max >= snr_threshold)) return PV_OK;
    const pv_event& e = h_events[best];
    const double t = start_timestamp + (double)(unsigned)(e.t + first_sample) * block_rate;
    const float dm = (float)(dm_low + dm_step * e.dm);
    const std::string msg = std::string("artemis:") + station + "##ID:" + id_root +
                            zero_pad(std::to_string(message_number), 4) + "##cFreqMHz:" + zero_pad(cfreq_mhz, 10) +
                            "##beamRA:" + zero_pad(beam_ra, 10) + "##beamDec:" + zero_pad(beam_dec, 9) +
                            "##eTime:" + zero_pad(fixed(t, 9), 20) + "##eDM:" + zero_pad(fixed(dm, 3), 9) +
                            "##eSNR:" + zero_pad(fixed(snr_max, 2), 6);
    *h_len = (long long)msg.size();
    if ((long long)msg.size() > cap) {
        if (!h_buf) return PV_OK;  // size query
        pv::set_error("pv_trigger_message: %lld bytes needed", (long long)msg.size());
        return PV_ERR_ARG;
    }
    if (h_buf) std::memcpy(h_buf, msg.data(), msg.size());
    return PV_OK;
}
