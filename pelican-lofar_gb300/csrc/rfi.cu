// K2/K3: RFI_Clipper (lib/src/RFI_Clipper.cpp:22-573) with its bandpass model
// (lib/src/BandPass.cpp, BandPassAdapter.cpp:30-108, BinMap.cpp).
//
// The clipper is a sequential state machine over spectra: every spectrum's
// channel-clip margin, bandpass level and rejection test depend on running
// averages updated by the previous spectrum.  One CTA, or for a wide beam a
// cluster of CTAs, walks a beam's spectra in order; partial p (P = 256, 512
// or 1024 by channel count) owns channels p, p+P, ... of each spectrum.  The
// state (running mean/RMS, their history rings, the last good spectrum, the
// bandpass offset) lives in device memory between calls, so a stream of
// chunks gives the same result as one long chunk.
//
// Arithmetic.  This is the FP64 variant of the reference: per-spectrum
// statistics and running averages are double, channel values and the
// bandpass are float as in the reference.  Channel sums use a fixed order
// (partial p's sequential sum, a halving tree of offsets 16..1 inside each
// warp, then offsets P/64..1 over the P/32 warp sums) so results are
// deterministic and independent of how the partials are spread over CTAs.  Clip flags therefore match the reference's FP32 arithmetic
// except for channels or spectra within rounding distance of a threshold.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include <cooperative_groups.h>

#include "pv_internal.cuh"

namespace {


// ---------------------------------------------------------------------------
// Host: BinMap / BandPass (BinMap.cpp:37-68, BandPass.cpp:26-166)
// ---------------------------------------------------------------------------
float powi(float a, int b) {  // C++98 std::pow(float,int): binary exponentiation in float
    float r = 1.0f;
    for (;;) {
        if (b & 1) r *= a;
        b /= 2;
        if (b == 0) break;
        a *= a;
    }
    return r;
}

struct Map {
    unsigned n = 0;
    double lower = 0.0, width = 1.0, half = 0.0;
    void set_width(double w) { width = w; half = w / 2.0; }
    int index(double v) const { return (int)(0.5 + ((v - lower) / width)); }
    double value(int i) const { return lower + (width * i); }
    std::tuple<unsigned, double, double> key() const { return std::make_tuple(n, lower, width); }
};

struct Bandpass {
    Map primary, current;
    std::vector<float> params{0.0f};
    std::map<std::tuple<unsigned, double, double>, std::vector<float>> sets;
    std::map<std::tuple<unsigned, double, double>, float> rms, median, mean;
    std::vector<std::pair<float, float>> killed;

    static float at(const std::map<std::tuple<unsigned, double, double>, float>& m,
                    const std::tuple<unsigned, double, double>& k) {
        auto it = m.find(k);
        return it == m.end() ? 0.0f : it->second;
    }
    float evaluate(float v) const {
        float tot = 0.0f;
        for (size_t i = 0; i < params.size(); ++i) tot += params[i] * powi(v, (int)i);
        return tot;
    }
    void zero_killed(const Map& m) {
        std::vector<float>& d = sets[m.key()];
        for (auto& r : killed) {
            int lo = m.index(r.first), hi = m.index(r.second);
            if (hi < lo) std::swap(lo, hi);
            lo = std::max(lo, 0);
            if ((int)d.size() < hi) d.resize(hi + 1);
            do { if (lo < (int)d.size()) d[lo] = 0.0f; } while (++lo <= hi);
        }
    }
    void build(const Map& m, float scale) {
        std::vector<float>& d = sets[m.key()];
        d.assign(m.n, 0.0f);
        for (unsigned i = 0; i < m.n; ++i) d[i] = scale * evaluate((float)m.value(i));
        zero_killed(m);
    }
    void rebin(const Map& m) {
        current = m;
        if (!sets.count(m.key())) {
            const double scale = m.width / primary.width;
            rms[m.key()] = (float)(at(rms, primary.key()) * std::sqrt(1.0 / scale));
            median[m.key()] = (float)(at(median, primary.key()) * scale);
            mean[m.key()] = (float)(at(mean, primary.key()) * scale);
            build(current, (float)scale);
        }
    }
    void set_data(const Map& m, const std::vector<float>& p) {
        primary = m;
        params = p;
        rebin(m);
        const std::vector<float>& d = sets[m.key()];
        float sum = 0.0f;
        std::vector<float> copy(d.begin(), d.end());
        for (unsigned i = 0; i < m.n; ++i) sum += d[i];
        mean[m.key()] = sum / m.n;
        std::nth_element(copy.begin(), copy.begin() + copy.size() / 2, copy.end());
        median[m.key()] = copy[copy.size() / 2];
    }
    void set_median(float med) {
        const float delta = med - median[current.key()];
        if (std::fabs(delta) > 0.0f) {
            const float scale = (float)(current.width / primary.width);
            median[current.key()] = med;
            median[primary.key()] = med / scale;
            params[0] += delta / scale;
            mean[current.key()] += delta;
            mean[primary.key()] += delta / scale;
            sets.clear();
            build(current, scale);
        }
    }
    void set_rms(float r) { rms[current.key()] = r; }
};

int parse_bandpass(const char* text, Bandpass& bp) {
    std::vector<float> params;
    std::vector<unsigned> kills;
    int count = 0, line = 0;
    const char* p = text;
    auto trim = [](const std::string& s) {
        const size_t a = s.find_first_not_of(" \t\r\v\f"), b = s.find_last_not_of(" \t\r\v\f");
        return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
    };
    while (*p) {
        ++line;
        const char* eol = std::strchr(p, '\n');
        const std::string ln = eol ? std::string(p, eol) : std::string(p);
        p = eol ? eol + 1 : p + ln.size();
        if (ln[0] == '#') continue;
        if (ln[0] == 'K') {
            unsigned idx = 0;
            double fq = 0.0;
            if (std::sscanf(trim(ln.substr(1)).c_str(), "%u %lf", &idx, &fq) < 2) {
                pv::set_error("BandPassAdapter: syntax error on line %d: expecting two numbers on "
                              "Kill line: index frequency", line);
                return PV_ERR_CONFIG;
            }
            kills.push_back(idx);
            continue;
        }
        ++count;
        const std::string s = trim(ln);
        char* end = nullptr;
        const double v = s.empty() ? 0.0 : std::strtod(s.c_str(), &end);
        if (s.empty() || !end || *end != '\0') {
            pv::set_error("BandPassAdapter: syntax error on line %d", line);
            return PV_ERR_CONFIG;
        }
        params.push_back((float)v);
    }
    if (count < 6) {
        pv::set_error("BandPassAdapter: data format wrong : got %d parameters, expecting at least 6",
                      count);
        return PV_ERR_CONFIG;
    }
    Map m;
    m.n = (unsigned)params[0];
    m.lower = params[1];
    m.set_width(params[3]);
    const float rms = params[4], median = params[5];
    params.erase(params.begin(), params.begin() + 5);  // the median is the first coefficient
    bp.set_data(m, params);
    bp.set_median(median);
    bp.set_rms(rms);
    for (unsigned idx : kills) {
        // The reference reads the kill line's index as its frequency too
        // (BandPassAdapter.cpp:67), so the check below rejects it unless the
        // index happens to name its own bin.
        if (m.index((double)idx) != (int)idx) {
            pv::set_error("BandPassAdapter:  Frequency kill mismatch: index %u does not match "
                          "frequency %u", idx, idx);
            return PV_ERR_CONFIG;
        }
        bp.killed.push_back({(float)(m.value(idx) - m.half), (float)(m.value(idx) + m.half)});
        for (auto& kv : bp.sets) {
            Map mm;
            mm.n = std::get<0>(kv.first); mm.lower = std::get<1>(kv.first); mm.set_width(std::get<2>(kv.first));
            bp.zero_killed(mm);
        }
    }
    return PV_OK;
}

// ---------------------------------------------------------------------------
// Device state
// ---------------------------------------------------------------------------
struct RfiState {
    double mean_run, rms_run, mean_over_rms, inv_mor, rms_carry;
    double mean_acc, mean_acc_prev, rms_acc, rms_acc_prev;
    int mean_head, mean_size, rms_head, rms_size;
    int num, bad_spectra, remaining_zeros;
    float frac_bad_channels;
    float params0, bp_mean, bp_rms;
};

struct RfiConfig {
    int nbins, history, zero_dming, use_mor, deg;
    float cr, sr, scale, mmm_f;
    double inv_sqrt_nbins;
};

struct RfiBuffers {
    RfiState* state;
    double* mean_buf;   // [history]
    double* rms_buf;    // [history]
    float* last_good;   // [nbins]
    const float* terms; // [deg][nbins]: params[k]*powi(f_i,k), k >= 1
    const unsigned char* killed;  // [nbins] or null
};

// ---------------------------------------------------------------------------
// Block reductions.  Every thread holds one FP32 partial per quantity (thread
// p sums channels p, p+P, ... in order).  The canonical order reduces each
// warp's 32 partials by the halving tree of offsets 16..1 and the NW warp
// sums by offsets NW/2..1 (warp 0, lane_tree below).
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void warp_tree(float (&v)[K], float* red /*[32][K]*/) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const float o = __shfl_down_sync(0xffffffffu, v[k], off);
            if (lane < off) v[k] = __fadd_rn(v[k], o);
        }
    }
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) red[warp * K + k] = v[k];
}

__device__ __forceinline__ float bp_value(const RfiConfig& cfg, const RfiBuffers& b, float params0, int i) {
    if (b.killed && b.killed[i]) return 0.0f;
    float tot = params0;  // 0 + params[0]*1
    for (int k = 0; k < cfg.deg; ++k) tot = __fadd_rn(tot, b.terms[(long long)k * cfg.nbins + i]);
    return __fmul_rn(cfg.scale, tot);
}

__device__ __forceinline__ void cp_async4(float* smem_dst, const float* gmem_src) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(gmem_src) : "memory");
}
// both addresses 16-byte aligned
__device__ __forceinline__ void cp_async16(float* smem_dst, const float* gmem_src) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(gmem_src) : "memory");
}

// Ring index x in [0, 2H) reduced to [0, H).
__device__ __forceinline__ int wrap_h(int x, int H) { return x >= H ? x - H : x; }

// Values warp 0 derives from the scalar state and broadcasts.
struct Bcast {
    float dm_f, margin_f;        // for the next clip pass
    float sub_f, rms_f, params0; // for the normalise pass
    int adapt;                   // next spectrum starts in the adaptive phase
    int spectrum_clip, do_fill, rebuild_bp;
};

// Channel geometry: bin -> pol-0 element offset within a spectrum, and band.
struct Geo {
    int nsub, npol, nchan, lg_nchan;  // lg_nchan < 0: nchan is not a power of two
    int cpb;
    // RFI_Clipper.cpp:383-394 compares good-channel counts with 0.8 * cpb and
    // 0.8 * nbins in double: for an integer count n, n < x exactly when
    // n < ceil(x), so the thresholds are these integers.
    int band_good_min, good_min;
    __device__ __forceinline__ long long off(int bin) const {
        int sb, c;
        if (lg_nchan >= 0) { sb = bin >> lg_nchan; c = bin & (nchan - 1); }
        else { sb = bin / nchan; c = bin - sb * nchan; }
        return ((long long)sb * npol) * nchan + c;
    }
    __device__ __forceinline__ int band(int bin) const {
        int b = 0;
#pragma unroll
        for (int k = 1; k < 8; ++k) b += bin >= k * cpb;
        return b;
    }
};

Geo make_geo(int nsub, int npol, int nchan) {
    const int nbins = nsub * nchan;
    Geo g{nsub, npol, nchan, (nchan & (nchan - 1)) == 0 ? __builtin_ctz((unsigned)nchan) : -1, nbins / 8, 0, 0};
    g.band_good_min = (int)std::ceil(0.8 * g.cpb);
    g.good_min = (int)std::ceil(0.8 * nbins);
    return g;
}

// The band of a thread's current channel as its channels rise: band b holds
// channels [b*cpb, (b+1)*cpb), band 7 the rest (Geo::band).
struct BandRun {
    int band, end;  // end: first channel of the next band (INT_MAX for band 7)
    __device__ __forceinline__ BandRun(const Geo& g, int i) { set(g, g.band(i)); }
    __device__ __forceinline__ void set(const Geo& g, int b) {
        band = b;
        end = b < 7 ? (b + 1) * g.cpb : 0x7fffffff;
    }
    __device__ __forceinline__ bool ends_before(int i) const { return i >= end; }
    __device__ __forceinline__ void advance(const Geo& g, int i) { set(g, g.band(i)); }
};

// A beam's clipper may span a cluster of C CTAs of T threads: partial p =
// rank * T + thread, so the P = C * T partials, their channels and the
// canonical sums are those of one CTA of P threads.  Warp 0 of every CTA
// reads the NW = P / 32 warp partials of the whole cluster (distributed
// shared memory) and runs the same scalar chain on them, so every CTA holds
// the same state without a broadcast.
template <int C, typename V>
__device__ __forceinline__ const V* cta_buf(const V* p, int rank) {
    if constexpr (C == 1) return p;
    else return cooperative_groups::this_cluster().map_shared_rank(p, (unsigned)rank);
}
// Barrier after the warp partials are written: the whole cluster's.
template <int C>
__device__ __forceinline__ void partials_barrier() {
    if constexpr (C == 1) __syncthreads();
    else cooperative_groups::this_cluster().sync();
}
// Warp 0: lane g < NW takes the K partials of warp g of the cluster (the
// loads are independent: one round trip to the other CTAs for all of them);
// lanes from NW on take `fill`.
template <int C, int WPC, int K, typename V>
__device__ __forceinline__ void lane_partials(const V* buf, V (&out)[K], V fill) {
    constexpr int NW = C * WPC;
    const int lane = threadIdx.x & 31;
    if (lane < NW) {
        const V* src = cta_buf<C>(buf, lane / WPC) + (lane % WPC) * K;
#pragma unroll
        for (int k = 0; k < K; ++k) out[k] = src[k];
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k) out[k] = fill;
    }
}
// The canonical second stage over the lanes' warp sums (offsets NW/2..1);
// every lane returns the total.
template <int NW>
__device__ __forceinline__ float lane_tree(float w) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int off = NW / 2; off >= 1; off >>= 1) {
        const float o = __shfl_down_sync(0xffffffffu, w, off);
        if (lane < off) w = __fadd_rn(w, o);
    }
    return __shfl_sync(0xffffffffu, w, 0);
}
__device__ __forceinline__ float lane_min(float m) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, off));
    return m;
}
// Shared words of the reduction buffers (one set per phase: a CTA rewrites a
// phase's buffer only after a later cluster barrier, which every reader of
// the previous contents has passed).
constexpr int kRedWords = 32 * 16 * 2 + 32 + 32 * 8 + 32 * 2 + 32;

// History rings of the running averages as warp 0 sees them: the newest two
// entries and the prefetched oldest entry stay in registers.
struct Hist {
    double last, prev, front;
};

// Steady-phase start of a spectrum (RFI_Clipper.cpp:279-307), run by warp 0
// at the end of the previous spectrum: update rmsRunAve, push the spectrum's
// RMS estimate and derive the channel margin.
__device__ __forceinline__ void steady_start(RfiState& st, Hist& hr, const RfiConfig& cfg,
                                             const RfiBuffers& bufs, double inv_h, Bcast& bc) {
    const int H = cfg.history;
    const int lane = threadIdx.x & 31;
    st.rms_run = st.rms_run - hr.front * inv_h;
    st.rms_run = st.rms_run + hr.last * inv_h;
    const double spectrum_rms = cfg.use_mor ? fabs(st.mean_run * st.inv_mor) : st.rms_carry;
    if (lane == 0) bufs.rms_buf[st.rms_head] = spectrum_rms;  // full: overwrite the oldest
    st.rms_head = wrap_h(st.rms_head + 1, H);
    hr.prev = hr.last;
    hr.last = spectrum_rms;
    hr.front = bufs.rms_buf[st.rms_head];  // oldest entry for the spectrum after next
    if (lane == 0) {
        bc.dm_f = 0.0f;
        bc.margin_f = __fmul_rn(cfg.cr, (float)st.rms_run);
        bc.adapt = 0;
    }
}

// One CTA per beam; blockDim.x == the partial count of the canonical sums.
// Each thread owns channels tid, tid+P, ... in every pass, so per-channel data
// (the spectrum, the bandpass, the last good value) never crosses threads and
// the passes of consecutive spectra need barriers only around the block
// reductions and warp 0's scalar work.
template <int T, int C>
__device__ __forceinline__ void rfi_body(const RfiConfig& cfg, const RfiBuffers& bufs,
                                         float* __restrict__ data, int nt, const Geo& geo,
                                         unsigned char* __restrict__ flags, int rank) {
    extern __shared__ __align__(16) float sh[];
    __shared__ Bcast bc;
    constexpr int P = T * C, WPC = T / 32;
    constexpr int UR = T >= 1024 ? 1 : 4;  // channel loops unrolled where registers allow
    const int nbins = cfg.nbins, H = cfg.history;
    const int nloc = (nbins + P - 1) / P * T;  // this CTA's channels: m * P + rank * T + tid -> m * T + tid
    float* bp = sh;                                         // [nloc]
    float* specs = sh + nloc;                               // [2][nloc]
    float* red_a = sh + 3 * nloc;                           // [32][16] adaptive band sums
    float* redm = red_a + 32 * 16;                          // [32][16] adaptive band minima
    float* red_c = redm + 32 * 16;                          // [32] clip pass: good sum
    int* redi_c = reinterpret_cast<int*>(red_c + 32);       // [32][8] clip pass: good per band
    float* red_f = reinterpret_cast<float*>(redi_c + 32 * 8);  // [32][2] fill pass: sums
    int* redi_f = reinterpret_cast<int*>(red_f + 32 * 2);   // [32] fill pass: filled
    // The last good spectrum of this CTA's channels, staged in shared memory
    // when the launch gave room for it (rfi_smem_bytes): a clipped channel
    // then costs no global load in the clip pass.
    unsigned dsm;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dsm));
    float* lgood = dsm >= sizeof(float) * (4 * (size_t)nloc + kRedWords) ? sh + 3 * nloc + kRedWords : nullptr;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int tg = rank * T + tid;  // the thread's partial
    const double inv_h = 1.0 / (double)H;
    // A flat bandpass (no polynomial terms, no killed channels) has one value
    // for every channel, scale * params[0] (bp_value): the passes then use
    // that scalar instead of a per-channel array.
    const bool flat = cfg.deg == 0 && bufs.killed == nullptr;
    const float bp_scale = cfg.scale;
    // pol-0 element offset of the thread's channels: geo.off(i), which rises
    // by P * npol from one of its channels to the next when nchan divides P
    const int npol = geo.npol, nchan_g = geo.nchan;
    const bool off_step = geo.lg_nchan >= 0 && P % geo.nchan == 0;
    const long long off0 = tg < nbins ? geo.off(tg) : 0;
    const long long off_inc = (long long)P * npol;
    const long long spec_elems = (long long)geo.nsub * geo.npol * geo.nchan;

    RfiState st;   // warp 0 only (every lane the same)
    Hist hm, hr;   // mean and rms rings, warp 0 only
    if (warp == 0) {
        st = *bufs.state;
        hm.last = st.mean_size > 0 ? bufs.mean_buf[(st.mean_head + st.mean_size - 1) % H] : 0.0;
        hm.prev = st.mean_size > 1 ? bufs.mean_buf[(st.mean_head + st.mean_size - 2) % H] : 0.0;
        hm.front = bufs.mean_buf[st.mean_head];
        hr.last = st.rms_size > 0 ? bufs.rms_buf[(st.rms_head + st.rms_size - 1) % H] : 0.0;
        hr.prev = st.rms_size > 1 ? bufs.rms_buf[(st.rms_head + st.rms_size - 2) % H] : 0.0;
        hr.front = bufs.rms_buf[st.rms_head];
        if (lane == 0) bc.params0 = st.params0;
    }
    // Every CTA of a cluster reads the oldest rms entry before any CTA's
    // steady_start overwrites it.
    if constexpr (C > 1) cooperative_groups::this_cluster().sync();
    if (warp == 0 && nt > 0) {
        if (st.rms_size < H) {
            if (lane == 0) bc.adapt = 1;
        } else {
            steady_start(st, hr, cfg, bufs, inv_h, bc);
        }
    }
    __syncthreads();
    float bp_flat = __fmul_rn(bp_scale, bc.params0);  // the flat bandpass's value
    // Spectrum t's channels are copied into specs[t & 1] by cp.async, in
    // units of 4 channels (16 bytes) where a subband's channels come in
    // fours: channels i..i+3 (i a multiple of 4) are then adjacent both in
    // the spectrum and in the CTA's slots (li = m * T + k for i = m * P +
    // rank * T + k).  Any thread may copy any unit; the copies are completed
    // by their issuers and published by a barrier before the passes read them.
    const bool vec4 = (nchan_g & 3) == 0 && (reinterpret_cast<unsigned long long>(data) & 15) == 0;
    const int unit = vec4 ? 4 : 1;
    const int nunits = nloc / unit;
    auto stage = [&](int t, int first, int stride) {
        float* buf = specs + (t & 1) * nloc;
        const float* src = data + (long long)t * spec_elems;
        for (int u = first; u < nunits; u += stride) {
            const int li = u * unit, m = li / T, k = li - m * T;
            const int i = m * P + rank * T + k;  // rises with u
            if (i >= nbins) break;
            if (vec4) cp_async16(buf + li, src + geo.off(i));
            else cp_async4(buf + li, src + geo.off(i));
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    if (nt > 0) stage(0, tid, T);
    for (int i = tg, li = tid; i < nbins; i += P, li += T) {
        if (!flat) bp[li] = bp_value(cfg, bufs, bc.params0, i);
        if (lgood) lgood[li] = bufs.last_good[i];
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();

    for (int t = 0; t < nt; ++t) {
        float* spec = specs + (t & 1) * nloc;
        float* dst = data + (long long)t * spec_elems;
        // ---- adaptive phase start, RFI_Clipper.cpp:214-278 ----
        if (bc.adapt) {
            float mins[16], part[16];
#pragma unroll
            for (int b = 0; b < 8; ++b) { mins[b] = 1e6f; mins[8 + b] = 1e6f; part[b] = 0.0f; part[8 + b] = 0.0f; }
            // A thread's channels rise, so each band's are consecutive in its loop: the band's
            // statistics accumulate in registers (sums from +0, minima from 1e6, in channel
            // order) and go to their band's slot when the band ends.
            BandRun run(geo, tg);
            float s1 = 0.0f, s2 = 0.0f, m1 = 1e6f, m2 = 1e6f;
            auto flush = [&]() {
#pragma unroll
                for (int b = 0; b < 8; ++b)
                    if (b == run.band) {
                        part[b] = s1;
                        part[8 + b] = s2;
                        mins[b] = m1;
                        mins[8 + b] = m2;
                    }
                s1 = s2 = 0.0f;
                m1 = m2 = 1e6f;
            };
#pragma unroll UR
            for (int i = tg, li = tid; i < nbins; i += P, li += T) {
                if (run.ends_before(i)) {
                    flush();
                    run.advance(geo, i);
                }
                const float v = spec[li];
                m1 = fminf(m1, v);
                m2 = fminf(m2, flat ? bp_flat : bp[li]);
                s1 = __fadd_rn(s1, v);
                s2 = __fadd_rn(s2, __fmul_rn(v, v));
            }
            if (tg < nbins) flush();
#pragma unroll
            for (int k = 0; k < 16; ++k)
#pragma unroll
                for (int off = 16; off >= 1; off >>= 1) mins[k] = fminf(mins[k], __shfl_xor_sync(0xffffffffu, mins[k], off));
            warp_tree<16>(part, red_a);
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < 16; ++k) redm[warp * 16 + k] = mins[k];
            partials_barrier<C>();
            if (warp == 0) {
                float dmm[8], srms = 0.0f, pa[16], pm[16];
                lane_partials<C, WPC>(red_a, pa, 0.0f);
                lane_partials<C, WPC>(redm, pm, 1e30f);
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    const float s1 = lane_tree<C * WPC>(pa[b]);
                    const float s2 = lane_tree<C * WPC>(pa[8 + b]);
                    const float md = lane_min(pm[b]);
                    const float mm = lane_min(pm[8 + b]);
                    dmm[b] = __fsub_rn(md, mm);
                    const float a = __fdiv_rn(s2, (float)geo.cpb);
                    const float m = __fdiv_rn(s1, (float)geo.cpb);
                    const float sg = __fsqrt_rn(__fsub_rn(a, __fmul_rn(m, m)));
                    srms = (b == 0 || sg < srms) ? sg : srms;
                }
                for (int i = 1; i < 8; ++i)  // insertion sort: dmm[4] is the fifth smallest
                    for (int j = i; j > 0 && dmm[j - 1] > dmm[j]; --j) {
                        const float x = dmm[j]; dmm[j] = dmm[j - 1]; dmm[j - 1] = x;
                    }
                const int pos = wrap_h(st.rms_head + st.rms_size, H);
                if (lane == 0) bufs.rms_buf[pos] = (double)srms;
                st.rms_acc_prev = st.rms_acc;
                st.rms_acc = st.rms_acc + (double)srms;
                st.rms_size += 1;
                st.rms_run = st.rms_acc / (double)st.rms_size;
                if (st.rms_size == H) {
                    st.mean_over_rms = st.mean_run / st.rms_run;
                    st.inv_mor = 1.0 / st.mean_over_rms;
                }
                hr.prev = hr.last;
                hr.last = (double)srms;
                hr.front = bufs.rms_buf[st.rms_head];
                if (lane == 0) {
                    bc.dm_f = __fadd_rn(dmm[4], __fmul_rn(cfg.mmm_f, (float)st.rms_run));
                    bc.margin_f = __fmul_rn(cfg.cr, (float)st.rms_run);
                }
            }
            __syncthreads();
        }
        const float dm_f = bc.dm_f, margin_f = bc.margin_f;
        // ---- channel clipping (RFI_Clipper.cpp:313-342), FP32 as the reference ----
        float gpart[1] = {0.0f};
        int good[8];
#pragma unroll
        for (int b = 0; b < 8; ++b) good[b] = 0;
        {
            // good channels per band: counted for the current band, stored when it ends
            BandRun run(geo, tg);
            int g = 0;
            auto flush = [&]() {
#pragma unroll
                for (int b = 0; b < 8; ++b) good[b] += b == run.band ? g : 0;
                g = 0;
            };
            const float bpf = bp_flat;
            unsigned char* fl = flags ? flags + (long long)t * nbins : nullptr;
            long long o = off0;
#pragma unroll UR
            for (int i = tg, li = tid; i < nbins; i += P, li += T, o += off_inc) {
                if (run.ends_before(i)) {
                    flush();
                    run.advance(geo, i);
                }
                const float v = spec[li];
                const bool clip = __fsub_rn(__fsub_rn(v, dm_f), flat ? bpf : bp[li]) > margin_f;
                if (clip) {  // the channel takes its last good value, every polarisation
                    const float lg = lgood ? lgood[li] : bufs.last_good[i];
                    if (npol > 1) {
                        const long long oo = off_step ? o : geo.off(i);
                        for (int p = 1; p < npol; ++p) dst[oo + (long long)p * nchan_g] = lg;
                    }
                    spec[li] = lg;
                } else {
                    gpart[0] = __fadd_rn(gpart[0], v);
                    ++g;
                }
                if (fl) fl[i] = clip ? 1 : 0;
            }
            flush();
        }
        warp_tree<1>(gpart, red_c);
#pragma unroll
        for (int k = 0; k < 8; ++k) good[k] = __reduce_add_sync(0xffffffffu, good[k]);
        if (lane == 0)
#pragma unroll
            for (int k = 0; k < 8; ++k) redi_c[warp * 8 + k] = good[k];
        partials_barrier<C>();
        // Every thread has finished spectrum t-1, whose slots spectrum t+1
        // takes: the other warps copy it in while warp 0 runs its chain, and
        // complete their copies before the barrier ahead of the normalise pass.
        if (warp != 0 && t + 1 < nt) stage(t + 1, tid - 32, T - 32);
        // ---- warp 0: spectrum mean, history, rejection (RFI_Clipper.cpp:343-470) ----
        if (warp == 0) {
            float pc[1];
            int pi[8];
            lane_partials<C, WPC>(red_c, pc, 0.0f);
            lane_partials<C, WPC>(redi_c, pi, 0);
            const float gsum = lane_tree<C * WPC>(pc[0]);
            int gb[8], total_good = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                gb[k] = __reduce_add_sync(0xffffffffu, pi[k]);
                total_good += gb[k];
            }
            st.frac_bad_channels = __fadd_rn(st.frac_bad_channels,
                                             __fdiv_rn((float)(nbins - total_good), (float)nbins));
            const float spectrum_sum = __fdiv_rn(gsum, (float)total_good);
            int bad_bands = 0;
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                if (gb[b] < geo.band_good_min) ++bad_bands;
                if (gb[b] == 0) bad_bands += 4;
            }
            if (total_good < geo.good_min) bad_bands += 4;
            if (st.mean_size < H) {
                const int pos = wrap_h(st.mean_head + st.mean_size, H);
                if (lane == 0) bufs.mean_buf[pos] = (double)spectrum_sum;
                st.mean_acc_prev = st.mean_acc;
                st.mean_acc = st.mean_acc + (double)spectrum_sum;
                st.mean_size += 1;
                st.mean_run = st.mean_acc / (double)st.mean_size;
            } else {
                st.mean_run = st.mean_run - hm.front * inv_h;
                st.mean_run = st.mean_run + hm.last * inv_h;
                if (lane == 0) bufs.mean_buf[st.mean_head] = (double)spectrum_sum;
                st.mean_head = wrap_h(st.mean_head + 1, H);
            }
            hm.prev = hm.last;
            hm.last = (double)spectrum_sum;
            const float tol = (float)((double)__fmul_rn(cfg.sr, st.bp_rms) * cfg.inv_sqrt_nbins);
            int sclip = 0, fill = 0;
            if (st.mean_size < 1000) {
                sclip = 1;
            } else if ((double)spectrum_sum - st.mean_run > (double)tol || bad_bands >= 4) {
                sclip = 1;
                st.bad_spectra += 1;
                // pop_back + push_back(back()): the newest entry takes the previous one's value
                const int mlast = wrap_h(st.mean_head + st.mean_size - 1, H);
                const int rlast = wrap_h(st.rms_head + st.rms_size - 1, H);
                if (lane == 0) {
                    bufs.mean_buf[mlast] = hm.prev;
                    bufs.rms_buf[rlast] = hr.prev;
                }
                hm.last = hm.prev;
                hr.last = hr.prev;
                st.mean_acc = st.mean_acc_prev + hm.prev;
                st.rms_acc = st.rms_acc_prev + hr.prev;
            } else if (st.remaining_zeros != 0) {
                fill = 1;
            }
            hm.front = bufs.mean_buf[st.mean_head];  // oldest entry for the next spectrum
            if (lane == 0) {
                bc.spectrum_clip = sclip;
                bc.do_fill = fill;
            }
        }
        __syncthreads();
        const bool spectrum_clip = bc.spectrum_clip != 0;
        const bool do_fill = bc.do_fill != 0;
        // ---- last good spectrum, clipSample, flatten (RFI_Clipper.cpp:441-494) ----
        int filled = 0;
        float s12[2] = {0.0f, 0.0f};
        const float bpd = __fadd_rn(bp_flat, dm_f);  // bandpass + dataModel of a flat bandpass
        long long of = off0;
#pragma unroll UR
        for (int i = tg, li = tid; i < nbins; i += P, li += T, of += off_inc) {
            float v = spec[li];
            if (do_fill && (lgood ? lgood[li] : bufs.last_good[i]) == 0.0f && v != 0.0f) {
                bufs.last_good[i] = v;
                if (lgood) lgood[li] = v;
                ++filled;
            }
            if (spectrum_clip) {
                const long long o = off_step ? of : geo.off(i);
                for (int p = 1; p < npol; ++p) dst[o + (long long)p * nchan_g] = -0.2f;
                v = -0.2f;
                if (flags) flags[(long long)t * nbins + i] |= 2;
            }
            v = __fsub_rn(v, flat ? bpd : __fadd_rn(bp[li], dm_f));
            spec[li] = v;
            s12[0] = __fadd_rn(s12[0], v);
            s12[1] = __fadd_rn(s12[1], __fmul_rn(v, v));
        }
        warp_tree<2>(s12, red_f);
        filled = __reduce_add_sync(0xffffffffu, filled);
        if (lane == 0) redi_f[warp] = filled;
        partials_barrier<C>();
        // ---- warp 0: normalisation constants, statistics, bandpass, next start ----
        if (warp == 0) {
            float pf[2];
            int pz[1];
            lane_partials<C, WPC>(red_f, pf, 0.0f);
            lane_partials<C, WPC>(redi_f, pz, 0);
            const float s1 = lane_tree<C * WPC>(pf[0]);
            const float s2 = lane_tree<C * WPC>(pf[1]);
            st.remaining_zeros -= __reduce_add_sync(0xffffffffu, pz[0]);
            const float m = __fdiv_rn(s1, (float)nbins);
            const float ms = __fdiv_rn(s2, (float)nbins);
            float srms = __fsqrt_rn(__fsub_rn(ms, __fmul_rn(m, m)));
            if (srms == 0.0f) srms = 1.0f;
            st.rms_carry = (double)srms;
            const float sub_f = cfg.zero_dming == 1 ? m : (float)st.mean_run;
            // statistics (RFI_Clipper.cpp:535-560)
            if (st.num == 0) {
                const float frac = (float)(100.0 * (float)st.bad_spectra / (float)(10 * H));
                if (frac > 99.0f) {
                    st.mean_size = st.rms_size = 0;
                    st.mean_head = st.rms_head = 0;
                    st.mean_acc = st.mean_acc_prev = st.rms_acc = st.rms_acc_prev = 0.0;
                    hm.front = bufs.mean_buf[0];
                    hr.front = bufs.rms_buf[0];
                }
                st.bad_spectra = 0;
                st.frac_bad_channels = 0.0f;
            }
            // BandPass::setMean / setRMS (BandPass.cpp:44-74)
            const float mean_f = (float)st.mean_run;
            const float delta = __fsub_rn(mean_f, st.bp_mean);
            int rebuild = 0;
            if (fabsf(delta) > 0.0f) {
                st.params0 = __fadd_rn(st.params0, __fdiv_rn(delta, cfg.scale));
                st.bp_mean = mean_f;
                rebuild = 1;
            }
            st.bp_rms = (float)st.rms_run;
            st.num = (st.num + 1) % (10 * H);
            if (lane == 0) {
                bc.sub_f = sub_f;
                bc.rms_f = srms;
                bc.rebuild_bp = rebuild;
                bc.params0 = st.params0;
            }
            // the next spectrum's start (its margin needs only this state)
            if (t + 1 < nt) {
                if (st.rms_size < H) {
                    if (lane == 0) bc.adapt = 1;
                } else {
                    steady_start(st, hr, cfg, bufs, inv_h, bc);
                }
            }
        }
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");  // spectrum t+1 in its slots
        __syncthreads();
        // ---- normalise and store (RFI_Clipper.cpp:507-532); rebuild the bandpass ----
        const float sub_f = bc.sub_f, rms_f = bc.rms_f;
        const bool rebuild = bc.rebuild_bp != 0;
        const float p0 = bc.params0;
        const float cr = cfg.cr;
        long long on = off0;
#pragma unroll UR
        for (int i = tg, li = tid; i < nbins; i += P, li += T, on += off_inc) {
            float v = spec[li];
            if (!spectrum_clip) {
                v = __fdiv_rn(__fsub_rn(v, sub_f), rms_f);
                if (v > cr) v = 0.0f;
            }
            dst[off_step ? on : geo.off(i)] = v;
            if (rebuild && !flat) bp[li] = bp_value(cfg, bufs, p0, i);
        }
        if (rebuild && flat) bp_flat = __fmul_rn(bp_scale, p0);  // bp_value of a flat bandpass
    }
    if (tid == 0) *bufs.state = st;  // every CTA of a cluster holds the same state
    if constexpr (C > 1) cooperative_groups::this_cluster().sync();  // no CTA leaves while others read it
}

// T threads per CTA (which sets the register budget), C CTAs per beam (a
// cluster); T * C is the partial count.
template <int T, int C>
__global__ void __launch_bounds__(T, 1)
rfi_kernel(RfiConfig cfg, RfiBuffers bufs, float* __restrict__ data, int nt, Geo geo,
           unsigned char* __restrict__ flags) {
    rfi_body<T, C>(cfg, bufs, data, nt, geo, flags, C > 1 ? (int)cooperative_groups::this_cluster().block_rank() : 0);
}

// One beam's clipper in a batched launch.
struct RfiJob {
    RfiConfig cfg;
    RfiBuffers bufs;
    float* data;
    unsigned char* flags;
    Geo geo;
    int nt;
    int beam;  // index into the batch's BeamStep array
};

// The clippers of many beams at once: cluster b (CTAs b*C .. b*C+C-1) runs
// job b (every job of a launch has the same partial count); beams without a
// chunk this step return at once.
template <int T, int C>
__global__ void __launch_bounds__(T, 1) rfi_batch_kernel(const RfiJob* __restrict__ jobs,
                                                         const pv::BeamStep* __restrict__ bs) {
    const int job = blockIdx.x / C;
    if (bs && !bs[jobs[job].beam].active) return;  // the whole cluster returns
    const RfiConfig cfg = jobs[job].cfg;
    const RfiBuffers bufs = jobs[job].bufs;
    const Geo geo = jobs[job].geo;
    rfi_body<T, C>(cfg, bufs, jobs[job].data, jobs[job].nt, geo, jobs[job].flags, (int)(blockIdx.x % C));
}

// Threads per CTA and CTAs per beam for a partial count.  split 0: one CTA
// of `parts` threads; 1: beams of 1024 partials on a cluster of 4 CTAs of
// 256 threads; 2: beams of 512 or 1024 partials on clusters of 128-thread
// CTAs (4 or 8).  The partials, and so every sum, are the same.
void rfi_shape(int parts, int split, int* threads, int* ctas) {
    *threads = parts;
    *ctas = 1;
    if (split == 1 && parts == 1024) {
        *threads = 256;
        *ctas = 4;
    } else if (split == 2 && parts >= 512) {
        *threads = 128;
        *ctas = parts / 128;
    }
}

// Shared bytes of a clipper CTA: bandpass, two spectra and the reduction
// buffers, plus the last good spectrum's copy when that still fits.
size_t rfi_smem_bytes(int nbins, int parts, int threads) {
    const size_t nloc = (size_t)((nbins + parts - 1) / parts) * threads;
    const size_t staged = sizeof(float) * (4 * nloc + kRedWords);
    return staged <= 227 * 1024 ? staged : sizeof(float) * (3 * nloc + kRedWords);
}

template <typename K>
int rfi_set_smem(K kern, size_t smem) {
    size_t limit = 0;
    PV_CUDA(pv::allow_max_dynamic_smem(kern, &limit), "cudaFuncSetAttribute(rfi)");
    if (smem > limit) {
        pv::set_error("RFI_Clipper: %zu bytes of shared memory exceed one CTA's %zu", smem, limit);
        return PV_ERR_ARG;
    }
    return PV_OK;
}

template <typename K, typename... Args>
int rfi_launch_ex(K kern, int clusters, int C, int T, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3((unsigned)(clusters * C));
    lc.blockDim = dim3((unsigned)T);
    lc.dynamicSmemBytes = smem;
    lc.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    lc.attrs = at;
    lc.numAttrs = C > 1 ? 1 : 0;
    PV_CUDA(cudaLaunchKernelEx(&lc, kern, args...), "launch RFI clipper");
    return PV_OK;
}

// Sets the shared-memory attribute of both kernels of a shape and launches
// one of them: jobs != null selects the batched kernel (nblocks jobs;
// nblocks == 0: the attribute only, before any stream capture).
template <int T, int C>
int rfi_launch_t(size_t smem, int nblocks, const RfiJob* jobs, const pv::BeamStep* bs,
                 const RfiConfig& cfg, const RfiBuffers& bufs, float* data, int nt, const Geo& geo,
                 unsigned char* flags, cudaStream_t s) {
    if (jobs) {
        if (nblocks == 0) return rfi_set_smem(rfi_batch_kernel<T, C>, smem);
        PV_TRY(rfi_launch_ex(rfi_batch_kernel<T, C>, nblocks, C, T, smem, s, jobs, bs));
        return pv::check_launch("rfi_batch_kernel");
    }
    PV_TRY(rfi_set_smem(rfi_kernel<T, C>, smem));
    PV_TRY(rfi_launch_ex(rfi_kernel<T, C>, 1, C, T, smem, s, cfg, bufs, data, nt, geo, flags));
    return pv::check_launch("rfi_kernel");
}

int rfi_launch(int parts, int split, size_t smem, int nblocks, const RfiJob* jobs, const pv::BeamStep* bs,
               const RfiConfig& cfg, const RfiBuffers& bufs, float* data, int nt, const Geo& geo,
               unsigned char* flags, cudaStream_t s) {
    int T = 0, C = 0;
    rfi_shape(parts, split, &T, &C);
#define PV_RFI_SHAPE(TT, CC)                                                                          \
    if (T == TT && C == CC)                                                                          \
        return rfi_launch_t<TT, CC>(smem, nblocks, jobs, bs, cfg, bufs, data, nt, geo, flags, s);
    PV_RFI_SHAPE(256, 1)
    PV_RFI_SHAPE(512, 1)
    PV_RFI_SHAPE(1024, 1)
    PV_RFI_SHAPE(256, 4)
    PV_RFI_SHAPE(128, 4)
    PV_RFI_SHAPE(128, 8)
#undef PV_RFI_SHAPE
    pv::set_error("RFI_Clipper: no kernel for %d partial sums", parts);
    return PV_ERR_ARG;
}

}  // namespace

// ---------------------------------------------------------------------------
// Handle
// ---------------------------------------------------------------------------
struct pv_rfi {
    Bandpass bp;
    float cr = 10.0f, sr = 4.0f;
    int history = 10, zero_dming = 0, use_mor = 1, band_matching = 0, active = 1;
    int split = 1;  // rfi_shape's split of a wide beam over a cluster
    float start_freq = 0.0f, end_freq = 0.0f;
    int nbins = 0;
    RfiConfig cfg{};
    RfiBuffers dev{};
    float* d_terms = nullptr;
    unsigned char* d_killed = nullptr;
    std::vector<float> h_bp;  // bandpass after rebinning (host copy)
    std::vector<float> h_terms;          // host copy of the device terms [deg][nbins]
    std::vector<unsigned char> h_killed; // [nbins]
};

namespace {

void free_device(pv_rfi* h) {
    if (h->dev.state) cudaFree(h->dev.state);
    if (h->dev.mean_buf) cudaFree(h->dev.mean_buf);
    if (h->dev.rms_buf) cudaFree(h->dev.rms_buf);
    if (h->dev.last_good) cudaFree(h->dev.last_good);
    if (h->d_terms) cudaFree(h->d_terms);
    if (h->d_killed) cudaFree(h->d_killed);
    h->dev = RfiBuffers{};
    h->d_terms = nullptr;
    h->d_killed = nullptr;
}

// First run with this channel count: rebin the model (RFI_Clipper.cpp:184-187)
// and set up the device state.
int setup(pv_rfi* h, int nbins, cudaStream_t s) {
    if (h->nbins == nbins && h->dev.state) return PV_OK;
    if (nbins % 8 != 0 || nbins <= 0) {
        pv::set_error("RFI_Clipper: %d channels do not split into 8 equal bands", nbins);
        return PV_ERR_ARG;
    }
    free_device(h);
    Map m;
    m.n = (unsigned)nbins;
    m.lower = h->start_freq;
    m.set_width((h->end_freq - m.lower) / nbins);  // BinMap::setEnd
    h->bp.rebin(m);
    const std::vector<float>& set = h->bp.sets[m.key()];
    h->h_bp.assign(set.begin(), set.begin() + std::min<size_t>(set.size(), nbins));
    h->h_bp.resize(nbins, 0.0f);
    const int deg = (int)h->bp.params.size() - 1;
    std::vector<float> terms((size_t)std::max(deg, 0) * nbins);
    std::vector<unsigned char> killed(nbins, 0);
    bool any_killed = false;
    const float scale = (float)(h->bp.current.width / h->bp.primary.width);
    for (int i = 0; i < nbins; ++i) {
        const float v = (float)m.value(i);
        for (int k = 1; k <= deg; ++k) terms[(size_t)(k - 1) * nbins + i] = h->bp.params[k] * powi(v, k);
    }
    // channels the kill list zeroes stay zero in every rebuilt model
    {
        Bandpass probe = h->bp;
        probe.params.assign(probe.params.size(), 1.0f);
        probe.sets.clear();
        probe.build(m, 1.0f);
        const std::vector<float>& d = probe.sets[m.key()];
        for (int i = 0; i < nbins && i < (int)d.size(); ++i)
            if (d[i] == 0.0f && !h->bp.killed.empty()) { killed[i] = 1; any_killed = true; }
    }
    h->cfg.nbins = nbins;
    h->cfg.history = h->history;
    h->cfg.zero_dming = h->zero_dming;
    h->cfg.use_mor = h->use_mor;
    h->cfg.deg = std::max(deg, 0);
    h->cfg.cr = h->cr;
    h->cfg.sr = h->sr;
    h->cfg.scale = scale;
    h->cfg.mmm_f = (float)(4.0f / std::sqrt(2.0 * 4.0f));  // k/sqrt(2k), k = 4 degrees of freedom
    h->cfg.inv_sqrt_nbins = 1.0 / std::sqrt((double)nbins);
    RfiState st{};
    st.remaining_zeros = nbins;
    st.params0 = h->bp.params[0];
    st.bp_mean = Bandpass::at(h->bp.mean, m.key());
    st.bp_rms = Bandpass::at(h->bp.rms, m.key());
    PV_CUDA(cudaMalloc(&h->dev.state, sizeof(RfiState)), "allocate RFI state");
    PV_CUDA(cudaMalloc(&h->dev.mean_buf, sizeof(double) * h->history), "allocate RFI history");
    PV_CUDA(cudaMalloc(&h->dev.rms_buf, sizeof(double) * h->history), "allocate RFI history");
    PV_CUDA(cudaMalloc(&h->dev.last_good, sizeof(float) * nbins), "allocate RFI last good spectrum");
    PV_CUDA(cudaMemcpyAsync(h->dev.state, &st, sizeof(st), cudaMemcpyHostToDevice, s), "copy RFI state");
    PV_CUDA(cudaMemsetAsync(h->dev.last_good, 0, sizeof(float) * nbins, s), "clear last good spectrum");
    PV_CUDA(cudaMemsetAsync(h->dev.mean_buf, 0, sizeof(double) * h->history, s), "clear history");
    PV_CUDA(cudaMemsetAsync(h->dev.rms_buf, 0, sizeof(double) * h->history, s), "clear history");
    h->h_terms = terms;
    h->h_killed = killed;
    if (!terms.empty()) {
        PV_CUDA(cudaMalloc(&h->d_terms, sizeof(float) * terms.size()), "allocate bandpass terms");
        PV_CUDA(cudaMemcpyAsync(h->d_terms, terms.data(), sizeof(float) * terms.size(),
                                cudaMemcpyHostToDevice, s), "copy bandpass terms");
    }
    if (any_killed) {
        PV_CUDA(cudaMalloc(&h->d_killed, nbins), "allocate kill mask");
        PV_CUDA(cudaMemcpyAsync(h->d_killed, killed.data(), nbins, cudaMemcpyHostToDevice, s),
                "copy kill mask");
    }
    PV_CUDA(cudaStreamSynchronize(s), "synchronise");
    h->dev.terms = h->d_terms;
    h->dev.killed = h->d_killed;
    h->nbins = nbins;
    return PV_OK;
}

}  // namespace

extern "C" int pv_rfi_create(pv_rfi** out, const char* bp_text, float channel_rejection_rms,
                             float spectrum_rejection_rms, int history, int zero_dming,
                             int compute_rms_from_mean, int band_matching, int active) {
    if (!out) return PV_ERR_ARG;
    auto* h = new pv_rfi;
    h->active = active;
    h->cr = channel_rejection_rms;
    h->sr = spectrum_rejection_rms;
    h->history = history;
    h->zero_dming = zero_dming ? 1 : 0;
    h->use_mor = compute_rms_from_mean ? 1 : 0;
    h->band_matching = band_matching;
    if (active) {
        if (!bp_text || !*bp_text) {
            pv::set_error("RFI_Clipper: <BandPassData file=?> not defined");
            delete h;
            return PV_ERR_CONFIG;
        }
        if (history < 2) {
            pv::set_error("RFI_Clipper: History maximum must be at least 2");
            delete h;
            return PV_ERR_CONFIG;
        }
        const int rc = parse_bandpass(bp_text, h->bp);
        if (rc != PV_OK) { delete h; return rc; }
        if (band_matching) {  // RFI_Clipper.cpp:76-79
            h->start_freq = (float)h->bp.current.lower;
            h->end_freq = (float)(h->bp.current.lower + h->bp.current.width * h->bp.current.n);
        }
    }
    *out = h;
    return PV_OK;
}

extern "C" void pv_rfi_destroy(pv_rfi* h) {
    if (!h) return;
    free_device(h);
    delete h;
}

extern "C" int pv_rfi_run(pv_rfi* h, float* d_data, int nt, int nsub, int npol, int nchan,
                          unsigned char* d_flags, void* stream) {
    if (!h || nt < 0 || nsub <= 0 || npol <= 0 || nchan <= 0 || (nt > 0 && !d_data)) {
        pv::set_error("pv_rfi_run: invalid arguments");
        return PV_ERR_ARG;
    }
    if (!h->active) return PV_OK;
    cudaStream_t s = pv::as_stream(stream);
    const int nbins = nsub * nchan;
    PV_TRY(setup(h, nbins, s));
    if (nt == 0) return PV_OK;
    // A wide beam alone spreads its channels over a cluster of CTAs.
    const int parts = pv_rfi_parts(nbins);
    int T = 0, C = 0;
    rfi_shape(parts, h->split, &T, &C);
    const size_t smem = rfi_smem_bytes(nbins, parts, T);
    if (smem > 227 * 1024) {
        pv::set_error("RFI_Clipper: %d channels exceed the shared memory of %d CTAs", nbins, C);
        return PV_ERR_ARG;
    }
    const Geo geo = make_geo(nsub, npol, nchan);
    return rfi_launch(parts, h->split, smem, 1, nullptr, nullptr, h->cfg, h->dev, d_data, nt, geo, d_flags, s);
}

// Back to the state of a clipper that has seen no spectrum (the running
// averages, histories and last good spectrum of setup()), asynchronously.
int pv::rfi_reset(pv_rfi* h, cudaStream_t s) {
    if (!h || !h->dev.state) return PV_OK;
    RfiState st{};
    st.remaining_zeros = h->nbins;
    st.params0 = h->bp.params[0];
    st.bp_mean = Bandpass::at(h->bp.mean, h->bp.current.key());
    st.bp_rms = Bandpass::at(h->bp.rms, h->bp.current.key());
    // st is a stack value: copy synchronously with respect to the host
    PV_CUDA(cudaStreamSynchronize(s), "synchronise");
    PV_CUDA(cudaMemcpy(h->dev.state, &st, sizeof(st), cudaMemcpyHostToDevice), "reset RFI state");
    PV_CUDA(cudaMemsetAsync(h->dev.last_good, 0, sizeof(float) * h->nbins, s), "clear last good spectrum");
    PV_CUDA(cudaMemsetAsync(h->dev.mean_buf, 0, sizeof(double) * h->history, s), "clear history");
    PV_CUDA(cudaMemsetAsync(h->dev.rms_buf, 0, sizeof(double) * h->history, s), "clear history");
    return PV_OK;
}

long long pv::rfi_state_bytes(const pv_rfi* h, int nbins) {
    return (long long)sizeof(RfiState) + 2LL * h->history * (long long)sizeof(double) +
           (long long)nbins * (long long)sizeof(float);
}

// Copies the running state (RfiState, both history buffers and the last good
// spectrum) to or from host memory, in that order.  A clipper that has run
// no spectrum yet is set up first, so its initial state is what is saved.
int pv::rfi_state_io(pv_rfi* h, int nbins, void* h_buf, bool save, cudaStream_t s) {
    PV_TRY(setup(h, nbins, s));
    char* p = static_cast<char*>(h_buf);
    const size_t hist = sizeof(double) * (size_t)h->history;
    struct Part { void* dev; size_t bytes; };
    const Part parts[4] = {{h->dev.state, sizeof(RfiState)}, {h->dev.mean_buf, hist}, {h->dev.rms_buf, hist},
                           {h->dev.last_good, sizeof(float) * (size_t)nbins}};
    for (const Part& q : parts) {
        if (save)
            PV_CUDA(cudaMemcpyAsync(p, q.dev, q.bytes, cudaMemcpyDeviceToHost, s), "save RFI state");
        else
            PV_CUDA(cudaMemcpyAsync(q.dev, p, q.bytes, cudaMemcpyHostToDevice, s), "load RFI state");
        p += q.bytes;
    }
    return PV_OK;
}

extern "C" int pv_rfi_set_split(pv_rfi* h, int split) {
    if (!h || split < 0 || split > 2) {
        pv::set_error("pv_rfi_set_split: split must be 0, 1 or 2");
        return PV_ERR_ARG;
    }
    h->split = split;
    return PV_OK;
}

extern "C" int pv_rfi_parts(int nbins) { return nbins <= 1024 ? 256 : (nbins <= 4096 ? 512 : 1024); }

extern "C" int pv_rfi_state(pv_rfi* h, double* out10) {
    if (!h || !out10) return PV_ERR_ARG;
    if (!h->dev.state) {
        std::memset(out10, 0, sizeof(double) * 10);
        return PV_OK;
    }
    RfiState st{};
    PV_CUDA(cudaMemcpy(&st, h->dev.state, sizeof(st), cudaMemcpyDeviceToHost), "read RFI state");
    out10[0] = st.mean_run;
    out10[1] = st.rms_run;
    out10[2] = st.bp_mean;
    out10[3] = st.bp_rms;
    out10[4] = st.params0;
    out10[5] = st.num;
    out10[6] = st.bad_spectra;
    out10[7] = st.mean_size;
    out10[8] = st.rms_size;
    out10[9] = st.remaining_zeros;
    return PV_OK;
}

extern "C" int pv_rfi_bandpass_current(pv_rfi* h, float* h_out, int nbins, float* h_stats4) {
    if (!h || nbins != h->nbins || !h->dev.state) {
        pv::set_error("pv_rfi_bandpass_current: run the clipper on %d channels first", nbins);
        return PV_ERR_STATE;
    }
    RfiState st{};
    PV_CUDA(cudaMemcpy(&st, h->dev.state, sizeof(st), cudaMemcpyDeviceToHost), "read RFI state");
    const int deg = h->cfg.deg;
    if (h_out) {
        // the device's bp_value: params[0] + the k >= 1 terms in order, times the rebin scale
        for (int i = 0; i < nbins; ++i) {
            if (!h->h_killed.empty() && h->h_killed[i] && !h->bp.killed.empty()) {
                h_out[i] = 0.0f;
                continue;
            }
            float tot = st.params0;
            for (int k = 0; k < deg; ++k) tot = tot + h->h_terms[(size_t)k * nbins + i];
            h_out[i] = h->cfg.scale * tot;
        }
    }
    if (h_stats4) {
        h_stats4[0] = st.bp_mean;
        h_stats4[1] = st.bp_rms;
        h_stats4[2] = Bandpass::at(h->bp.median, h->bp.current.key());
        h_stats4[3] = st.params0;
    }
    return PV_OK;
}

extern "C" int pv_rfi_bandpass(pv_rfi* h, float* out, int nbins) {
    if (!h || !out || nbins != h->nbins) {
        pv::set_error("pv_rfi_bandpass: run the clipper on %d channels first", nbins);
        return PV_ERR_STATE;
    }
    std::copy(h->h_bp.begin(), h->h_bp.end(), out);
    return PV_OK;
}

// ---------------------------------------------------------------------------
// Batched clippers: the RFI_Clipper of every beam of a batch, one CTA per
// beam, one launch per class of beams with the same channel count (so the
// same partial-sum count and about the same time per spectrum): the SMs of a
// class are free for other work as soon as its own beams are done.  Classes
// run largest channel count first.
// ---------------------------------------------------------------------------
namespace pv {

struct RfiBatch {
    struct Class {
        int parts = 0, nbins = 0, threads = 0, ctas = 1;  // ctas: CTAs (a cluster) per beam
        size_t smem = 0;
        RfiJob* d_jobs = nullptr;
        int njobs = 0;
    };
    std::vector<Class> classes;
    const BeamStep* bs = nullptr;
    int split = 1;
};

void rfi_batch_destroy(RfiBatch* b) {
    if (!b) return;
    for (auto& c : b->classes)
        if (c.d_jobs) cudaFree(c.d_jobs);
    delete b;
}

int rfi_batch_create(RfiBatch** out, pv_rfi* const* handles, float* const* data, const int* nsub,
                     const int* nchan, int n, int nt, const BeamStep* bs, int split, cudaStream_t s) {
    auto* b = new RfiBatch;
    b->bs = bs;
    b->split = split;
    std::vector<std::vector<RfiJob>> jobs;
    for (int i = 0; i < n; ++i) {
        pv_rfi* h = handles[i];
        if (!h || !h->active) continue;
        const int nbins = nsub[i] * nchan[i];
        int rc = setup(h, nbins, s);
        const int parts = pv_rfi_parts(nbins);
        int T = 0, C = 0;
        rfi_shape(parts, split, &T, &C);
        const size_t smem = rfi_smem_bytes(nbins, parts, T);
        if (rc == PV_OK && smem > 227 * 1024) {
            set_error("RFI_Clipper: %d channels exceed the shared memory of %d CTAs", nbins, C);
            rc = PV_ERR_ARG;
        }
        if (rc != PV_OK) {
            rfi_batch_destroy(b);
            return rc;
        }
        size_t k = 0;
        while (k < b->classes.size() && b->classes[k].nbins != nbins) ++k;
        if (k == b->classes.size()) {
            b->classes.emplace_back();
            b->classes[k].parts = parts;
            b->classes[k].nbins = nbins;
            b->classes[k].threads = T;
            b->classes[k].ctas = C;
            jobs.emplace_back();
        }
        b->classes[k].smem = std::max(b->classes[k].smem, smem);
        RfiJob j{};
        j.cfg = h->cfg;
        j.bufs = h->dev;
        j.data = data[i];
        j.flags = nullptr;
        j.geo = make_geo(nsub[i], 1, nchan[i]);
        j.nt = nt;
        j.beam = i;
        jobs[k].push_back(j);
    }
    {  // largest channel count first
        std::vector<size_t> order(b->classes.size());
        for (size_t k = 0; k < order.size(); ++k) order[k] = k;
        std::stable_sort(order.begin(), order.end(),
                         [&](size_t x, size_t y) { return b->classes[x].nbins > b->classes[y].nbins; });
        std::vector<RfiBatch::Class> cs;
        std::vector<std::vector<RfiJob>> js;
        for (size_t k : order) {
            cs.push_back(b->classes[k]);
            js.push_back(std::move(jobs[k]));
        }
        b->classes.swap(cs);
        jobs.swap(js);
    }
    for (size_t k = 0; k < b->classes.size(); ++k) {
        auto& c = b->classes[k];
        c.njobs = (int)jobs[k].size();
        cudaError_t e = cudaMalloc(&c.d_jobs, sizeof(RfiJob) * jobs[k].size());
        if (e == cudaSuccess)
            e = cudaMemcpy(c.d_jobs, jobs[k].data(), sizeof(RfiJob) * jobs[k].size(),
                           cudaMemcpyHostToDevice);
        int rc = e == cudaSuccess ? PV_OK : cuda_status(e, "RFI batch jobs");
        // set the kernel attribute now, outside any stream capture
        if (rc == PV_OK)
            rc = rfi_launch(c.parts, b->split, c.smem, 0, c.d_jobs, nullptr, RfiConfig{}, RfiBuffers{}, nullptr, 0,
                            Geo{}, nullptr, s);
        if (rc != PV_OK) {
            rfi_batch_destroy(b);
            return rc;
        }
    }
    *out = b;
    return PV_OK;
}

int rfi_batch_launches(const RfiBatch* b) { return (int)b->classes.size(); }

int rfi_batch_ctas(const RfiBatch* b, int k) { return b->classes[k].njobs * b->classes[k].ctas; }

int rfi_batch_launch_one(RfiBatch* b, int k, cudaStream_t s) {
    auto& c = b->classes[k];
    if (c.njobs == 0) return PV_OK;
    return rfi_launch(c.parts, b->split, c.smem, c.njobs, c.d_jobs, b->bs, RfiConfig{}, RfiBuffers{}, nullptr, 0,
                      Geo{}, nullptr, s);
}

}  // namespace pv
