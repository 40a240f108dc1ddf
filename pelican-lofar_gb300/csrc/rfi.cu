// K2/K3: RFI_Clipper (lib/src/RFI_Clipper.cpp:22-573) with its bandpass model
// (lib/src/BandPass.cpp, BandPassAdapter.cpp:30-108, BinMap.cpp).
//
// The clipper is a sequential state machine over spectra: every spectrum's
// channel-clip margin, bandpass level and rejection test depend on running
// averages updated by the previous spectrum.  One CTA of 256 threads walks a
// beam's spectra in order; thread p owns channels p, p+256, ... of each
// spectrum.  The state (running mean/RMS, their history rings, the last good
// spectrum, the bandpass offset) lives in device memory between calls, so a
// stream of chunks gives the same result as one long chunk.
//
// Arithmetic.  This is the FP64 variant of the reference: per-spectrum
// statistics and running averages are double, channel values and the
// bandpass are float as in the reference.  Channel sums use a fixed order
// (thread p's sequential partial, a halving tree of offsets 16..1 inside each
// warp, then offsets 4, 2, 1 over the 8 warp sums) so results are
// deterministic.  Clip flags therefore match the reference's FP32 arithmetic
// except for channels or spectra within rounding distance of a threshold.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "pv_common.cuh"

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
        // (BandPassAdapter.cpp:555), so the check below rejects it unless the
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
    double mean_run, rms_run, mean_over_rms, rms_carry;
    double mean_acc, mean_acc_prev, rms_acc, rms_acc_prev;
    int mean_head, mean_size, rms_head, rms_size;
    int num, bad_spectra, remaining_zeros;
    float frac_bad_channels;
    float params0, bp_mean, bp_rms;
};

struct RfiConfig {
    int nbins, history, zero_dming, use_mor, deg;
    float cr, sr, scale;
    double mmm, sqrt_nbins;
};

struct RfiBuffers {
    RfiState* state;
    double* mean_buf;   // [history]
    double* rms_buf;    // [history]
    float* last_good;   // [nbins]
    const float* terms; // [deg][nbins]: params[k]*powi(f_i,k), k >= 1
    const unsigned char* killed;  // [nbins] or null
};

// Canonical reduction: every thread holds one FP32 partial per quantity; the
// partials are widened to double and reduced by the halving tree of offsets
// 16..1 inside each warp, then offsets NW/2..1 over the NW warp sums.
template <int K>
__device__ __forceinline__ void reduce_sum(const float (&part)[K], double (&out)[K], double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        v[k] = (double)part[k];
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) {
            const double o = __shfl_down_sync(0xffffffffu, v[k], off);
            if (lane < off) v[k] = __dadd_rn(v[k], o);
        }
    }
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) red[warp * K + k] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            double w = lane < nw ? red[lane * K + k] : 0.0;
            for (int off = nw / 2; off >= 1; off >>= 1) {
                const double o = __shfl_down_sync(0xffffffffu, w, off);
                if (lane < off) w = __dadd_rn(w, o);
            }
            if (lane == 0) red[32 * K + k] = w;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = red[32 * K + k];
    __syncthreads();
}

template <int K>
__device__ __forceinline__ void reduce_int(int (&v)[K], int* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = __reduce_add_sync(0xffffffffu, v[k]);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) red[warp * K + k] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        int s = 0;
        for (int g = 0; g < nw; ++g) s += red[g * K + k];
        v[k] = s;
    }
    __syncthreads();
}

template <int K>
__device__ __forceinline__ void reduce_min(float (&v)[K], float* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
        for (int off = 16; off >= 1; off >>= 1) v[k] = fminf(v[k], __shfl_xor_sync(0xffffffffu, v[k], off));
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) red[warp * K + k] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        float m = red[k];
        for (int g = 1; g < nw; ++g) m = fminf(m, red[g * K + k]);
        v[k] = m;
    }
    __syncthreads();
}

__device__ __forceinline__ long long elem(int t, int bin, int p, int nsub, int npol, int nchan) {
    const int s = bin / nchan, c = bin - s * nchan;
    return (((long long)t * nsub + s) * npol + p) * nchan + c;
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

// Stages spectrum t (pol 0) into buf with cp.async.
__device__ __forceinline__ void prefetch_spectrum(float* buf, const float* data, int t, int nbins,
                                                  int nsub, int npol, int nchan) {
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) cp_async4(buf + i, data + elem(t, i, 0, nsub, npol, nchan));
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// One CTA per beam; blockDim.x == the partial count of the canonical sums.
__global__ void __launch_bounds__(1024, 1)
rfi_kernel(RfiConfig cfg, RfiBuffers bufs, float* __restrict__ data, int nt, int nsub, int npol,
           int nchan, unsigned char* __restrict__ flags) {
    extern __shared__ float sh[];
    const int nbins = cfg.nbins, H = cfg.history;
    const int P = blockDim.x;
    float* bp = sh;                   // [nbins]
    float* specs = sh + nbins;        // [2][nbins] double-buffered spectra
    double* red = reinterpret_cast<double*>(sh + 3 * nbins + (nbins & 1));  // [33*16]
    int* redi = reinterpret_cast<int*>(red + 33 * 16);                       // [32*8]
    float* redf = reinterpret_cast<float*>(redi + 32 * 8);                   // [32*16]
    const int tid = threadIdx.x;
    const int cpb = nbins / 8;

    RfiState st = *bufs.state;  // every thread keeps the same copy of the scalar state
    for (int i = tid; i < nbins; i += P) bp[i] = bp_value(cfg, bufs, st.params0, i);
    if (nt > 0) prefetch_spectrum(specs, data, 0, nbins, nsub, npol, nchan);

    for (int t = 0; t < nt; ++t) {
        float* spec = specs + (t & 1) * nbins;
        if (t + 1 < nt) {
            prefetch_spectrum(specs + ((t + 1) & 1) * nbins, data, t + 1, nbins, nsub, npol, nchan);
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();
        double data_model;
        double spectrum_rms = st.rms_carry;
        if (st.rms_size < H) {
            // adaptive phase, RFI_Clipper.cpp:214-278
            float mins[16], part[16];
#pragma unroll
            for (int b = 0; b < 8; ++b) { mins[b] = 1e6f; mins[8 + b] = 1e6f; part[b] = 0.0f; part[8 + b] = 0.0f; }
            for (int i = tid; i < nbins; i += P) {
                const int band = i / cpb;
                const float v = spec[i];
#pragma unroll
                for (int b = 0; b < 8; ++b) {
                    if (b == band) {
                        mins[b] = fminf(mins[b], v);
                        mins[8 + b] = fminf(mins[8 + b], bp[i]);
                        part[b] = __fadd_rn(part[b], v);
                        part[8 + b] = __fadd_rn(part[8 + b], __fmul_rn(v, v));
                    }
                }
            }
            double sums[16];
            reduce_min<16>(mins, redf);
            reduce_sum<16>(part, sums, red);
            double sig_min = 0.0, dmm[8];
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const double a = sums[8 + b] / cpb, m = sums[b] / cpb;
                const double sg = sqrt(a - m * m);
                sig_min = (b == 0 || sg < sig_min) ? sg : sig_min;
                dmm[b] = (double)mins[b] - (double)mins[8 + b];
            }
            // the fifth smallest of the eight (std::nth_element at size/2)
#pragma unroll
            for (int i = 1; i < 8; ++i)
#pragma unroll
                for (int j = i; j > 0; --j) {
                    const double lo = fmin(dmm[j - 1], dmm[j]), hi = fmax(dmm[j - 1], dmm[j]);
                    dmm[j - 1] = lo;
                    dmm[j] = hi;
                }
            spectrum_rms = sig_min;
            data_model = dmm[4];
            const int pos = (st.rms_head + st.rms_size) % H;
            if (tid == 0) bufs.rms_buf[pos] = spectrum_rms;
            st.rms_acc_prev = st.rms_acc;
            st.rms_acc = st.rms_acc + spectrum_rms;
            st.rms_size += 1;
            st.rms_run = st.rms_acc / st.rms_size;
            if (st.rms_size == H) st.mean_over_rms = st.mean_run / st.rms_run;
            data_model = data_model + cfg.mmm * st.rms_run;
        } else {
            // steady phase, RFI_Clipper.cpp:279-307
            const double front = bufs.rms_buf[st.rms_head];
            const double back = bufs.rms_buf[(st.rms_head + st.rms_size - 1) % H];
            st.rms_run -= front / (double)st.rms_size;
            st.rms_run += back / (double)H;
            if (cfg.use_mor) spectrum_rms = fabs(st.mean_run / st.mean_over_rms);
            __syncthreads();
            if (tid == 0) bufs.rms_buf[st.rms_head] = spectrum_rms;  // full: overwrite the oldest
            st.rms_head = (st.rms_head + 1) % H;
            data_model = 0.0;
        }
        const float dm_f = (float)data_model;
        const float margin_f = (float)((double)cfg.cr * st.rms_run);
        // channel clipping, RFI_Clipper.cpp:313-342 (FP32 as the reference)
        float gpart[1] = {0.0f};
        int good[8];
#pragma unroll
        for (int b = 0; b < 8; ++b) good[b] = 0;
        for (int i = tid; i < nbins; i += P) {
            const float v = spec[i];
            const bool clip = __fsub_rn(__fsub_rn(v, dm_f), bp[i]) > margin_f;
            if (clip) {
                const float lg = bufs.last_good[i];
                for (int p = 1; p < npol; ++p) data[elem(t, i, p, nsub, npol, nchan)] = lg;
                spec[i] = lg;
            } else {
                gpart[0] = __fadd_rn(gpart[0], v);
                const int band = i / cpb;
#pragma unroll
                for (int b = 0; b < 8; ++b) good[b] += (b == band);
            }
            if (flags) flags[(long long)t * nbins + i] = clip ? 1 : 0;
        }
        double gsum[1];
        reduce_sum<1>(gpart, gsum, red);
        reduce_int<8>(good, redi);
        int total_good = 0;
#pragma unroll
        for (int b = 0; b < 8; ++b) total_good += good[b];
        st.frac_bad_channels += (float)(nbins - total_good) / (float)nbins;
        const double spectrum_sum = gsum[0] / (double)total_good;
        int bad_bands = 0;
#pragma unroll
        for (int b = 0; b < 8; ++b) {
            if ((double)good[b] < 0.8 * cpb) ++bad_bands;
            if (good[b] == 0) bad_bands += 4;
        }
        if ((double)total_good < 0.8 * nbins) bad_bands += 4;
        // mean history, RFI_Clipper.cpp:383-400
        if (st.mean_size < H) {
            const int pos = (st.mean_head + st.mean_size) % H;
            if (tid == 0) bufs.mean_buf[pos] = spectrum_sum;
            st.mean_acc_prev = st.mean_acc;
            st.mean_acc = st.mean_acc + spectrum_sum;
            st.mean_size += 1;
            st.mean_run = st.mean_acc / st.mean_size;
        } else {
            const double front = bufs.mean_buf[st.mean_head];
            const double back = bufs.mean_buf[(st.mean_head + st.mean_size - 1) % H];
            st.mean_run -= front / (double)st.mean_size;
            st.mean_run += back / (double)st.mean_size;
            __syncthreads();  // every thread has read front/back before the overwrite
            if (tid == 0) bufs.mean_buf[st.mean_head] = spectrum_sum;
            st.mean_head = (st.mean_head + 1) % H;
        }
        __syncthreads();  // history writes visible
        const double tol = (double)cfg.sr * (double)st.bp_rms / cfg.sqrt_nbins;
        bool spectrum_clip = false;
        if (st.mean_size < 1000) {
            spectrum_clip = true;
        } else if (spectrum_sum - st.mean_run > tol || bad_bands >= 4) {
            spectrum_clip = true;
            st.bad_spectra += 1;
            // pop_back + push_back(back()): the newest entry takes the previous one's value
            const int mlast = (st.mean_head + st.mean_size - 1) % H;
            const int rlast = (st.rms_head + st.rms_size - 1) % H;
            const double mprev = bufs.mean_buf[(mlast + H - 1) % H];
            const double rprev = bufs.rms_buf[(rlast + H - 1) % H];
            __syncthreads();
            if (tid == 0) { bufs.mean_buf[mlast] = mprev; bufs.rms_buf[rlast] = rprev; }
            st.mean_acc = st.mean_acc_prev + mprev;
            st.rms_acc = st.rms_acc_prev + rprev;
            __syncthreads();
        } else if (st.remaining_zeros != 0) {
            int filled[1] = {0};
            for (int i = tid; i < nbins; i += P) {
                const float v = spec[i];
                if (bufs.last_good[i] == 0.0f && v != 0.0f) {
                    bufs.last_good[i] = v;
                    filled[0] += 1;
                }
            }
            reduce_int<1>(filled, redi);
            st.remaining_zeros -= filled[0];
        }
        if (spectrum_clip) {  // clipSample, RFI_Clipper.cpp:127-150
            for (int i = tid; i < nbins; i += P) {
                for (int p = 1; p < npol; ++p) data[elem(t, i, p, nsub, npol, nchan)] = -0.2f;
                spec[i] = -0.2f;
                if (flags) flags[(long long)t * nbins + i] |= 2;
            }
        }
        // flatten and normalise, RFI_Clipper.cpp:478-532 (FP32 per channel)
        float s12[2] = {0.0f, 0.0f};
        for (int i = tid; i < nbins; i += P) {
            const float v = __fsub_rn(spec[i], __fadd_rn(bp[i], dm_f));
            spec[i] = v;
            s12[0] = __fadd_rn(s12[0], v);
            s12[1] = __fadd_rn(s12[1], __fmul_rn(v, v));
        }
        double sums2[2];
        reduce_sum<2>(s12, sums2, red);
        const double m = sums2[0] / nbins;
        double rms = sqrt(sums2[1] / nbins - m * m);
        if (rms == 0.0) rms = 1.0;
        st.rms_carry = rms;
        const float sub_f = (float)(cfg.zero_dming == 1 ? m : st.mean_run);
        const float rms_f = (float)rms;
        for (int i = tid; i < nbins; i += P) {
            float v = spec[i];
            if (!spectrum_clip) {
                v = __fdiv_rn(__fsub_rn(v, sub_f), rms_f);
                if (v > cfg.cr) v = 0.0f;
            }
            data[elem(t, i, 0, nsub, npol, nchan)] = v;
        }
        // statistics, RFI_Clipper.cpp:535-560
        if (st.num == 0) {
            const float frac = (float)(100.0 * (float)st.bad_spectra / (float)(10 * H));
            if (frac > 99.0) {
                st.mean_size = st.rms_size = 0;
                st.mean_head = st.rms_head = 0;
                st.mean_acc = st.mean_acc_prev = st.rms_acc = st.rms_acc_prev = 0.0;
            }
            st.bad_spectra = 0;
            st.frac_bad_channels = 0.0f;
        }
        // BandPass::setMean / setRMS (BandPass.cpp:44-74)
        const float mean_f = (float)st.mean_run;
        const float delta = mean_f - st.bp_mean;
        if (fabsf(delta) > 0.0f) {
            st.params0 = st.params0 + delta / cfg.scale;
            st.bp_mean = mean_f;
            for (int i = tid; i < nbins; i += P) bp[i] = bp_value(cfg, bufs, st.params0, i);
        }
        st.bp_rms = (float)st.rms_run;
        st.num = (st.num + 1) % (10 * H);
        __syncthreads();
    }
    if (tid == 0) *bufs.state = st;
}

}  // namespace

// ---------------------------------------------------------------------------
// Handle
// ---------------------------------------------------------------------------
struct pv_rfi {
    Bandpass bp;
    float cr = 10.0f, sr = 4.0f;
    int history = 10, zero_dming = 0, use_mor = 1, band_matching = 0, active = 1;
    float start_freq = 0.0f, end_freq = 0.0f;
    int nbins = 0;
    RfiConfig cfg{};
    RfiBuffers dev{};
    float* d_terms = nullptr;
    unsigned char* d_killed = nullptr;
    std::vector<float> h_bp;  // bandpass after rebinning (host copy)
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
    h->cfg.mmm = 4.0 / std::sqrt(8.0);  // k/sqrt(2k) with k = 4 degrees of freedom
    h->cfg.sqrt_nbins = std::sqrt((double)nbins);
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
    const int threads = pv_rfi_parts(nbins);
    const size_t smem = sizeof(float) * (3 * (size_t)nbins + 2) + sizeof(double) * 33 * 16 +
                        sizeof(int) * 32 * 8 + sizeof(float) * 32 * 16;
    if (smem > 227 * 1024) {
        pv::set_error("RFI_Clipper: %d channels exceed one CTA's shared memory", nbins);
        return PV_ERR_ARG;
    }
    PV_CUDA(cudaFuncSetAttribute(rfi_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
            "cudaFuncSetAttribute(rfi)");
    rfi_kernel<<<1, threads, smem, s>>>(h->cfg, h->dev, d_data, nt, nsub, npol, nchan, d_flags);
    return pv::check_launch("rfi_kernel");
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

extern "C" int pv_rfi_bandpass(pv_rfi* h, float* out, int nbins) {
    if (!h || !out || nbins != h->nbins) {
        pv::set_error("pv_rfi_bandpass: run the clipper on %d channels first", nbins);
        return PV_ERR_STATE;
    }
    std::copy(h->h_bp.begin(), h->h_bp.end(), out);
    return PV_OK;
}
