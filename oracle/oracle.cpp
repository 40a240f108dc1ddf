// CPU oracle for the pelican-lofar beam-processing hot path.
//
// TEST INFRASTRUCTURE ONLY: this is the checker.  Only the test-suite, the
// smoke check and the benchmark's CPU-baseline leg load it; the product
// library never does.
//
// Each section restates one reference function from its observable
// behaviour; citations are relative to the reference's src/ directory.
// Arithmetic follows the reference's types and evaluation order: the
// reference builds as C++98 (PPFChanneliser.cpp:285 assigns through
// std::complex::real(), which only C++98 allows), so std::pow(float,int)
// returns float, unqualified sqrt() is ::sqrt(double), and x86-64 SSE has
// no fused multiply-add.  Build with -ffp-contract=off.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <numeric>
#include <string>
#include <tuple>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kDispersion = 4148.741601;  // DedispersionModule.cpp:154

int threads_or_default(int n) {
#ifdef _OPENMP
    return n > 0 ? n : omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// libgcc's __powisf2 (binary exponentiation in float): what C++98
// std::pow(float, int) lowers to.
float powi_f(float a, int b) {
    const bool recip = b < 0;
    if (recip) b = -b;
    float r = 1.0f;
    for (;;) {
        if (b & 1) r *= a;
        b /= 2;
        if (b == 0) break;
        a *= a;
    }
    return recip ? 1.0f / r : r;
}

}  // namespace

// ===========================================================================
// A7 delay table
// ===========================================================================
extern "C" int or_dm_shifts(double fch1, double foff, int nchan, float* dmshift) {
    // DedispersionModule.cpp:153-157.  Inverted bands are re-expressed with
    // the highest frequency first so that all delays are non-negative.
    int inverted = foff >= 0 ? 1 : 0;
    if (inverted) {
        fch1 = fch1 + foff * (nchan - 1);
        foff = -foff;
    }
    for (int c = 0; c < nchan; ++c) {
        double f = fch1 + (foff * c);
        dmshift[c] = (float)(kDispersion * ((1.0 / f / f) - (1.0 / fch1 / fch1)));
    }
    return inverted;
}

extern "C" void or_maxshift(float dm_low, float dm_step, int tdms, const float* dmshift,
                            int nchan, double tsamp, int buffer_samples, int* maxshift,
                            int* remaining) {
    // DedispersionModule.cpp:159 (non-inverted branch), :162.
    float dm_max = dm_low + dm_step * (float)(unsigned)(tdms - 1);
    float prod = dm_max * dmshift[nchan - 1];
    int ms = (int)((double)prod / tsamp);
    *maxshift = ms;
    *remaining = (int)(((unsigned)buffer_samples - (unsigned)ms) % (14u * 16u));
}

static inline int shift_f32(float dmshift, int d, float start, float step) {
    // DedispersionKernel.cu:29 (mstartdm + d*mdmstep, contracted to one FMA
    // by nvcc's default -fmad) and :36 (__float2int_rz of the product).
    float dmv = std::fmaf((float)d, step, start);
    float p = dmshift * dmv;
    return (int)p;
}

extern "C" void or_shift_table(const float* dmshift, int nchan, int tdms, float start,
                               float step, int* shifts) {
    for (int d = 0; d < tdms; ++d)
        for (int c = 0; c < nchan; ++c)
            shifts[(long long)d * nchan + c] = shift_f32(dmshift[c], d, start, step);
}

extern "C" void or_shift_table_f64(double fch1, double foff, int nchan, int tdms,
                                   double dm_low, double dm_step, double tsamp,
                                   int* shifts) {
    if (foff >= 0) {
        fch1 = fch1 + foff * (nchan - 1);
        foff = -foff;
    }
    for (int c = 0; c < nchan; ++c) {
        double f = fch1 + foff * c;
        double k = kDispersion * ((1.0 / f / f) - (1.0 / fch1 / fch1));
        for (int d = 0; d < tdms; ++d)
            shifts[(long long)d * nchan + c] = (int)(k * (dm_low + d * dm_step) / tsamp);
    }
}

// ===========================================================================
// A9 dedispersion
// ===========================================================================
extern "C" void or_dedisperse(const float* buf, int nchan, long long ld, int nout, int tdms,
                              const float* dmshift, float start, float step, float* out,
                              int nthreads) {
    int nt = threads_or_default(nthreads);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int d = 0; d < tdms; ++d) {
        float* row = out + (long long)d * nout;
        for (int t = 0; t < nout; ++t) row[t] = 0.0f;
        // Per output the sum runs over channels in order 0..nchan-1, exactly
        // the accumulation order of DedispersionKernel.cu:32-43.
        for (int c = 0; c < nchan; ++c) {
            const float* src = buf + (long long)c * ld + shift_f32(dmshift[c], d, start, step);
            for (int t = 0; t < nout; ++t) row[t] += src[t];
        }
    }
}

extern "C" void or_dedisperse_f64(const float* buf, int nchan, long long ld, int nout,
                                  int tdms, const float* dmshift, float start, float step,
                                  double* out, int nthreads) {
    int nt = threads_or_default(nthreads);
#pragma omp parallel for schedule(dynamic, 1) num_threads(nt)
    for (int d = 0; d < tdms; ++d) {
        double* row = out + (long long)d * nout;
        for (int t = 0; t < nout; ++t) row[t] = 0.0;
        for (int c = 0; c < nchan; ++c) {
            const float* src = buf + (long long)c * ld + shift_f32(dmshift[c], d, start, step);
            for (int t = 0; t < nout; ++t) row[t] += (double)src[t];
        }
    }
}

// ===========================================================================
// A11 analyser
// ===========================================================================
extern "C" void or_thresholds(float thr, float rms, int bin_pow2, float* out) {
    // DedispersionAnalyser.cpp:112 (level 0, float) and :121 (levels >= 1:
    // float product times ::sqrt(double), rounded on assignment).
    float base = thr * rms;
    out[0] = base;
    for (int n = 1; n <= bin_pow2; ++n) {
        unsigned bin_factor = 1u << n;
        out[n] = (float)((double)base * ::sqrt((double)(float)bin_factor));
    }
}

extern "C" long long or_analyse(const float* data, int tdms, int nsamp, float thr, float rms,
                                int bin_pow2, or_event* events, long long cap) {
    long long n_ev = 0;
    auto add = [&](int dm, int t, float bf, float v) {
        if (n_ev < cap) events[n_ev] = or_event{dm, t, bf, v};
        ++n_ev;
    };
    add(0, 0, 1.0f, 0.0f);  // DedispersionAnalyser.cpp:69
    std::vector<float> thr_n(bin_pow2 + 1);
    or_thresholds(thr, rms, bin_pow2, thr_n.data());
    const unsigned max_pow2 = 1u << bin_pow2;
    const int nblocks = (int)((unsigned)nsamp / max_pow2);  // tail dropped
    std::vector<std::vector<float>> binned(bin_pow2 + 1, std::vector<float>(max_pow2));
    for (int dm = 0; dm < tdms; ++dm) {
        const float* row = data + (long long)dm * nsamp;
        for (int i = 0; i < nblocks; ++i) {
            unsigned cur = max_pow2;
            for (unsigned j = 0; j < max_pow2; ++j) {
                int index = i * (int)max_pow2 + (int)j;
                binned[0][j] = row[index];
                if (binned[0][j] >= thr_n[0]) add(dm, index, 1.0f, binned[0][j]);
            }
            for (int n = 1; n <= bin_pow2; ++n) {
                cur /= 2;
                for (unsigned j = 0; j < cur; ++j) {
                    unsigned bin_factor = max_pow2 / cur;
                    int index = i * (int)max_pow2 + (int)(bin_factor * j);
                    binned[n][j] = binned[n - 1][2 * j] + binned[n - 1][2 * j + 1];
                    if (binned[n][j] >= thr_n[n]) add(dm, index, (float)bin_factor, binned[n][j]);
                }
            }
        }
    }
    return n_ev;
}

// ===========================================================================
// A2 polyphase coefficients
// ===========================================================================
namespace {

double bessel_i0(double x) {  // PolyphaseCoefficients.cpp:77-103
    const double p1 = 1.0, p2 = 3.5156229, p3 = 3.0899424, p4 = 1.2067492, p5 = 0.2659732,
                 p6 = 3.60768e-2, p7 = 4.5813e-3;
    const double q1 = 0.39894228, q2 = 1.328592e-2, q3 = 2.25319e-3, q4 = -1.57565e-3,
                 q5 = 9.16281e-3, q6 = -2.057706e-2, q7 = 2.635537e-2, q8 = -1.647633e-2,
                 q9 = 3.92377e-3;
    const double k1 = 3.75;
    double ax = std::fabs(x);
    if (ax < k1) {
        double xx = x / k1;
        double y = xx * xx;
        return p1 + y * (p2 + y * (p3 + y * (p4 + y * (p5 + y * (p6 + y * p7)))));
    }
    double y = k1 / ax;
    return (std::exp(ax) / std::sqrt(ax)) *
           (q1 + y * (q2 + y * (q3 + y * (q4 + y * (q5 + y * (q6 + y * (q7 + y * (q8 + y * q9))))))));
}

void window_fn(int n, int type, double* d) {
    switch (type) {
        case 0: {  // Hamming, :139-149
            if (n == 1) { d[0] = 1.0; return; }
            unsigned m = (unsigned)n - 1;
            for (unsigned i = 0; i < (unsigned)n; ++i)
                d[i] = 0.54 - 0.46 * std::cos((2.0 * M_PI * i) / m);
            return;
        }
        case 1: {  // Blackman with the integer division i/m kept, :152-163
            if (n == 1) { d[0] = 1.0; return; }
            unsigned m = (unsigned)n - 1;
            for (unsigned i = 0; i < (unsigned)n; ++i) {
                double k = i / m;
                d[i] = 0.42 - 0.5 * std::cos(2.0 * M_PI * k) + 0.08 * std::cos(4.0 * M_PI * k);
            }
            return;
        }
        case 2: {  // Gaussian alpha = 3.5, :130-136
            double a = 3.5;
            int index = 0;
            for (int i = -(n - 1); i <= n - 1; i += 2) {
                double x = a / n * i;
                d[index++] = std::exp(-0.5 * (x * x));
            }
            return;
        }
        default: {  // Kaiser beta = 9.0695, :114-127
            double beta = 9.0695;
            if (n == 1) { d[0] = 1.0; return; }
            int m = n - 1;
            for (int i = 0; i < n; ++i) {
                double k = 2.0 * beta / m * std::sqrt(double(i * (m - i)));
                d[i] = bessel_i0(k) / bessel_i0(beta);
            }
        }
    }
}

// In-place complex FFT in double; sign -1 forward, +1 backward.  Power of two
// lengths use an iterative radix-2; other lengths a direct DFT.
void fft_f64(std::vector<double>& re, std::vector<double>& im, int sign) {
    const size_t n = re.size();
    if ((n & (n - 1)) == 0) {
        for (size_t i = 1, j = 0; i < n; ++i) {
            size_t bit = n >> 1;
            for (; j & bit; bit >>= 1) j ^= bit;
            j ^= bit;
            if (i < j) { std::swap(re[i], re[j]); std::swap(im[i], im[j]); }
        }
        for (size_t len = 2; len <= n; len <<= 1) {
            for (size_t i = 0; i < n; i += len) {
                for (size_t k = 0; k < len / 2; ++k) {
                    double ang = sign * 2.0 * M_PI * (double)k / (double)len;
                    double wr = std::cos(ang), wi = std::sin(ang);
                    size_t a = i + k, b = i + k + len / 2;
                    double xr = re[b] * wr - im[b] * wi;
                    double xi = re[b] * wi + im[b] * wr;
                    re[b] = re[a] - xr; im[b] = im[a] - xi;
                    re[a] += xr; im[a] += xi;
                }
            }
        }
        return;
    }
    std::vector<double> r2(n), i2(n);
    for (size_t k = 0; k < n; ++k) {
        double sr = 0, si = 0;
        for (size_t j = 0; j < n; ++j) {
            double ang = sign * 2.0 * M_PI * (double)((j * k) % n) / (double)n;
            sr += re[j] * std::cos(ang) - im[j] * std::sin(ang);
            si += re[j] * std::sin(ang) + im[j] * std::cos(ang);
        }
        r2[k] = sr; i2[k] = si;
    }
    re = r2; im = i2;
}

unsigned next_pow2(unsigned n) {
    unsigned r = 1;
    while (r < n) r *= 2;
    return r;
}

void interpolate(const double* x, const double* y, unsigned nx, unsigned n, double* result) {
    unsigned next = 0, index = 0;
    for (double ix = 0.0; ix <= 1.0; ix += 1.0 / (n - 1), index++) {
        while (x[next] <= ix && next < nx - 1) next++;
        if (next == 0) return;
        double rc = (y[next] - y[next - 1]) / (x[next] - x[next - 1]);
        result[index] = y[next - 1] + (ix - x[next - 1]) * rc;
    }
}

void fir_filter(unsigned n, double w, const double* window, double* result) {
    // PolyphaseCoefficients.cpp:216-304 (fir2 with ramp_n/grid_n == 0).
    unsigned grid_n = next_pow2(n + 1);
    unsigned ramp_n = 2;
    double f[] = {0.0, w - ramp_n / grid_n / 2.0, w, w + ramp_n / grid_n / 2.0, 1.0};
    double m[] = {1.0, 1.0, 0.0, 0.0, 0.0};
    std::vector<double> grid(grid_n + 1, 0.0);
    interpolate(f, m, 5, grid_n + 1, grid.data());
    const unsigned L = grid_n * 4;
    // The reference stores the IFFT input and output in float (fftwf).
    std::vector<double> re(L, 0.0), im(L, 0.0);
    for (unsigned i = 0; i < grid_n + 1; ++i) re[i] = (float)grid[i];
    for (unsigned i = grid_n - 1, index = 0; i >= 1; i--, index++)
        re[grid_n * 3 + 1 + index] = (float)grid[i];
    fft_f64(re, im, +1);
    unsigned index = 0;
    for (unsigned i = 4 * grid_n - n; i < 4 * grid_n; i += 2) result[index++] = (float)re[i];
    for (unsigned i = 1; i <= n; i += 2) result[index++] = (float)re[i];
    for (unsigned i = 0; i <= n; ++i) result[i] *= window[i];
    double factor = result[n / 2];
    for (unsigned i = 0; i <= n; ++i) result[i] /= factor;
}

}  // namespace

extern "C" int or_fir_coefficients(int ntaps, int nchan, int window, double* coeffs) {
    // PolyphaseCoefficients.cpp:308-364
    unsigned n = (unsigned)nchan * (unsigned)ntaps;
    if (n < 2) return -1;
    std::vector<double> win(n), result(n);
    window_fn((int)n, window, win.data());
    fir_filter(n - 1, 1.0 / nchan, win.data(), result.data());
    for (int t = 0; t < ntaps; ++t)
        for (int c = 0; c < nchan; ++c) {
            unsigned idx = t * nchan + c;
            coeffs[idx] = (c % 2 == 0) ? result[idx] / nchan : -result[idx] / nchan;
        }
    return 0;
}

// ===========================================================================
// A3 PPF channeliser
// ===========================================================================
struct or_ppf {
    int nchan, ntaps;
    std::vector<float> coeffs;
    int nsub = -1, npol = -1;
    std::vector<std::vector<float>> work;  // per (s,p): ntaps*nchan complex
    std::vector<int> oldest;               // per (s,p) ring position
};

extern "C" or_ppf* or_ppf_create(int nchan, int ntaps, const float* coeffs) {
    or_ppf* p = new or_ppf;
    p->nchan = nchan;
    p->ntaps = ntaps;
    p->coeffs.assign(coeffs, coeffs + (size_t)nchan * ntaps);
    return p;
}
extern "C" void or_ppf_destroy(or_ppf* p) { delete p; }

extern "C" int or_ppf_run(or_ppf* p, const float* in, int nsub, int npol, int nblocks,
                          float* out) {
    // PPFChanneliser.cpp:81-187, _updateBuffer :247-254, _filter :266-290.
    const int N = p->nchan, T = p->ntaps;
    if (nsub <= 0 || npol <= 0 || nblocks <= 0) return -1;
    if (N == 1) {  // :108-131
        for (int s = 0; s < nsub; ++s)
            for (int q = 0; q < npol; ++q)
                for (int b = 0; b < nblocks; ++b) {
                    const float* src = in + 2 * ((long long)nblocks * (s * npol + q) + b);
                    float* dst = out + 2 * ((long long)npol * (nsub * b + s) + q);
                    dst[0] = src[0]; dst[1] = src[1];
                }
        return 0;
    }
    if (p->nsub != nsub || p->npol != npol) {
        p->nsub = nsub; p->npol = npol;
        p->work.assign((size_t)nsub * npol, std::vector<float>((size_t)2 * N * T, 0.0f));
        p->oldest.assign((size_t)nsub * npol, 0);
    }
    // Subband/polarisation streams are independent (PPFChanneliser.cpp:139-183
    // splits subbands over OpenMP threads).
#pragma omp parallel for schedule(dynamic, 1)
    for (int sq = 0; sq < nsub * npol; ++sq) {
        const int s = sq / npol, q = sq % npol;
        std::vector<float> y(2 * N);
        std::vector<double> re(N), im(N);
            std::vector<float>& wb = p->work[s * npol + q];
            int& old = p->oldest[s * npol + q];
            for (int b = 0; b < nblocks; ++b) {
                const float* src = in + 2 * (long long)N * ((long long)nblocks * (s * npol + q) + b);
                std::memcpy(&wb[2 * (size_t)old * N], src, sizeof(float) * 2 * N);
                old = (old + 1) % T;
                std::fill(y.begin(), y.end(), 0.0f);
                for (int i = 0, t = 0; t < T; ++t) {
                    int ib = ((old + t) % T) * N;
                    for (int c = 0; c < N; ++c, ++i) {
                        float coeff = p->coeffs[i];
                        float r = wb[2 * (ib + c)] * coeff;
                        float m = wb[2 * (ib + c) + 1] * coeff;
                        y[2 * c] += r;
                        y[2 * c + 1] += m;
                    }
                }
                for (int c = 0; c < N; ++c) { re[c] = y[2 * c]; im[c] = y[2 * c + 1]; }
                fft_f64(re, im, -1);  // FFTW_FORWARD, unnormalised
                float* dst = out + 2 * (long long)N * ((long long)npol * ((long long)nsub * b + s) + q);
                for (int c = 0; c < N; ++c) { dst[2 * c] = (float)re[c]; dst[2 * c + 1] = (float)im[c]; }
            }
        }
    return 0;
}

// ===========================================================================
// A4 Stokes, A5 integrator
// ===========================================================================
extern "C" void or_stokes(const float* spectra, int nt, int nsub, int nchan, int nstokes,
                          float* stokes) {
    // StokesGenerator.cpp:40-108
    for (int t = 0; t < nt; ++t)
        for (int s = 0; s < nsub; ++s) {
            const float* X = spectra + 2 * (long long)nchan * (2 * ((long long)nsub * t + s) + 0);
            const float* Y = spectra + 2 * (long long)nchan * (2 * ((long long)nsub * t + s) + 1);
            float* base = stokes + (long long)nchan * (nstokes * ((long long)nsub * t + s));
            for (int c = 0; c < nchan; ++c) {
                float Xr = X[2 * c], Xi = X[2 * c + 1], Yr = Y[2 * c], Yi = Y[2 * c + 1];
                float xyr = Xr * Yr + Xi * Yi;
                float xyi = Xi * Yr - Xr * Yi;
                float px = Xr * Xr + Xi * Xi;
                float py = Yr * Yr + Yi * Yi;
                base[c] = px + py;
                if (nstokes == 4) {
                    base[nchan + c] = px - py;
                    base[2 * nchan + c] = 2.0f * xyr;
                    base[3 * nchan + c] = 2.0f * xyi;
                }
            }
        }
}

extern "C" int or_integrate(const float* in, int nt, int nsub, int npol, int nchan, int window,
                            int bin_chans, float* out) {
    // StokesIntegrator.cpp:32-119
    if (window > nt) window = nt;
    if (window <= 0 || bin_chans <= 0) return 0;
    int nu = nt / window, nc_out = nchan / bin_chans;
    std::fill(out, out + (long long)nu * nsub * npol * nc_out, 0.0f);
    for (int u = 0; u < nu; ++u)
        for (int t = u * window; t < (u + 1) * window; ++t)
            for (int s = 0; s < nsub; ++s)
                for (int q = 0; q < npol; ++q) {
                    const float* v = in + (long long)nchan * (npol * ((long long)nsub * t + s) + q);
                    float* o = out + (long long)nc_out * (npol * ((long long)nsub * u + s) + q);
                    int c0 = 0;
                    for (int nc = 0; nc < nc_out; ++nc) {
                        for (int c = c0; c < c0 + bin_chans; ++c) o[nc] += v[c];
                        c0 += bin_chans;
                    }
                }
    return nu;
}

// ===========================================================================
// A6 BinMap / BandPass (BinMap.cpp, BandPass.cpp, Range.h)
// ===========================================================================
namespace {

struct BinMapR {
    unsigned n = 0;
    double lower = 0.0, width = 1.0, half = 0.0;
    int bin_index(double v) const { return (int)(0.5 + ((v - lower) / width)); }
    double assign(int i) const { return lower + (width * i); }
    std::tuple<unsigned, double, double> key() const { return std::make_tuple(n, lower, width); }
    void set_width(double w) { width = w; half = w / 2.0; }
};

struct BandPassR {
    BinMapR primary, current;
    std::vector<float> params{0.0f};
    std::map<std::tuple<unsigned, double, double>, std::vector<float>> data;
    std::map<std::tuple<unsigned, double, double>, float> rms_, median_, mean_;
    std::vector<std::pair<float, float>> killed;

    float get(const std::map<std::tuple<unsigned, double, double>, float>& m,
              const std::tuple<unsigned, double, double>& k) const {
        auto it = m.find(k);
        return it == m.end() ? 0.0f : it->second;
    }
    float evaluate(float v) const {  // BandPass.cpp:159-166
        float tot = 0.0f;
        for (size_t i = 0; i < params.size(); ++i) tot += params[i] * powi_f(v, (int)i);
        return tot;
    }
    void zero_killed(const BinMapR& map) {  // :111-123
        std::vector<float>& d = data[map.key()];
        for (auto& r : killed) {
            int lo = map.bin_index(r.first), hi = map.bin_index(r.second);
            if (hi < lo) std::swap(lo, hi);
            if (lo < 0) lo = 0;
            if ((int)d.size() < hi) d.resize(hi + 1);
            do { if (lo < (int)d.size()) d[lo] = 0.0f; } while (++lo <= hi);
        }
    }
    void build(const BinMapR& map, float scale) {  // :101-108
        std::vector<float>& d = data[map.key()];
        d.assign(map.n, 0.0f);
        for (unsigned i = 0; i < map.n; ++i) d[i] = scale * evaluate((float)map.assign(i));
        zero_killed(map);
    }
    void rebin(const BinMapR& map) {  // :81-99
        current = map;
        if (!data.count(map.key())) {
            double scale = map.width / primary.width;
            rms_[map.key()] = (float)(get(rms_, primary.key()) * std::sqrt(1.0 / scale));
            median_[map.key()] = (float)(get(median_, primary.key()) * scale);
            mean_[map.key()] = (float)(get(mean_, primary.key()) * scale);
            build(current, (float)scale);
        }
    }
    void set_data(const BinMapR& map, const std::vector<float>& p) {  // :26-42
        primary = map;
        params = p;
        rebin(map);
        const std::vector<float>& d = data[primary.key()];
        float m = 0.0f;
        std::vector<float> copy;
        for (unsigned i = 0; i < map.n; ++i) { m += d[i]; copy.push_back(d[i]); }
        m /= map.n;
        mean_[primary.key()] = m;
        std::nth_element(copy.begin(), copy.begin() + copy.size() / 2, copy.end());
        median_[primary.key()] = *(copy.begin() + copy.size() / 2);
    }
    void set_rms(float r) { rms_[current.key()] = r; }
    void set_median(float median) {  // :48-61
        float delta = median - median_[current.key()];
        if (std::fabs(delta) > 0.0f) {
            float scale = (float)(current.width / primary.width);
            median_[current.key()] = median;
            median_[primary.key()] = median / scale;
            params[0] += delta / scale;
            mean_[current.key()] += delta;
            mean_[primary.key()] += delta / scale;
            data.clear();
            build(current, scale);
        }
    }
    void set_mean(float mean) {  // :63-74
        float delta = mean - mean_[current.key()];
        if (std::fabs(delta) > 0.0f) {
            float scale = (float)(current.width / primary.width);
            params[0] += delta / scale;
            mean_[current.key()] = mean;
            mean_[primary.key()] = mean / scale;
            data.clear();
            build(current, scale);
        }
    }
    void kill_band(float a, float b) {  // :151-157 with Range<float> min/max ordering
        if (b < a) std::swap(a, b);
        killed.push_back({a, b});
        std::vector<BinMapR> maps;
        for (auto& kv : data) {
            BinMapR m;
            m.n = std::get<0>(kv.first); m.lower = std::get<1>(kv.first); m.set_width(std::get<2>(kv.first));
            maps.push_back(m);
        }
        for (auto& m : maps) zero_killed(m);
    }
    const std::vector<float>& current_set() { return data[current.key()]; }
    float rms() const { return get(rms_, current.key()); }
    float median() const { return get(median_, current.key()); }
    float mean() const { return get(mean_, current.key()); }
};

// BandPassAdapter.cpp:30-108.  Returns false with a message on error.
bool parse_bp(const char* text, BandPassR& bp, std::string& err) {
    std::vector<float> params;
    std::vector<std::pair<unsigned, double>> kills;
    int count = 0, line = 0;
    const char* p = text;
    while (*p) {
        ++line;
        const char* eol = std::strchr(p, '\n');
        std::string ln = eol ? std::string(p, eol) : std::string(p);
        p = eol ? eol + 1 : p + ln.size();
        if (ln[0] == '#') continue;
        auto trim = [](std::string s) {
            size_t a = s.find_first_not_of(" \t\r\v\f"), b = s.find_last_not_of(" \t\r\v\f");
            return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
        };
        if (ln[0] == 'K') {
            std::string rest = trim(ln.substr(1));
            unsigned idx; double fq;
            if (std::sscanf(rest.c_str(), "%u %lf", &idx, &fq) < 2) {
                err = "BandPassAdapter: syntax error on line " + std::to_string(line) +
                      ": expecting two numbers on Kill line: index frequency";
                return false;
            }
            kills.push_back({idx, (double)idx});  // the reference reads nums[0] twice
            continue;
        }
        ++count;
        std::string s = trim(ln);
        char* end = nullptr;
        double v = s.empty() ? 0.0 : std::strtod(s.c_str(), &end);
        if (s.empty() || end == nullptr || *end != '\0') {
            err = "BandPassAdapter: syntax error on line " + std::to_string(line);
            return false;
        }
        params.push_back((float)v);
    }
    if (count < 6) {
        err = "BandPassAdapter: data format wrong : got " + std::to_string(count) +
              " parameters, expecting at least 6";
        return false;
    }
    unsigned nchan = (unsigned)params[0];
    float start = params[1], delta = params[3], rms = params[4], median = params[5];
    params.erase(params.begin(), params.begin() + 5);
    BinMapR map;
    map.n = nchan;
    map.lower = start;
    map.set_width(delta);
    bp.set_data(map, params);
    bp.set_median(median);
    bp.set_rms(rms);
    for (auto& k : kills) {
        if (map.bin_index(k.second) != (int)k.first) {
            err = "BandPassAdapter:  Frequency kill mismatch: index " + std::to_string(k.first) +
                  " does not match frequency " + std::to_string(k.second);
            return false;
        }
        bp.kill_band((float)(map.assign(k.first) - map.half), (float)(map.assign(k.first) + map.half));
    }
    return true;
}

// boost::circular_buffer semantics used by RFI_Clipper.h:627.
template <typename T>
struct CircBuf {
    std::deque<T> q;
    size_t cap = 0;
    bool full() const { return q.size() == cap; }
    void push_back(T v) {
        if (cap == 0) return;
        if (q.size() == cap) q.pop_front();
        q.push_back(v);
    }
    void pop_back() { if (!q.empty()) q.pop_back(); }
    T front() const { return q.empty() ? T(0) : q.front(); }
    T back() const { return q.empty() ? T(0) : q.back(); }
    size_t size() const { return q.size(); }
    double accumulate() const {  // std::accumulate(begin, end, 0.0)
        double s = 0.0;
        for (auto v : q) s += v;
        return s;
    }
};

}  // namespace

// Canonical FP32 reduction of the RFI variant over P partials (P a multiple
// of 32): each group of 32 consecutive partials is reduced by the halving
// tree of offsets 16, 8, 4, 2, 1, then the P/32 group sums by offsets
// P/64, ..., 1.
static float tree_p(float* part, int P) {
    const int nw = P / 32;
    float w[32];
    for (int g = 0; g < nw; ++g) {
        float* q = part + 32 * g;
        for (int off = 16; off >= 1; off >>= 1)
            for (int l = 0; l < off; ++l) q[l] = q[l] + q[l + off];
        w[g] = q[0];
    }
    for (int off = nw / 2; off >= 1; off >>= 1)
        for (int l = 0; l < off; ++l) w[l] = w[l] + w[l + off];
    return w[0];
}

// Sum of n floats: partial p is the FP32 sum of x[p], x[p+P], ... in order
// (from +0), reduced by tree_p.
extern "C" double or_sum_canonical(const float* x, int n, int P) {
    float part[1024];
    for (int p = 0; p < P; ++p) {
        float s = 0.0f;
        for (int i = p; i < n; i += P) s += x[i];
        part[p] = s;
    }
    return tree_p(part, P);
}

// ===========================================================================
// A6 RFI_Clipper::run (RFI_Clipper.cpp:154-573)
// ===========================================================================
namespace {

struct RfiBase {
    virtual ~RfiBase() {}
    virtual int run(float* I, float* W, int nt, int nsub, int npol, int nchan, uint8_t* flags) = 0;
    virtual void state(double* out) const = 0;
    BandPassR bp;
    BinMapR map;
    float start_freq = 0.0f, end_freq = 0.0f;
};

// The reference's arithmetic (mode 0) and the library's variant (mode 1).
// Mode 1 keeps every per-channel and per-spectrum expression in the
// reference's FP32 form, replaces the sequential channel sums by `parts`
// FP32 partials reduced by tree_p, and keeps the running averages and their
// history buffers in FP64, updated with multiplications by 1/H and by the
// reciprocal of meanOverRMS.
struct Rfi : RfiBase {
    bool f64;
    int parts = 256;
    float cr, sr;
    int max_history, zero_dming, use_mor;
    CircBuf<double> mean_buf, rms_buf;   // mode 0 stores float values exactly
    double rms_run = 0, mean_run = 0, mean_over_rms = 0, inv_mor = 0;
    double rms_carry = 0;  // function-scope spectrumRMS carried between spectra
    double acc_mean = 0, acc_mean_prev = 0, acc_rms = 0, acc_rms_prev = 0;
    float frac_bad_channels = 0.0f;
    int bad_spectra = 0, num = 0, remaining_zeros = 0;
    std::vector<float> last_good;

    // Guided run (test infrastructure for the "bit-exact except within eps of
    // threshold" bar): hint holds another implementation's flags [t][nbins]
    // (bit 0 channel, bit 1 spectrum).  Where this run's decision differs
    // from the hint and its decision statistic lies within eps of the
    // threshold, the hint is taken (an allowed near-threshold difference);
    // any other difference is counted as a mismatch and the hint is taken
    // too, so that both runs keep the same state and every later decision is
    // still compared.  Channel statistic: (I - dataModel - bp) - margin in
    // units of rmsRunAve; spectrum statistic: (mean - meanRunAve) - tolerance
    // in units of bandpass rms / sqrt(nBins) (RFI_Clipper.cpp:315,415-419).
    const uint8_t* hint = nullptr;
    double eps_c = 0.0, eps_s = 0.0;
    double rep[12] = {0};
    void guide_reset() {
        for (double& r : rep) r = 0.0;
        rep[8] = rep[9] = 1e300;
        rep[10] = -1.0;
    }
    bool guide(bool own, bool want, double stat, double scale, long long t, bool spectrum,
               bool integral) {
        const int base = spectrum ? 4 : 0;
        const double z = scale > 0.0 ? std::fabs(stat) / scale : std::fabs(stat);
        rep[base] += 1.0;
        if (!integral && z < rep[spectrum ? 9 : 8]) rep[spectrum ? 9 : 8] = z;
        if (own == want) return own;
        if (!integral && z <= (spectrum ? eps_s : eps_c)) {
            rep[base + 1] += 1.0;
            if (z > rep[base + 3]) rep[base + 3] = z;
        } else {
            rep[base + 2] += 1.0;
        }
        if (rep[10] < 0.0) rep[10] = (double)t;
        return want;
    }

    // mode 0: one sequential FP32 sum; mode 1: canonical partials + tree
    template <typename F>
    float channel_sum(int n, F f) const {
        if (!f64) {
            float s = 0.0f;
            for (int i = 0; i < n; ++i) s += f(i);
            return s;
        }
        float part[1024];
        for (int p = 0; p < parts; ++p) {
            float s = 0.0f;
            for (int i = p; i < n; i += parts) s += f(i);
            part[p] = s;
        }
        return tree_p(part, parts);
    }
    // mode 1 running sums: reference's accumulate() is the sequential sum of
    // the buffer; the variant keeps it incrementally with the same order.
    int run(float* I, float* W, int nt, int nsub, int npol, int nchan, uint8_t* flags) override {
        const unsigned nbins = (unsigned)(nchan * nsub);
        if (nbins % 8 != 0) return -2;
        const float k = 4;
        const float mmm = (float)(k / ::sqrt(2.0 * k));
        const double inv_h = 1.0 / (double)max_history;
        const double inv_sqrt_nbins = 1.0 / std::sqrt((double)nbins);
        if (last_good.size() != nbins) {
            last_good.resize(nbins, 0.0f);
            remaining_zeros = (int)nbins;
        }
        map.n = nbins; map.lower = 0.0; map.width = 1.0;  // BinMap::reset
        map.lower = start_freq;
        map.set_width((end_freq - map.lower) / nbins);  // setEnd
        bp.rebin(map);
        const unsigned cpb = nbins / 8;
        auto idx = [&](unsigned t, unsigned s, unsigned p) -> long long {
            return (long long)nchan * (npol * ((long long)nsub * t + s) + p);
        };
        std::vector<float> vals(nbins);
        for (unsigned t = 0; t < (unsigned)nt; ++t) {
            const std::vector<float> bandpass = bp.current_set();
            auto at = [&](unsigned bin) -> float& {
                unsigned s = bin / nchan, c = bin % nchan;
                return I[idx(t, s, 0) + c];
            };
            bool good_spectrum = true;
            float data_model;
            double spectrum_rms = rms_carry;
            if (!rms_buf.full()) {
                // adaptive phase, RFI_Clipper.cpp:214-278
                float mini_data[8], mini_model[8], band_sigma[8], dmm[8];
                for (int b = 0; b < 8; ++b) { mini_data[b] = 1e6f; mini_model[b] = 1e6f; }
                for (unsigned bin = 0; bin < nbins; ++bin) {
                    unsigned band = bin / cpb;
                    float v = at(bin);
                    if (v < mini_data[band]) mini_data[band] = v;
                    if (bandpass[bin] < mini_model[band]) mini_model[band] = bandpass[bin];
                }
                for (int b = 0; b < 8; ++b) {
                    float bm, bms;
                    if (!f64) {
                        float s1 = 0.0f, s2 = 0.0f;
                        for (unsigned bin = b * cpb; bin < (b + 1) * cpb; ++bin) {
                            float v = at(bin);
                            s1 += v;
                            s2 += (v * v);
                        }
                        bm = s1; bms = s2;
                    } else {
                        // partial p: FP32 sums of the band's bins with bin % parts == p
                        float f1[1024] = {0}, f2[1024] = {0};
                        for (unsigned bin = b * cpb; bin < (b + 1) * cpb; ++bin) {
                            const float v = at(bin);
                            f1[bin % parts] += v;
                            f2[bin % parts] += v * v;
                        }
                        bm = tree_p(f1, parts); bms = tree_p(f2, parts);
                    }
                    dmm[b] = mini_data[b] - mini_model[b];
                    const float a = bms / cpb;
                    const float m = bm / cpb;
                    const float diff = a - m * m;  // std::pow(float,2) == m*m in float
                    band_sigma[b] = (float)::sqrt((double)diff);
                }
                const float srms = *std::min_element(band_sigma, band_sigma + 8);
                std::nth_element(dmm, dmm + 4, dmm + 8);
                data_model = dmm[4];
                if (!f64) {
                    rms_buf.push_back(srms);
                    rms_run = (float)(rms_buf.accumulate() / rms_buf.size());
                    if (rms_buf.full()) mean_over_rms = (float)((float)mean_run / (float)rms_run);
                    data_model = data_model + mmm * (float)rms_run;
                } else {
                    acc_rms_prev = acc_rms;
                    acc_rms = acc_rms + (double)srms;
                    rms_buf.push_back(srms);
                    rms_run = acc_rms / (double)rms_buf.size();
                    if (rms_buf.full()) {
                        mean_over_rms = mean_run / rms_run;
                        inv_mor = 1.0 / mean_over_rms;
                    }
                    data_model = data_model + mmm * (float)rms_run;
                }
                spectrum_rms = srms;
            } else {
                // steady phase, RFI_Clipper.cpp:279-307
                if (!f64) {
                    float r = (float)rms_run;
                    r -= ((float)rms_buf.front() / (float)rms_buf.size());
                    r += ((float)rms_buf.back() / (float)rms_buf.cap);
                    rms_run = r;
                    if (use_mor) spectrum_rms = std::fabs((float)mean_run / (float)mean_over_rms);
                    rms_buf.push_back((float)spectrum_rms);
                } else {
                    rms_run = rms_run - rms_buf.front() * inv_h;
                    rms_run = rms_run + rms_buf.back() * inv_h;
                    if (use_mor) spectrum_rms = std::fabs(mean_run * inv_mor);
                    rms_buf.push_back(spectrum_rms);
                }
                data_model = 0.0f;
            }
            const float margin = cr * (float)rms_run;
            // channel clipping, :315-342
            std::vector<unsigned char> clipped(nbins, 0);
            int good_per_band[8] = {0};
            for (unsigned bin = 0; bin < nbins; ++bin) {
                float v = at(bin);
                const float x = (float)((float)(v - data_model) - bandpass[bin]);
                bool clip = x > margin;
                if (hint)
                    clip = guide(clip, (hint[(long long)t * nbins + bin] & 1) != 0,
                                 (double)x - (double)margin, std::fabs(rms_run), t, false, false);
                if (clip) {
                    clipped[bin] = 1;
                    unsigned s = bin / nchan, c = bin % nchan;
                    for (int q = 0; q < npol; ++q) {
                        I[idx(t, s, q) + c] = last_good[bin];
                        W[idx(t, s, q) + c] = 1.0f;
                    }
                } else {
                    ++good_per_band[bin / cpb];
                }
            }
            float spectrum_sum = channel_sum((int)nbins, [&](int bin) -> float {
                return clipped[bin] ? 0.0f : at(bin);
            });
            unsigned total_good = 0;
            for (int b = 0; b < 8; ++b) total_good += good_per_band[b];
            frac_bad_channels += (float)(nbins - total_good) / nbins;
            spectrum_sum /= total_good;
            unsigned bad_bands = 0;
            for (int b = 0; b < 8; ++b) {
                if ((double)good_per_band[b] < 0.8 * cpb) ++bad_bands;
                if (good_per_band[b] == 0) bad_bands += 4;
            }
            if (total_good < 0.8 * nbins) bad_bands += 4;
            // mean history, :383-400
            if (!mean_buf.full()) {
                if (!f64) {
                    mean_buf.push_back(spectrum_sum);
                    mean_run = (float)(mean_buf.accumulate() / mean_buf.size());
                } else {
                    acc_mean_prev = acc_mean;
                    acc_mean = acc_mean + (double)spectrum_sum;
                    mean_buf.push_back(spectrum_sum);
                    mean_run = acc_mean / (double)mean_buf.size();
                }
            } else {
                if (!f64) {
                    float mr = (float)mean_run;
                    mr -= (float)mean_buf.front() / (float)mean_buf.size();
                    mr += (float)mean_buf.back() / (float)mean_buf.size();
                    mean_run = mr;
                } else {
                    mean_run = mean_run - mean_buf.front() * inv_h;
                    mean_run = mean_run + mean_buf.back() * inv_h;
                }
                mean_buf.push_back(spectrum_sum);
            }
            bool reject;
            double reject_stat;
            if (!f64) {
                const float tol = (float)((double)(sr * bp.rms()) / ::sqrt((double)nbins));
                const float dev = (float)(spectrum_sum - (float)mean_run);
                reject = dev > tol;
                reject_stat = (double)dev - (double)tol;
            } else {
                const float tol = (float)((double)(sr * bp.rms()) * inv_sqrt_nbins);
                reject = (double)spectrum_sum - mean_run > (double)tol;
                reject_stat = ((double)spectrum_sum - mean_run) - (double)tol;
            }
            bool spectrum_clip = false;
            if (hint) {
                // the 1000-spectrum gate and the bad-band count are integer
                // decisions: any difference there is a mismatch
                const bool want = (hint[(long long)t * nbins] & 2) != 0;
                const bool gate = mean_buf.size() < 1000;
                const bool integral = gate || bad_bands >= 4;
                const bool own = gate || reject || bad_bands >= 4;
                const bool take = guide(own, want, reject_stat,
                                        std::fabs((double)bp.rms()) * inv_sqrt_nbins, t, true, integral);
                // follow the hint past the gate (inside the gate it cannot be followed)
                if (!gate && take != own) {
                    reject = take;
                    if (!take) bad_bands = 0;
                }
            }
            if (mean_buf.size() < 1000) {
                spectrum_clip = true;
            } else if (reject || bad_bands >= 4) {
                spectrum_clip = true;
                ++bad_spectra;
                mean_buf.pop_back();
                rms_buf.pop_back();
                mean_buf.push_back(mean_buf.back());
                rms_buf.push_back(rms_buf.back());
                if (f64) {
                    acc_mean = acc_mean_prev + mean_buf.back();
                    acc_rms = acc_rms_prev + rms_buf.back();
                }
            } else if (remaining_zeros != 0) {
                for (unsigned bin = 0; bin < nbins; ++bin) {
                    float v = at(bin);
                    if (last_good[bin] == 0.0f && v != 0.0f) {
                        last_good[bin] = v;
                        --remaining_zeros;
                    }
                }
            }
            if (spectrum_clip) {  // clipSample, :127-150
                good_spectrum = false;
                for (int s = 0; s < nsub; ++s)
                    for (int q = 0; q < npol; ++q)
                        for (int c = 0; c < nchan; ++c) {
                            W[idx(t, s, q) + c] = 1.0f;
                            I[idx(t, s, q) + c] = -0.2f;
                        }
            }
            // flatten, :478-494
            for (unsigned bin = 0; bin < nbins; ++bin) {
                float& v = at(bin);
                v -= (float)(bandpass[bin] + data_model);
                vals[bin] = v;
            }
            const float s1 = channel_sum((int)nbins, [&](int bin) -> float { return vals[bin]; });
            const float s2 = channel_sum((int)nbins, [&](int bin) -> float { return vals[bin] * vals[bin]; });
            const float m = s1 / nbins;
            const float ms = s2 / nbins;
            float srms = (float)::sqrt((double)(ms - m * m));
            if (srms == 0.0f) srms = 1.0f;
            rms_carry = srms;
            if (good_spectrum) {
                const float sub = (zero_dming == 1) ? (float)(zero_dming * m) : (float)mean_run;
                for (unsigned bin = 0; bin < nbins; ++bin) {
                    float& v = at(bin);
                    v -= sub;
                    v /= srms;
                    if (v > cr) v = 0.0f;
                }
            }
            if (flags) {
                for (unsigned bin = 0; bin < nbins; ++bin)
                    flags[(long long)t * nbins + bin] =
                        (uint8_t)(clipped[bin] | (spectrum_clip ? 2 : 0));
            }
            // statistics, :535-560
            unsigned report_every = 10 * max_history;
            if (num == 0) {
                float frac_bad_spectra = (float)(100.0 * (float)bad_spectra / (float)report_every);
                if (frac_bad_spectra > 99.0) {
                    rms_buf.q.clear();
                    mean_buf.q.clear();
                    acc_mean = acc_mean_prev = acc_rms = acc_rms_prev = 0.0;
                }
                bad_spectra = 0;
                frac_bad_channels = 0.0f;
            }
            bp.set_mean((float)mean_run);
            bp.set_rms((float)rms_run);
            ++num;
            num = num % (int)report_every;
        }
        return 0;
    }

    void state(double* out) const override {
        out[0] = mean_run;
        out[1] = rms_run;
        out[2] = bp.mean();
        out[3] = bp.rms();
        out[4] = bp.params.empty() ? 0.0 : bp.params[0];
        out[5] = num;
        out[6] = bad_spectra;
        out[7] = (double)mean_buf.size();
        out[8] = (double)rms_buf.size();
        out[9] = remaining_zeros;
    }
};

}  // namespace

struct or_rfi {
    RfiBase* impl;
};

extern "C" or_rfi* or_rfi_create(const char* bp_text, float cr_factor, float sr_factor,
                                 int max_history, int zero_dming, int use_mean_over_rms,
                                 int band_matching, int mode, int parts, char* err, int errlen) {
    if (parts != 256 && parts != 512 && parts != 1024) parts = 256;
    Rfi* r = new Rfi;
    r->f64 = mode == 1;
    r->parts = parts;
    r->cr = cr_factor; r->sr = sr_factor; r->max_history = max_history;
    r->zero_dming = zero_dming; r->use_mor = use_mean_over_rms;
    r->mean_buf.cap = r->rms_buf.cap = (size_t)max_history;
    RfiBase* impl = r;
    std::string e;
    if (!parse_bp(bp_text, impl->bp, e)) {
        if (err && errlen > 0) std::snprintf(err, errlen, "%s", e.c_str());
        delete impl;
        return nullptr;
    }
    if (band_matching) {
        impl->start_freq = (float)impl->bp.current.lower;
        impl->end_freq = (float)(impl->bp.current.lower + impl->bp.current.width * impl->bp.current.n);
    }
    or_rfi* h = new or_rfi;
    h->impl = impl;
    return h;
}

extern "C" void or_rfi_destroy(or_rfi* r) {
    if (r) { delete r->impl; delete r; }
}

extern "C" int or_rfi_run(or_rfi* r, float* data, float* weights, int nt, int nsub, int npol,
                          int nchan, uint8_t* flags) {
    return r->impl->run(data, weights, nt, nsub, npol, nchan, flags);
}

extern "C" int or_rfi_run_guided(or_rfi* r, float* data, float* weights, int nt, int nsub, int npol,
                                 int nchan, const uint8_t* hint, double eps_chan, double eps_spec,
                                 uint8_t* flags, double* report12) {
    Rfi* g = static_cast<Rfi*>(r->impl);
    g->hint = hint;
    g->eps_c = eps_chan;
    g->eps_s = eps_spec;
    g->guide_reset();
    const int rc = g->run(data, weights, nt, nsub, npol, nchan, flags);
    g->hint = nullptr;
    for (int i = 0; i < 12; ++i) report12[i] = g->rep[i];
    return rc;
}

extern "C" void or_rfi_state(const or_rfi* r, double* out10) { r->impl->state(out10); }

extern "C" int or_rfi_bandpass(const or_rfi* r, float* out, int nbins) {
    const std::vector<float>& d = r->impl->bp.current_set();
    if ((int)d.size() < nbins) return -1;
    std::copy(d.begin(), d.begin() + nbins, out);
    return 0;
}

// BandPass checks -----------------------------------------------------------
struct or_bandpass { BandPassR bp; };

extern "C" or_bandpass* or_bandpass_create(int nbins, double start, double width,
                                           const float* params, int nparams) {
    or_bandpass* b = new or_bandpass;
    BinMapR map;
    map.n = (unsigned)nbins; map.lower = start; map.set_width(width);
    b->bp.set_data(map, std::vector<float>(params, params + nparams));
    return b;
}
extern "C" void or_bandpass_destroy(or_bandpass* b) { delete b; }
extern "C" void or_bandpass_set_rms(or_bandpass* b, float v) { b->bp.set_rms(v); }
extern "C" void or_bandpass_set_median(or_bandpass* b, float v) { b->bp.set_median(v); }
extern "C" void or_bandpass_set_mean(or_bandpass* b, float v) { b->bp.set_mean(v); }
extern "C" void or_bandpass_kill_band(or_bandpass* b, float s, float e) { b->bp.kill_band(s, e); }
extern "C" void or_bandpass_rebin(or_bandpass* b, int nbins, double start, double width) {
    BinMapR map;
    map.n = (unsigned)nbins; map.lower = start; map.set_width(width);
    b->bp.rebin(map);
}
extern "C" float or_bandpass_intensity(const or_bandpass* b, float freq) {
    auto it = b->bp.data.find(b->bp.current.key());
    int i = b->bp.current.bin_index(freq);
    if (it == b->bp.data.end() || i < 0 || i >= (int)it->second.size()) return NAN;
    return it->second[i];
}
extern "C" float or_bandpass_intensity_of_bin(const or_bandpass* b, int i) {
    auto it = b->bp.data.find(b->bp.current.key());
    if (it == b->bp.data.end() || i < 0 || i >= (int)it->second.size()) return NAN;
    return it->second[i];
}
extern "C" float or_bandpass_median(const or_bandpass* b) { return b->bp.median(); }
extern "C" float or_bandpass_rms(const or_bandpass* b) { return b->bp.rms(); }
extern "C" float or_bandpass_mean(const or_bandpass* b) { return b->bp.mean(); }
extern "C" int or_binmap_index(double start, double width, double value) {
    BinMapR m; m.lower = start; m.set_width(width);
    return m.bin_index(value);
}

// ===========================================================================
// A8/A10 DedispersionBuffer + DedispersionModule (DedispersionModule.cpp:109-297,
// DedispersionBuffer.cpp:65-245)
// ===========================================================================
struct or_ddmod {
    int B, tdms;
    float dm_low, dm_step;
    double fch1, foff;
    int nchan_total = 0, maxshift = 0, remaining = 0, inverted = 0;
    double tsamp = 0.0;
    std::vector<float> dmshift;
    std::vector<float> buf;  // [nchan_total][B]
    int count = 0;
    long long first_abs = 0, next_abs = 0;
    struct Done { std::vector<float> data; int nout; long long first; };
    std::deque<Done> done;
};

extern "C" or_ddmod* or_ddmod_create(int buffer_samples, int tdms, float dm_low, float dm_step,
                                     double fch1, double foff) {
    or_ddmod* m = new or_ddmod;
    m->B = buffer_samples;
    m->tdms = tdms;
    m->dm_low = dm_low < 0.0f ? 0.0f : dm_low;  // :57
    m->dm_step = dm_step;
    m->fch1 = fch1;
    m->foff = foff;
    return m;
}
extern "C" void or_ddmod_destroy(or_ddmod* m) { delete m; }

extern "C" int or_ddmod_add(or_ddmod* m, const float* stokes, int nt, int nsub, int npol,
                            int nchan, double tsamp) {
    const int nbins = nsub * nchan;
    if (nbins != m->nchan_total) {  // resize(), :109-190
        m->nchan_total = nbins;
        m->dmshift.assign(nbins, 0.0f);
        m->inverted = or_dm_shifts(m->fch1, m->foff, nbins, m->dmshift.data());
        m->tsamp = tsamp;
        or_maxshift(m->dm_low, m->dm_step, m->tdms, m->dmshift.data(), nbins, tsamp, m->B,
                    &m->maxshift, &m->remaining);
        if (m->B <= m->maxshift) return -1;
        m->buf.assign((size_t)nbins * m->B + 1, 0.0f);  // +1: zero pad after the last row
        m->count = 0;
        m->first_abs = m->next_abs;
    }
    int produced = 0;
    const float start = m->dm_low / (float)m->tsamp, step = m->dm_step / (float)m->tsamp;
    for (int t = 0; t < nt; ++t) {
        for (int r = 0; r < nbins; ++r) {
            int bin = m->inverted ? nbins - 1 - r : r;
            int s = bin / nchan, c = bin % nchan;
            m->buf[(size_t)r * m->B + m->count] =
                stokes[(long long)nchan * (npol * ((long long)nsub * t + s) + 0) + c];
        }
        ++m->count;
        ++m->next_abs;
        if (m->count == m->B) {
            const int overlap = m->maxshift + m->remaining;
            const int nout = m->B - overlap;
            or_ddmod::Done d;
            d.nout = nout;
            d.first = m->first_abs;
            d.data.assign((size_t)m->tdms * nout, 0.0f);
            or_dedisperse(m->buf.data(), nbins, m->B, nout, m->tdms, m->dmshift.data(), start, step,
                          d.data.data(), 0);
            m->done.push_back(std::move(d));
            ++produced;
            for (int r = 0; r < nbins; ++r)
                std::memmove(&m->buf[(size_t)r * m->B], &m->buf[(size_t)r * m->B + nout],
                             sizeof(float) * overlap);
            m->count = overlap;
            m->first_abs += nout;
        }
    }
    return produced;
}

extern "C" int or_ddmod_pop(or_ddmod* m, float* out, long long cap, long long* first_sample) {
    if (m->done.empty()) return 0;
    or_ddmod::Done& d = m->done.front();
    int nout = d.nout;
    if (out && cap >= (long long)d.data.size()) std::copy(d.data.begin(), d.data.end(), out);
    if (first_sample) *first_sample = d.first;
    m->done.pop_front();
    return nout;
}

extern "C" void or_ddmod_params(const or_ddmod* m, int* maxshift, int* remaining, int* nout,
                                int* nchan_total, int* inverted) {
    if (maxshift) *maxshift = m->maxshift;
    if (remaining) *remaining = m->remaining;
    if (nout) *nout = m->B - m->maxshift - m->remaining;
    if (nchan_total) *nchan_total = m->nchan_total;
    if (inverted) *inverted = m->inverted;
}

extern "C" int or_num_threads(void) { return threads_or_default(0); }

// ===========================================================================
// F1 LOFAR UDP packets -> TimeSeriesDataSetC32 (AdapterTimeSeriesDataSet)
// ===========================================================================
// A packet is the 16-byte header (LofarUdpHeader.h:25-35: version u8,
// sourceInfo u8, configuration u16, station u16, nrBeamlets u8, nrBlocks u8,
// timestamp u32, blockSequenceNumber u32; little endian), the data and, for
// fixed-size packets, padding up to sizeof(UDPPacket) = 8148 bytes (16 + 8130
// rounded to the struct's 4-byte alignment).

// AdapterTimeSeriesDataSet::_checkData (AdapterTimeSeriesDataSet.cpp:152-191).
// Returns 0, or the number of the first failing check: 1 sample bits, 2 chunk
// size, 3 data larger than a packet, 4 time samples not a multiple of the
// block length.  packet_bytes and nblocks are written when the check passes.
extern "C" int or_udp_check(int fixed, int bits, int npackets, int spp, int nchan, int nsub,
                            int npol, long long chunk_bytes, long long* packet_bytes, int* nblocks) {
    if (bits != 8 && bits != 16) return 1;
    const long long samples = (long long)nsub * npol * spp;
    const long long useful_bits = samples * bits * 2;
    const long long useful_bytes = useful_bits / 8;
    const long long psize = fixed ? 8148 : 16 + useful_bytes;
    const long long udp_bits = fixed ? 8130LL * 8 : useful_bits;
    if (chunk_bytes != psize * npackets) return 2;
    if (useful_bits > udp_bits) return 3;
    const long long times = (long long)spp * npackets;
    if (nchan <= 0 || times % nchan != 0) return 4;
    if (packet_bytes) *packet_bytes = psize;
    if (nblocks) *nblocks = (int)(times / nchan);
    return 0;
}

// AdapterTimeSeriesDataSet::_readData (AdapterTimeSeriesDataSet.cpp:217-293):
// each packet's data is read in the order subband, time, polarisation, one
// complex int8 or int16 per (s, t, p); time t of packet k is sample
// k*spp + t of the series [s][p] (TimeSeriesDataSet.h:145-151 with blocks of
// nchan samples: the series is contiguous in time).  The 16-bit reader reads
// two polarisations per time (:240-258), so 16-bit data needs npol == 2.
extern "C" int or_udp_unpack(const unsigned char* chunk, long long packet_bytes, int npackets,
                             int bits, int nsub, int npol, int spp, float* out) {
    if (bits == 16 && npol != 2) return 1;
    const long long nt = (long long)npackets * spp;
    for (int k = 0; k < npackets; ++k) {
        const unsigned char* d = chunk + (long long)k * packet_bytes + 16;
        long long ip = 0;
        for (int s = 0; s < nsub; ++s)
            for (int t = 0; t < spp; ++t)
                for (int p = 0; p < npol; ++p) {
                    float re, im;
                    if (bits == 8) {
                        re = (float)(signed char)d[ip];
                        im = (float)(signed char)d[ip + 1];
                        ip += 2;
                    } else {
                        int16_t v[2];
                        std::memcpy(v, d + ip, 4);
                        re = (float)v[0];
                        im = (float)v[1];
                        ip += 4;
                    }
                    float* o = out + 2 * (((long long)s * npol + p) * nt + (long long)k * spp + t);
                    o[0] = re;
                    o[1] = im;
                }
    }
    return 0;
}

// The chunk's time stamp from its first packet (AdapterTimeSeriesDataSet.cpp:
// 108-120): blocks per second are 156250 at the 160 MHz clock, else 195313 in
// even seconds and 195312 in odd ones.
extern "C" void or_udp_time(const unsigned char* header, int clock_mhz, double* timestamp,
                            double* block_rate) {
    uint32_t ts, seq;
    std::memcpy(&ts, header + 8, 4);
    std::memcpy(&seq, header + 12, 4);
    const unsigned tot = clock_mhz == 160 ? 156250u : (ts % 2 == 0 ? 195313u : 195312u);
    *timestamp = ts + (1.0 * seq) / tot;
    *block_rate = 1.0 / tot;
}

// ===========================================================================
// F2 SigprocStokesWriter data block (SigprocStokesWriter.cpp:187-236, 288-293)
// ===========================================================================
// Per spectrum t, per written polarisation p, subbands s = nsub-1..0 and
// channels i = nchan-1..0 of the Stokes set (index nchan*(npol*(nsub*t+s)+p),
// SpectrumDataSet.h:229-235): the float itself (32 bits) or the low byte of
// (int)rint((min(x, max) - min) * nRange / (max - min)), 0 below min (8
// bits); nRange = (int)pow(2, nbits) - 1.0 held in a float member, the
// product and quotient in float, rint on the double.
extern "C" long long or_sigproc_pack(const float* stokes, int nt, int nsub, int npol, int nchan, int npw,
                                     int nbits, float cmin, float cmax, unsigned char* out) {
    const float nrange = (float)((int)std::pow(2.0, (double)nbits) - 1.0);
    const float delta = cmax - cmin;
    long long o = 0;
    for (int t = 0; t < nt; ++t)
        for (int p = 0; p < npw; ++p)
            for (int s = nsub - 1; s >= 0; --s) {
                const long long index = (long long)nchan * (npol * ((long long)nsub * t + s) + p);
                for (int i = nchan - 1; i >= 0; --i) {
                    const float x = stokes[index + i];
                    if (nbits == 32) {
                        std::memcpy(out + o, &x, 4);
                        o += 4;
                    } else {
                        const float f = (x > cmax) ? cmax : x;
                        int ci = 0;
                        if (!(f < cmin)) {
                            const float q = (f - cmin) * nrange / delta;
                            const double r = ::rint((double)q);
                            ci = std::isnan(r) ? 0 : (int)r;  // the conversion of NaN gives a zero low byte
                        }
                        out[o++] = (unsigned char)(ci & 0xff);
                    }
                }
            }
    return o;
}
