// K1: the channeliser chain.
//
//   PPFChanneliser::run   (lib/src/PPFChanneliser.cpp:81-290)
//   StokesGenerator::run  (lib/src/StokesGenerator.cpp:40-108)
//   StokesIntegrator::run (lib/src/StokesIntegrator.cpp:32-119)
//
// One CTA takes one subband and a tile of BT consecutive PPF blocks (N
// samples each) of both polarisations.  It stages the tile plus the T-1
// preceding blocks (from the previous call's history where the tile starts
// the chunk) in shared memory, applies the T-tap polyphase FIR per channel
// (oldest tap first in the reference's order, each product added by one FP32
// fused multiply-add), transforms every block with a shared-memory radix-2
// decimation-in-frequency FFT (forward, unnormalised, as FFTW_FORWARD) and then either writes the
// complex spectra (SpectrumDataSetC32 layout) or forms Stokes parameters and
// integrates them over `window` blocks and `bin` channels (the
// SpectrumDataSetStokes layout), so the channelised voltages never reach
// HBM.  Raw int16 station samples are accepted directly (the conversion to
// float is exact).
#include <algorithm>
#include <cstring>
#include <cstdlib>
#include <vector>

#include "pv_internal.cuh"

namespace pv {
int fir_coefficients(int ntaps, int nchan, int window, std::vector<double>& out);
}

namespace {

struct ChanArgs {
    const void* in;          // [sub][pol][block*N] complex (float2 or short2)
    int in_int16;            // 1: short2 samples
    const float2* hist_in;   // [sub][pol][T-1][N] previous blocks (may be null: zeros)
    float2* hist_out;        // [sub][pol][T-1][N] blocks carried to the next call
    const float* coeffs;     // [T][N]
    const float2* twiddle;   // [N/2] exp(-2 pi i k / N) ([N] when N is not a power of two)
    int nsub, npol, nblocks, N, T, log2n, BT;  // log2n < 0: N is not a power of two (direct DFT)
    // output
    int mode;                // 0: complex spectra, 1: Stokes + integration
    float2* spectra;         // mode 0: [block][sub][pol][N]
    float* stokes;           // mode 1: [u][sub][nstokes][N/bin]
    int nstokes, window, bin, nu;  // nu: complete windows written
};

__device__ __forceinline__ float2 load_sample(const ChanArgs& a, long long idx) {
    if (a.in_int16) {
        const short2 v = reinterpret_cast<const short2*>(a.in)[idx];
        return make_float2((float)v.x, (float)v.y);
    }
    return reinterpret_cast<const float2*>(a.in)[idx];
}

// The upper output of a radix-2 decimation-in-frequency butterfly,
// (u - v) * w, with the rounding every channeliser kernel uses: the lower
// output is u + v.  Both kernels evaluate each butterfly identically, so their
// spectra agree bit for bit.  The last two stages (spans 1 and 2) only meet
// the twiddles 1 and -i (held exactly in the table): d and (d.y, -d.x), with
// no multiplication.
__device__ __forceinline__ float2 twiddle_mul(float2 d, float2 w) {
    return make_float2(fmaf(d.x, w.x, __fmul_rn(-d.y, w.y)), fmaf(d.x, w.y, __fmul_rn(d.y, w.x)));
}
__device__ __forceinline__ float2 dif_upper(float2 u, float2 v, float2 w) {
    return twiddle_mul(make_float2(__fsub_rn(u.x, v.x), __fsub_rn(u.y, v.y)), w);
}
__device__ __forceinline__ float2 times_minus_i(float2 d) { return make_float2(d.y, -d.x); }

__global__ void __launch_bounds__(256) channelise_kernel(const ChanArgs a) {
    extern __shared__ float2 sm[];
    const int N = a.N, T = a.T, BT = a.BT, P = a.npol;
    const int s = blockIdx.y;
    const int b0 = blockIdx.x * BT;
    const int nb = min(BT, a.nblocks - b0);  // blocks of this tile
    const int H = T - 1;
    const int rows = nb + H;                 // staged blocks per polarisation
    float2* x = sm;                          // [P][BT+H][N]
    float2* y = sm + (size_t)P * (BT + H) * N;    // [P][BT][N]
    float2* tw = y + (size_t)P * BT * N;          // [N/2], or [N] for the direct DFT
    const int ntw = a.log2n < 0 ? N : N / 2;
    float* cf = reinterpret_cast<float*>(tw + N);  // [T][N]
    const int tid = threadIdx.x, nt = blockDim.x;

    for (int i = tid; i < ntw; i += nt) tw[i] = a.twiddle[i];
    for (int i = tid; i < T * N; i += nt) cf[i] = a.coeffs[i];
    // stage blocks b0-H .. b0+nb-1; negative blocks come from the history
    for (int p = 0; p < P; ++p) {
        const long long base = ((long long)s * P + p) * (long long)a.nblocks * N;
        for (int i = tid; i < rows * N; i += nt) {
            const int r = i / N, c = i - r * N;
            const int b = b0 - H + r;
            float2 v;
            if (b >= 0) {
                v = load_sample(a, base + (long long)b * N + c);
            } else {
                v = a.hist_in ? a.hist_in[(((long long)s * P + p) * H + (H + b)) * N + c]
                              : make_float2(0.0f, 0.0f);
            }
            x[((size_t)p * (BT + H) + r) * N + c] = v;
        }
    }
    __syncthreads();
    // the last tile carries its final T-1 blocks (old history included when
    // the chunk is shorter than that) to the next call
    if (b0 + nb == a.nblocks && a.hist_out) {
        for (int p = 0; p < P; ++p)
            for (int i = tid; i < H * N; i += nt) {
                const int r = i / N, c = i - r * N;
                a.hist_out[(((long long)s * P + p) * H + r) * N + c] =
                    x[((size_t)p * (BT + H) + nb + r) * N + c];
            }
    }
    // FIR: y[p][b][c] = sum_t coeff[t][c] * x[p][b+t][c], oldest tap first
    for (int i = tid; i < P * nb * N; i += nt) {
        const int c = i % N, pb = i / N;
        const int p = pb / nb, b = pb - p * nb;
        const float2* xs = x + ((size_t)p * (BT + H) + b) * N + c;
        if (N == 1) {  // PPFChanneliser.cpp:108-131: one channel is the time series itself
            y[(size_t)p * BT + b] = xs[(size_t)H * N];
            continue;
        }
        float re = 0.0f, im = 0.0f;
        for (int t = 0; t < T; ++t) {
            const float k = cf[t * N + c];
            const float2 v = xs[(size_t)t * N];
            re = __fmaf_rn(v.x, k, re);
            im = __fmaf_rn(v.y, k, im);
        }
        y[((size_t)p * BT + b) * N + c] = make_float2(re, im);
    }
    __syncthreads();
    if (a.log2n < 0) {
        // N not a power of two: the forward DFT sum_j y[j] exp(-2 pi i j k / N) of every row
        // into x (no longer needed), in natural channel order
        for (int i = tid; i < P * nb * N; i += nt) {
            const int k = i % N, pb = i / N;
            const int p = pb / nb, b = pb - p * nb;
            const float2* r = y + ((size_t)p * BT + b) * N;
            float re = 0.0f, im = 0.0f;
            int m = 0;  // j * k mod N
            for (int j = 0; j < N; ++j) {
                const float2 v = r[j], w = tw[m];
                re = __fadd_rn(re, __fsub_rn(__fmul_rn(v.x, w.x), __fmul_rn(v.y, w.y)));
                im = __fadd_rn(im, __fadd_rn(__fmul_rn(v.x, w.y), __fmul_rn(v.y, w.x)));
                m += k;
                if (m >= N) m -= N;
            }
            x[((size_t)p * BT + b) * N + k] = make_float2(re, im);
        }
        __syncthreads();
    }
    // In-place radix-2 decimation-in-frequency FFT of every (pol, block) row
    // of y (dif_upper gives the butterfly arithmetic); row position i then
    // holds channel bitrev(i).
    const int half = N / 2, lg = a.log2n;
    for (int lh = lg - 1; lh >= 0; --lh) {  // no stage when lg <= 0
        const int h = 1 << lh;
        for (int i = tid; i < P * nb * half; i += nt) {
            const int j = i & (half - 1), row = i >> (lg - 1);
            const int p = row / nb, b = row - p * nb;
            float2* r = y + ((size_t)p * BT + b) * N;
            const int lo = ((j >> lh) << (lh + 1)) + (j & (h - 1));
            const float2 u = r[lo], v = r[lo + h];
            r[lo] = make_float2(__fadd_rn(u.x, v.x), __fadd_rn(u.y, v.y));
            const float2 d = make_float2(__fsub_rn(u.x, v.x), __fsub_rn(u.y, v.y));
            if (lh == 0) r[lo + h] = d;                                   // twiddle 1
            else if (lh == 1) r[lo + h] = (j & 1) ? times_minus_i(d) : d;  // 1 or -i
            else r[lo + h] = twiddle_mul(d, tw[(j & (h - 1)) << (lg - 1 - lh)]);
        }
        __syncthreads();
    }
    const float2* src = lg < 0 ? x : y;
    // row position of channel c: bit-reversed after the radix-2 FFT, natural after the DFT
    auto pos = [lg](int c) { return lg > 0 ? (int)(__brev((unsigned)c) >> (32 - lg)) : c; };
    // src holds the spectra, rows of stride N with pol stride BT*N
    if (a.mode == 0) {
        for (int i = tid; i < P * nb * N; i += nt) {
            const int c = i % N, pb = i / N;
            const int b = pb % nb, p = pb / nb;
            a.spectra[(((long long)(b0 + b) * a.nsub + s) * P + p) * N + c] =
                src[((size_t)p * BT + b) * N + pos(c)];
        }
        return;
    }
    // Stokes (StokesGenerator.cpp:93-104) integrated over window blocks and bin
    // channels in the integrator's order (StokesIntegrator.cpp:97-115).
    const int nco = N / a.bin;
    const int u0 = b0 / a.window;
    const int nu_tile = nb / a.window;
    for (int i = tid; i < nu_tile * a.nstokes * nco; i += nt) {
        const int nc = i % nco, rest = i / nco;
        const int k = rest % a.nstokes, ul = rest / a.nstokes;
        const int u = u0 + ul;
        if (u >= a.nu) continue;
        float acc = 0.0f;
        for (int tb = 0; tb < a.window; ++tb) {
            const int b = ul * a.window + tb;
            const float2* X = src + (size_t)b * N;
            const float2* Y = src + ((size_t)BT + b) * N;
            for (int c = nc * a.bin; c < (nc + 1) * a.bin; ++c) {
                const int i = pos(c);
                const float xr = X[i].x, xi = X[i].y, yr = Y[i].x, yi = Y[i].y;
                const float px = __fadd_rn(__fmul_rn(xr, xr), __fmul_rn(xi, xi));
                const float py = __fadd_rn(__fmul_rn(yr, yr), __fmul_rn(yi, yi));
                float v;
                if (k == 0) v = __fadd_rn(px, py);
                else if (k == 1) v = __fsub_rn(px, py);
                else if (k == 2) v = __fmul_rn(2.0f, __fadd_rn(__fmul_rn(xr, yr), __fmul_rn(xi, yi)));
                else v = __fmul_rn(2.0f, __fsub_rn(__fmul_rn(xi, yr), __fmul_rn(xr, yi)));
                acc = __fadd_rn(acc, v);
            }
        }
        a.stokes[(((long long)u * a.nsub + s) * a.nstokes + k) * nco + nc] = acc;
    }
}

// ---------------------------------------------------------------------------
// K1 fast path: Stokes I of a dual-polarisation, 8-tap PPF with N = 16, 32 or
// 64 channels, integrated over `window` blocks without channel binning -- the
// beam pipelines' configuration.  One warp runs one subband over a range of
// kRangeBlocks consecutive blocks: lanes 0-15 hold polarisation X and lanes
// 16-31 polarisation Y, lane j holding channels j, j+16, ... (M = N/16 of
// them).  The 8-block FIR window stays in registers, the FFT's stages of
// stride >= 16 run inside each lane and those of stride 8..1 across lanes
// with shuffles, and lane j+16 hands |Y|^2 to lane j, which integrates
// I = |X|^2 + |Y|^2.  Every FIR product and sum, FFT butterfly, Stokes and
// integration step is evaluated exactly as channelise_kernel evaluates it, so
// the two kernels' outputs are bit-identical.  Inputs are read once (plus 7
// warm-up blocks per range); raw loads run 8 blocks ahead of the arithmetic
// (4 for 64 channels, whose int16 kernel is held to 168 registers so that
// three CTAs share an SM).
//
// Jobs (one per beam) are laid out one after another in warp space, so one
// launch channelises any number of beams with the same N.
// ---------------------------------------------------------------------------
constexpr int kRangeBlocks = 256;
constexpr int kFastTaps = 8;

template <bool I16>
struct RawSample;
template <>
struct RawSample<true> {
    using type = int;  // short2 bits
    static __device__ __forceinline__ float2 f2(int v) {
        const short2 s = *reinterpret_cast<const short2*>(&v);
        return make_float2((float)s.x, (float)s.y);
    }
};
template <>
struct RawSample<false> {
    using type = float2;
    static __device__ __forceinline__ float2 f2(float2 v) { return v; }
};

// Packed FP32 pairs for the FIR (Blackwell fma .f32x2): each half is rounded
// as the scalar __fmaf_rn, so the sums are bit-identical to channelise_kernel's.
__device__ __forceinline__ unsigned long long pk2(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 upk2(unsigned long long v) {
    float2 f;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(f.x), "=f"(f.y) : "l"(v));
    return f;
}
// round(a * b + s) per half
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b,
                                                   unsigned long long s) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(s));
    return r;
}

// The FIR window of one lane as packed pairs.  M == 1: (re, im) of the lane's
// channel, coefficients duplicated.  M >= 2: channels 2k and 2k+1 (strided
// by 16) side by side, real parts and imaginary parts in separate pairs, so
// coefficient pairs are two distinct taps' values of the same slot.
template <int M, int T>
struct FirWindow {
    static constexpr int K = M == 1 ? 1 : M / 2;
    unsigned long long re[T][K], im[T][M == 1 ? 1 : K], cf[T][K];
    __device__ __forceinline__ void coeffs(const float (&c)[T][M]) {
#pragma unroll
        for (int t = 0; t < T; ++t)
#pragma unroll
            for (int k = 0; k < K; ++k) cf[t][k] = M == 1 ? pk2(c[t][0], c[t][0]) : pk2(c[t][2 * k], c[t][2 * k + 1]);
    }
    __device__ __forceinline__ void set(int q, const float2 (&v)[M]) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (M == 1) {
                re[q][0] = pk2(v[0].x, v[0].y);
            } else {
                re[q][k] = pk2(v[2 * k].x, v[2 * k + 1].x);
                im[q][k] = pk2(v[2 * k].y, v[2 * k + 1].y);
            }
        }
    }
    // y[m] = sum over taps t (oldest first: slot (q + 1 + t) & (T - 1)) of x * coeff[t]
    __device__ __forceinline__ void fir(int q, float2 (&y)[M]) const {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            unsigned long long ar = 0ull, ai = 0ull;  // +0.0f pairs
#pragma unroll
            for (int t = 0; t < T; ++t) {
                const int slot = (q + 1 + t) & (T - 1);
                ar = fma2(re[slot][k], cf[t][k], ar);
                if (M != 1) ai = fma2(im[slot][k], cf[t][k], ai);
            }
            if (M == 1) {
                y[0] = upk2(ar);
            } else {
                const float2 r = upk2(ar), i = upk2(ai);
                y[2 * k] = make_float2(r.x, i.x);
                y[2 * k + 1] = make_float2(r.y, i.y);
            }
        }
    }
};

template <int N, bool I16, bool PKT>
__global__ void __launch_bounds__(128, N == 64 && I16 ? 3 : 1)  // 3 CTAs of 168 registers
chan_stokes_i_kernel(const pv::ChanJob* __restrict__ jobs, const __grid_constant__ pv::ChanJob one, int njobs,
                     long long nwarps, const pv::BeamStep* __restrict__ bs) {
    constexpr int M = N / 16, T = kFastTaps, H = T - 1;
    constexpr int LOGN = M == 1 ? 4 : (M == 2 ? 5 : 6);
    using Raw = typename RawSample<I16>::type;
    const long long gw = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (gw >= nwarps) return;
    int lo = 0, hi = njobs - 1;  // the job whose warps include gw
    while (jobs && lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].warp_begin <= gw) lo = mid;
        else hi = mid - 1;
    }
    const pv::ChanJob& J = jobs ? jobs[lo] : one;
    const int nblocks = J.nblocks, window = J.window, nu = J.nu, nsub = J.nsub;
    const long long local = gw - J.warp_begin;
    const int s = (int)(local / J.nranges);
    const int r = (int)(local - (long long)s * J.nranges);
    const int B0 = r * kRangeBlocks;
    const int B1 = min(B0 + kRangeBlocks, nblocks);
    const int lane = threadIdx.x & 31, pol = lane >> 4, j = lane & 15;
    const long long row = (long long)s * 2 + pol;
    int par = 0;  // step parity of this beam: input buffer and history double buffer
    if (bs) {
        const pv::BeamStep& B = bs[J.beam];
        if (!B.active) return;
        par = (int)((B.written - B.base) & 1);
    }
    const float2* hin = J.hist[par];
    float2* hout = J.hist[par ^ 1];
    const void* src = (par && J.in_odd) ? J.in_odd : J.in;
    // Raw element (block b, channel-lane m) at in[b * sb + m * sm].  Voltages: the row
    // [sub][pol][t] with t = b*N + j + 16m.  Packets (int16, 16 samples per packet, subband-major
    // [subband][t][pol] after a 16-byte header; AdapterTimeSeriesDataSet.cpp:246-288): sample t is
    // time j of packet b*(N/16) + m of the subband's stream.
    const Raw* in;
    long long sb;
    int sm;  // channel-group stride (a packet: under 64 KiB of words)
    if (PKT) {
        const long long pw = J.pkt_bytes / 4;  // 4-byte words per packet
        const long long npk = (long long)nblocks * (N / 16);
        const int stream = s / J.pkt_nsub, ls = s - stream * J.pkt_nsub;
        in = reinterpret_cast<const Raw*>(src) + stream * npk * pw + 4 + (ls * 16 + j) * 2 + pol;
        sb = (N / 16) * pw;
        sm = (int)pw;
    } else {
        in = reinterpret_cast<const Raw*>(src) + row * nblocks * N + j;
        sb = N;
        sm = 16;
    }

    float cf[T][M];
#pragma unroll
    for (int t = 0; t < T; ++t)
#pragma unroll
        for (int m = 0; m < M; ++m) cf[t][m] = J.coeffs[t * N + j + 16 * m];
    // twiddles: in-lane stages (stride 16*hm, hm = M/2..1) then lane stages
    float2 twr[M > 1 ? M - 1 : 1];
#pragma unroll
    for (int hm = M / 2; hm >= 1; hm >>= 1)
#pragma unroll
        for (int q = 0; q < hm; ++q) twr[M - 2 * hm + q] = J.twiddle[(j + 16 * q) * (M / (2 * hm))];
    float2 tws[4];
    float sgn[4];
    const bool rot = (j & 3) == 3;  // upper lane of the stride-2 stage with twiddle -i
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int h = 8 >> q;
        const bool upper = (j & h) != 0;
        tws[q] = upper ? J.twiddle[(j & (h - 1)) * (N / (2 * h))] : make_float2(1.0f, 0.0f);
        sgn[q] = upper ? -1.0f : 1.0f;
    }

    // FIR window: slot b & 7 holds block b (B0 is a multiple of 8)
    FirWindow<M, T> win;
    win.coeffs(cf);
#pragma unroll
    for (int q = 1; q < T; ++q) {
        const int b = B0 - T + q;
        float2 v[M];
#pragma unroll
        for (int m = 0; m < M; ++m) {
            if (b >= 0) v[m] = RawSample<I16>::f2(in[(long long)b * sb + m * sm]);
            else v[m] = hin ? hin[(row * H + (H + b)) * N + j + 16 * m] : make_float2(0.0f, 0.0f);
        }
        win.set(q, v);
    }
    constexpr int PF = M == 4 ? 4 : T;  // raw loads run PF blocks ahead
    Raw cur[PF][M];
#pragma unroll
    for (int q = 0; q < PF; ++q)
#pragma unroll
        for (int m = 0; m < M; ++m)
            if (B0 + q < B1) cur[q][m] = in[(long long)(B0 + q) * sb + m * sm];
    const Raw* nxt = in + (long long)(B0 + PF) * sb;  // packets: block b + PF, advanced by sb per block

    float acc[M];
#pragma unroll
    for (int m = 0; m < M; ++m) acc[m] = 0.0f;
    int wleft = window;
    int u = B0 / window;
    for (int g0 = B0; g0 < B1; g0 += T) {
#pragma unroll
        for (int q = 0; q < T; ++q) {
            const int b = g0 + q;
            if (b >= B1) break;
            {
                float2 v[M];
#pragma unroll
                for (int m = 0; m < M; ++m) v[m] = RawSample<I16>::f2(cur[q % PF][m]);
                win.set(q, v);
            }
            if (b + PF < B1) {
#pragma unroll
                for (int m = 0; m < M; ++m)
                    cur[q % PF][m] = PKT ? nxt[m * sm] : in[(long long)(b + PF) * sb + m * sm];
            }
            if (PKT) nxt += sb;
            // FIR, oldest tap (block b-7, slot q+1) first, in packed pairs
            float2 y[M];
            win.fir(q, y);
            // FFT stages of stride 16*hm inside the lane
#pragma unroll
            for (int hm = M / 2; hm >= 1; hm >>= 1)
#pragma unroll
                for (int m = 0; m < M; ++m)
                    if ((m & hm) == 0) {
                        const float2 a = y[m], c = y[m + hm];
                        y[m] = make_float2(__fadd_rn(a.x, c.x), __fadd_rn(a.y, c.y));
                        y[m + hm] = dif_upper(a, c, twr[M - 2 * hm + (m & (hm - 1))]);
                    }
            // stages of stride 8..1 across lanes: d = a + b (lower lane) or
            // a - b (upper lane) -- exact sign flips -- then (d * w), w = 1 below;
            // stride 2 meets only w = 1 and -i, stride 1 only w = 1
#pragma unroll
            for (int q2 = 0; q2 < 4; ++q2) {
                const int h = 8 >> q2;
#pragma unroll
                for (int m = 0; m < M; ++m) {
                    const float ox = __shfl_xor_sync(0xffffffffu, y[m].x, h);
                    const float oy = __shfl_xor_sync(0xffffffffu, y[m].y, h);
                    const float2 d = make_float2(fmaf(sgn[q2], y[m].x, ox), fmaf(sgn[q2], y[m].y, oy));
                    if (h == 1) y[m] = d;
                    else if (h == 2) y[m] = rot ? times_minus_i(d) : d;
                    else y[m] = twiddle_mul(d, tws[q2]);
                }
            }
            // Stokes I = |X|^2 + |Y|^2 and integration
#pragma unroll
            for (int m = 0; m < M; ++m) {
                const float p = __fadd_rn(__fmul_rn(y[m].x, y[m].x), __fmul_rn(y[m].y, y[m].y));
                const float py = __shfl_down_sync(0xffffffffu, p, 16);
                acc[m] = __fadd_rn(acc[m], __fadd_rn(p, py));
            }
            if (--wleft == 0) {
                if (pol == 0 && u < nu) {
                    float* o = J.out + ((long long)u * nsub + s) * N;
#pragma unroll
                    for (int m = 0; m < M; ++m) o[__brev(j + 16 * m) >> (32 - LOGN)] = acc[m];
                }
#pragma unroll
                for (int m = 0; m < M; ++m) acc[m] = 0.0f;
                wleft = window;
                ++u;
            }
        }
    }
    // the range that ends the chunk carries its last 7 blocks to the next call
    if (hout && B1 == nblocks) {
#pragma unroll
        for (int q = 0; q < H; ++q)
#pragma unroll
            for (int m = 0; m < M; ++m)
                hout[(row * H + q) * N + j + 16 * m] =
                    RawSample<I16>::f2(in[(long long)(nblocks - H + q) * sb + m * sm]);
    }
}

// StokesGenerator::run on complex spectra [t][sub][2][N] (module-level call).
__global__ void stokes_kernel(const float2* __restrict__ spectra, int nt, int nsub, int N, int nstokes,
                              float* __restrict__ out) {
    const long long n = (long long)nt * nsub * N;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % N);
        const long long ts = i / N;
        const float2 X = spectra[(ts * 2 + 0) * N + c];
        const float2 Y = spectra[(ts * 2 + 1) * N + c];
        const float xyr = __fadd_rn(__fmul_rn(X.x, Y.x), __fmul_rn(X.y, Y.y));
        const float xyi = __fsub_rn(__fmul_rn(X.y, Y.x), __fmul_rn(X.x, Y.y));
        const float px = __fadd_rn(__fmul_rn(X.x, X.x), __fmul_rn(X.y, X.y));
        const float py = __fadd_rn(__fmul_rn(Y.x, Y.x), __fmul_rn(Y.y, Y.y));
        float* o = out + ts * nstokes * N;
        o[c] = __fadd_rn(px, py);
        if (nstokes == 4) {
            o[N + c] = __fsub_rn(px, py);
            o[2 * N + c] = __fmul_rn(2.0f, xyr);
            o[3 * N + c] = __fmul_rn(2.0f, xyi);
        }
    }
}

// StokesIntegrator::run on [t][sub][pol][nchan] (module-level call).
__global__ void integrate_kernel(const float* __restrict__ in, int nsub, int npol, int nchan,
                                 int window, int bin, int nu, float* __restrict__ out) {
    const int nco = nchan / bin;
    const long long n = (long long)nu * nsub * npol * nco;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int nc = (int)(i % nco);
        const long long usp = i / nco;  // (u*nsub + s)*npol + p
        const int p = (int)(usp % npol);
        const long long us = usp / npol;
        const int s = (int)(us % nsub);
        const long long u = us / nsub;
        float acc = 0.0f;
        for (int tb = 0; tb < window; ++tb) {
            const long long t = u * window + tb;
            const float* v = in + (((t * nsub + s) * npol) + p) * nchan;
            for (int c = nc * bin; c < (nc + 1) * bin; ++c) acc = __fadd_rn(acc, v[c]);
        }
        out[i] = acc;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// PPF state object
// ---------------------------------------------------------------------------
struct pv_ppf {
    int nchan = 0, ntaps = 0, log2n = 0;
    float* d_coeffs = nullptr;
    float2* d_twiddle = nullptr;
    float2* d_hist[2] = {nullptr, nullptr};
    int cur = 0;
    int nsub = 0, npol = 0;
    bool have_hist = false;
    std::vector<float> h_coeffs;
};

namespace {

int tile_blocks(int N, int T, int P, int window, size_t* smem_out) {
    // largest power-of-two tile (a multiple of the integration window) that
    // fits in shared memory
    for (int bt = 128; bt >= 1; bt /= 2) {
        if (window > 0 && bt % window != 0) continue;
        const size_t smem = ((size_t)P * (bt + T - 1) * N + (size_t)P * bt * N + N) * sizeof(float2) +
                            (size_t)T * N * sizeof(float);
        if (smem <= 200 * 1024 && (size_t)P * bt * N <= 256 * 256) {
            *smem_out = smem;
            return bt;
        }
    }
    return 0;
}

int prepare_history(pv_ppf* h, int nsub, int npol, cudaStream_t s) {
    if (h->nsub == nsub && h->npol == npol && h->d_hist[0]) return PV_OK;
    for (auto& p : h->d_hist)
        if (p) { cudaFree(p); p = nullptr; }
    const size_t bytes = (size_t)nsub * npol * (h->ntaps - 1) * h->nchan * sizeof(float2);
    for (auto& p : h->d_hist) {
        if (bytes == 0) continue;
        PV_CUDA(cudaMalloc(&p, bytes), "allocate PPF history");
        PV_CUDA(cudaMemsetAsync(p, 0, bytes, s), "clear PPF history");
    }
    h->nsub = nsub;
    h->npol = npol;
    h->cur = 0;
    h->have_hist = false;
    return PV_OK;
}

}  // namespace

namespace pv {

bool chan_fast_supported(int nchan, int ntaps, int npol, int nstokes, int window, int bin,
                         int nblocks) {
    return (nchan == 16 || nchan == 32 || nchan == 64) && ntaps == kFastTaps && npol == 2 &&
           nstokes == 1 && bin == 1 && window > 0 && kRangeBlocks % window == 0 &&
           nblocks >= kFastTaps - 1;
}

int chan_job_warps(ChanJob& job) {
    job.nranges = ceil_div(job.nblocks, kRangeBlocks);
    return job.nsub * job.nranges;
}

int launch_chan_fast(int nchan, int input, const ChanJob* d_jobs, const ChanJob& one, int njobs,
                     long long nwarps, const BeamStep* bs, cudaStream_t s) {
    if (nwarps <= 0) return PV_OK;
    const unsigned grid = (unsigned)ceil_div<long long>(nwarps, 4);
#define PV_CHAN_FAST(NN)                                                                         \
    if (nchan == NN) {                                                                           \
        if (input == 2)                                                                          \
            chan_stokes_i_kernel<NN, true, true><<<grid, 128, 0, s>>>(d_jobs, one, njobs, nwarps, bs);  \
        else if (input == 1)                                                                     \
            chan_stokes_i_kernel<NN, true, false><<<grid, 128, 0, s>>>(d_jobs, one, njobs, nwarps, bs); \
        else                                                                                     \
            chan_stokes_i_kernel<NN, false, false><<<grid, 128, 0, s>>>(d_jobs, one, njobs, nwarps, bs);\
        return check_launch("chan_stokes_i_kernel");                                            \
    }
    PV_CHAN_FAST(16)
    PV_CHAN_FAST(32)
    PV_CHAN_FAST(64)
#undef PV_CHAN_FAST
    set_error("channelise: no fast kernel for %d channels", nchan);
    return PV_ERR_ARG;
}

}  // namespace pv

namespace {

int run_channelise(pv_ppf* h, const void* d_in, int in_int16, int nsub, int npol, int nblocks,
                   int mode, float2* d_spectra, float* d_stokes, int nstokes, int window, int bin,
                   int* nu_out, cudaStream_t s, long long pkt_bytes = 0, int pkt_nsub = 0) {
    if (!h || !d_in || nsub <= 0 || npol <= 0 || nblocks <= 0) {
        pv::set_error("PPFChanneliser: Empty time data blob");
        return PV_ERR_ARG;
    }
    if (mode == 1 && (npol != 2 || (nstokes != 1 && nstokes != 4) || window <= 0 || bin <= 0 ||
                      h->nchan % bin != 0)) {
        pv::set_error("channelise: Stokes output needs 2 polarisations, 1 or 4 Stokes, "
                      "window > 0 and a channel bin dividing nChannels");
        return PV_ERR_ARG;
    }
    size_t smem = 0;
    const int win_tile = mode == 1 ? std::min(window, nblocks) : 0;
    const int bt = tile_blocks(h->nchan, h->ntaps, npol, win_tile, &smem);
    if (bt == 0) {
        pv::set_error("channelise: %d channels x window %d do not fit one tile", h->nchan, window);
        return PV_ERR_ARG;
    }
    PV_TRY(prepare_history(h, nsub, npol, s));
    const int w = mode == 1 ? std::min(window, nblocks) : 1;  // StokesIntegrator.cpp:53-59
    const int nu = mode == 1 ? nblocks / w : 0;
    const bool fast = mode == 1 && pv::chan_fast_supported(h->nchan, h->ntaps, npol, nstokes, w, bin, nblocks);
    if (pkt_bytes > 0 && (!fast || !in_int16)) {
        pv::set_error("channelise: packet input needs int16 samples, 16/32/64 channels, 8 taps, Stokes I");
        return PV_ERR_ARG;
    }
    if (fast && (pkt_bytes > 0 || getenv("PV_CHAN_GENERIC") == nullptr)) {
        pv::ChanJob job{};
        job.in = d_in;
        job.hist[0] = h->have_hist ? h->d_hist[h->cur] : nullptr;
        job.hist[1] = h->d_hist[h->cur ^ 1];
        job.coeffs = h->d_coeffs;
        job.twiddle = h->d_twiddle;
        job.out = d_stokes;
        job.nsub = nsub;
        job.nblocks = nblocks;
        job.window = w;
        job.nu = nu;
        job.pkt_bytes = pkt_bytes;
        job.pkt_nsub = pkt_nsub;
        const long long nwarps = pv::chan_job_warps(job);
        PV_TRY(pv::launch_chan_fast(h->nchan, pkt_bytes > 0 ? 2 : (in_int16 ? 1 : 0), nullptr, job, 1, nwarps,
                                    nullptr, s));
        h->cur ^= 1;
        h->have_hist = true;
        if (nu_out) *nu_out = nu;
        return PV_OK;
    }
    ChanArgs a{};
    a.in = d_in;
    a.in_int16 = in_int16;
    a.hist_in = h->have_hist ? h->d_hist[h->cur] : nullptr;
    a.hist_out = h->d_hist[h->cur ^ 1];
    a.coeffs = h->d_coeffs;
    a.twiddle = h->d_twiddle;
    a.nsub = nsub; a.npol = npol; a.nblocks = nblocks;
    a.N = h->nchan; a.T = h->ntaps; a.log2n = h->log2n; a.BT = bt;
    a.mode = mode; a.spectra = d_spectra; a.stokes = d_stokes;
    a.nstokes = nstokes; a.window = w; a.bin = bin; a.nu = nu;
    PV_CUDA(cudaFuncSetAttribute(channelise_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem), "cudaFuncSetAttribute(channelise)");
    dim3 grid((unsigned)pv::ceil_div(nblocks, bt), (unsigned)nsub);
    if (nsub > 65535) {
        pv::set_error("channelise: too many subbands");
        return PV_ERR_ARG;
    }
    channelise_kernel<<<grid, 256, smem, s>>>(a);
    PV_TRY(pv::check_launch("channelise_kernel"));
    if (h->ntaps > 1) {
        h->cur ^= 1;
        h->have_hist = true;
    }
    if (nu_out) *nu_out = nu;
    return PV_OK;
}

}  // namespace

namespace pv {
int ppf_tables(const pv_ppf* h, const float** d_coeffs, const float2** d_twiddle, int* nchan,
               int* ntaps) {
    if (!h) return PV_ERR_ARG;
    *d_coeffs = h->d_coeffs;
    *d_twiddle = h->d_twiddle;
    *nchan = h->nchan;
    *ntaps = h->ntaps;
    return PV_OK;
}
}  // namespace pv

extern "C" int pv_ppf_create(pv_ppf** out, int nchan, int ntaps, int window,
                             const float* h_coeffs) {
    // PPFChanneliser.cpp:42-44: one channel or an even number of them
    if (!out || nchan < 1 || (nchan != 1 && nchan % 2 != 0) || ntaps < 1 || nchan > 1024) {
        pv::set_error("PPFChanneliser: Number of channels needs to be even (1 or 2..1024, got %d)", nchan);
        return PV_ERR_CONFIG;
    }
    auto* h = new pv_ppf;
    h->nchan = nchan;
    h->ntaps = ntaps;
    const bool pow2 = (nchan & (nchan - 1)) == 0;
    while ((1 << h->log2n) < nchan) ++h->log2n;
    if (!pow2) h->log2n = -1;  // direct DFT
    if (nchan == 1) {
        // The time series is the spectrum (PPFChanneliser.cpp:108-131): no filter, no history.
        h->ntaps = 1;
        h->h_coeffs.assign(1, 1.0f);
    } else if (h_coeffs) {
        h->h_coeffs.assign(h_coeffs, h_coeffs + (size_t)nchan * ntaps);
    } else {
        std::vector<double> c;
        int rc = pv::fir_coefficients(ntaps, nchan, window, c);
        if (rc != PV_OK) { delete h; return rc; }
        h->h_coeffs.resize(c.size());
        for (size_t i = 0; i < c.size(); ++i) h->h_coeffs[i] = (float)c[i];  // PPFChanneliser.cpp:212-217
    }
    std::vector<float2> tw(std::max(1, pow2 ? nchan / 2 : nchan));
    for (int k = 0; k < (int)tw.size(); ++k) {
        const double ang = -2.0 * M_PI * k / nchan;
        tw[k] = make_float2((float)std::cos(ang), (float)std::sin(ang));
    }
    if (nchan % 4 == 0) tw[nchan / 4] = make_float2(0.0f, -1.0f);  // exactly -i (cos(pi/2) is not 0 in FP64)
    cudaError_t e = cudaMalloc(&h->d_coeffs, sizeof(float) * h->h_coeffs.size());
    if (e == cudaSuccess) e = cudaMalloc(&h->d_twiddle, sizeof(float2) * tw.size());
    if (e == cudaSuccess)
        e = cudaMemcpy(h->d_coeffs, h->h_coeffs.data(), sizeof(float) * h->h_coeffs.size(),
                       cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(h->d_twiddle, tw.data(), sizeof(float2) * tw.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        pv::set_error("pv_ppf_create: %s", cudaGetErrorString(e));
        if (h->d_coeffs) cudaFree(h->d_coeffs);
        if (h->d_twiddle) cudaFree(h->d_twiddle);
        delete h;
        return PV_ERR_CUDA;
    }
    *out = h;
    return PV_OK;
}

extern "C" void pv_ppf_destroy(pv_ppf* h) {
    if (!h) return;
    cudaFree(h->d_coeffs);
    cudaFree(h->d_twiddle);
    for (auto p : h->d_hist)
        if (p) cudaFree(p);
    delete h;
}

extern "C" int pv_ppf_coefficients(const pv_ppf* h, float* out) {
    if (!h || !out) return PV_ERR_ARG;
    std::copy(h->h_coeffs.begin(), h->h_coeffs.end(), out);
    return PV_OK;
}

extern "C" int pv_ppf_reset(pv_ppf* h) {
    if (!h) return PV_ERR_ARG;
    h->have_hist = false;
    for (auto p : h->d_hist)
        if (p) cudaMemset(p, 0, (size_t)h->nsub * h->npol * (h->ntaps - 1) * h->nchan * sizeof(float2));
    return PV_OK;
}

extern "C" int pv_ppf_run(pv_ppf* h, const float* d_in, int nsub, int npol, int nblocks,
                          float* d_out, void* stream) {
    return run_channelise(h, d_in, 0, nsub, npol, nblocks, 0, reinterpret_cast<float2*>(d_out),
                          nullptr, 1, 1, 1, nullptr, pv::as_stream(stream));
}

long long pv::ppf_state_bytes(const pv_ppf* h, int nsub, int npol) {
    return (long long)nsub * npol * (h->ntaps - 1) * h->nchan * (long long)sizeof(float2);
}

// Copies the tap history [sub][pol][T-1][N] (complex float) to or from host
// memory.  A channeliser that has run no block yet has an all-zero history.
int pv::ppf_state_io(pv_ppf* h, int nsub, int npol, void* h_buf, bool save, cudaStream_t s) {
    PV_TRY(prepare_history(h, nsub, npol, s));
    const size_t bytes = (size_t)ppf_state_bytes(h, nsub, npol);
    if (bytes == 0) return PV_OK;
    if (save) {
        if (!h->have_hist) {
            PV_CUDA(cudaStreamSynchronize(s), "synchronise");
            std::memset(h_buf, 0, bytes);
            return PV_OK;
        }
        PV_CUDA(cudaMemcpyAsync(h_buf, h->d_hist[h->cur], bytes, cudaMemcpyDeviceToHost, s), "save PPF history");
        return PV_OK;
    }
    PV_CUDA(cudaMemcpyAsync(h->d_hist[h->cur], h_buf, bytes, cudaMemcpyHostToDevice, s), "load PPF history");
    h->have_hist = true;
    return PV_OK;
}

int pv::channelise_stokes_i(pv_ppf* h, const void* d_in, int nsub, int nblocks, int window, int bin, float* d_stokes,
                            int* nu_out, long long pkt_bytes, int pkt_nsub, cudaStream_t s) {
    return run_channelise(h, d_in, 1, nsub, 2, nblocks, 1, nullptr, d_stokes, 1, window, bin, nu_out, s, pkt_bytes,
                          pkt_nsub);
}

extern "C" int pv_channelise(pv_ppf* h, const void* d_in, int in_int16, int nsub, int nblocks,
                             int nstokes, int window, int bin, float* d_stokes, int* nu_out,
                             void* stream) {
    return run_channelise(h, d_in, in_int16, nsub, 2, nblocks, 1, nullptr, d_stokes, nstokes,
                          window, bin, nu_out, pv::as_stream(stream));
}

extern "C" int pv_stokes(const float* d_spectra, int nt, int nsub, int nchan, int nstokes,
                         float* d_out, void* stream) {
    if (nstokes != 1 && nstokes != 4) {
        pv::set_error("StokesGenerator: You can either generate 1 or 4 Stokes parameters.");
        return PV_ERR_CONFIG;
    }
    if (!d_spectra || !d_out || nt < 0 || nsub <= 0 || nchan <= 0) {
        pv::set_error("pv_stokes: invalid arguments");
        return PV_ERR_ARG;
    }
    const long long n = (long long)nt * nsub * nchan;
    if (n == 0) return PV_OK;
    const int blocks = (int)std::min<long long>(pv::ceil_div<long long>(n, 256), pv::sm_count() * 16LL);
    stokes_kernel<<<blocks, 256, 0, pv::as_stream(stream)>>>(
        reinterpret_cast<const float2*>(d_spectra), nt, nsub, nchan, nstokes, d_out);
    return pv::check_launch("stokes_kernel");
}

extern "C" int pv_integrate(const float* d_in, int nt, int nsub, int npol, int nchan, int window,
                            int bin, float* d_out, int* nu_out, void* stream) {
    if (!d_in || !d_out || nt < 0 || nsub <= 0 || npol <= 0 || nchan <= 0 || window <= 0 ||
        bin <= 0 || nchan % bin != 0) {
        pv::set_error("pv_integrate: invalid arguments");
        return PV_ERR_ARG;
    }
    const int w = std::min(window, std::max(nt, 1));  // StokesIntegrator.cpp:53-59
    const int nu = nt / w;
    if (nu_out) *nu_out = nu;
    const long long n = (long long)nu * nsub * npol * (nchan / bin);
    if (n == 0) return PV_OK;
    const int blocks = (int)std::min<long long>(pv::ceil_div<long long>(n, 256), pv::sm_count() * 16LL);
    integrate_kernel<<<blocks, 256, 0, pv::as_stream(stream)>>>(d_in, nsub, npol, nchan, w, bin, nu,
                                                               d_out);
    return pv::check_launch("integrate_kernel");
}
