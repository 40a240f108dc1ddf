// K5: DedispersionAnalyser (lib/src/DedispersionAnalyser.cpp:30-203).
//
// For each DM row and each block of 2^P samples (a trailing partial block is
// dropped) the reference builds a dyadic boxcar tree, level n holding sums of
// 2^n samples formed as b_n[j] = b_{n-1}[2j] + b_{n-1}[2j+1] in FP32, and
// records every value at or above level n's threshold.  Events are listed
// after a dummy (0,0,1,0) by DM, block, level and position.
//
// One thread owns one (DM, block) pair: it loads the 2^P samples, builds the
// tree in registers with the reference's pairing (bit-identical sums) and
// counts its events.  An exclusive scan over the pairs in (DM, block) order
// gives every pair its output offset, and a second pass rebuilds the tree and
// writes the events in the reference order.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "pv_common.cuh"

namespace {

constexpr int kMaxPow2 = 8;

struct Thresholds {
    float v[kMaxPow2 + 1];
};

template <int P>
__device__ __forceinline__ void load_block(float (&b)[1 << P], const float* __restrict__ src,
                                           bool vec4) {
    constexpr int M = 1 << P;
    if (M >= 4 && vec4) {
        const float4* s4 = reinterpret_cast<const float4*>(src);
#pragma unroll
        for (int q = 0; q < M / 4; ++q) {
            const float4 v = __ldg(s4 + q);
            b[4 * q] = v.x; b[4 * q + 1] = v.y; b[4 * q + 2] = v.z; b[4 * q + 3] = v.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < M; ++j) b[j] = __ldg(src + j);
    }
}

// Level N of the tree: b[j] = b[2j] + b[2j+1] for j < 2^(P-N), then the
// threshold test; recursion keeps every index a compile-time constant so the
// block stays in registers.
template <int P, int N, typename F>
struct TreeLevel {
    __device__ __forceinline__ static void run(float (&b)[1 << P], const Thresholds& thr, F& emit) {
        constexpr int cur = (1 << P) >> N;
#pragma unroll
        for (int j = 0; j < cur; ++j) {
            b[j] = __fadd_rn(b[2 * j], b[2 * j + 1]);
            if (b[j] >= thr.v[N]) emit((1 << N) * j, 1 << N, b[j]);
        }
        TreeLevel<P, N + 1, F>::run(b, thr, emit);
    }
};
template <int P, typename F>
struct TreeLevel<P, P + 1, F> {
    __device__ __forceinline__ static void run(float (&)[1 << P], const Thresholds&, F&) {}
};

// Walks the tree of one block; calls emit(t_in_block, width, value) for each
// value at or above its threshold in the reference order.
template <int P, typename F>
__device__ __forceinline__ void walk_block(float (&b)[1 << P], const Thresholds& thr, F emit) {
    constexpr int M = 1 << P;
#pragma unroll
    for (int j = 0; j < M; ++j)
        if (b[j] >= thr.v[0]) emit(j, 1, b[j]);
    TreeLevel<P, 1, F>::run(b, thr, emit);
}

template <int P>
__global__ void analyse_count(const float* __restrict__ data, long long ld, int tdms, int nblocks,
                              Thresholds thr, bool vec4, int* __restrict__ counts) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long npairs = (long long)tdms * nblocks;
    if (g >= npairs) return;
    const int dm = (int)(g / nblocks), i = (int)(g % nblocks);
    float b[1 << P];
    load_block<P>(b, data + dm * ld + (long long)i * (1 << P), vec4);
    int n = 0;
    walk_block<P>(b, thr, [&](int, int, float) { ++n; });
    counts[g] = n;
}

template <int P>
__global__ void analyse_emit(const float* __restrict__ data, long long ld, int tdms, int nblocks,
                             Thresholds thr, bool vec4, const int* __restrict__ counts,
                             const long long* __restrict__ offsets, pv_event* __restrict__ ev,
                             long long cap) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (g == 0 && cap > 0) ev[0] = pv_event{0, 0, 1.0f, 0.0f};
    const long long npairs = (long long)tdms * nblocks;
    if (g >= npairs || counts[g] == 0) return;
    const int dm = (int)(g / nblocks), i = (int)(g % nblocks);
    float b[1 << P];
    load_block<P>(b, data + dm * ld + (long long)i * (1 << P), vec4);
    long long o = 1 + offsets[g];
    const int base = i * (1 << P);
    walk_block<P>(b, thr, [&](int t, int w, float v) {
        if (o < cap) ev[o] = pv_event{dm, base + t, (float)w, v};
        ++o;
    });
}

// ---------------------------------------------------------------------------
// Exclusive scan of n values into long long offsets (1024 per block, block
// totals scanned recursively).
// ---------------------------------------------------------------------------
constexpr int kScanBlock = 1024;

template <typename T>
__global__ void scan_block(const T* __restrict__ in, long long* __restrict__ out,
                           long long* __restrict__ block_sums, long long n) {
    __shared__ long long warp_tot[32];
    const long long g = blockIdx.x * (long long)kScanBlock + threadIdx.x;
    const long long v = g < n ? (long long)in[g] : 0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        long long w = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_tot[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    const long long before = warp == 0 ? 0 : warp_tot[warp - 1];
    if (g < n) out[g] = before + x - v;
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = warp_tot[31];
}

__global__ void scan_add(long long* __restrict__ out, const long long* __restrict__ block_off,
                         long long n) {
    const long long g = blockIdx.x * (long long)kScanBlock + threadIdx.x;
    if (g < n && blockIdx.x > 0) out[g] += block_off[blockIdx.x];
}

// total = 1 (the dummy) + events of every (DM, block) pair
__global__ void analyse_total(const int* __restrict__ counts, const long long* __restrict__ offsets,
                              long long npairs, long long* __restrict__ total) {
    *total = npairs > 0 ? 1 + offsets[npairs - 1] + counts[npairs - 1] : 1;
}

// Block sums and their scans of every level of the scan of n values.
constexpr long long scan_workspace(long long n) {
    return n > 1 ? 2 * ((n + kScanBlock - 1) / kScanBlock) + scan_workspace((n + kScanBlock - 1) / kScanBlock)
                 : 0;
}

// Scratch bytes of the analyser for npairs (trial, block) pairs: per-pair
// counts and offsets, the scan workspace and two totals, rounded to 256.
constexpr size_t scratch_bytes_for(long long npairs) {
    return (((size_t)(npairs > 1 ? npairs : 1) * (sizeof(int) + sizeof(long long)) +
             (size_t)(scan_workspace(npairs > 1 ? npairs : 1) + 2) * sizeof(long long) + 256) + 255) /
           256 * 256;
}

// Exclusive scan of in[0..n) into out; ws holds scan_workspace(n) values.
template <typename T>
int exclusive_scan(const T* in, long long* out, long long n, long long* ws, cudaStream_t s) {
    const long long nb = pv::ceil_div<long long>(n, kScanBlock);
    long long* sums = ws;
    long long* sums_scan = ws + nb;
    scan_block<T><<<(unsigned)nb, kScanBlock, 0, s>>>(in, out, sums, n);
    PV_TRY(pv::check_launch("scan_block"));
    if (nb > 1) {
        PV_TRY(exclusive_scan<long long>(sums, sums_scan, nb, ws + 2 * nb, s));
        scan_add<<<(unsigned)nb, kScanBlock, 0, s>>>(out, sums_scan, n);
        PV_TRY(pv::check_launch("scan_add"));
    }
    return PV_OK;
}

template <int P>
int run_analyse(const float* data, long long ld, int tdms, int nsamp, const Thresholds& thr,
                pv_event* ev, long long cap, long long* d_total, int* counts, long long* offsets,
                long long* ws, cudaStream_t s) {
    const int nblocks = nsamp >> P;
    const long long npairs = (long long)tdms * nblocks;
    const bool vec4 = (ld % 4 == 0) && ((reinterpret_cast<uintptr_t>(data) & 15) == 0);
    const int threads = 128;
    if (npairs > 0) {
        const unsigned blocks = (unsigned)pv::ceil_div<long long>(npairs, threads);
        analyse_count<P><<<blocks, threads, 0, s>>>(data, ld, tdms, nblocks, thr, vec4, counts);
        PV_TRY(pv::check_launch("analyse_count"));
        PV_TRY(exclusive_scan<int>(counts, offsets, npairs, ws, s));
        analyse_emit<P><<<blocks, threads, 0, s>>>(data, ld, tdms, nblocks, thr, vec4, counts,
                                                   offsets, ev, cap);
        PV_TRY(pv::check_launch("analyse_emit"));
    } else if (cap > 0) {
        analyse_emit<P><<<1, 32, 0, s>>>(data, ld, tdms, 0, thr, false, counts, offsets, ev, cap);
        PV_TRY(pv::check_launch("analyse_emit"));
    }
    analyse_total<<<1, 1, 0, s>>>(counts, offsets, npairs, d_total);
    return pv::check_launch("analyse_total");
}

}  // namespace

namespace pv {

// Scratch bytes the analyser needs for tdms x nsamp at 2^bin_pow2 blocks.
size_t analyse_scratch_bytes(int tdms, int nsamp, int bin_pow2) {
    // rounded to 256 bytes: keeps anything placed after it aligned
    return scratch_bytes_for((long long)tdms * (nsamp >> bin_pow2));
}

// Analyser with caller-provided scratch (analyse_scratch_bytes bytes);
// asynchronous: the event total (dummy included) lands in *d_total.
int analyse_launch(const float* data, long long ld, int tdms, int nsamp, float threshold,
                   float rms, int bin_pow2, pv_event* ev, long long cap, long long* d_total,
                   void* scratch, cudaStream_t s) {
    Thresholds thr{};
    PV_TRY(pv_analyser_thresholds(threshold, rms, bin_pow2, thr.v));
    const long long npairs = std::max<long long>((long long)tdms * (nsamp >> bin_pow2), 1);
    char* p = static_cast<char*>(scratch);
    long long* offsets = reinterpret_cast<long long*>(p);
    p += npairs * sizeof(long long);
    long long* ws = reinterpret_cast<long long*>(p);
    p += (scan_workspace(npairs) + 2) * sizeof(long long);
    int* counts = reinterpret_cast<int*>(p);
    switch (bin_pow2) {
#define PV_CASE(P) \
    case P: return run_analyse<P>(data, ld, tdms, nsamp, thr, ev, cap, d_total, counts, offsets, ws, s);
        PV_CASE(0) PV_CASE(1) PV_CASE(2) PV_CASE(3) PV_CASE(4) PV_CASE(5) PV_CASE(6) PV_CASE(7)
        PV_CASE(8)
#undef PV_CASE
        default:
            set_error("pv_analyse: power2ForBinning must be in 0..%d", kMaxPow2);
            return PV_ERR_ARG;
    }
}

}  // namespace pv

extern "C" int pv_analyser_thresholds(float threshold, float rms, int bin_pow2, float* h_thr) {
    if (bin_pow2 < 0 || bin_pow2 > kMaxPow2 || !h_thr) {
        pv::set_error("pv_analyser_thresholds: power2ForBinning must be in 0..%d", kMaxPow2);
        return PV_ERR_ARG;
    }
    // Level 0 is the float product; wider boxcars multiply it by ::sqrt of
    // the (float) width in double and round once (DedispersionAnalyser.cpp:121).
    const float base = threshold * rms;
    h_thr[0] = base;
    for (int n = 1; n <= bin_pow2; ++n)
        h_thr[n] = (float)((double)base * std::sqrt((double)(float)(1u << n)));
    return PV_OK;
}

extern "C" int pv_analyse(const float* d_data, long long ld, int tdms, int nsamp, float threshold,
                          float rms, int bin_pow2, pv_event* d_events, long long cap,
                          long long* h_count, void* stream) {
    if (!h_count || tdms < 0 || nsamp < 0 || ld < nsamp || (cap > 0 && !d_events) ||
        (tdms > 0 && nsamp > 0 && !d_data)) {
        pv::set_error("pv_analyse: invalid arguments");
        return PV_ERR_ARG;
    }
    if (bin_pow2 < 0 || bin_pow2 > kMaxPow2) {
        pv::set_error("pv_analyse: power2ForBinning must be in 0..%d", kMaxPow2);
        return PV_ERR_ARG;
    }
    cudaStream_t s = pv::as_stream(stream);
    void* scratch = nullptr;
    PV_TRY(pv::scratch_alloc(&scratch, pv::analyse_scratch_bytes(tdms, nsamp, bin_pow2) + 64, s));
    long long* d_total = reinterpret_cast<long long*>(static_cast<char*>(scratch) +
                                                      pv::analyse_scratch_bytes(tdms, nsamp, bin_pow2));
    int rc = pv::analyse_launch(d_data, ld, tdms, nsamp, threshold, rms, bin_pow2, d_events, cap,
                                d_total, scratch, s);
    if (rc == PV_OK) {
        rc = pv::cuda_status(cudaMemcpyAsync(h_count, d_total, sizeof(long long),
                                             cudaMemcpyDeviceToHost, s), "read event count");
        if (rc == PV_OK) rc = pv::cuda_status(cudaStreamSynchronize(s), "synchronise");
    }
    pv::scratch_free(scratch, s);
    return rc;
}

// ---------------------------------------------------------------------------
// pv_analyse_noalloc: the analyser with its scratch in a fixed device array
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kNoAllocPairs = PV_ANALYSE_NOALLOC_MAX_PAIRS;
// the same formula as pv_analyse's scratch at the largest pair count: a call
// within the pair limit always fits
constexpr size_t kNoAllocScratch = scratch_bytes_for((long long)kNoAllocPairs);
static_assert(scratch_bytes_for((long long)kNoAllocPairs) >= scratch_bytes_for((long long)kNoAllocPairs - 1),
              "scratch grows with the pair count");
// Scratch (counts, offsets, scan workspace) followed by the event total.
// Every GPU that loads the library keeps this array until the process exits.
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratch + 256];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.  The host-side
// name is only a stand-in, so the address is looked up once per device with
// that device current.
int noalloc_scratch(void** out) {
    int dev = 0;
    PV_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) {
        pv::set_error("pv_analyse_noalloc: device %d out of range", dev);
        return PV_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            pv::set_error("pv_analyse_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return PV_ERR_CUDA;
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return PV_OK;
}

}  // namespace

extern "C" int pv_analyse_noalloc(const float* d_data, long long ld, int tdms, int nsamp,
                                  float threshold, float rms, int bin_pow2, pv_event* d_events,
                                  long long cap, long long* h_count, void* stream) {
    if (!h_count || tdms < 0 || nsamp < 0 || ld < nsamp || (cap > 0 && !d_events) ||
        (tdms > 0 && nsamp > 0 && !d_data)) {
        pv::set_error("pv_analyse_noalloc: invalid arguments");
        return PV_ERR_ARG;
    }
    if (bin_pow2 < 0 || bin_pow2 > kMaxPow2) {
        pv::set_error("pv_analyse_noalloc: power2ForBinning must be in 0..%d", kMaxPow2);
        return PV_ERR_ARG;
    }
    const long long pairs = (long long)tdms * (nsamp >> bin_pow2);
    if (pairs > (long long)kNoAllocPairs) {
        pv::set_error("pv_analyse_noalloc: %d trials x %d blocks of 2^%d samples = %lld pairs "
                      "exceeds the fixed scratch limit of %lld pairs; use pv_analyse",
                      tdms, nsamp >> bin_pow2, bin_pow2, pairs, (long long)kNoAllocPairs);
        return PV_ERR_ARG;
    }
    void* scratch = nullptr;
    PV_TRY(noalloc_scratch(&scratch));
    // Nothing in the scratch needs clearing: the launch writes every count,
    // offset, workspace entry and the total before it reads them.
    long long* d_total = reinterpret_cast<long long*>(static_cast<char*>(scratch) + kNoAllocScratch);
    cudaStream_t s = pv::as_stream(stream);
    PV_TRY(pv::analyse_launch(d_data, ld, tdms, nsamp, threshold, rms, bin_pow2, d_events, cap,
                              d_total, scratch, s));
    PV_CUDA(cudaMemcpyAsync(h_count, d_total, sizeof(long long), cudaMemcpyDeviceToHost, s),
            "read event count");
    PV_CUDA(cudaStreamSynchronize(s), "synchronise");
    return PV_OK;
}
