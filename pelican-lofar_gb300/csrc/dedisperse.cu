// K0 delay table and K4 brute-force dedispersion for sm_103a.
//
// out[d][t] = sum_{c=0..nchan-1} in[c][t + shift(c,d)]
// (lib/DedispersionKernel.cu:15-50).  Each output is accumulated in one
// register in channel order 0..nchan-1 with plain FP32 adds, the same order
// as the reference kernel, so results are bit-identical to it.
//
// Tiling.  A CTA owns DMS consecutive trials (one warp each) and a time tile
// of 32*R samples (lane l holds samples l, l+32, ...).  Channels are streamed
// through shared memory CS at a time, double buffered with cp.async: for
// channel c the CTA needs in[c][t0 + s(c,d0) .. t0 + s(c,d_last) + 32R),
// whose length is 32R plus the delay spread of the tile's trials at c; that
// spread is bounded on the host (delay_spread) and sizes the slot.  Every
// shared-memory read of a warp is 32 consecutive words, so the loop has no
// bank conflicts; the kernel is bounded by shared-memory bandwidth
// (one 4-byte read per add).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <map>
#include <vector>

#include <cuda_fp16.h>

#include "pv_internal.cuh"

namespace {

// ---------------------------------------------------------------------------
// K0: delay table
// ---------------------------------------------------------------------------
__global__ void delay_table_kernel(int* __restrict__ shifts, const float* __restrict__ dmshift,
                                   int nchan, int tdms, float start, float step) {
    const long long n = (long long)nchan * tdms;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int d = (int)(i / nchan), c = (int)(i % nchan);
        shifts[i] = pv_shift(dmshift[c], pv_trial_value(d, start, step));
    }
}

// ---------------------------------------------------------------------------
// K4: dedispersion
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async4(float* smem_dst, const float* gmem_src) {
    const unsigned dst = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(gmem_src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

struct DedispArgs {
    float* out;
    long long out_stride;
    const float* in;
    long long row_stride;
    long long row_len;   // linear mode: valid samples per row
    long long ring_len;  // ring mode (> 0): rows are rings of ring_len samples
    long long t_base;    // ring mode: physical position of output sample 0
    const float* dmshift;
    int nchan, nout, tdms;
    float start, step;
    int slot;  // floats per channel slot in shared memory
    unsigned long long wait_ns;  // limit of each pipeline wait
    int stall;                   // failure-path test: the first stage's copies are withheld
};

template <int DMS, int R, int CS>
__global__ void __launch_bounds__(DMS * 32)
dedisperse_kernel(const DedispArgs a) {
    extern __shared__ float smem[];
    constexpr int NT = DMS * 32;
    constexpr int TT = 32 * R;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long t0 = (long long)blockIdx.x * TT;
    const int d0 = blockIdx.y * DMS;
    const int d_last = min(d0 + DMS, a.tdms) - 1;
    const int d = d0 + warp;
    const float dv0 = pv_trial_value(d0, a.start, a.step);
    const float dv_last = pv_trial_value(d_last, a.start, a.step);
    const float dv = pv_trial_value(d, a.start, a.step);

    // Issues the copies of channels [c_begin, c_begin+CS) into buffer b.
    auto load_stage = [&](int c_begin, float* buf) {
        const int c_end = min(c_begin + CS, a.nchan);
        for (int c = c_begin; c < c_end; ++c) {
            const float k = a.dmshift[c];
            const int s0 = pv_shift(k, dv0);
            // Samples the tile's stored outputs need: the last tile may be short.
            const int valid = (int)min((long long)TT, (long long)a.nout - t0);
            const int span = min(valid + pv_shift(k, dv_last) - s0, a.slot);
            const float* src = a.in + (long long)c * a.row_stride;
            float* dst = buf + (c - c_begin) * a.slot;
            if (a.ring_len > 0) {
                // Ring rows: positions wrap modulo ring_len (span <= ring_len).
                long long g0 = (a.t_base + t0 + s0) % a.ring_len;
                for (int j = threadIdx.x; j < span; j += NT) {
                    long long g = g0 + j;
                    if (g >= a.ring_len) g -= a.ring_len;
                    cp_async4(dst + j, src + g);
                }
            } else {
                // Contiguous rows (row_len == row_stride, the DedispersionBuffer
                // layout) read on into the next row as the reference kernel
                // does; only reads past the whole buffer become zeros.
                const long long g0 = t0 + s0;
                const long long lim = a.row_len == a.row_stride
                                          ? (long long)(a.nchan - c) * a.row_stride
                                          : a.row_len;
                for (int j = threadIdx.x; j < span; j += NT) {
                    const long long g = g0 + j;
                    if (g < lim) cp_async4(dst + j, src + g);
                    else dst[j] = 0.0f;
                }
            }
        }
    };

    float acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = 0.0f;

    const int nstages = (a.nchan + CS - 1) / CS;
    load_stage(0, smem);
    cp_async_commit();
    for (int st = 0; st < nstages; ++st) {
        if (st + 1 < nstages) {
            load_stage((st + 1) * CS, smem + ((st + 1) & 1) * CS * a.slot);
            cp_async_commit();
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const float* buf = smem + (st & 1) * CS * a.slot;
        const int c_begin = st * CS;
        const int c_end = min(c_begin + CS, a.nchan);
        if (d <= d_last) {
            for (int c = c_begin; c < c_end; ++c) {
                const float k = a.dmshift[c];
                // off <= slot - TT by the host's spread bound; the clamp keeps
                // every read inside the slot regardless.
                const int off = min(pv_shift(k, dv) - pv_shift(k, dv0), a.slot - TT);
                const float* row = buf + (c - c_begin) * a.slot + off + lane;
#pragma unroll
                for (int r = 0; r < R; ++r) acc[r] = __fadd_rn(acc[r], row[32 * r]);
            }
        }
        __syncthreads();
    }
    if (d <= d_last) {
        float* o = a.out + (long long)d * a.out_stride;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const long long t = t0 + lane + 32 * r;
            if (t < a.nout) o[t] = acc[r];
        }
    }
}

// ---------------------------------------------------------------------------
// K4 v2 (ring rows): TMA bulk copies into an mbarrier pipeline.
//
// Warp DMS is a producer: for every stage of CS channels it waits until the
// consumers have released the stage buffer, posts the byte count on the
// stage's "full" barrier and issues one cp.async.bulk per channel span (two
// where the span wraps the ring).  Warps 0..DMS-1 are consumers (one trial
// each): they wait on "full", add 32*R samples per channel from shared
// memory in channel order and release the buffer on "empty".  Span starts are
// rounded down to 16 bytes; the rounding offset is folded into the per-channel
// offset table the producer writes beside the data.  Every wait is bounded by
// %globaltimer; a wait that gives up records PV_ERR_TIMEOUT in *status.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes) : "memory");
}
// A waiting thread sleeps until the phase completes or for up to 100 us
// (the suspend-time hint) instead of polling: a warp that waits for a stage
// or a free slot issues no instructions meanwhile.
constexpr unsigned kSuspendHintNs = 100000u;
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok) : "r"(smem_u32(bar)), "r"(parity), "n"(kSuspendHintNs) : "memory");
    return ok != 0;
}
// Whole-warp wait for the phase of the given parity.  Every lane observes the
// completion itself (acquire), and the give-up decision comes from lane 0's
// clock, so the warp leaves the wait together.  Gives up after limit_ns.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, unsigned parity, unsigned long long limit_ns) {
    const unsigned long long t_end = global_ns() + limit_ns;
    bool done = false;
    for (;;) {
        if (!done) done = mbar_try_wait(bar, parity);
        if (__all_sync(0xffffffffu, done)) return true;
        const bool expired = __shfl_sync(0xffffffffu, global_ns() > t_end, 0);
        if (expired) return false;
    }
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}


template <int DMS, int R, int CS, int ST>
__global__ void __launch_bounds__((DMS + 1) * 32, 1)
dedisperse_tma_kernel(const DedispArgs a, int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int TT = 32 * R;
    float* slots = reinterpret_cast<float*>(smem_raw);
    int* meta_off = reinterpret_cast<int*>(slots + (size_t)ST * CS * a.slot);
    float* meta_k = reinterpret_cast<float*>(meta_off + ST * CS);
    // slot is a multiple of 4 floats and 2*ST*CS words follow: 8-byte aligned
    uint64_t* full = reinterpret_cast<uint64_t*>(meta_k + ST * CS);
    uint64_t* empty = full + ST;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long long t0 = (long long)blockIdx.x * TT;
    const int d0 = blockIdx.y * DMS;
    const int d_last = min(d0 + DMS, a.tdms) - 1;
    const float dv0 = pv_trial_value(d0, a.start, a.step);
    const float dv_last = pv_trial_value(d_last, a.start, a.step);
    const int nstages = (a.nchan + CS - 1) / CS;

    __shared__ int s_abort;
    if (threadIdx.x == 0) {
        // a launch in which some CTA already gave up stops here
        s_abort = *(volatile int*)status;
        for (int b = 0; b < ST; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], DMS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    __syncthreads();
    if (s_abort != 0) return;

    if (warp == DMS) {
        // ---------------- producer ----------------
        const int valid = (int)min((long long)TT, (long long)a.nout - t0);
        int issued = 0;
        bool ok = true;
        for (int st = 0; st < nstages && ok; ++st) {
            const int b = st % ST;
            const unsigned round = (unsigned)(st / ST);
            if (!mbar_wait_warp(&empty[b], (round & 1u) ^ 1u, a.wait_ns)) {
                if (lane == 0) atomicExch(status, PV_ERR_TIMEOUT);
                ok = false;
                break;
            }
            if (a.stall && st == 0) {  // nothing completes this stage: its consumers' wait runs out
                issued = st + 1;
                continue;
            }
            const int c = st * CS + lane;
            unsigned bytes = 0, piece1 = 0, piece2 = 0;
            long long g_al = 0;
            if (lane < CS && c < a.nchan) {
                const float k = a.dmshift[c];
                const int s0 = pv_shift(k, dv0);
                const int span = valid + pv_shift(k, dv_last) - s0;
                const long long g0 = (a.t_base + t0 + s0) % a.ring_len;
                g_al = g0 & ~3LL;
                const int base = (int)(g0 - g_al);
                const unsigned n = (unsigned)((base + span + 3) & ~3);
                piece1 = (unsigned)min((long long)n, a.ring_len - g_al);
                piece2 = n - piece1;
                bytes = n * 4u;
                meta_off[b * CS + lane] = s0 - base;
                meta_k[b * CS + lane] = k;
                __threadfence_block();
            }
            unsigned total = bytes;
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
            __syncwarp();
            if (lane == 0) mbar_arrive_expect_tx(&full[b], total);
            __syncwarp();
            if (bytes) {
                const float* src = a.in + (long long)c * a.row_stride;
                float* dst = slots + (size_t)(b * CS + lane) * a.slot;
                bulk_g2s(dst, src + g_al, piece1 * 4u, &full[b]);
                if (piece2) bulk_g2s(dst + piece1, src, piece2 * 4u, &full[b]);
            }
            issued = st + 1;
        }
        // Before the producer leaves, its last copies have landed (bounded):
        // consumers that give up return at once, and the CTA's shared memory
        // must not be released under copies in flight.
        (void)ok;
        for (int st = max(0, issued - ST); st < issued; ++st)
            if (!(a.stall && st == 0))  // the withheld stage has no copies in flight
                mbar_wait_warp(&full[st % ST], (unsigned)(st / ST) & 1u, pv::kDrainWaitNs);
        return;
    }

    // ---------------- consumers ----------------
    const int d = d0 + warp;
    const bool active = d <= d_last;
    const float dv = pv_trial_value(d, a.start, a.step);
    float acc[R];
#pragma unroll
    for (int r = 0; r < R; ++r) acc[r] = 0.0f;
    bool ok = true;
    for (int st = 0; st < nstages; ++st) {
        const int b = st % ST;
        if (!mbar_wait_warp(&full[b], (unsigned)(st / ST) & 1u, a.wait_ns)) {
            if (lane == 0) atomicExch(status, PV_ERR_TIMEOUT);
            ok = false;
            break;
        }
        if (active) {
            const int c_end = min(CS, a.nchan - st * CS);
            // lane j computes channel j's row offset once per stage; the warp
            // takes it by shuffle (no shared-memory wavefront per channel)
            const int my_off =
                lane < c_end ? min(pv_shift(meta_k[b * CS + lane], dv) - meta_off[b * CS + lane], a.slot - TT) : 0;
            for (int j = 0; j < c_end; ++j) {
                const int off = __shfl_sync(0xffffffffu, my_off, j);
                const float* row = slots + (size_t)(b * CS + j) * a.slot + off + lane;
#pragma unroll
                for (int r = 0; r < R; ++r) acc[r] = __fadd_rn(acc[r], row[32 * r]);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[b]);
    }
    if (ok && active) {
        float* o = a.out + (long long)d * a.out_stride;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const long long t = t0 + lane + 32 * r;
            if (t < a.nout) o[t] = acc[r];
        }
    }
}

// ---------------------------------------------------------------------------
// K4 batched (ring rows of many beams): one persistent launch works through a
// list of (beam, DM tile, time tile) tiles taken from a global counter, so
// beams of any channel count, trial count and delay range share the GPU in
// one launch.  The pipeline is the one of dedisperse_tma_kernel and runs on
// across tile boundaries: the producer warp takes the next tile, records it
// beside the tile's first stage and streams its channel spans; consumers
// learn the tile from that record when the stage arrives.  A beam's DM tile
// height (1..16 trials, one warp each) is chosen on the host so that its
// delay spread fits the launch's channel slot; warps above it idle on that
// beam's tiles.  Only beams whose BeamStep selects a window this step are
// dedispersed (window w reads ring columns from w*chunk on).  All waits are
// bounded as in dedisperse_tma_kernel.
// ---------------------------------------------------------------------------
// Packed FP32 pairs (Blackwell fma .f32x2): two independent IEEE
// operations, each rounded as the scalar one.
__device__ __forceinline__ unsigned long long f2_pack(float lo, float hi) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long v) {
    float2 f;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(f.x), "=f"(f.y) : "l"(v));
    return f;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// Mixed-precision add (sm_100+): float(h) + a with one rounding, h an FP16 bit pattern
__device__ __forceinline__ float add_f16(unsigned short h, float a) {
    float r;
    asm("add.rn.f32.f16 %0, %1, %2;" : "=f"(r) : "h"(h), "f"(a));
    return r;
}
__device__ __forceinline__ void f16_halves(unsigned w, unsigned short& lo, unsigned short& hi) {
    asm("mov.b32 {%0, %1}, %2;" : "=h"(lo), "=h"(hi) : "r"(w));
}
// byte i of w as float (q - 128): 0x4B0000qq is 2^23 + q exactly
__device__ __forceinline__ float u8_centered(unsigned w, int i) {
    return __int_as_float((int)__byte_perm(w, 0x4B000000u, 0x7540u | (unsigned)i)) - 8388736.0f;
}

// Ring storage of the batched kernel: element bytes and TMA alignment unit.
template <int STORE>
struct Store {
    static constexpr int E = STORE == PV_STORE_F32 ? 4 : (STORE == PV_STORE_F16 ? 2 : 1);
    static constexpr int AU = 16 / E;  // elements per 16 bytes
};

// The producer warp of the batched kernels: takes (beam, DM tile, time tile)
// tiles of beams that dedisperse a window this step from the global counter,
// records each tile beside its first stage and streams the tile's channel
// spans (TT samples plus the tile's delay spread) into the stage slots with
// bulk copies, CS channels per stage, ST stages in flight.  Waits are
// bounded; the last copies have landed before it returns.
template <int TT, int CS, int ST, int STORE>
__device__ __forceinline__ void batch_producer(const pv::DdJob* __restrict__ jobs,
                                               const pv::DdTile* __restrict__ tiles, int ntiles, int slot,
                                               int* __restrict__ counter, const pv::BeamStep* __restrict__ bs,
                                               int* __restrict__ status, unsigned long long wait_ns,
                                               unsigned char* slots, int* meta_off, float* meta_k,
                                               float* meta_sc, int* s_first, uint64_t* full, uint64_t* empty,
                                               int lane) {
    constexpr int E = Store<STORE>::E, AU = Store<STORE>::AU;
    unsigned gs = 0;
    bool ok = true, sentinel = false;
    for (;;) {
        int tile = -1;  // next tile of a beam that has a window at this step
        for (;;) {
            int t = 0;
            if (lane == 0) t = atomicAdd(counter, 1);
            t = __shfl_sync(0xffffffffu, t, 0);
            if (t >= ntiles) break;
            if (bs[jobs[tiles[t].job].beam].sel) {
                tile = t;
                break;
            }
        }
        const int b_first = gs % ST;
        if (!mbar_wait_warp(&empty[b_first], ((gs / ST) & 1u) ^ 1u, wait_ns)) {
            if (lane == 0) atomicExch(status, PV_ERR_TIMEOUT);
            ok = false;
            break;
        }
        if (tile < 0) {  // no work left: release the consumers
            if (lane == 0) {
                s_first[b_first] = -1;
                mbar_arrive(&full[b_first]);
            }
            sentinel = true;
            break;
        }
        const pv::DdTile tt = tiles[tile];
        const pv::DdJob& J = jobs[tt.job];
        const int d_last = min(tt.d0 + J.dms, J.tdms) - 1;
        const float dv0 = pv_trial_value(tt.d0, J.start, J.step);
        const float dv_last = pv_trial_value(d_last, J.start, J.step);
        const int valid = min(TT, J.nout - tt.t0);
        const long long t_base = (bs[J.beam].window * J.chunk) % J.ring_len;
        const int nst = (J.nchan + CS - 1) / CS;
        const unsigned char* ring = reinterpret_cast<const unsigned char*>(J.ring);
        for (int st = 0; st < nst; ++st) {
            const int b = gs % ST;
            if (st > 0 && !mbar_wait_warp(&empty[b], ((gs / ST) & 1u) ^ 1u, wait_ns)) {
                if (lane == 0) atomicExch(status, PV_ERR_TIMEOUT);
                ok = false;
                break;
            }
            if (st == 0 && lane == 0) s_first[b] = tile;
            const int c = st * CS + lane;
            unsigned bytes = 0, piece1 = 0, piece2 = 0;
            long long g_al = 0;
            if (lane < CS && c < J.nchan) {
                const float k = J.dmshift[c];
                const int s0 = pv_shift(k, dv0);
                const int span = valid + pv_shift(k, dv_last) - s0;
                const long long g0 = (t_base + tt.t0 + s0) % J.ring_len;
                g_al = g0 & ~(long long)(AU - 1);
                const int base = (int)(g0 - g_al);
                const unsigned n = (unsigned)((base + span + AU - 1) & ~(AU - 1));
                piece1 = (unsigned)min((long long)n, J.ring_len - g_al);
                piece2 = n - piece1;
                bytes = n * (unsigned)E;
                meta_off[b * CS + lane] = s0 - base;
                meta_k[b * CS + lane] = k;
                if (STORE == PV_STORE_U8) meta_sc[b * CS + lane] = J.scale[c];
            }
            __threadfence_block();
            unsigned total = bytes;
#pragma unroll
            for (int o = 16; o >= 1; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
            __syncwarp();
            if (lane == 0) mbar_arrive_expect_tx(&full[b], total);
            __syncwarp();
            if (bytes) {
                const unsigned char* src = ring + (long long)c * J.row_stride * E;
                unsigned char* dst = slots + (size_t)(b * CS + lane) * slot * E;
                bulk_g2s(dst, src + g_al * E, piece1 * (unsigned)E, &full[b]);
                if (piece2) bulk_g2s(dst + (size_t)piece1 * E, src, piece2 * (unsigned)E, &full[b]);
            }
            ++gs;
        }
        if (!ok) break;
    }
    // The last copies have landed (bounded) before the producer leaves.  The
    // end-of-work record re-armed the slot of stage gs - ST, whose copies had
    // landed before its consumers released the slot: that stage is skipped
    // (its barrier's parity now names the newer phase).
    (void)ok;
    unsigned g0 = gs > (unsigned)ST ? gs - ST : 0;
    if (sentinel && gs >= (unsigned)ST) g0 = gs - ST + 1;
    for (unsigned g = g0; g < gs; ++g)
        mbar_wait_warp(&full[g % ST], (g / ST) & 1u, pv::kDrainWaitNs);
}

template <int R, int CS, int ST, int STORE>
__global__ void __launch_bounds__(17 * 32, 1)
dedisperse_batch_kernel(const pv::DdJob* __restrict__ jobs, const pv::DdTile* __restrict__ tiles,
                        int ntiles, int slot, int* __restrict__ counter,
                        const pv::BeamStep* __restrict__ bs, int* __restrict__ status,
                        unsigned long long wait_ns) {
    constexpr int DMS = 16;
    constexpr int TT = 32 * R;
    constexpr int E = Store<STORE>::E, AU = Store<STORE>::AU;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* slots = smem_raw;  // [ST*CS][slot] elements of E bytes
    int* meta_off = reinterpret_cast<int*>(slots + (size_t)ST * CS * slot * E);
    float* meta_k = reinterpret_cast<float*>(meta_off + ST * CS);
    float* meta_sc = meta_k + ST * CS;
    int* s_first = reinterpret_cast<int*>(meta_sc + ST * CS);  // [2*ST], ST used
    uint64_t* full = reinterpret_cast<uint64_t*>(s_first + 2 * ST);
    uint64_t* empty = full + ST;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    __shared__ int s_abort;
    if (threadIdx.x == 0) {
        s_abort = *(volatile int*)status;
        for (int b = 0; b < ST; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], DMS);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    __syncthreads();
    if (s_abort != 0) return;

    if (warp == DMS) {
        batch_producer<TT, CS, ST, STORE>(jobs, tiles, ntiles, slot, counter, bs, status, wait_ns, slots,
                                         meta_off, meta_k, meta_sc, s_first, full, empty, lane);
        return;
    }

    // ---------------- consumers ----------------
    // FP32 rows: lane l adds samples l + 32r.  FP16 rows: lane l adds samples
    // 2l, 2l+1 (+64p) from one 4-byte word, or from two when the row offset is
    // odd.  u8 rows: lane l adds samples 4l..4l+3 (+128q) from one word, or a
    // funnel shift of two when the offset is not a multiple of 4; a byte q
    // stands for (q - 128) * scale + offset of its channel, the offsets of all
    // channels being added once per output.  When every row of the beam has
    // the same scale, the codes themselves are summed exactly as integers:
    // bytes 0 and 2 (1 and 3) of a word go to the two 16-bit halves of one
    // register, which take 257 codes before a carry could cross, so the
    // halves move into 32-bit sums every 256 channels; the output is then
    // scale * (sum - 128 * nchan) + offset sum.
    unsigned gs = 0;
    for (;;) {
        const int b0 = gs % ST;
        if (!mbar_wait_warp(&full[b0], (gs / ST) & 1u, wait_ns)) {
            if (lane == 0) atomicExch(status, PV_ERR_TIMEOUT);
            return;
        }
        const int tile = *(volatile int*)&s_first[b0];
        if (tile < 0) return;
        const pv::DdTile tt = tiles[tile];
        const pv::DdJob& J = jobs[tt.job];
        const int d = tt.d0 + warp;
        const int d_last = min(tt.d0 + J.dms, J.tdms) - 1;
        const bool active = warp < J.dms && d <= d_last;
        const float dv = pv_trial_value(d, J.start, J.step);
        const int nchan = J.nchan;
        const int nst = (nchan + CS - 1) / CS;
        if (STORE == PV_STORE_U8 && J.uniform) {
            unsigned pk[R / 2];  // [2q]: samples 4l, 4l+2 of group q; [2q+1]: 4l+1, 4l+3
            int isum[R];
#pragma unroll
            for (int r = 0; r < R / 2; ++r) pk[r] = 0u;
#pragma unroll
            for (int r = 0; r < R; ++r) isum[r] = 0;
            auto flush = [&]() {
#pragma unroll
                for (int q = 0; q < R / 4; ++q) {
                    isum[4 * q + 0] += (int)(pk[2 * q] & 0xffffu);
                    isum[4 * q + 2] += (int)(pk[2 * q] >> 16);
                    isum[4 * q + 1] += (int)(pk[2 * q + 1] & 0xffffu);
                    isum[4 * q + 3] += (int)(pk[2 * q + 1] >> 16);
                    pk[2 * q] = 0u;
                    pk[2 * q + 1] = 0u;
                }
            };
            for (int st = 0; st < nst; ++st) {
                const int b = gs % ST;
                if (st > 0 && !mbar_wait_warp(&full[b], (gs / ST) & 1u, wait_ns)) {
                    if (lane == 0) atomicExch(status, PV_ERR_TIMEOUT);
                    return;
                }
                if (active) {
                    const int c_end = min(CS, nchan - st * CS);
                    const int my_off =
                        lane < c_end ? min(pv_shift(meta_k[b * CS + lane], dv) - meta_off[b * CS + lane], slot - TT - 4)
                                     : 0;
                    for (int j = 0; j < c_end; ++j) {
                        const int off = __shfl_sync(0xffffffffu, my_off, j);
                        const unsigned* wr =
                            reinterpret_cast<const unsigned*>(slots + (size_t)(b * CS + j) * slot) + (off >> 2) + lane;
                        const int m = off & 3;
#pragma unroll
                        for (int q = 0; q < R / 4; ++q) {
                            unsigned x = wr[32 * q];
                            if (m) x = __funnelshift_r(x, wr[32 * q + 1], 8 * m);
                            pk[2 * q] += __byte_perm(x, 0u, 0x4240u);
                            pk[2 * q + 1] += __byte_perm(x, 0u, 0x4341u);
                        }
                    }
                    if ((st + 1) % (256 / CS) == 0) flush();
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&empty[b]);
                ++gs;
            }
            if (active) {
                flush();
                float* o = J.out + (long long)d * J.out_stride;
                const float sc = J.scale[0], os = *J.off_sum;
                const int bias = 128 * nchan;
#pragma unroll
                for (int q = 0; q < R / 4; ++q) {
                    const long long t = tt.t0 + 128 * q + 4 * lane;
                    if (t < J.nout)
                        *reinterpret_cast<float4*>(o + t) =
                            make_float4(fmaf(sc, (float)(isum[4 * q + 0] - bias), os),
                                        fmaf(sc, (float)(isum[4 * q + 1] - bias), os),
                                        fmaf(sc, (float)(isum[4 * q + 2] - bias), os),
                                        fmaf(sc, (float)(isum[4 * q + 3] - bias), os));
                }
            }
            continue;
        }
        float acc[R];
        unsigned long long acc2[R / 2];
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r] = 0.0f;
#pragma unroll
        for (int r = 0; r < R / 2; ++r) acc2[r] = 0ull;
        for (int st = 0; st < nst; ++st) {
            const int b = gs % ST;
            if (st > 0 && !mbar_wait_warp(&full[b], (gs / ST) & 1u, wait_ns)) {
                if (lane == 0) atomicExch(status, PV_ERR_TIMEOUT);
                return;
            }
            if (active) {
                const int c_end = min(CS, nchan - st * CS);
                // lane j computes channel j's row offset once per stage (see the single-beam kernel)
                const int my_off =
                    lane < c_end ? min(pv_shift(meta_k[b * CS + lane], dv) - meta_off[b * CS + lane], slot - TT - 4) : 0;
                for (int j = 0; j < c_end; ++j) {
                    const int off = __shfl_sync(0xffffffffu, my_off, j);
                    const unsigned char* rowb = slots + (size_t)(b * CS + j) * slot * E;
                    if (STORE == PV_STORE_F32) {
                        const float* row = reinterpret_cast<const float*>(rowb) + off + lane;
#pragma unroll
                        for (int r = 0; r < R; ++r) acc[r] = __fadd_rn(acc[r], row[32 * r]);
                    } else if (STORE == PV_STORE_F16) {
                        // each half is added to its FP32 sum by one mixed-precision add
                        // (exactly fadd(float(h), sum)); odd offsets take the high half of
                        // one word and the low half of the next
                        const unsigned* w = reinterpret_cast<const unsigned*>(rowb);
                        if ((off & 1) == 0) {
                            const unsigned* wr = w + (off >> 1) + lane;
#pragma unroll
                            for (int p = 0; p < R / 2; ++p) {
                                unsigned short lo, hi;
                                f16_halves(wr[32 * p], lo, hi);
                                acc[2 * p] = add_f16(lo, acc[2 * p]);
                                acc[2 * p + 1] = add_f16(hi, acc[2 * p + 1]);
                            }
                        } else {
                            const unsigned* wr = w + ((off - 1) >> 1) + lane;
#pragma unroll
                            for (int p = 0; p < R / 2; ++p) {
                                unsigned short lo0, hi0, lo1, hi1;
                                f16_halves(wr[32 * p], lo0, hi0);
                                f16_halves(wr[32 * p + 1], lo1, hi1);
                                acc[2 * p] = add_f16(hi0, acc[2 * p]);
                                acc[2 * p + 1] = add_f16(lo1, acc[2 * p + 1]);
                            }
                        }
                    } else {
                        const unsigned* wr = reinterpret_cast<const unsigned*>(rowb) + (off >> 2) + lane;
                        const int m = off & 3;
                        const float sc = meta_sc[b * CS + j];
                        const unsigned long long sc2 = f2_pack(sc, sc);
#pragma unroll
                        for (int q = 0; q < R / 4; ++q) {
                            unsigned x = wr[32 * q];
                            if (m) x = __funnelshift_r(x, wr[32 * q + 1], 8 * m);
                            acc2[2 * q] = f2_fma(f2_pack(u8_centered(x, 0), u8_centered(x, 1)), sc2, acc2[2 * q]);
                            acc2[2 * q + 1] =
                                f2_fma(f2_pack(u8_centered(x, 2), u8_centered(x, 3)), sc2, acc2[2 * q + 1]);
                        }
                    }
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[b]);
            ++gs;
        }
        if (active) {
            float* o = J.out + (long long)d * J.out_stride;
            if (STORE == PV_STORE_F32) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const long long t = tt.t0 + lane + 32 * r;
                    if (t < J.nout) o[t] = acc[r];
                }
            } else if (STORE == PV_STORE_F16) {
#pragma unroll
                for (int p = 0; p < R / 2; ++p) {
                    const long long t = tt.t0 + 64 * p + 2 * lane;
                    if (t < J.nout) *reinterpret_cast<float2*>(o + t) = make_float2(acc[2 * p], acc[2 * p + 1]);
                }
            } else {
                const float os = *J.off_sum;
#pragma unroll
                for (int q = 0; q < R / 4; ++q) {
                    const long long t = tt.t0 + 128 * q + 4 * lane;
                    if (t < J.nout) {
                        const float2 a = f2_unpack(acc2[2 * q]), c = f2_unpack(acc2[2 * q + 1]);
                        *reinterpret_cast<float4*>(o + t) =
                            make_float4(a.x + os, a.y + os, c.x + os, c.y + os);
                    }
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// K4 batched, FP32 rows, trial pairs.  The batched producer fills the same
// stage slots; eight consumer warps each take two adjacent trials of the
// tile (d, d+1) and lane l the 33 consecutive output samples 33l..33l+32 of
// a 1056-sample time tile.  For each channel the lane reads the 33 + delta
// words row[o_d + 33l + j], delta = o_(d+1) - o_d the channel's shift
// difference between the two trials, once into registers and adds word j
// to trial d's sample j and to trial d+1's sample j - delta: up to
// delta = 32, 33 + delta shared-memory words feed 66 adds (the one-trial
// consumers read one word per add).  delta selects a fully unrolled variant
// (a warp-uniform jump), larger shifts take two separate 33-word reads.
// Lanes 33 words apart read distinct banks, so every read is one
// conflict-free wavefront.  Each output still adds its channels 0..nchan-1
// in order with FP32 adds: the results are bit-identical to the other
// kernels.
// ---------------------------------------------------------------------------
constexpr int kPairS = 33;  // output samples per lane

// w holds row[0..32], read before the jump: every delta needs them.
template <int D>
__device__ __forceinline__ void pair_add(const float* __restrict__ row, const float (&w)[kPairS],
                                         float (&a0)[kPairS], float (&a1)[kPairS]) {
#pragma unroll
    for (int j = 0; j < kPairS; ++j) {
        a0[j] = __fadd_rn(a0[j], w[j]);
        if (j >= D) a1[j - D] = __fadd_rn(a1[j - D], w[j]);
    }
#pragma unroll
    for (int j = kPairS; j < kPairS + D; ++j) a1[j - D] = __fadd_rn(a1[j - D], row[j]);
}

__device__ __forceinline__ void pair_add_far(const float* __restrict__ row, int dl, const float (&w)[kPairS],
                                             float (&a0)[kPairS], float (&a1)[kPairS]) {
#pragma unroll
    for (int j = 0; j < kPairS; ++j) a0[j] = __fadd_rn(a0[j], w[j]);
    const float* rb = row + dl;
#pragma unroll
    for (int j = 0; j < kPairS; ++j) a1[j] = __fadd_rn(a1[j], rb[j]);
}

// The jump over the shift difference dl: 0..LIM from registers, larger
// differences read trial b's 33 words separately.  LIM 15 halves the jump's
// code, which the instruction cache of a sub-partition then holds.
template <int LIM>
__device__ __forceinline__ void pair_dispatch(const float* __restrict__ row, int dl, const float (&w)[kPairS],
                                              float (&a0)[kPairS], float (&a1)[kPairS]) {
#define PV_PAIR(D) \
    case D:        \
        pair_add<D>(row, w, a0, a1); \
        break;
    if constexpr (LIM == 32) {
        switch (dl) {
            PV_PAIR(0) PV_PAIR(1) PV_PAIR(2) PV_PAIR(3) PV_PAIR(4) PV_PAIR(5) PV_PAIR(6) PV_PAIR(7) PV_PAIR(8)
            PV_PAIR(9) PV_PAIR(10) PV_PAIR(11) PV_PAIR(12) PV_PAIR(13) PV_PAIR(14) PV_PAIR(15) PV_PAIR(16)
            PV_PAIR(17) PV_PAIR(18) PV_PAIR(19) PV_PAIR(20) PV_PAIR(21) PV_PAIR(22) PV_PAIR(23) PV_PAIR(24)
            PV_PAIR(25) PV_PAIR(26) PV_PAIR(27) PV_PAIR(28) PV_PAIR(29) PV_PAIR(30) PV_PAIR(31) PV_PAIR(32)
            default:
                pair_add_far(row, dl, w, a0, a1);
        }
    } else {
        static_assert(LIM == 15, "shift-difference limits 15 and 32");
        switch (dl) {
            PV_PAIR(0) PV_PAIR(1) PV_PAIR(2) PV_PAIR(3) PV_PAIR(4) PV_PAIR(5) PV_PAIR(6) PV_PAIR(7) PV_PAIR(8)
            PV_PAIR(9) PV_PAIR(10) PV_PAIR(11) PV_PAIR(12) PV_PAIR(13) PV_PAIR(14) PV_PAIR(15)
            default:
                pair_add_far(row, dl, w, a0, a1);
        }
    }
#undef PV_PAIR
}

// PAIRS trial pairs per tile (2 * PAIRS trials) and HALVES parts of the
// time tile (HALVES x 1056 samples): consumer warp w takes pair w % PAIRS in
// part w / PAIRS.  8 x 1: 8 consumer warps; 6 x 2: 12; 7 x 2: 14, more warps
// to hide each channel's offset shuffle, jump and first reads within the
// register file's share of one SM sub-partition (13 to 16 warps: up to 128
// registers).
template <int CS, int ST, int PAIRS, int HALVES, int LIM>
__global__ void __launch_bounds__((PAIRS * HALVES + 1) * 32, 1)
dedisperse_pair_kernel(const pv::DdJob* __restrict__ jobs, const pv::DdTile* __restrict__ tiles, int ntiles,
                       int slot, int* __restrict__ counter, const pv::BeamStep* __restrict__ bs,
                       int* __restrict__ status, unsigned long long wait_ns) {
    constexpr int NW = PAIRS * HALVES;
    constexpr int TT = 32 * kPairS * HALVES;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned char* slots = smem_raw;  // [ST*CS][slot] floats
    int* meta_off = reinterpret_cast<int*>(slots + (size_t)ST * CS * slot * 4);
    float* meta_k = reinterpret_cast<float*>(meta_off + ST * CS);
    float* meta_sc = meta_k + ST * CS;
    int* s_first = reinterpret_cast<int*>(meta_sc + ST * CS);
    uint64_t* full = reinterpret_cast<uint64_t*>(s_first + 2 * ST);
    uint64_t* empty = full + ST;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

    __shared__ int s_abort;
    if (threadIdx.x == 0) {
        s_abort = *(volatile int*)status;
        for (int b = 0; b < ST; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], NW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    }
    __syncthreads();
    if (s_abort != 0) return;
    if (warp == NW) {
        batch_producer<TT, CS, ST, PV_STORE_F32>(jobs, tiles, ntiles, slot, counter, bs, status, wait_ns, slots,
                                                 meta_off, meta_k, meta_sc, s_first, full, empty, lane);
        return;
    }
    const float* slotf = reinterpret_cast<const float*>(slots);
    unsigned gs = 0;
    for (;;) {
        const int b0 = gs % ST;
        if (!mbar_wait_warp(&full[b0], (gs / ST) & 1u, wait_ns)) {
            if (lane == 0) atomicExch(status, PV_ERR_TIMEOUT);
            return;
        }
        const int tile = *(volatile int*)&s_first[b0];
        if (tile < 0) return;
        const pv::DdTile tt = tiles[tile];
        const pv::DdJob& J = jobs[tt.job];
        const int d_last = min(tt.d0 + J.dms, J.tdms) - 1;
        const int pair = warp % PAIRS, half = warp / PAIRS;
        const int da = tt.d0 + 2 * pair;
        const bool act_a = 2 * pair < J.dms && da <= d_last;
        const bool act_b = 2 * pair + 1 < J.dms && da + 1 <= d_last;
        const int lane_t = half * 32 * kPairS + kPairS * lane;  // the lane's first sample in the tile
        const float dva = pv_trial_value(min(da, d_last), J.start, J.step);
        const float dvb = pv_trial_value(min(da + 1, d_last), J.start, J.step);
        const int nst = (J.nchan + CS - 1) / CS;
        float a0[kPairS], a1[kPairS];
#pragma unroll
        for (int j = 0; j < kPairS; ++j) a0[j] = a1[j] = 0.0f;
        for (int st = 0; st < nst; ++st) {
            const int b = gs % ST;
            if (st > 0 && !mbar_wait_warp(&full[b], (gs / ST) & 1u, wait_ns)) {
                if (lane == 0) atomicExch(status, PV_ERR_TIMEOUT);
                return;
            }
            if (act_a) {
                const int c_end = min(CS, J.nchan - st * CS);
                // lane j computes channel j's two row offsets; the warp takes them by shuffle
                int my_oa = 0, my_dl = 0;
                if (lane < c_end) {
                    const float k = meta_k[b * CS + lane];
                    const int mo = meta_off[b * CS + lane];
                    my_oa = min(pv_shift(k, dva) - mo, slot - TT - 16);
                    my_dl = min(pv_shift(k, dvb) - mo, slot - TT - 16) - my_oa;
                }
                // channel j+1's offsets are taken while channel j is added
                int oa = __shfl_sync(0xffffffffu, my_oa, 0);
                int dl = __shfl_sync(0xffffffffu, my_dl, 0);
                for (int j = 0; j < c_end; ++j) {
                    const int oa_n = __shfl_sync(0xffffffffu, my_oa, (j + 1) & 31);
                    const int dl_n = __shfl_sync(0xffffffffu, my_dl, (j + 1) & 31);
                    const float* row = slotf + (size_t)(b * CS + j) * slot + oa + lane_t;
                    float w[kPairS];
#pragma unroll
                    for (int q = 0; q < kPairS; ++q) w[q] = row[q];
                    pair_dispatch<LIM>(row, dl, w, a0, a1);
                    oa = oa_n;
                    dl = dl_n;
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[b]);
            ++gs;
        }
        float* oa_p = J.out + (long long)da * J.out_stride;
#pragma unroll
        for (int j = 0; j < kPairS; ++j) {
            const long long t = tt.t0 + lane_t + j;
            if (t < J.nout) {
                if (act_a) oa_p[t] = a0[j];
                if (act_b) oa_p[J.out_stride + t] = a1[j];
            }
        }
    }
}

// Largest delay spread s(c, d0+DMS-1) - s(c, d0) over channels and DM tiles,
// evaluated with the kernel's own float arithmetic on the host.
int delay_spread(const std::vector<float>& dmshift, int tdms, int dms, float start, float step) {
    int spread = 0;
    for (int d0 = 0; d0 < tdms; d0 += dms) {
        const int dl = std::min(d0 + dms, tdms) - 1;
        const float v0 = std::fmaf((float)d0, step, start);
        const float vl = std::fmaf((float)dl, step, start);
        for (float k : dmshift) {
            const float p0 = k * v0, pl = k * vl;
            spread = std::max(spread, (int)pl - (int)p0);
        }
    }
    return spread;
}

template <int DMS, int R, int CS>
int launch_dedisperse(DedispArgs a, int spread, cudaStream_t s) {
    constexpr int TT = 32 * R;
    a.slot = TT + spread;
    const size_t smem = (size_t)2 * CS * a.slot * sizeof(float);
    if (smem > 227 * 1024) {
        pv::set_error("dedispersion: delay spread %d per tile needs %zu bytes of shared memory",
                      spread, smem);
        return PV_ERR_ARG;
    }
    if (a.ring_len > 0 && a.ring_len < std::min(TT, a.nout) + spread) {
        pv::set_error("dedispersion: ring of %lld samples is shorter than one tile span (%d)",
                      a.ring_len, std::min(TT, a.nout) + spread);
        return PV_ERR_ARG;
    }
    auto kern = dedisperse_kernel<DMS, R, CS>;
    PV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
            "cudaFuncSetAttribute(dedisperse)");
    dim3 grid((unsigned)pv::ceil_div<long long>(a.nout, TT), (unsigned)pv::ceil_div(a.tdms, DMS));
    if (grid.y > 65535u) {
        pv::set_error("dedispersion: too many DM tiles");
        return PV_ERR_ARG;
    }
    kern<<<grid, DMS * 32, smem, s>>>(a);
    return pv::check_launch("dedisperse_kernel");
}

template <int DMS, int R, int CS, int ST>
int launch_dedisperse_tma(DedispArgs a, int spread, int* status, cudaStream_t s) {
    constexpr int TT = 32 * R;
    a.slot = (TT + spread + 8 + 3) & ~3;
    const size_t smem = (size_t)ST * CS * a.slot * sizeof(float) + (size_t)ST * CS * 8 + 8 +
                        (size_t)2 * ST * sizeof(uint64_t);
    auto kern = dedisperse_tma_kernel<DMS, R, CS, ST>;
    PV_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
            "cudaFuncSetAttribute(dedisperse_tma)");
    dim3 grid((unsigned)pv::ceil_div<long long>(a.nout, TT), (unsigned)pv::ceil_div(a.tdms, DMS));
    kern<<<grid, (DMS + 1) * 32, smem, s>>>(a, status);
    return pv::check_launch("dedisperse_tma_kernel");
}

}  // namespace

namespace pv {

// Shared-memory bytes of the TMA kernel for a given slot size.
static size_t tma_smem(int st, int cs, int slot_floats) {
    return (size_t)st * cs * slot_floats * sizeof(float) + (size_t)st * cs * 8 + 8 + 2 * st * 8;
}

// Chooses the tile for the delay spread: the widest trial tile whose channel
// slots fit in shared memory with two buffers of CS channels.
int dedisperse_device(float* out, long long out_stride, const float* in, long long row_stride,
                      long long row_len, long long ring_len, long long t_base, int nchan, int nout,
                      int tdms, const float* d_dmshift, const std::vector<float>& h_dmshift,
                      float start, float step, cudaStream_t s, int* status) {
    if (ring_len > 0 && (ring_len > row_stride || t_base < 0)) {
        set_error("dedispersion: ring of %lld samples does not fit rows of %lld", ring_len, row_stride);
        return PV_ERR_ARG;
    }
    DedispArgs a{out, out_stride, in, row_stride, row_len, ring_len, t_base % std::max(ring_len, 1LL),
                 d_dmshift, nchan, nout, tdms, start, step, 0, wait_ns(), 0};
    // Ring rows with 16-byte aligned spans go through the TMA pipeline.
    if (status && ring_len > 0 && ring_len % 4 == 0 && row_stride % 4 == 0 &&
        (reinterpret_cast<uintptr_t>(in) & 15) == 0 && getenv("PV_DEDISP_V1") == nullptr) {
        a.stall = take_stall();
        const int spread16 = delay_spread(h_dmshift, tdms, 16, start, step);
        const int slot = (1024 + spread16 + 8 + 3) & ~3;
        // every copy (span + 16-byte rounding) must fit in one ring turn
        const bool fits = ring_len >= (long long)std::min(1024, nout) + spread16 + 8;
        if (fits && tma_smem(4, 4, slot) <= 220 * 1024)
            return launch_dedisperse_tma<16, 32, 4, 4>(a, spread16, status, s);
        if (fits && tma_smem(4, 2, slot) <= 220 * 1024)
            return launch_dedisperse_tma<16, 32, 2, 4>(a, spread16, status, s);
    }
    const int spread16 = delay_spread(h_dmshift, tdms, 16, start, step);
    if ((size_t)2 * 4 * (1024 + spread16) * 4 <= 200 * 1024)
        return launch_dedisperse<16, 32, 4>(a, spread16, s);
    const int spread8 = delay_spread(h_dmshift, tdms, 8, start, step);
    if ((size_t)2 * 4 * (1024 + spread8) * 4 <= 220 * 1024)
        return launch_dedisperse<8, 32, 4>(a, spread8, s);
    const int spread4 = delay_spread(h_dmshift, tdms, 4, start, step);
    if ((size_t)2 * 2 * (512 + spread4) * 4 <= 220 * 1024)
        return launch_dedisperse<4, 16, 2>(a, spread4, s);
    const int spread1 = delay_spread(h_dmshift, tdms, 1, start, step);
    return launch_dedisperse<1, 16, 1>(a, spread1, s);
}

}  // namespace pv

// ---------------------------------------------------------------------------
// Batched dedispersion set-up and the DM x time tile autotuner
// ---------------------------------------------------------------------------
namespace {

struct Variant {
    int R, CS, ST;
    bool pair; // FP32 trial-pair consumers (dedisperse_pair_kernel, R = 33 per part of the time tile)
    int dmax;  // trials per tile at most
};
// Time tile 32R samples, CS channels per pipeline stage, ST stages in flight.
constexpr Variant kVariants[] = {{32, 4, 4, false, 16}, {32, 2, 4, false, 16}, {16, 4, 4, false, 16},
                                 {32, 8, 2, false, 16}, {33, 8, 2, true, 16},  {66, 8, 2, true, 12},
                                 {66, 8, 2, true, 12},  {66, 8, 2, true, 14},  {66, 4, 4, true, 14}};
constexpr int kNumVariants = 9;
static_assert(kNumVariants == PV_BATCH_VARIANTS, "variant count of the C ABI");
constexpr size_t kBatchSmemBudget = 220 * 1024;

int store_bytes(int store) { return store == PV_STORE_F32 ? 4 : (store == PV_STORE_F16 ? 2 : 1); }

// slots, per-channel offsets, delay constants and scales, tile records, barriers
size_t batch_smem(const Variant& v, int slot, int store) {
    return (size_t)store_bytes(store) * v.ST * v.CS * slot + (size_t)12 * v.ST * v.CS + (size_t)8 * v.ST +
           16 * v.ST;
}

template <int R, int CS, int ST, int STORE>
int launch_batch_t(const pv::DdJob* jobs, const pv::DdTile* tiles, int ntiles, int slot, size_t smem,
                   int grid, int* counter, const pv::BeamStep* bs, int* status, cudaStream_t s,
                   bool set_attr) {
    auto kern = dedisperse_batch_kernel<R, CS, ST, STORE>;
    if (set_attr) {
        size_t limit = 0;
        PV_CUDA(pv::allow_max_dynamic_smem(kern, &limit), "cudaFuncSetAttribute(dedisperse_batch)");
        if (smem > limit) {
            pv::set_error("dedisperse_batch: %zu bytes of shared memory exceed one CTA's %zu", smem, limit);
            return PV_ERR_ARG;
        }
        return PV_OK;
    }
    if (grid < 0) {  // the counter was reset beforehand: this launch joins the same tile queue
        grid = -grid;
    } else {
        PV_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), s), "reset tile counter");
    }
    kern<<<grid, 17 * 32, smem, s>>>(jobs, tiles, ntiles, slot, counter, bs, status, pv::wait_ns());
    return pv::check_launch("dedisperse_batch_kernel");
}

template <int CS, int ST, int PAIRS, int HALVES, int LIM>
int launch_pair_t(const pv::DdJob* jobs, const pv::DdTile* tiles, int ntiles, int slot, size_t smem, int grid,
                  int* counter, const pv::BeamStep* bs, int* status, cudaStream_t s, bool set_attr) {
    constexpr int NW = PAIRS * HALVES;
    auto kern = dedisperse_pair_kernel<CS, ST, PAIRS, HALVES, LIM>;
    if (set_attr) {
        size_t limit = 0;
        PV_CUDA(pv::allow_max_dynamic_smem(kern, &limit), "cudaFuncSetAttribute(dedisperse_pair)");
        if (smem > limit) {
            pv::set_error("dedisperse_pair: %zu bytes of shared memory exceed one CTA's %zu", smem, limit);
            return PV_ERR_ARG;
        }
        return PV_OK;
    }
    if (grid < 0) {
        grid = -grid;
    } else {
        PV_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), s), "reset tile counter");
    }
    kern<<<grid, (NW + 1) * 32, smem, s>>>(jobs, tiles, ntiles, slot, counter, bs, status, pv::wait_ns());
    return pv::check_launch("dedisperse_pair_kernel");
}

int launch_batch(int variant, int store, const pv::DdJob* jobs, const pv::DdTile* tiles, int ntiles,
                 int slot, size_t smem, int grid, int* counter, const pv::BeamStep* bs, int* status,
                 cudaStream_t s, bool set_attr) {
    if (store == PV_STORE_F32 && variant >= 4 && variant <= 8) {
#define PV_PAIRV(I, CS, ST, P, H, L)                                                                   \
    if (variant == I)                                                                                 \
        return launch_pair_t<CS, ST, P, H, L>(jobs, tiles, ntiles, slot, smem, grid, counter, bs, status, s, \
                                              set_attr);
        PV_PAIRV(4, 8, 2, 8, 1, 32)
        PV_PAIRV(5, 8, 2, 6, 2, 32)
        PV_PAIRV(6, 8, 2, 6, 2, 15)
        PV_PAIRV(7, 8, 2, 7, 2, 15)
        PV_PAIRV(8, 4, 4, 7, 2, 15)
#undef PV_PAIRV
    }
    switch (variant * 3 + store) {
#define PV_VAR(I, R, CS, ST, SS)                                                                 \
    case I * 3 + SS:                                                                            \
        return launch_batch_t<R, CS, ST, SS>(jobs, tiles, ntiles, slot, smem, grid, counter, bs, \
                                             status, s, set_attr);
#define PV_VARS(I, R, CS, ST) PV_VAR(I, R, CS, ST, 0) PV_VAR(I, R, CS, ST, 1) PV_VAR(I, R, CS, ST, 2)
        PV_VARS(0, 32, 4, 4)
        PV_VARS(1, 32, 2, 4)
        PV_VARS(2, 16, 4, 4)
        PV_VARS(3, 32, 8, 2)
#undef PV_VARS
#undef PV_VAR
    }
    pv::set_error("dedispersion: unknown tile variant %d", variant);
    return PV_ERR_ARG;
}

// Upper bound of delay_spread from the largest delay constant alone (the
// per-channel truncations differ from the exact products by under one sample
// each, plus the float rounding of the products).
int spread_bound(float kmax, int tdms, int dms, float start, float step) {
    double worst = 0.0;
    for (int d0 = 0; d0 < tdms; d0 += dms) {
        const int dl = std::min(d0 + dms, tdms) - 1;
        const float v0 = std::fmaf((float)d0, step, start);
        const float vl = std::fmaf((float)dl, step, start);
        worst = std::max(worst, (double)kmax * ((double)vl - (double)v0) +
                                    (double)kmax * ((double)vl + (double)v0) * 2.4e-7);
    }
    return (int)worst + 2;
}

}  // namespace

namespace pv {

struct DdBatch {
    int variant = 0, slot = 0, grid = 0, ntiles = 0, store = PV_STORE_F32;
    size_t smem = 0;
    DdJob* d_jobs = nullptr;
    DdTile* d_tiles = nullptr;
    int* d_counter = nullptr;
    int* d_status = nullptr;
    std::vector<int> dms;
    std::vector<float> tune_ms;
};

void dd_batch_destroy(DdBatch* b) {
    if (!b) return;
    for (void* p : {(void*)b->d_jobs, (void*)b->d_tiles, (void*)b->d_counter, (void*)b->d_status})
        if (p) cudaFree(p);
    delete b;
}

namespace {

struct Shape {
    int slot = 0;
    size_t smem = 0;
    std::vector<int> dms;
    std::vector<DdTile> tiles;
};

// DM tile heights, slot size and tile list of one variant; false if some beam
// cannot be tiled (its ring is shorter than a tile span).
// A slot holds the span (tile + delay spread), up to one alignment unit in
// front of it and 16 more elements for the reduced-precision readers.
bool build_shape(const Variant& v, int store, const DdBeam* beams, int n,
                 std::vector<std::map<int, int>>& exact, Shape& out) {
    if (v.pair && store != PV_STORE_F32) return false;
    const int TT = 32 * v.R;
    const size_t fixed = batch_smem(v, 0, store);
    const int E = store_bytes(store);
    const int pad = 16 / E + 16;
    const int slot_cap =
        (int)(((kBatchSmemBudget - fixed) / ((size_t)E * v.ST * v.CS)) & ~(size_t)15);
    if (slot_cap < TT + pad) return false;
    out.dms.assign(n, 1);
    out.slot = 0;
    for (int i = 0; i < n; ++i) {
        const DdBeam& B = beams[i];
        float kmax = 0.0f;
        for (int c = 0; c < B.nchan; ++c) kmax = std::max(kmax, B.h_dmshift[c]);
        int dms = v.dmax, sp = 0;
        for (; dms >= 1; --dms) {
            if (TT + spread_bound(kmax, B.tdms, dms, B.start, B.step) + pad > slot_cap) continue;
            auto it = exact[i].find(dms);
            if (it == exact[i].end()) {
                std::vector<float> k(B.h_dmshift, B.h_dmshift + B.nchan);
                it = exact[i].emplace(dms, delay_spread(k, B.tdms, dms, B.start, B.step)).first;
            }
            sp = it->second;
            if (TT + sp + pad <= slot_cap) break;
        }
        if (dms < 1) return false;
        if (B.ring_len < (long long)std::min(TT, B.nout) + sp + pad) return false;
        out.dms[i] = dms;
        out.slot = std::max(out.slot, (TT + sp + pad + 15) & ~15);
    }
    out.smem = batch_smem(v, out.slot, store);
    // tiles, beams with the most work per tile first, time tiles outer
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (long long)beams[a].nchan * out.dms[a] > (long long)beams[b].nchan * out.dms[b];
    });
    out.tiles.clear();
    for (int i : order)
        for (int t0 = 0; t0 < beams[i].nout; t0 += TT)
            for (int d0 = 0; d0 < beams[i].tdms; d0 += out.dms[i]) out.tiles.push_back({i, d0, t0});
    return true;
}

int upload(DdBatch* b, const DdBeam* beams, int n, const Shape& sh, int variant) {
    std::vector<DdJob> jobs(n);
    for (int i = 0; i < n; ++i) {
        const DdBeam& B = beams[i];
        jobs[i] = DdJob{B.out, B.out_stride, B.ring, B.row_stride, B.ring_len, B.d_dmshift, B.scale,
                        B.off_sum, B.nchan, B.nout, B.tdms, B.chunk, sh.dms[i], i, B.start, B.step,
                        b->store == PV_STORE_U8 ? B.uniform : 0};
    }
    if (b->d_jobs) cudaFree(b->d_jobs);
    if (b->d_tiles) cudaFree(b->d_tiles);
    b->d_jobs = nullptr;
    b->d_tiles = nullptr;
    PV_CUDA(cudaMalloc(&b->d_jobs, sizeof(DdJob) * n), "allocate dedispersion jobs");
    PV_CUDA(cudaMalloc(&b->d_tiles, sizeof(DdTile) * std::max<size_t>(sh.tiles.size(), 1)),
            "allocate dedispersion tiles");
    PV_CUDA(cudaMemcpy(b->d_jobs, jobs.data(), sizeof(DdJob) * n, cudaMemcpyHostToDevice),
            "copy dedispersion jobs");
    PV_CUDA(cudaMemcpy(b->d_tiles, sh.tiles.data(), sizeof(DdTile) * sh.tiles.size(),
                       cudaMemcpyHostToDevice), "copy dedispersion tiles");
    b->variant = variant;
    b->slot = sh.slot;
    b->smem = sh.smem;
    b->ntiles = (int)sh.tiles.size();
    b->dms = sh.dms;
    b->grid = std::max(1, std::min(b->ntiles, sm_count()));
    return launch_batch(variant, b->store, nullptr, nullptr, 0, 0, b->smem, 0, nullptr, nullptr,
                        nullptr, nullptr, true);
}

}  // namespace

int dd_batch_create(DdBatch** out, const DdBeam* beams, int n, int variant, int store, cudaStream_t s) {
    if (!out || !beams || n <= 0) {
        set_error("dedispersion batch: no beams");
        return PV_ERR_ARG;
    }
    for (int i = 0; i < n; ++i) {
        const DdBeam& B = beams[i];
        const int au = 16 / store_bytes(store < 0 || store > 2 ? 0 : store);
        if (B.ring_len <= 0 || B.ring_len % au != 0 || B.row_stride % au != 0 || B.ring_len > B.row_stride ||
            (store == PV_STORE_U8 && (!B.scale || !B.off_sum)) || B.nout % 4 != 0 ||
            (reinterpret_cast<uintptr_t>(B.ring) & 15) != 0 || B.nout <= 0 || B.tdms <= 0 ||
            B.nchan <= 0 || B.chunk <= 0) {
            set_error("dedispersion batch: beam %d needs a 16-byte aligned ring of a multiple of 16 "
                      "bytes per row and a window of a multiple of 4 samples", i);
            return PV_ERR_ARG;
        }
    }
    if (store < PV_STORE_F32 || store > PV_STORE_U8) {
        set_error("dedispersion batch: unknown storage %d", store);
        return PV_ERR_ARG;
    }
    auto* b = new DdBatch;
    b->store = store;
    std::vector<std::map<int, int>> exact(n);
    int rc = PV_OK;
    if (cudaMalloc(&b->d_counter, sizeof(int)) != cudaSuccess ||
        cudaMalloc(&b->d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(b->d_status, 0, sizeof(int)) != cudaSuccess) {
        set_error("dedispersion batch: cannot allocate counters");
        dd_batch_destroy(b);
        return PV_ERR_NOMEM;
    }
    Shape sh;
    if (variant >= 0) {
        if (variant >= kNumVariants || !build_shape(kVariants[variant], store, beams, n, exact, sh)) {
            set_error("dedispersion batch: tile variant %d cannot hold these beams", variant);
            dd_batch_destroy(b);
            return PV_ERR_ARG;
        }
        rc = upload(b, beams, n, sh, variant);
    } else {
        // Autotuner: time every variant that can tile the beams on the rings as
        // they are, with every beam dedispersing window 0, and keep the fastest.
        BeamStep* d_tstep = nullptr;
        std::vector<BeamStep> all(n);
        for (auto& x : all) {
            x = BeamStep{};
            x.sel = 1;
        }
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        PV_CUDA(cudaMalloc(&d_tstep, sizeof(BeamStep) * n), "allocate tuning steps");
        PV_CUDA(cudaMemcpy(d_tstep, all.data(), sizeof(BeamStep) * n, cudaMemcpyHostToDevice),
                "copy tuning steps");
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best = 1e30f;
        int best_v = -1;
        b->tune_ms.assign(kNumVariants, -1.0f);
        for (int v = 0; v < kNumVariants && rc == PV_OK; ++v) {
            Shape cand;
            if (!build_shape(kVariants[v], store, beams, n, exact, cand)) continue;
            rc = upload(b, beams, n, cand, v);
            if (rc != PV_OK) break;
            float ms = 0.0f;
            for (int it = 0; it < 3 && rc == PV_OK; ++it) {
                if (it == 1) cudaEventRecord(e0, s);
                rc = launch_batch(v, store, b->d_jobs, b->d_tiles, b->ntiles, b->slot, b->smem, b->grid,
                                  b->d_counter, d_tstep, b->d_status, s, false);
            }
            if (rc != PV_OK) break;
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                rc = cuda_status(cudaGetLastError(), "dedispersion tuning");
                break;
            }
            cudaEventElapsedTime(&ms, e0, e1);
            ms *= 0.5f;
            b->tune_ms[v] = ms;
            if (ms < best) {
                best = ms;
                best_v = v;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(d_tstep);
        int st = 0;
        if (rc == PV_OK) rc = cuda_status(cudaMemcpy(&st, b->d_status, sizeof(int), cudaMemcpyDeviceToHost), "read status");
        if (rc == PV_OK && st != PV_OK) {
            set_error("dedispersion tuning: a pipeline wait gave up");
            rc = st;
        }
        if (rc == PV_OK && best_v < 0) {
            set_error("dedispersion batch: no tile variant can hold these beams");
            rc = PV_ERR_ARG;
        }
        if (rc == PV_OK) {
            build_shape(kVariants[best_v], store, beams, n, exact, sh);
            rc = upload(b, beams, n, sh, best_v);
        }
    }
    if (rc != PV_OK) {
        dd_batch_destroy(b);
        return rc;
    }
    *out = b;
    return PV_OK;
}

int dd_batch_launch(DdBatch* b, const BeamStep* bs, cudaStream_t s) {
    return launch_batch(b->variant, b->store, b->d_jobs, b->d_tiles, b->ntiles, b->slot, b->smem, b->grid,
                        b->d_counter, bs, b->d_status, s, false);
}

int dd_batch_reset(DdBatch* b, cudaStream_t s) {
    PV_CUDA(cudaMemsetAsync(b->d_counter, 0, sizeof(int), s), "reset tile counter");
    return PV_OK;
}

int dd_batch_launch_shared(DdBatch* b, const BeamStep* bs, int ctas, cudaStream_t s) {
    if (ctas <= 0) return PV_OK;
    return launch_batch(b->variant, b->store, b->d_jobs, b->d_tiles, b->ntiles, b->slot, b->smem,
                        -std::min(ctas, std::max(b->ntiles, 1)), b->d_counter, bs, b->d_status, s, false);
}

int dd_batch_grid(const DdBatch* b) { return b->grid; }

int dd_batch_status(const DdBatch* b, int* h_status) {
    PV_CUDA(cudaMemcpy(h_status, b->d_status, sizeof(int), cudaMemcpyDeviceToHost), "read status");
    return PV_OK;
}

int dd_batch_shape(const DdBatch* b, int* h8) {
    const Variant& v = kVariants[b->variant];
    h8[0] = b->variant;
    h8[1] = 32 * v.R;
    h8[2] = v.CS;
    h8[3] = v.ST;
    h8[4] = b->slot;
    h8[5] = b->ntiles;
    h8[6] = b->grid;
    h8[7] = (int)b->smem;
    return PV_OK;
}

const std::vector<int>& dd_batch_dms(const DdBatch* b) { return b->dms; }
const int* dd_batch_status_word(const DdBatch* b) { return b->d_status; }
const std::vector<float>& dd_batch_tune_ms(const DdBatch* b) { return b->tune_ms; }

}  // namespace pv

extern "C" int pv_delay_table(int* d_shifts, const float* d_dmshift, int nchan, int tdms,
                              float start_over_tsamp, float step_over_tsamp, void* stream) {
    if (!d_shifts || !d_dmshift || nchan <= 0 || tdms <= 0) {
        pv::set_error("pv_delay_table: invalid arguments");
        return PV_ERR_ARG;
    }
    const long long n = (long long)nchan * tdms;
    const int threads = 256;
    const int blocks = (int)std::min<long long>(pv::ceil_div<long long>(n, threads),
                                                (long long)pv::sm_count() * 8);
    delay_table_kernel<<<blocks, threads, 0, pv::as_stream(stream)>>>(
        d_shifts, d_dmshift, nchan, tdms, start_over_tsamp, step_over_tsamp);
    return pv::check_launch("delay_table_kernel");
}

extern "C" int pv_dedisperse_ex(float* d_out, long long out_stride, const float* d_in,
                                long long row_stride, long long row_len, int nchans, int nout,
                                int tdms, const float* d_dmshift, float start_over_tsamp,
                                float step_over_tsamp, void* stream) {
    if (!d_out || !d_in || !d_dmshift || nchans <= 0 || tdms < 0 || nout < 0 ||
        out_stride < nout || row_stride <= 0 || row_len < 0) {
        pv::set_error("pv_dedisperse_ex: invalid arguments");
        return PV_ERR_ARG;
    }
    if (tdms == 0 || nout == 0) return PV_OK;
    std::vector<float> h(nchans);
    cudaStream_t s = pv::as_stream(stream);
    PV_CUDA(cudaMemcpyAsync(h.data(), d_dmshift, sizeof(float) * nchans, cudaMemcpyDeviceToHost, s),
            "copy dmshift");
    PV_CUDA(cudaStreamSynchronize(s), "synchronise");
    // Every delay must be a finite, non-negative sample count: the tiles
    // address shared memory and the input relative to the first trial's delay.
    if (!(start_over_tsamp >= 0.0f) || !(step_over_tsamp >= 0.0f) ||
        !std::isfinite(start_over_tsamp) || !std::isfinite(step_over_tsamp) || row_len > row_stride) {
        pv::set_error("pv_dedisperse_ex: trial start/step must be finite and >= 0 and "
                      "row_len <= row_stride");
        return PV_ERR_ARG;
    }
    for (int c = 0; c < nchans; ++c) {
        if (!(h[c] >= 0.0f) || !std::isfinite(h[c])) {
            pv::set_error("pv_dedisperse_ex: dmshift[%d] = %g is not a finite value >= 0", c, h[c]);
            return PV_ERR_ARG;
        }
    }
    const float vmax = std::fmaf((float)(tdms - 1), step_over_tsamp, start_over_tsamp);
    for (int c = 0; c < nchans; ++c) {
        if ((double)h[c] * vmax > 2.0e9) {
            pv::set_error("pv_dedisperse_ex: delay of channel %d exceeds the int range", c);
            return PV_ERR_ARG;
        }
    }
    return pv::dedisperse_device(d_out, out_stride, d_in, row_stride, row_len, 0, 0, nchans, nout,
                                 tdms, d_dmshift, h, start_over_tsamp, step_over_tsamp, s, nullptr);
}

extern "C" int pv_dedisperse(float* d_out, long long out_bytes, const float* d_in,
                             float start_over_tsamp, float step_over_tsamp, int tdms,
                             int num_samples, const float* d_dmshift, int maxshift, int nchans,
                             void* stream) {
    const int nout = num_samples - maxshift;
    if (nout < 0 || (long long)nout * tdms * (long long)sizeof(float) > out_bytes) {
        pv::set_error("pv_dedisperse: output buffer of %lld bytes is smaller than %d trials x %d "
                      "samples", out_bytes, tdms, nout);
        return PV_ERR_ARG;
    }
    return pv_dedisperse_ex(d_out, nout, d_in, num_samples, num_samples, nchans, nout, tdms,
                            d_dmshift, start_over_tsamp, step_over_tsamp, stream);
}

// ---------------------------------------------------------------------------
// Plans
// ---------------------------------------------------------------------------
struct pv_dedisp_plan {
    std::vector<float> h_dmshift;
    float* d_dmshift = nullptr;
    int* d_status = nullptr;  // PV_ERR_TIMEOUT if a pipeline wait gave up
    int nchan = 0, tdms = 0, max_shift = 0;
    float start = 0.0f, step = 0.0f;
};

extern "C" int pv_dedisp_plan_create(pv_dedisp_plan** plan, const float* h_dmshift, int nchans,
                                     int tdms, float start_over_tsamp, float step_over_tsamp) {
    if (!plan || !h_dmshift || nchans <= 0 || tdms <= 0 || !(start_over_tsamp >= 0.0f) ||
        !(step_over_tsamp >= 0.0f) || !std::isfinite(start_over_tsamp) ||
        !std::isfinite(step_over_tsamp)) {
        pv::set_error("pv_dedisp_plan_create: invalid arguments");
        return PV_ERR_ARG;
    }
    const float vmax = std::fmaf((float)(tdms - 1), step_over_tsamp, start_over_tsamp);
    int max_shift = 0;
    for (int c = 0; c < nchans; ++c) {
        if (!(h_dmshift[c] >= 0.0f) || !std::isfinite(h_dmshift[c]) ||
            (double)h_dmshift[c] * vmax > 2.0e9) {
            pv::set_error("pv_dedisp_plan_create: dmshift[%d] = %g is not a usable delay", c,
                          h_dmshift[c]);
            return PV_ERR_ARG;
        }
        max_shift = std::max(max_shift, (int)(h_dmshift[c] * vmax));
    }
    auto* p = new pv_dedisp_plan;
    p->h_dmshift.assign(h_dmshift, h_dmshift + nchans);
    p->nchan = nchans;
    p->tdms = tdms;
    p->start = start_over_tsamp;
    p->step = step_over_tsamp;
    p->max_shift = max_shift;
    cudaError_t e = cudaMalloc(&p->d_dmshift, sizeof(float) * nchans);
    if (e == cudaSuccess)
        e = cudaMemcpy(p->d_dmshift, h_dmshift, sizeof(float) * nchans, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->d_status, 0, sizeof(int));
    if (e != cudaSuccess) {
        pv::set_error("pv_dedisp_plan_create: %s", cudaGetErrorString(e));
        if (p->d_dmshift) cudaFree(p->d_dmshift);
        if (p->d_status) cudaFree(p->d_status);
        delete p;
        return PV_ERR_CUDA;
    }
    *plan = p;
    return PV_OK;
}

extern "C" void pv_dedisp_plan_destroy(pv_dedisp_plan* p) {
    if (!p) return;
    if (p->d_dmshift) cudaFree(p->d_dmshift);
    if (p->d_status) cudaFree(p->d_status);
    delete p;
}

extern "C" int pv_dedisp_plan_status(const pv_dedisp_plan* p, int* h_status) {
    if (!p || !h_status) return PV_ERR_ARG;
    PV_CUDA(cudaMemcpy(h_status, p->d_status, sizeof(int), cudaMemcpyDeviceToHost), "read plan status");
    return PV_OK;
}

namespace pv {
int plan_tables(const pv_dedisp_plan* p, const float** d_dmshift, const float** h_dmshift,
                int* nchan, int* tdms, float* start, float* step) {
    if (!p) return PV_ERR_ARG;
    *d_dmshift = p->d_dmshift;
    *h_dmshift = p->h_dmshift.data();
    *nchan = p->nchan;
    *tdms = p->tdms;
    *start = p->start;
    *step = p->step;
    return PV_OK;
}
}  // namespace pv

extern "C" int pv_dedisp_plan_clear_status(pv_dedisp_plan* p, void* stream) {
    if (!p) return PV_ERR_ARG;
    PV_CUDA(cudaMemsetAsync(p->d_status, 0, sizeof(int), pv::as_stream(stream)), "clear plan status");
    return PV_OK;
}

extern "C" int pv_dedisp_plan_max_shift(const pv_dedisp_plan* p) { return p ? p->max_shift : -1; }

extern "C" int pv_dedisp_plan_run(const pv_dedisp_plan* p, float* d_out, long long out_stride,
                                  const float* d_in, long long row_stride, long long row_len,
                                  long long ring_len, long long t_base, int nout, void* stream) {
    if (!p || !d_out || !d_in || nout < 0 || out_stride < nout || row_stride <= 0 ||
        (ring_len == 0 && (row_len < 0 || row_len > row_stride))) {
        pv::set_error("pv_dedisp_plan_run: invalid arguments");
        return PV_ERR_ARG;
    }
    if (nout == 0) return PV_OK;
    return pv::dedisperse_device(d_out, out_stride, d_in, row_stride, row_len, ring_len, t_base,
                                 p->nchan, nout, p->tdms, p->d_dmshift, p->h_dmshift, p->start,
                                 p->step, pv::as_stream(stream), p->d_status);
}
