// A8: DedispersionBuffer::addSamples on the device
// (lib/src/DedispersionBuffer.cpp:98-180).
//
// Stokes samples [t][sub][pol][chan] (pol 0 used, DedispersionBuffer.cpp:116)
// are transposed into the per-channel dedispersion ring: row r holds bin r,
// or bin nbins-1-r for an inverted (ascending) band, and logical sample
// pos+t lands at physical column (pos+t) mod ring_len.  The noise-template
// substitution of DedispersionBuffer.cpp:169 is omitted: the reference's
// weights are always 1, which makes it the identity.
#include <cuda_fp16.h>

#include "pv_internal.cuh"

namespace {

constexpr int kTile = 32;

// One stored sample: float, half (round to nearest) or the u8 code
// q = clamp(rint((v - offset) / scale) + 128, 0, 255) of the row (128 while
// the row has no scale yet).
template <int STORE>
__device__ __forceinline__ void ring_store(float* ring, long long i, float v, const float* scale,
                                           const float* offset, int row) {
    if (STORE == PV_STORE_F32) {
        ring[i] = v;
    } else if (STORE == PV_STORE_F16) {
        reinterpret_cast<__half*>(ring)[i] = __float2half_rn(v);
    } else {
        const float sc = scale[row];
        float q = sc > 0.0f ? rintf(__fdiv_rn(__fsub_rn(v, offset[row]), sc)) + 128.0f : 128.0f;
        q = fminf(fmaxf(q, 0.0f), 255.0f);
        reinterpret_cast<unsigned char*>(ring)[i] = (unsigned char)(int)q;
    }
}

// One CTA of 32 x 8 threads moves a strip of 32 bins x kStrip samples:
// coalesced 128-byte reads of each sample's 32 bins into shared memory (rows
// padded to kStrip + 1 words: both phases are free of bank conflicts), then
// coalesced 128-byte writes of each bin's samples into its ring row.
constexpr int kStrip = 128;

template <int STORE = PV_STORE_F32>
__device__ __forceinline__ void ring_write_tile(float* __restrict__ ring, long long row_stride,
                                                long long ring_len, long long pos,
                                                const float* __restrict__ stokes, int nt, int nsub,
                                                int npol, int nchan, int inverted, int t0, int b0,
                                                const float* scale = nullptr,
                                                const float* offset = nullptr) {
    __shared__ float tile[kTile][kStrip + 1];
    const int nbins = nsub * nchan;
    const int b = b0 + threadIdx.x;
    if (b < nbins) {
        const int s = b / nchan, c = b - s * nchan;
        const long long base = (long long)nchan * npol * s + c;
        const long long tstride = (long long)nchan * npol * nsub;  // one spectrum
#pragma unroll 4
        for (int i = threadIdx.y; i < kStrip; i += blockDim.y) {
            const int t = t0 + i;
            if (t < nt) tile[threadIdx.x][i] = stokes[tstride * t + base];
        }
    }
    __syncthreads();
    long long col0 = pos + t0;
    if (ring_len > 0) col0 %= ring_len;
    for (int j = threadIdx.y; j < kTile; j += blockDim.y) {
        const int bb = b0 + j;
        if (bb >= nbins) break;
        const int row = inverted ? nbins - 1 - bb : bb;
        const long long rbase = (long long)row * row_stride;
#pragma unroll
        for (int k = 0; k < kStrip / 32; ++k) {
            const int i = threadIdx.x + 32 * k;
            if (t0 + i < nt) {
                long long col = col0 + i;
                if (ring_len > 0 && col >= ring_len) col = ring_len >= kStrip ? col - ring_len : col % ring_len;
                ring_store<STORE>(ring, rbase + col, tile[j][i], scale, offset, row);
            }
        }
    }
}

__global__ void ring_write_kernel(float* __restrict__ ring, long long row_stride, long long ring_len,
                                  long long pos, const float* __restrict__ stokes, int nt, int nsub,
                                  int npol, int nchan, int inverted) {
    ring_write_tile(ring, row_stride, ring_len, pos, stokes, nt, nsub, npol, nchan, inverted,
                    blockIdx.x * kStrip, blockIdx.y * kTile);
}

// The rings of many beams: CTAs are laid out job after job; an active beam's
// chunk lands at logical position written * nt.
template <int STORE>
__global__ void ring_write_batch_kernel(const pv::RingJob* __restrict__ jobs, int njobs,
                                        const pv::BeamStep* __restrict__ bs) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].block_begin <= (long long)blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const pv::RingJob& J = jobs[lo];
    const pv::BeamStep& B = bs[J.beam];
    if (!B.active) return;
    const int local = (int)(blockIdx.x - J.block_begin);
    const int tiles_t = (J.nt + kStrip - 1) / kStrip;
    const int bt = local / tiles_t, tt = local - bt * tiles_t;
    ring_write_tile<STORE>(J.ring, J.row_stride, J.ring_len, B.written * J.nt, J.stokes, J.nt, J.nsub,
                           1, J.nchan, J.inverted, tt * kStrip, bt * kTile, J.scale, J.offset);
}

// u8 rings of beams without a clipper: each row's offset (the median of its
// channel) and scale (6 sigma over 127 codes, sigma = 1.4826 times the median
// absolute deviation), from up to 1024 evenly spaced samples of the chunk.  A
// row is calibrated by the first chunk whose deviation is not 0 and keeps its
// scale and offset; until then its samples are stored as the code 128.  Rows
// with a scale already (every row of a clipped beam) return at once.  One CTA
// per channel, bitonic sorts in shared memory.
constexpr int kCalSamples = 1024;

__device__ void bitonic_sort(float* v) {
    for (int k = 2; k <= kCalSamples; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < kCalSamples; i += blockDim.x) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const float a = v[i], b = v[l];
                    if ((a > b) == up) {
                        v[i] = b;
                        v[l] = a;
                    }
                }
            }
            __syncthreads();
        }
}

__global__ void ring_calibrate_kernel(const pv::RingJob* __restrict__ jobs, int njobs,
                                      const pv::BeamStep* __restrict__ bs) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (jobs[mid].cal_begin <= (long long)blockIdx.x) lo = mid;
        else hi = mid - 1;
    }
    const pv::RingJob& J = jobs[lo];
    if (!bs[J.beam].active) return;
    const int nbins = J.nsub * J.nchan;
    const int b = (int)(blockIdx.x - J.cal_begin);
    const int row = J.inverted ? nbins - 1 - b : b;
    if (J.scale[row] > 0.0f) return;  // calibrated already
    __shared__ float v[kCalSamples];
    const int cnt = min(J.nt, kCalSamples);
    for (int i = threadIdx.x; i < kCalSamples; i += blockDim.x)
        v[i] = i < cnt ? J.stokes[(long long)((long long)i * J.nt / cnt) * nbins + b] : INFINITY;
    __syncthreads();
    bitonic_sort(v);
    const float med = v[cnt / 2];
    __syncthreads();
    for (int i = threadIdx.x; i < kCalSamples; i += blockDim.x)
        v[i] = i < cnt ? fabsf(v[i] - med) : INFINITY;
    __syncthreads();
    bitonic_sort(v);
    if (threadIdx.x == 0) {
        const float mad = v[cnt / 2];
        if (mad > 0.0f && mad < INFINITY) {
            J.offset[row] = med;
            J.scale[row] = 6.0f * 1.4826f * mad / 127.0f;
        }
    }
}

// Sum of each active beam's row offsets (added once per dedispersed output).
__global__ void offset_sum_kernel(const pv::RingJob* __restrict__ jobs, int njobs,
                                  const pv::BeamStep* __restrict__ bs) {
    const pv::RingJob& J = jobs[blockIdx.x];
    if (!bs[J.beam].active) return;
    __shared__ float part[256];
    const int nbins = J.nsub * J.nchan;
    float a = 0.0f;
    for (int i = threadIdx.x; i < nbins; i += blockDim.x) a += J.offset[i];
    part[threadIdx.x] = a;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *J.off_sum = part[0];
}

}  // namespace

namespace pv {

int ring_write_device(float* ring, long long row_stride, long long ring_len, long long pos,
                      const float* stokes, int nt, int nsub, int npol, int nchan, int inverted,
                      cudaStream_t s) {
    if (nt <= 0) return PV_OK;
    dim3 grid((unsigned)ceil_div(nt, kStrip), (unsigned)ceil_div(nsub * nchan, kTile));
    ring_write_kernel<<<grid, dim3(kTile, 8), 0, s>>>(ring, row_stride, ring_len, pos, stokes, nt,
                                                     nsub, npol, nchan, inverted);
    return check_launch("ring_write_kernel");
}

int ring_job_blocks(const RingJob& j) {
    return ceil_div(j.nt, kStrip) * ceil_div(j.nsub * j.nchan, kTile);
}

int ring_cal_blocks(const RingJob& j) { return j.nsub * j.nchan; }

int ring_write_batch(const RingJob* d_jobs, int njobs, long long nblocks, const BeamStep* bs,
                     int store, cudaStream_t s) {
    if (nblocks <= 0) return PV_OK;
    const dim3 grid((unsigned)nblocks), block(kTile, 8);
    if (store == PV_STORE_F16) ring_write_batch_kernel<PV_STORE_F16><<<grid, block, 0, s>>>(d_jobs, njobs, bs);
    else if (store == PV_STORE_U8) ring_write_batch_kernel<PV_STORE_U8><<<grid, block, 0, s>>>(d_jobs, njobs, bs);
    else ring_write_batch_kernel<PV_STORE_F32><<<grid, block, 0, s>>>(d_jobs, njobs, bs);
    return check_launch("ring_write_batch_kernel");
}

int ring_calibrate_batch(const RingJob* d_jobs, int njobs, long long nblocks, const BeamStep* bs,
                         cudaStream_t s) {
    if (nblocks <= 0) return PV_OK;
    ring_calibrate_kernel<<<(unsigned)nblocks, 256, 0, s>>>(d_jobs, njobs, bs);
    PV_TRY(check_launch("ring_calibrate_kernel"));
    offset_sum_kernel<<<njobs, 256, 0, s>>>(d_jobs, njobs, bs);
    return check_launch("offset_sum_kernel");
}

}  // namespace pv

extern "C" int pv_ring_write(float* d_ring, long long row_stride, long long ring_len, long long pos,
                             const float* d_stokes, int nt, int nsub, int npol, int nchan,
                             int inverted, void* stream) {
    if (!d_ring || (nt > 0 && !d_stokes) || nt < 0 || nsub <= 0 || npol <= 0 || nchan <= 0 ||
        pos < 0 || row_stride <= 0 || ring_len < 0 || ring_len > row_stride ||
        (ring_len == 0 && pos + nt > row_stride)) {
        pv::set_error("pv_ring_write: invalid arguments");
        return PV_ERR_ARG;
    }
    return pv::ring_write_device(d_ring, row_stride, ring_len, pos, d_stokes, nt, nsub, npol, nchan,
                                 inverted, pv::as_stream(stream));
}
