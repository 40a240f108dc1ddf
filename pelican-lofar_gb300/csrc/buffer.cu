// A8: DedispersionBuffer::addSamples on the device
// (lib/src/DedispersionBuffer.cpp:98-180).
//
// Stokes samples [t][sub][pol][chan] (pol 0 used, DedispersionBuffer.cpp:116)
// are transposed into the per-channel dedispersion ring: row r holds bin r,
// or bin nbins-1-r for an inverted (ascending) band, and logical sample
// pos+t lands at physical column (pos+t) mod ring_len.  The noise-template
// substitution of DedispersionBuffer.cpp:169 is omitted: the reference's
// weights are always 1, which makes it the identity.
#include "pv_internal.cuh"

namespace {

constexpr int kTile = 32;

__device__ __forceinline__ void ring_write_tile(float* __restrict__ ring, long long row_stride,
                                                long long ring_len, long long pos,
                                                const float* __restrict__ stokes, int nt, int nsub,
                                                int npol, int nchan, int inverted, int t0, int b0) {
    __shared__ float tile[kTile][kTile + 1];
    const int nbins = nsub * nchan;
    // read: rows of the tile are samples, columns are bins (coalesced in bins)
    for (int i = threadIdx.y; i < kTile; i += blockDim.y) {
        const int t = t0 + i, b = b0 + threadIdx.x;
        if (t < nt && b < nbins) {
            const int s = b / nchan, c = b - s * nchan;
            tile[i][threadIdx.x] = stokes[(long long)nchan * (npol * ((long long)nsub * t + s)) + c];
        }
    }
    __syncthreads();
    // write: rows of the ring are bins, columns samples (coalesced in samples)
    for (int i = threadIdx.y; i < kTile; i += blockDim.y) {
        const int b = b0 + i, t = t0 + threadIdx.x;
        if (t < nt && b < nbins) {
            const int row = inverted ? nbins - 1 - b : b;
            long long col = pos + t;
            if (ring_len > 0) col %= ring_len;
            ring[(long long)row * row_stride + col] = tile[threadIdx.x][i];
        }
    }
}

__global__ void ring_write_kernel(float* __restrict__ ring, long long row_stride, long long ring_len,
                                  long long pos, const float* __restrict__ stokes, int nt, int nsub,
                                  int npol, int nchan, int inverted) {
    ring_write_tile(ring, row_stride, ring_len, pos, stokes, nt, nsub, npol, nchan, inverted,
                    blockIdx.x * kTile, blockIdx.y * kTile);
}

// The rings of many beams: CTAs are laid out job after job; an active beam's
// chunk lands at logical position written * nt.
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
    const int tiles_t = (J.nt + kTile - 1) / kTile;
    const int bt = local / tiles_t, tt = local - bt * tiles_t;
    ring_write_tile(J.ring, J.row_stride, J.ring_len, B.written * J.nt, J.stokes, J.nt, J.nsub, 1,
                    J.nchan, J.inverted, tt * kTile, bt * kTile);
}

}  // namespace

namespace pv {

int ring_write_device(float* ring, long long row_stride, long long ring_len, long long pos,
                      const float* stokes, int nt, int nsub, int npol, int nchan, int inverted,
                      cudaStream_t s) {
    if (nt <= 0) return PV_OK;
    dim3 grid((unsigned)ceil_div(nt, kTile), (unsigned)ceil_div(nsub * nchan, kTile));
    ring_write_kernel<<<grid, dim3(kTile, 8), 0, s>>>(ring, row_stride, ring_len, pos, stokes, nt,
                                                     nsub, npol, nchan, inverted);
    return check_launch("ring_write_kernel");
}

int ring_job_blocks(const RingJob& j) {
    return ceil_div(j.nt, kTile) * ceil_div(j.nsub * j.nchan, kTile);
}

int ring_write_batch(const RingJob* d_jobs, int njobs, long long nblocks, const BeamStep* bs,
                     cudaStream_t s) {
    if (nblocks <= 0) return PV_OK;
    ring_write_batch_kernel<<<(unsigned)nblocks, dim3(kTile, 8), 0, s>>>(d_jobs, njobs, bs);
    return check_launch("ring_write_batch_kernel");
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
