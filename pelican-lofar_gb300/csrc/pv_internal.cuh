// Internal (non-ABI) entry points shared between translation units.
#pragma once

#include <vector>

#include "pv_common.cuh"

namespace pv {

int ring_write_device(float* ring, long long row_stride, long long ring_len, long long pos,
                      const float* stokes, int nt, int nsub, int npol, int nchan, int inverted,
                      cudaStream_t s);

size_t analyse_scratch_bytes(int tdms, int nsamp, int bin_pow2);
int analyse_launch(const float* data, long long ld, int tdms, int nsamp, float threshold, float rms,
                   int bin_pow2, pv_event* ev, long long cap, long long* d_total, void* scratch,
                   cudaStream_t s);

}  // namespace pv
