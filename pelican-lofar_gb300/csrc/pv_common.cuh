// Shared helpers of libpv: status codes, thread-local error text, launch
// accounting and small device utilities.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "pv.h"

namespace pv {

// Thread-local last error message returned by pv_last_error().
void set_error(const char* fmt, ...);
const char* last_error();

// Kernels launched by this library since load (pv_kernel_launches()).
extern std::atomic<long long> g_launches;

// Limit of a pipelined kernel's bounded device-side waits (ns), passed to
// each launch (pv_set_wait_limit).  The drain of a kernel's own copies in
// flight after a give-up always waits up to kDrainWaitNs.
constexpr unsigned long long kDefaultWaitNs = 500000000ull;  // 0.5 s
constexpr unsigned long long kDrainWaitNs = 500000000ull;
extern std::atomic<unsigned long long> g_wait_ns;
inline unsigned long long wait_ns() { return g_wait_ns.load(std::memory_order_relaxed); }
// Failure-path test hook (pv_stall_next_launches): the next n pipelined
// dedispersion launches withhold the copies of their first stage.
extern std::atomic<int> g_stall_launches;
inline int take_stall() {
    int n = g_stall_launches.load();
    while (n > 0 && !g_stall_launches.compare_exchange_weak(n, n - 1)) {
    }
    return n > 0 ? 1 : 0;
}
inline void count_launch(long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }

inline int cuda_status(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return PV_OK;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return PV_ERR_CUDA;
}

// Checks the launch that was just issued.
inline int check_launch(const char* what) {
    count_launch();
    return cuda_status(cudaGetLastError(), what);
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

template <typename T>
inline T ceil_div(T a, T b) { return (a + b - 1) / b; }

// Number of SMs of the current device (cached per device).
int sm_count();
// Largest dynamic shared memory a CTA may opt into on the current device.  The
// batched kernels set their attribute to it once: the attribute is global to
// the process, and launches captured into a graph for one batch must not
// depend on the shared memory another batch asked for afterwards.
int smem_optin();
// Sets kern's dynamic shared-memory limit to smem_optin() less its static
// shared memory; *limit (if given) receives that limit.
template <typename Kernel>
cudaError_t allow_max_dynamic_smem(Kernel kern, size_t* limit = nullptr) {
    cudaFuncAttributes a{};
    cudaError_t e = cudaFuncGetAttributes(&a, kern);
    if (e != cudaSuccess) return e;
    const int dyn = smem_optin() - (int)a.sharedSizeBytes;
    if (limit) *limit = (size_t)dyn;
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn);
}

// Stream-ordered scratch allocation (cudaMallocAsync / cudaFreeAsync).
int scratch_alloc(void** p, size_t bytes, cudaStream_t s);
void scratch_free(void* p, cudaStream_t s);

}  // namespace pv

#define PV_TRY(expr)                   \
    do {                               \
        int _rc = (expr);              \
        if (_rc != PV_OK) return _rc;  \
    } while (0)

#define PV_CUDA(expr, what) PV_TRY(pv::cuda_status((expr), (what)))

// The reference kernel's per-(channel, trial) integer delay
// (DedispersionKernel.cu:29,36): trunc(dmshift[c] * (start + d*step)), the
// trial value formed with one fused multiply-add as nvcc contracts it.
__device__ __forceinline__ float pv_trial_value(int d, float start, float step) {
    return fmaf((float)d, step, start);
}
__device__ __forceinline__ int pv_shift(float dmshift, float trial_value) {
    return __float2int_rz(__fmul_rn(dmshift, trial_value));
}
