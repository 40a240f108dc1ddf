// libpv runtime helpers: error text, launch counter, device queries,
// scratch memory and the host-side delay-table functions.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "pv_common.cuh"

namespace pv {

namespace {
thread_local char t_error[512] = "";
std::mutex g_sm_mutex;
std::vector<int> g_sm_counts;
}  // namespace

std::atomic<long long> g_launches{0};
std::atomic<unsigned long long> g_wait_ns{kDefaultWaitNs};
std::atomic<int> g_stall_launches{0};

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(t_error, sizeof(t_error), fmt, ap);
    va_end(ap);
}

const char* last_error() { return t_error; }

int sm_count() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 152;
    std::lock_guard<std::mutex> lk(g_sm_mutex);
    if ((int)g_sm_counts.size() <= dev) g_sm_counts.resize(dev + 1, 0);
    if (g_sm_counts[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 152;
        g_sm_counts[dev] = n;
    }
    return g_sm_counts[dev];
}

int smem_optin() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || n <= 0)
        return 227 * 1024;
    return n;
}

int scratch_alloc(void** p, size_t bytes, cudaStream_t s) {
    *p = nullptr;
    if (bytes == 0) return PV_OK;
    cudaError_t e = cudaMallocAsync(p, bytes, s);
    if (e != cudaSuccess) {
        set_error("scratch allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return PV_ERR_NOMEM;
    }
    return PV_OK;
}

void scratch_free(void* p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
}

}  // namespace pv

extern "C" const char* pv_last_error(void) { return pv::last_error(); }
extern "C" int pv_version(void) { return 100; }
extern "C" long long pv_kernel_launches(void) { return pv::g_launches.load(); }

extern "C" int pv_stall_next_launches(int n) {
    const int prev = pv::g_stall_launches.load();
    pv::g_stall_launches.store(n > 0 ? n : 0);
    return prev;
}

extern "C" long long pv_set_wait_limit(long long ns) {
    const unsigned long long prev = pv::g_wait_ns.load();
    pv::g_wait_ns.store(ns > 0 ? (unsigned long long)ns : pv::kDefaultWaitNs);
    return (long long)prev;
}

// ---------------------------------------------------------------------------
// Host-side delay table (DedispersionModule::resize, DedispersionModule.cpp:151-162)
// ---------------------------------------------------------------------------
extern "C" int pv_dm_shifts(double fch1, double foff, int nchan, float* h_dmshift, int* inverted) {
    if (nchan <= 0 || !h_dmshift) {
        pv::set_error("pv_dm_shifts: nchan must be > 0");
        return PV_ERR_ARG;
    }
    if (fch1 == 0.0) {
        pv::set_error("DedispersionModule: frequencyChannel1 must be a positve number");
        return PV_ERR_CONFIG;
    }
    // Channels of an ascending band are taken from the top down, so that the
    // reference frequency is the highest and every delay is non-negative.
    const int inv = foff >= 0 ? 1 : 0;
    const double f_top = inv ? fch1 + foff * (nchan - 1) : fch1;
    const double step = inv ? -foff : foff;
    const double k = 4148.741601;
    for (int c = 0; c < nchan; ++c) {
        const double f = f_top + (step * c);
        h_dmshift[c] = (float)(k * ((1.0 / f / f) - (1.0 / f_top / f_top)));
    }
    if (inverted) *inverted = inv;
    return PV_OK;
}

extern "C" int pv_maxshift(float dm_low, float dm_step, int tdms, const float* h_dmshift, int nchan,
                           double tsamp, int buffer_samples, int* maxshift, int* remaining) {
    if (nchan <= 0 || tdms <= 0 || tsamp <= 0.0 || !h_dmshift) {
        pv::set_error("pv_maxshift: invalid arguments");
        return PV_ERR_ARG;
    }
    // The largest trial's value times the last (largest) channel constant,
    // formed in float and divided by the double sample time.
    const float dm_max = dm_low + dm_step * (float)(unsigned)(tdms - 1);
    const float delay = dm_max * h_dmshift[nchan - 1];
    const int ms = (int)((double)delay / tsamp);
    if (maxshift) *maxshift = ms;
    // The reference keeps the dedispersed length a multiple of its 14x16
    // launch tile.
    if (remaining) *remaining = (int)(((unsigned)buffer_samples - (unsigned)ms) % 224u);
    if (buffer_samples <= ms) {
        pv::set_error("DedispersionModule: maxshift requirements (%d) are bigger than the number "
                      "of samples (%d)", ms, buffer_samples);
        return PV_ERR_CONFIG;
    }
    return PV_OK;
}

extern "C" int pv_device_copy(void* dst, const void* src, long long bytes, void* stream) {
    if ((!dst || !src) && bytes > 0) {
        pv::set_error("pv_device_copy: null pointer");
        return PV_ERR_ARG;
    }
    if (bytes <= 0) return PV_OK;
    PV_CUDA(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, pv::as_stream(stream)),
            "pv_device_copy");
    return PV_OK;
}

extern "C" int pv_host_alloc(void** h_ptr, long long bytes, int write_combined) {
    if (!h_ptr || bytes <= 0) {
        pv::set_error("pv_host_alloc: invalid arguments");
        return PV_ERR_ARG;
    }
    const unsigned flags = cudaHostAllocPortable | (write_combined ? cudaHostAllocWriteCombined : 0u);
    const cudaError_t e = cudaHostAlloc(h_ptr, (size_t)bytes, flags);
    if (e != cudaSuccess) {
        *h_ptr = nullptr;
        pv::set_error("pv_host_alloc: %s (%lld bytes)", cudaGetErrorString(e), bytes);
        return PV_ERR_NOMEM;
    }
    return PV_OK;
}

extern "C" void pv_host_free(void* h_ptr) {
    if (h_ptr) cudaFreeHost(h_ptr);
}

extern "C" int pv_device_alloc(void** d_ptr, long long bytes) {
    if (!d_ptr || bytes < 0) {
        pv::set_error("pv_device_alloc: invalid arguments");
        return PV_ERR_ARG;
    }
    *d_ptr = nullptr;
    if (bytes == 0) return PV_OK;
    const cudaError_t e = cudaMalloc(d_ptr, (size_t)bytes);
    if (e != cudaSuccess) {
        *d_ptr = nullptr;
        pv::set_error("pv_device_alloc: %s (%lld bytes)", cudaGetErrorString(e), bytes);
        return PV_ERR_NOMEM;
    }
    return PV_OK;
}

extern "C" void pv_device_free(void* d_ptr) {
    if (d_ptr) cudaFree(d_ptr);
}

extern "C" int pv_synchronize(void* stream) {
    PV_CUDA(cudaStreamSynchronize(pv::as_stream(stream)), "pv_synchronize");
    return PV_OK;
}
