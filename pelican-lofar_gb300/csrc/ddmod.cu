// A10: DedispersionModule::dedisperse with the reference's buffering
// (lib/src/DedispersionModule.cpp:109-325, lib/src/DedispersionBuffer.cpp:65-245).
//
// The reference fills host buffers of B = 2^timeBinsPerBufferPow2 samples,
// dedisperses nout = B - maxshift - remainingSamples outputs once a buffer is
// full and starts the next buffer with the last maxshift + remainingSamples
// samples.  Output window k therefore covers input samples
// [k*nout, k*nout + B).  Here the channel rows are a device ring of B samples:
// input blobs of any length are transposed into the ring in pieces that stop
// at each window boundary, every completed window is dedispersed straight
// from the ring, and its DedispersionSpectra waits in a queue until popped.
#include <algorithm>
#include <deque>
#include <vector>

#include "pv_internal.cuh"

struct pv_ddmod {
    int B = 0, tdms = 0;
    float dm_low = 0.0f, dm_step = 0.0f;
    double fch1 = 0.0, foff = 0.0;
    int nbins = 0, maxshift = 0, remaining = 0, nout = 0, inverted = 0;
    double tsamp = 0.0;
    pv_dedisp_plan* plan = nullptr;
    float* d_ring = nullptr;
    long long row_stride = 0;
    long long count = 0;        // samples written (logical)
    long long next_window = 0;  // index of the next window to complete
    float* d_stage = nullptr;
    size_t stage_bytes = 0;
    struct Window {
        float* d_out;
        long long first;
    };
    std::deque<Window> done;
    std::vector<float*> pool;
};

namespace {

void release(pv_ddmod* m) {
    if (m->plan) pv_dedisp_plan_destroy(m->plan);
    m->plan = nullptr;
    if (m->d_ring) cudaFree(m->d_ring);
    m->d_ring = nullptr;
    for (auto& w : m->done) cudaFree(w.d_out);
    m->done.clear();
    for (float* p : m->pool) cudaFree(p);
    m->pool.clear();
}

// DedispersionModule::resize (DedispersionModule.cpp:109-190).
int resize(pv_ddmod* m, int nbins, double tsamp) {
    release(m);
    std::vector<float> k(nbins);
    PV_TRY(pv_dm_shifts(m->fch1, m->foff, nbins, k.data(), &m->inverted));
    PV_TRY(pv_maxshift(m->dm_low, m->dm_step, m->tdms, k.data(), nbins, tsamp, m->B, &m->maxshift,
                       &m->remaining));
    m->nout = m->B - m->maxshift - m->remaining;
    m->tsamp = tsamp;
    // the reference kernel takes tsamp as float (DedispersionModule.cpp:181-184, :363-364)
    const float ts = (float)tsamp;
    PV_TRY(pv_dedisp_plan_create(&m->plan, k.data(), nbins, m->tdms, m->dm_low / ts, m->dm_step / ts));
    m->row_stride = (m->B + 3) / 4 * 4;
    PV_CUDA(cudaMalloc(&m->d_ring, sizeof(float) * (size_t)nbins * m->row_stride), "allocate ring");
    PV_CUDA(cudaMemset(m->d_ring, 0, sizeof(float) * (size_t)nbins * m->row_stride), "clear ring");
    m->nbins = nbins;
    m->count = 0;
    m->next_window = 0;
    return PV_OK;
}

}  // namespace

extern "C" int pv_ddmod_create(pv_ddmod** out, int buffer_samples, int tdms, float dm_low,
                               float dm_step, double fch1, double foff) {
    if (!out || buffer_samples <= 0 || tdms <= 0) {
        pv::set_error("DedispersionModule: invalid buffer or trial count");
        return PV_ERR_CONFIG;
    }
    if (fch1 == 0.0) {
        pv::set_error("DedispersionModule: frequencyChannel1 must be a positve number");
        return PV_ERR_CONFIG;
    }
    auto* m = new pv_ddmod;
    m->B = buffer_samples;
    m->tdms = tdms;
    m->dm_low = dm_low < 0.0f ? 0.0f : dm_low;  // DedispersionModule.cpp:57
    m->dm_step = dm_step;
    m->fch1 = fch1;
    m->foff = foff;
    *out = m;
    return PV_OK;
}

extern "C" void pv_ddmod_destroy(pv_ddmod* m) {
    if (!m) return;
    release(m);
    if (m->d_stage) cudaFree(m->d_stage);
    delete m;
}

extern "C" int pv_ddmod_add(pv_ddmod* m, const float* stokes, int nt, int nsub, int npol, int nchan,
                            double tsamp, int* completed, void* stream) {
    if (!m || !stokes || nt < 0 || nsub <= 0 || npol <= 0 || nchan <= 0) {
        pv::set_error("pv_ddmod_add: invalid arguments");
        return PV_ERR_ARG;
    }
    cudaStream_t s = pv::as_stream(stream);
    const int nbins = nsub * nchan;
    if (nbins != m->nbins) PV_TRY(resize(m, nbins, tsamp));
    const size_t bytes = sizeof(float) * (size_t)nt * nsub * npol * nchan;
    if (bytes > m->stage_bytes) {
        if (m->d_stage) cudaFree(m->d_stage);
        m->d_stage = nullptr;
        m->stage_bytes = 0;
        PV_CUDA(cudaMalloc(&m->d_stage, bytes), "allocate staging");
        m->stage_bytes = bytes;
    }
    // Host or device input (unified addressing decides the direction).
    PV_CUDA(cudaMemcpyAsync(m->d_stage, stokes, bytes, cudaMemcpyDefault, s), "stage Stokes data");
    int n_done = 0;
    int t = 0;
    const long long spectrum = (long long)nsub * npol * nchan;
    while (t < nt) {
        const long long boundary = m->next_window * m->nout + m->B;  // window completes here
        const int n = (int)std::min<long long>(nt - t, boundary - m->count);
        PV_TRY(pv::ring_write_device(m->d_ring, m->row_stride, m->B, m->count,
                                     m->d_stage + (long long)t * spectrum, n, nsub, npol, nchan,
                                     m->inverted, s));
        m->count += n;
        t += n;
        if (m->count == boundary) {
            float* out = nullptr;
            if (!m->pool.empty()) {
                out = m->pool.back();
                m->pool.pop_back();
            } else {
                PV_CUDA(cudaMalloc(&out, sizeof(float) * (size_t)m->tdms * m->nout),
                        "allocate DedispersionSpectra");
            }
            const long long first = m->next_window * m->nout;
            PV_TRY(pv_dedisp_plan_run(m->plan, out, m->nout, m->d_ring, m->row_stride, 0, m->B,
                                      first % m->B, m->nout, stream));
            m->done.push_back({out, first});
            m->next_window += 1;
            ++n_done;
        }
    }
    if (completed) *completed = n_done;
    return PV_OK;
}

extern "C" int pv_ddmod_pop(pv_ddmod* m, float* out, long long cap_floats, int* nout,
                            long long* first_sample, void* stream) {
    if (!m) return PV_ERR_ARG;
    if (m->done.empty()) {
        if (nout) *nout = 0;
        return PV_OK;
    }
    const pv_ddmod::Window w = m->done.front();
    const long long n = (long long)m->tdms * m->nout;
    if (out) {
        if (cap_floats < n) {
            pv::set_error("pv_ddmod_pop: output of %lld floats is smaller than %d x %d", cap_floats,
                          m->tdms, m->nout);
            return PV_ERR_ARG;
        }
        PV_CUDA(cudaMemcpyAsync(out, w.d_out, sizeof(float) * n, cudaMemcpyDefault,
                                pv::as_stream(stream)), "copy DedispersionSpectra");
        PV_CUDA(cudaStreamSynchronize(pv::as_stream(stream)), "synchronise");
    }
    int status = PV_OK;
    PV_TRY(pv_dedisp_plan_status(m->plan, &status));
    if (status != PV_OK) {
        pv::set_error("pv_ddmod_pop: a dedispersion pipeline wait gave up");
        return status;
    }
    m->done.pop_front();
    m->pool.push_back(w.d_out);
    if (nout) *nout = m->nout;
    if (first_sample) *first_sample = w.first;
    return PV_OK;
}

extern "C" int pv_ddmod_params(const pv_ddmod* m, int* h_out6) {
    if (!m || !h_out6) return PV_ERR_ARG;
    h_out6[0] = m->maxshift;
    h_out6[1] = m->remaining;
    h_out6[2] = m->nout;
    h_out6[3] = m->nbins;
    h_out6[4] = m->inverted;
    h_out6[5] = (int)m->done.size();
    return PV_OK;
}
