// The batched serving form of the beam chain: many beams of different
// channel counts, trial counts and delay ranges advance one chunk per step,
// each stage of all beams in as few launches as the kernels allow:
//
//   K1  chan_stokes_i_kernel   one launch per channels-per-subband class
//   K2  rfi_batch_kernel       one CTA per beam, one launch per CTA size
//   A8  ring_write_batch_kernel one launch
//   K4  dedisperse_batch_kernel one persistent launch over every beam's tiles,
//                              DM x time tile shape chosen by the autotuner
//   K5  analyser               per beam (count, scan, emit)
//
// Every launch reads the chunk index from a device step counter that the
// step's last kernel advances, so one captured CUDA graph replays every
// step unchanged.  The chain of each beam is the pv_beam chain: the same
// state layout (tap history, RFI state, delay ring) and the same arithmetic,
// so a beam's events in the batch equal its events run alone.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pv_internal.cuh"

namespace {

__global__ void step_advance_kernel(long long* step) { *step += 1; }

}  // namespace

struct pv_batch {
    int n = 0;
    int flags = 0;
    std::vector<pv_beam*> beams;
    std::vector<void*> d_in;
    std::vector<long long> in_bytes;
    std::vector<float2*> d_hist;  // two per beam
    struct ChanClass {
        int nchan = 0, njobs = 0;
        long long nwarps = 0;
        pv::ChanJob* d_jobs = nullptr;
    };
    std::vector<ChanClass> chan;
    pv::RfiBatch* rfi = nullptr;
    pv::RingJob* d_ring_jobs = nullptr;
    long long ring_blocks = 0;
    pv::DdBatch* dd = nullptr;
    long long* d_step = nullptr;
    long long* h_totals = nullptr;  // pinned, one per beam
    long long step = 0;             // steps issued
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long graph_kernels = 0;
    cudaEvent_t ev[6] = {};
    bool timed = false;
};

namespace {

void destroy(pv_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    for (auto e : b->ev)
        if (e) cudaEventDestroy(e);
    if (b->dd) pv::dd_batch_destroy(b->dd);
    if (b->rfi) pv::rfi_batch_destroy(b->rfi);
    for (auto& c : b->chan)
        if (c.d_jobs) cudaFree(c.d_jobs);
    if (b->d_ring_jobs) cudaFree(b->d_ring_jobs);
    if (b->d_step) cudaFree(b->d_step);
    if (b->h_totals) cudaFreeHost(b->h_totals);
    for (void* p : b->d_in)
        if (p) cudaFree(p);
    for (void* p : b->d_hist)
        if (p) cudaFree(p);
    for (pv_beam* x : b->beams)
        if (x) pv_beam_destroy(x);
    delete b;
}

// Issues one step of every beam on stream s.
int enqueue_step(pv_batch* b, cudaStream_t s, bool capture) {
    const bool timing = (b->flags & PV_BATCH_TIMING) != 0;
    auto mark = [&](int i) -> int {
        if (!timing) return PV_OK;
        return pv::cuda_status(capture ? cudaEventRecordWithFlags(b->ev[i], s, cudaEventRecordExternal)
                                       : cudaEventRecord(b->ev[i], s),
                               "record stage event");
    };
    PV_TRY(mark(0));
    for (auto& c : b->chan)
        PV_TRY(pv::launch_chan_fast(c.nchan, 1, c.d_jobs, pv::ChanJob{}, c.njobs, c.nwarps, b->d_step, s));
    PV_TRY(mark(1));
    if (b->rfi) PV_TRY(pv::rfi_batch_launch(b->rfi, s));
    PV_TRY(mark(2));
    PV_TRY(pv::ring_write_batch(b->d_ring_jobs, b->n, b->ring_blocks, b->d_step, s));
    PV_TRY(mark(3));
    PV_TRY(pv::dd_batch_launch(b->dd, b->d_step, s));
    PV_TRY(mark(4));
    for (int i = 0; i < b->n; ++i) {
        pv_beam* x = b->beams[i];
        const pv_beam_config& c = x->cfg;
        PV_TRY(pv::analyse_launch(x->d_out, c.chunk, c.tdms, c.chunk, c.threshold, x->rms, c.bin_pow2,
                                  x->d_events, x->cap, x->d_total, x->d_scratch, s));
        PV_CUDA(cudaMemcpyAsync(b->h_totals + i, x->d_total, sizeof(long long), cudaMemcpyDeviceToHost, s),
                "read event count");
    }
    PV_TRY(mark(5));
    step_advance_kernel<<<1, 1, 0, s>>>(b->d_step);
    return pv::check_launch("step_advance_kernel");
}

int capture(pv_batch* b) {
    PV_CUDA(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking), "create capture stream");
    const long long before = pv_kernel_launches();
    PV_CUDA(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal), "begin capture");
    const int rc = enqueue_step(b, b->cap_stream, true);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
    b->graph = g;
    const long long captured = pv_kernel_launches() - before;
    pv::g_launches.fetch_sub(captured);  // counted again at every replay
    if (rc != PV_OK) return rc;
    PV_CUDA(e, "end capture");
    PV_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0), "instantiate step graph");
    b->graph_kernels = captured;
    return PV_OK;
}

}  // namespace

extern "C" int pv_batch_create(pv_batch** out, const pv_beam_config* configs, int nbeams, int flags) {
    if (!out || !configs || nbeams <= 0) {
        pv::set_error("pv_batch_create: no beams");
        return PV_ERR_ARG;
    }
    *out = nullptr;
    auto* b = new pv_batch;
    b->n = nbeams;
    b->flags = flags;
    b->beams.assign(nbeams, nullptr);
    b->d_in.assign(nbeams, nullptr);
    b->in_bytes.assign(nbeams, 0);
    b->d_hist.assign(2 * nbeams, nullptr);
    int rc = PV_OK;
    auto fail = [&](int code) {
        destroy(b);
        return code;
    };
    const int chunk = configs[0].chunk;
    for (int i = 0; i < nbeams; ++i) {
        pv_beam_config c = configs[i];
        c.timing = 0;
        c.debug_taps = 0;
        if (c.chunk != chunk || c.chunk % 4 != 0) {
            pv::set_error("pv_batch_create: every beam needs the same chunk, a multiple of 4 spectra "
                          "(beam %d: %d)", i, c.chunk);
            return fail(PV_ERR_CONFIG);
        }
        if (!pv::chan_fast_supported(c.nchan_sub, c.ntaps, 2, 1, c.int_time, c.int_chan,
                                     c.chunk * c.int_time)) {
            pv::set_error("pv_batch_create: beam %d: the batched channeliser takes 16, 32 or 64 "
                          "channels, 8 taps, no channel binning and a time window dividing 256",
                          i);
            return fail(PV_ERR_CONFIG);
        }
        rc = pv_beam_create(&b->beams[i], &c);
        if (rc != PV_OK) return fail(rc);
        pv_beam* x = b->beams[i];
        b->in_bytes[i] = pv_beam_input_bytes(x, 1);
        const size_t hist = sizeof(float2) * (size_t)c.nsub * 2 * 7 * c.nchan_sub;
        cudaError_t e = cudaMalloc(&b->d_in[i], b->in_bytes[i]);
        for (int h = 0; h < 2 && e == cudaSuccess; ++h) {
            e = cudaMalloc(&b->d_hist[2 * i + h], hist);
            if (e == cudaSuccess) e = cudaMemset(b->d_hist[2 * i + h], 0, hist);
        }
        if (e == cudaSuccess) e = cudaMemset(x->d_out, 0, sizeof(float) * (size_t)c.tdms * c.chunk);
        if (e != cudaSuccess) {
            pv::set_error("pv_batch_create: beam %d: %s", i, cudaGetErrorString(e));
            return fail(PV_ERR_NOMEM);
        }
    }
    cudaStream_t s0 = nullptr;
    // K1 jobs, one launch per channel count
    std::vector<std::vector<pv::ChanJob>> cj;
    for (int i = 0; i < nbeams; ++i) {
        pv_beam* x = b->beams[i];
        const float* coeffs = nullptr;
        const float2* tw = nullptr;
        int nchan = 0, ntaps = 0;
        rc = pv::ppf_tables(x->ppf, &coeffs, &tw, &nchan, &ntaps);
        if (rc != PV_OK) return fail(rc);
        size_t k = 0;
        while (k < b->chan.size() && b->chan[k].nchan != nchan) ++k;
        if (k == b->chan.size()) {
            b->chan.emplace_back();
            b->chan[k].nchan = nchan;
            cj.emplace_back();
        }
        pv::ChanJob j{};
        j.in = b->d_in[i];
        j.hist[0] = b->d_hist[2 * i];
        j.hist[1] = b->d_hist[2 * i + 1];
        j.coeffs = coeffs;
        j.twiddle = tw;
        j.out = x->d_fb;
        j.nsub = x->cfg.nsub;
        j.nblocks = x->cfg.chunk * x->cfg.int_time;
        j.window = x->cfg.int_time;
        j.nu = x->cfg.chunk;
        j.warp_begin = b->chan[k].nwarps;
        b->chan[k].nwarps += pv::chan_job_warps(j);
        cj[k].push_back(j);
    }
    for (size_t k = 0; k < b->chan.size(); ++k) {
        auto& c = b->chan[k];
        c.njobs = (int)cj[k].size();
        if (cudaMalloc(&c.d_jobs, sizeof(pv::ChanJob) * cj[k].size()) != cudaSuccess ||
            cudaMemcpy(c.d_jobs, cj[k].data(), sizeof(pv::ChanJob) * cj[k].size(),
                       cudaMemcpyHostToDevice) != cudaSuccess) {
            pv::set_error("pv_batch_create: cannot upload channeliser jobs");
            return fail(PV_ERR_CUDA);
        }
    }
    // K2: clippers
    {
        std::vector<pv_rfi*> hs(nbeams);
        std::vector<float*> data(nbeams);
        std::vector<int> nsub(nbeams), nch(nbeams);
        for (int i = 0; i < nbeams; ++i) {
            hs[i] = b->beams[i]->rfi;
            data[i] = b->beams[i]->d_fb;
            nsub[i] = b->beams[i]->cfg.nsub;
            nch[i] = b->beams[i]->nchan_fb;
        }
        rc = pv::rfi_batch_create(&b->rfi, hs.data(), data.data(), nsub.data(), nch.data(), nbeams,
                                  chunk, s0);
        if (rc != PV_OK) return fail(rc);
    }
    // A8: ring writes
    {
        std::vector<pv::RingJob> rj(nbeams);
        for (int i = 0; i < nbeams; ++i) {
            pv_beam* x = b->beams[i];
            rj[i] = pv::RingJob{x->d_ring, x->row_stride, x->ring_len, x->d_fb, chunk, x->cfg.nsub,
                                x->nchan_fb, x->inverted, b->ring_blocks, x->chunks};
            b->ring_blocks += pv::ring_job_blocks(rj[i]);
        }
        if (cudaMalloc(&b->d_ring_jobs, sizeof(pv::RingJob) * nbeams) != cudaSuccess ||
            cudaMemcpy(b->d_ring_jobs, rj.data(), sizeof(pv::RingJob) * nbeams, cudaMemcpyHostToDevice) !=
                cudaSuccess) {
            pv::set_error("pv_batch_create: cannot upload ring jobs");
            return fail(PV_ERR_CUDA);
        }
    }
    // K4: dedispersion tiles (autotuned unless a variant is forced)
    {
        std::vector<pv::DdBeam> db(nbeams);
        for (int i = 0; i < nbeams; ++i) {
            pv_beam* x = b->beams[i];
            pv::DdBeam& d = db[i];
            int nchan = 0, tdms = 0;
            rc = pv::plan_tables(x->plan, &d.d_dmshift, &d.h_dmshift, &nchan, &tdms, &d.start, &d.step);
            if (rc != PV_OK) return fail(rc);
            d.out = x->d_out;
            d.out_stride = chunk;
            d.ring = x->d_ring;
            d.row_stride = x->row_stride;
            d.ring_len = x->ring_len;
            d.nchan = nchan;
            d.nout = chunk;
            d.tdms = tdms;
            d.lag = x->lag;
            d.chunk = chunk;
            d.base = (int)x->chunks;  // lag when the beam starts prefilled, else 0
        }
        const int variant = (flags & PV_BATCH_TUNE) ? -1 : PV_BATCH_VARIANT_OF(flags);
        rc = pv::dd_batch_create(&b->dd, db.data(), nbeams, variant, s0);
        if (rc != PV_OK) return fail(rc);
    }
    if (cudaMalloc(&b->d_step, sizeof(long long)) != cudaSuccess ||
        cudaMemset(b->d_step, 0, sizeof(long long)) != cudaSuccess ||
        cudaMallocHost(&b->h_totals, sizeof(long long) * nbeams) != cudaSuccess) {
        pv::set_error("pv_batch_create: cannot allocate the step counter");
        return fail(PV_ERR_NOMEM);
    }
    std::fill(b->h_totals, b->h_totals + nbeams, 0LL);
    if (flags & PV_BATCH_TIMING) {
        for (auto& e : b->ev)
            if (cudaEventCreate(&e) != cudaSuccess) {
                pv::set_error("pv_batch_create: cudaEventCreate failed");
                return fail(PV_ERR_CUDA);
            }
    }
    if (cudaDeviceSynchronize() != cudaSuccess) {
        rc = pv::cuda_status(cudaGetLastError(), "pv_batch_create");
        return fail(rc);
    }
    if (flags & PV_BATCH_GRAPH) {
        rc = capture(b);
        if (rc != PV_OK) return fail(rc);
    }
    *out = b;
    return PV_OK;
}

extern "C" void pv_batch_destroy(pv_batch* b) {
    if (b) destroy(b);
}

extern "C" int pv_batch_input(pv_batch* b, int beam, void** d_voltages, long long* bytes) {
    if (!b || beam < 0 || beam >= b->n) return PV_ERR_ARG;
    if (d_voltages) *d_voltages = b->d_in[beam];
    if (bytes) *bytes = b->in_bytes[beam];
    return PV_OK;
}

extern "C" int pv_batch_run(pv_batch* b, void* stream) {
    if (!b) return PV_ERR_ARG;
    cudaStream_t s = pv::as_stream(stream);
    if (b->exec) {
        PV_CUDA(cudaGraphLaunch(b->exec, s), "launch step graph");
        pv::count_launch(b->graph_kernels);
    } else {
        PV_TRY(enqueue_step(b, s, false));
    }
    b->step += 1;
    b->timed = (b->flags & PV_BATCH_TIMING) != 0;
    return PV_OK;
}

extern "C" int pv_batch_run_host(pv_batch* b, const void* const* h_voltages, void* stream) {
    if (!b || !h_voltages) return PV_ERR_ARG;
    cudaStream_t s = pv::as_stream(stream);
    for (int i = 0; i < b->n; ++i) {
        if (!h_voltages[i]) {
            pv::set_error("pv_batch_run_host: no voltages for beam %d", i);
            return PV_ERR_ARG;
        }
        PV_CUDA(cudaMemcpyAsync(b->d_in[i], h_voltages[i], b->in_bytes[i], cudaMemcpyHostToDevice, s),
                "copy voltages to the device");
    }
    return pv_batch_run(b, stream);
}

extern "C" int pv_batch_events(pv_batch* b, int beam, pv_event* h_events, long long cap,
                               long long* h_count, long long* h_first_sample, void* stream) {
    if (!b || beam < 0 || beam >= b->n || !h_count) return PV_ERR_ARG;
    PV_CUDA(cudaStreamSynchronize(pv::as_stream(stream)), "synchronise");
    int status = PV_OK;
    PV_TRY(pv::dd_batch_status(b->dd, &status));
    if (status != PV_OK) {
        pv::set_error("pv_batch_events: a dedispersion pipeline wait gave up (status %d)", status);
        return status;
    }
    pv_beam* x = b->beams[beam];
    const long long w = b->step + x->chunks - 1 - x->lag;  // x->chunks: prefilled chunks
    if (w < 0) {
        *h_count = 0;
        if (h_first_sample) *h_first_sample = -1;
        return PV_OK;
    }
    *h_count = b->h_totals[beam];
    if (h_first_sample) *h_first_sample = w * x->cfg.chunk;
    const long long n = std::min(std::min(b->h_totals[beam], x->cap), cap);
    if (h_events && n > 0)
        PV_CUDA(cudaMemcpy(h_events, x->d_events, sizeof(pv_event) * n, cudaMemcpyDeviceToHost),
                "copy events");
    return PV_OK;
}

extern "C" int pv_batch_info(const pv_batch* b, int beam, long long* h_info8) {
    if (!b || beam < 0 || beam >= b->n || !h_info8) return PV_ERR_ARG;
    const pv_beam* x = b->beams[beam];
    h_info8[0] = x->nbins;
    h_info8[1] = x->max_shift;
    h_info8[2] = x->lag;
    h_info8[3] = x->ring_len;
    h_info8[4] = x->inverted;
    h_info8[5] = b->step + x->chunks;
    h_info8[6] = b->step + x->chunks - 1 - x->lag;
    h_info8[7] = (long long)x->nbins * x->row_stride * (long long)sizeof(float);
    return PV_OK;
}

extern "C" int pv_batch_tiles(const pv_batch* b, int* h_shape8, int* h_dms, float* h_tune_ms4,
                              long long* h_graph_kernels) {
    if (!b) return PV_ERR_ARG;
    if (h_shape8) PV_TRY(pv::dd_batch_shape(b->dd, h_shape8));
    if (h_dms) {
        const auto& d = pv::dd_batch_dms(b->dd);
        std::copy(d.begin(), d.end(), h_dms);
    }
    if (h_tune_ms4) {
        const auto& t = pv::dd_batch_tune_ms(b->dd);
        for (int i = 0; i < 4; ++i) h_tune_ms4[i] = i < (int)t.size() ? t[i] : -1.0f;
    }
    if (h_graph_kernels) *h_graph_kernels = b->exec ? b->graph_kernels : 0;
    return PV_OK;
}

extern "C" int pv_batch_stage_ms(pv_batch* b, float* h_ms5) {
    if (!b || !h_ms5) return PV_ERR_ARG;
    if (!b->timed) {
        pv::set_error("pv_batch_stage_ms: timing is off or no step ran");
        return PV_ERR_STATE;
    }
    for (int i = 0; i < 5; ++i) {
        PV_CUDA(cudaEventSynchronize(b->ev[i + 1]), "synchronise stage event");
        PV_CUDA(cudaEventElapsedTime(&h_ms5[i], b->ev[i], b->ev[i + 1]), "stage time");
    }
    return PV_OK;
}

extern "C" int pv_batch_buffers(const pv_batch* b, int beam, float** d_filterbank,
                                float** d_dedispersed, float** d_ring) {
    if (!b || beam < 0 || beam >= b->n) return PV_ERR_ARG;
    const pv_beam* x = b->beams[beam];
    if (d_filterbank) *d_filterbank = x->d_fb;
    if (d_dedispersed) *d_dedispersed = x->d_out;
    if (d_ring) *d_ring = x->d_ring;
    return PV_OK;
}
