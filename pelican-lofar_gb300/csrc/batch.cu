// The batched serving form of the beam chain: many beams of different
// channel counts, trial counts and delay ranges advance one chunk per step,
// each stage of all beams in as few launches as the kernels allow:
//
//   K1  chan_stokes_i_kernel   one launch per channels-per-subband class
//   K2  rfi_batch_kernel       one CTA per beam, one launch per channel count
//   A8  ring_write_batch_kernel one launch
//   K4  dedisperse_batch_kernel one persistent launch over every beam's tiles,
//                              DM x time tile shape chosen by the autotuner
//   K5  analyser               per beam (count, scan, emit)
//
// Pipelined mode (PV_BATCH_PIPELINED) splits a step into two concurrent
// branches after the channeliser: clip and ring-write chunk k, and meanwhile
// dedisperse and search window k-lag-1 (complete since the previous step).
// The clippers run one CTA per beam, so the persistent dedispersion launch
// fills the SMs they leave idle; every ring holds one more chunk so that the
// branches never touch the same ring positions, and a window's events come
// one step later.
// Every launch reads the chunk index from a device step counter that the
// step's last kernel advances, so one captured CUDA graph replays every
// step unchanged.  Inputs and event outputs are double buffered by step
// parity: the host copies the next step's voltages (on the batch's copy
// stream) while the current step computes, and each step's events land in
// host-mapped pinned memory, readable while the next step runs.  The chain of each beam is the pv_beam chain: the same
// state layout (tap history, RFI state, delay ring) and the same arithmetic,
// so a beam's events in the batch equal its events run alone.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pv_internal.cuh"

namespace {

// First kernel of a step: which beams process a chunk (the host's mask for
// this step, read from host-mapped memory) and which dedisperse a window.
// Window w needs ring chunks w..w+lag; pipelined, the chunk written in this
// step is not yet usable.
__global__ void plan_kernel(pv::BeamStep* __restrict__ bs, int n, const long long* __restrict__ d_step,
                            const int* h_mask, int pipelined) {
    const int par = (int)(*d_step & 1);
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
        pv::BeamStep& B = bs[b];
        const int active = ((const volatile int*)h_mask)[par * n + b] != 0;
        const long long avail = B.written + (pipelined ? 0 : active);
        B.active = active;
        B.sel = B.done + B.lag + 1 <= avail;
        B.window = B.done;
    }
}

// Last kernel of a step: advance every beam's counters and the step.
__global__ void advance_kernel(pv::BeamStep* __restrict__ bs, int n, long long* d_step) {
    for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n; b += gridDim.x * blockDim.x) {
        bs[b].written += bs[b].active;
        bs[b].done += bs[b].sel;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) *d_step += 1;
}

struct ExportJob {
    const pv_event* d_events;
    const long long* d_total;
    long long cap;  // device event capacity of the beam
};

// Copies every beam's event count (-1: no window this step), window index and
// first events of this step into the host-mapped slot of the step's parity,
// with the dedispersion status word.
__global__ void event_export_kernel(const ExportJob* __restrict__ jobs, int n,
                                    const long long* __restrict__ d_step,
                                    const pv::BeamStep* __restrict__ bs,
                                    const int* __restrict__ d_status, long long* h_counts,
                                    long long* h_windows, pv_event* h_events, long long host_cap,
                                    int* h_status) {
    const int b = blockIdx.x;
    const int par = (int)(*d_step & 1);
    const bool sel = bs[b].sel != 0;
    const long long total = sel ? *jobs[b].d_total : -1;
    const long long k = sel ? min(min(total, jobs[b].cap), host_cap) : 0;
    pv_event* dst = h_events + ((long long)par * n + b) * host_cap;
    for (long long i = threadIdx.x; i < k; i += blockDim.x) dst[i] = jobs[b].d_events[i];
    if (threadIdx.x == 0) {
        h_counts[(long long)par * n + b] = total;
        h_windows[(long long)par * n + b] = bs[b].window;
        if (b == 0) h_status[par] = *d_status;
    }
}

}  // namespace

struct pv_batch {
    int n = 0;
    int flags = 0;
    std::vector<pv_beam*> beams;
    std::vector<void*> d_in;  // [2][n]: inputs of even and odd steps
    std::vector<long long> in_bytes;
    std::vector<float2*> d_hist;  // two per beam
    struct ChanClass {
        int nchan = 0, njobs = 0;
        int packets = 0;  // the class's beams take LOFAR packets (one kernel per input layout)
        long long nwarps = 0;
        pv::ChanJob* d_jobs = nullptr;
    };
    std::vector<ChanClass> chan;
    pv::RfiBatch* rfi = nullptr;
    pv::RingJob* d_ring_jobs = nullptr;
    long long ring_blocks = 0, cal_blocks = 0;
    int store = PV_STORE_F32;
    std::vector<float*> d_scale;  // u8 rings: per beam [scale rows][offset rows][offset sum]
    pv::DdBatch* dd = nullptr;
    long long* d_step = nullptr;    // steps issued (parity of the host slots)
    pv::BeamStep* d_bs = nullptr;   // per-beam progress
    ExportJob* d_export = nullptr;
    void* h_mapped = nullptr;       // host-mapped pinned: counts, windows, masks, status, events
    long long* h_counts = nullptr;  // [2][n]
    long long* h_windows = nullptr; // [2][n]
    int* h_mask = nullptr;          // [2][n]
    int* h_status = nullptr;        // [2]
    std::vector<pv::BeamStep> mirror;  // host copy of the per-beam progress after the last step issued
    std::vector<long long> processed;  // chunks processed per beam (input parity)
    pv_event* h_events = nullptr;
    long long host_cap = 0;
    long long step = 0;             // steps issued
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t done[2] = {};       // step of each parity finished on the device
    cudaEvent_t copied[2] = {};     // inputs of each parity copied
    bool done_valid[2] = {false, false};
    cudaStream_t cap_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long graph_kernels = 0;
    cudaEvent_t ev[7] = {};
    bool timed = false;
    bool pipelined = false;
    cudaStream_t side = nullptr;     // second branch of a pipelined step
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    std::vector<cudaStream_t> rfi_side;  // pipelined: one stream per clipper class after the first
    std::vector<cudaEvent_t> rfi_join;
    std::vector<cudaEvent_t> rfi_tail;   // pipelined: end of the dedispersion helper after each class
    cudaStream_t branch_a = nullptr; // pipelined: clippers and ring write (high priority)
    cudaEvent_t join_a = nullptr;
};

namespace {

void destroy(pv_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    if (b->side) cudaStreamDestroy(b->side);
    for (cudaStream_t x : b->rfi_side)
        if (x) cudaStreamDestroy(x);
    for (cudaEvent_t x : b->rfi_join)
        if (x) cudaEventDestroy(x);
    for (cudaEvent_t x : b->rfi_tail)
        if (x) cudaEventDestroy(x);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->branch_a) cudaStreamDestroy(b->branch_a);
    if (b->join_a) cudaEventDestroy(b->join_a);
    if (b->join_ev) cudaEventDestroy(b->join_ev);
    for (auto e : b->ev)
        if (e) cudaEventDestroy(e);
    if (b->dd) pv::dd_batch_destroy(b->dd);
    if (b->rfi) pv::rfi_batch_destroy(b->rfi);
    for (auto& c : b->chan)
        if (c.d_jobs) cudaFree(c.d_jobs);
    if (b->d_ring_jobs) cudaFree(b->d_ring_jobs);
    for (float* p : b->d_scale)
        if (p) cudaFree(p);
    if (b->d_step) cudaFree(b->d_step);
    if (b->d_bs) cudaFree(b->d_bs);
    if (b->d_export) cudaFree(b->d_export);
    if (b->h_mapped) cudaFreeHost(b->h_mapped);
    if (b->copy_stream) cudaStreamDestroy(b->copy_stream);
    for (int i = 0; i < 2; ++i) {
        if (b->done[i]) cudaEventDestroy(b->done[i]);
        if (b->copied[i]) cudaEventDestroy(b->copied[i]);
    }
    for (void* p : b->d_in)
        if (p) cudaFree(p);
    for (void* p : b->d_hist)
        if (p) cudaFree(p);
    for (pv_beam* x : b->beams)
        if (x) pv_beam_destroy(x);
    delete b;
}

// Issues one step of every beam on stream s.  Pipelined, the channeliser
// runs first on the whole GPU.  Then the clippers (one CTA, one SM, per beam)
// run on high-priority streams beside a persistent dedispersion launch with
// one CTA for each SM they leave free; as each clipper class ends, a
// dedispersion launch of as many CTAs joins the same tile queue on its
// stream, so no SM idles and a dedispersion CTA never holds an SM a clipper
// needs.  Both branches join s before the step counter advances.
int enqueue_step(pv_batch* b, cudaStream_t s, bool capture) {
    const bool timing = (b->flags & PV_BATCH_TIMING) != 0;
    auto mark = [&](int i, cudaStream_t st) -> int {
        if (!timing) return PV_OK;
        return pv::cuda_status(capture ? cudaEventRecordWithFlags(b->ev[i], st, cudaEventRecordExternal)
                                       : cudaEventRecord(b->ev[i], st),
                               "record stage event");
    };
    cudaStream_t sd = b->pipelined ? b->side : s;      // dedispersion branch (low priority)
    cudaStream_t sa = b->pipelined ? b->branch_a : s;  // clippers and ring write (high priority)
    plan_kernel<<<1, 256, 0, s>>>(b->d_bs, b->n, b->d_step, b->h_mask, b->pipelined ? 1 : 0);
    PV_TRY(pv::check_launch("plan_kernel"));
    PV_TRY(mark(0, s));
    for (auto& c : b->chan)
        PV_TRY(pv::launch_chan_fast(c.nchan, c.packets ? 2 : 1, c.d_jobs, pv::ChanJob{}, c.njobs, c.nwarps,
                                    b->d_bs, s));
    PV_TRY(mark(1, s));
    const int nk = b->rfi ? pv::rfi_batch_launches(b->rfi) : 0;
    int rfi_ctas = 0;
    for (int k = 0; k < nk; ++k) rfi_ctas += pv::rfi_batch_ctas(b->rfi, k);
    if (b->pipelined) {
        PV_TRY(pv::dd_batch_reset(b->dd, s));  // one tile queue for every dedispersion launch
        PV_CUDA(cudaEventRecord(b->fork_ev, s), "fork");
        PV_CUDA(cudaStreamWaitEvent(sa, b->fork_ev, 0), "fork");
        PV_CUDA(cudaStreamWaitEvent(sd, b->fork_ev, 0), "fork");
    }
    if (b->rfi && b->pipelined) {
        // every clipper class resident at once (class 0 on branch A, the
        // others on their own streams); as a class finishes, a dedispersion
        // launch of as many CTAs takes its SMs and joins the tile queue
        for (int k = 1; k < nk; ++k) {
            cudaStream_t sk = b->rfi_side[k - 1];
            PV_CUDA(cudaStreamWaitEvent(sk, b->fork_ev, 0), "fork clipper");
            PV_TRY(pv::rfi_batch_launch_one(b->rfi, k, sk));
            PV_CUDA(cudaEventRecord(b->rfi_join[k - 1], sk), "join clipper");
            PV_TRY(pv::dd_batch_launch_shared(b->dd, b->d_bs, pv::rfi_batch_ctas(b->rfi, k), sk));
            PV_CUDA(cudaEventRecord(b->rfi_tail[k - 1], sk), "join helper");
        }
        if (nk > 0) PV_TRY(pv::rfi_batch_launch_one(b->rfi, 0, sa));
        for (int k = 1; k < nk; ++k) PV_CUDA(cudaStreamWaitEvent(sa, b->rfi_join[k - 1], 0), "join clipper");
    } else if (b->rfi) {
        // the classes side by side, joined before the dedispersion
        if (nk > 1) PV_CUDA(cudaEventRecord(b->fork_ev, s), "fork");
        for (int k = 1; k < nk; ++k) {
            PV_CUDA(cudaStreamWaitEvent(b->rfi_side[k - 1], b->fork_ev, 0), "fork clipper");
            PV_TRY(pv::rfi_batch_launch_one(b->rfi, k, b->rfi_side[k - 1]));
            PV_CUDA(cudaEventRecord(b->rfi_join[k - 1], b->rfi_side[k - 1]), "join clipper");
        }
        if (nk > 0) PV_TRY(pv::rfi_batch_launch_one(b->rfi, 0, s));
        for (int k = 1; k < nk; ++k) PV_CUDA(cudaStreamWaitEvent(s, b->rfi_join[k - 1], 0), "join clipper");
    }
    PV_TRY(mark(2, sa));
    auto dedisperse_branch = [&]() -> int {
        PV_TRY(mark(6, sd));
        if (b->pipelined) {
            // the SMs the clippers leave free; the clippers' SMs join later
            const int free_sms = std::max(8, pv::sm_count() - rfi_ctas);
            PV_TRY(pv::dd_batch_launch_shared(b->dd, b->d_bs, std::min(free_sms, pv::dd_batch_grid(b->dd)), sd));
        } else {
            PV_TRY(pv::dd_batch_launch(b->dd, b->d_bs, sd));
        }
        PV_TRY(mark(4, sd));
        for (int i = 0; i < b->n; ++i) {
            pv_beam* x = b->beams[i];
            const pv_beam_config& c = x->cfg;
            PV_TRY(pv::analyse_launch(x->d_out, c.chunk, c.tdms, c.chunk, c.threshold, x->rms,
                                      c.bin_pow2, x->d_events, x->cap, x->d_total, x->d_scratch, sd));
        }
        event_export_kernel<<<b->n, 256, 0, sd>>>(b->d_export, b->n, b->d_step, b->d_bs,
                                                 pv::dd_batch_status_word(b->dd), b->h_counts,
                                                 b->h_windows, b->h_events, b->host_cap,
                                                 b->h_status);
        PV_TRY(pv::check_launch("event_export_kernel"));
        return mark(5, sd);
    };
    if (b->pipelined) PV_TRY(dedisperse_branch());
    if (b->store == PV_STORE_U8)
        PV_TRY(pv::ring_calibrate_batch(b->d_ring_jobs, b->n, b->cal_blocks, b->d_bs, sa));
    PV_TRY(pv::ring_write_batch(b->d_ring_jobs, b->n, b->ring_blocks, b->d_bs, b->store, sa));
    PV_TRY(mark(3, sa));
    if (b->pipelined) {
        if (nk > 0) PV_TRY(pv::dd_batch_launch_shared(b->dd, b->d_bs, pv::rfi_batch_ctas(b->rfi, 0), sa));
        PV_CUDA(cudaEventRecord(b->join_a, sa), "join");
        PV_CUDA(cudaEventRecord(b->join_ev, sd), "join");
        PV_CUDA(cudaStreamWaitEvent(s, b->join_a, 0), "join");
        PV_CUDA(cudaStreamWaitEvent(s, b->join_ev, 0), "join");
        for (int k = 1; k < nk; ++k) PV_CUDA(cudaStreamWaitEvent(s, b->rfi_tail[k - 1], 0), "join helper");
    } else {
        PV_TRY(dedisperse_branch());
    }
    advance_kernel<<<1, 256, 0, s>>>(b->d_bs, b->n, b->d_step);
    return pv::check_launch("advance_kernel");
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

// How the clippers of wide beams spread over the GPU (rfi_batch_create's
// split).  Pipelined, the clippers share the GPU with the dedispersion,
// whose time is what a cluster's extra SMs take: one CTA per beam.
// Unpipelined, the clippers run alone and their longest beam sets the
// stage's time: beams of 1024 partial sums over a cluster of 4 CTAs.
static int rfi_split(int flags) {
    if (flags & PV_BATCH_RFI_ONE_CTA) return 0;
    if (flags & PV_BATCH_RFI_CLUSTER8) return 2;
    if (flags & PV_BATCH_RFI_CLUSTER4) return 1;
    return (flags & PV_BATCH_PIPELINED) ? 0 : 1;
}

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
    b->d_in.assign(2 * nbeams, nullptr);
    b->in_bytes.assign(nbeams, 0);
    b->d_hist.assign(2 * nbeams, nullptr);
    b->mirror.assign(nbeams, pv::BeamStep{});
    b->processed.assign(nbeams, 0);
    b->store = (flags & PV_BATCH_STORE_U8) ? PV_STORE_U8 : ((flags & PV_BATCH_STORE_F16) ? PV_STORE_F16
                                                                                         : PV_STORE_F32);
    b->d_scale.assign(nbeams, nullptr);
    const int elem = b->store == PV_STORE_F32 ? 4 : (b->store == PV_STORE_F16 ? 2 : 1);
    b->pipelined = (flags & PV_BATCH_PIPELINED) != 0;
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
        if (c.chunk != chunk || c.chunk % 16 != 0) {
            pv::set_error("pv_batch_create: every beam needs the same chunk, a multiple of 16 spectra "
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
        const int extra = (flags & PV_BATCH_PIPELINED) ? 1 : 0;
        rc = pv::beam_create(&b->beams[i], &c, extra, elem);
        if (rc != PV_OK) return fail(rc);
        pv_beam* x = b->beams[i];
        pv::BeamStep& m = b->mirror[i];
        m.base = x->chunks;  // lag when prefilled, else 0
        m.written = m.base;
        m.lag = x->lag;
        b->in_bytes[i] = pv_beam_input_bytes(x, 1);
        const size_t hist = sizeof(float2) * (size_t)c.nsub * 2 * 7 * c.nchan_sub;
        cudaError_t e = cudaMalloc(&b->d_in[i], b->in_bytes[i]);
        if (e == cudaSuccess) e = cudaMalloc(&b->d_in[nbeams + i], b->in_bytes[i]);
        for (int h = 0; h < 2 && e == cudaSuccess; ++h) {
            e = cudaMalloc(&b->d_hist[2 * i + h], hist);
            if (e == cudaSuccess) e = cudaMemset(b->d_hist[2 * i + h], 0, hist);
        }
        if (e == cudaSuccess) e = cudaMemset(x->d_out, 0, sizeof(float) * (size_t)c.tdms * c.chunk);
        if (e == cudaSuccess && b->store == PV_STORE_U8) {
            // With zero-DMing the clipper leaves every good spectrum at zero mean and unit RMS
            // (RFI_Clipper.cpp:507-532), so the rows share the scale 6 sigma / 127 = 6/127 and
            // offset 0; otherwise both come from the data (scale 0: not calibrated yet).
            std::vector<float> so(2 * (size_t)x->nbins + 1, 0.0f);
            if (c.rfi_active && c.zero_dming) std::fill(so.begin(), so.begin() + x->nbins, 6.0f / 127.0f);
            e = cudaMalloc(&b->d_scale[i], sizeof(float) * so.size());
            if (e == cudaSuccess)
                e = cudaMemcpy(b->d_scale[i], so.data(), sizeof(float) * so.size(), cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess) {
            pv::set_error("pv_batch_create: beam %d: %s", i, cudaGetErrorString(e));
            return fail(PV_ERR_NOMEM);
        }
    }
    cudaStream_t s0 = nullptr;
    if (cudaMalloc(&b->d_bs, sizeof(pv::BeamStep) * nbeams) != cudaSuccess ||
        cudaMemcpy(b->d_bs, b->mirror.data(), sizeof(pv::BeamStep) * nbeams, cudaMemcpyHostToDevice) !=
            cudaSuccess) {
        pv::set_error("pv_batch_create: cannot allocate the beam progress");
        return fail(PV_ERR_NOMEM);
    }
    // K1 jobs, one launch per channel count
    std::vector<std::vector<pv::ChanJob>> cj;
    for (int i = 0; i < nbeams; ++i) {
        pv_beam* x = b->beams[i];
        const float* coeffs = nullptr;
        const float2* tw = nullptr;
        int nchan = 0, ntaps = 0;
        rc = pv::ppf_tables(x->ppf, &coeffs, &tw, &nchan, &ntaps);
        if (rc != PV_OK) return fail(rc);
        const int packets = x->cfg.udp_packet_bytes > 0 ? 1 : 0;
        size_t k = 0;
        while (k < b->chan.size() && (b->chan[k].nchan != nchan || b->chan[k].packets != packets)) ++k;
        if (k == b->chan.size()) {
            b->chan.emplace_back();
            b->chan[k].nchan = nchan;
            b->chan[k].packets = packets;
            cj.emplace_back();
        }
        pv::ChanJob j{};
        j.in = b->d_in[i];
        j.in_odd = b->d_in[nbeams + i];
        j.hist[0] = b->d_hist[2 * i];
        j.hist[1] = b->d_hist[2 * i + 1];
        j.coeffs = coeffs;
        j.twiddle = tw;
        j.out = x->d_fb;
        j.nsub = x->cfg.nsub;
        j.nblocks = x->cfg.chunk * x->cfg.int_time;
        j.window = x->cfg.int_time;
        j.nu = x->cfg.chunk;
        j.beam = i;
        j.pkt_bytes = x->cfg.udp_packet_bytes;
        j.pkt_nsub = x->cfg.udp_subbands;
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
                                  chunk, b->d_bs, rfi_split(flags), s0);
        if (rc != PV_OK) return fail(rc);
    }
    // A8: ring writes
    {
        std::vector<pv::RingJob> rj(nbeams);
        for (int i = 0; i < nbeams; ++i) {
            pv_beam* x = b->beams[i];
            float* so = b->d_scale[i];
            rj[i] = pv::RingJob{x->d_ring, x->row_stride, x->ring_len, x->d_fb, chunk, x->cfg.nsub,
                                x->nchan_fb, x->inverted, b->ring_blocks, i, so,
                                so ? so + x->nbins : nullptr, so ? so + 2 * x->nbins : nullptr,
                                b->cal_blocks};
            b->ring_blocks += pv::ring_job_blocks(rj[i]);
            b->cal_blocks += pv::ring_cal_blocks(rj[i]);
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
            d.chunk = chunk;
            d.scale = b->d_scale[i];
            d.off_sum = b->d_scale[i] ? b->d_scale[i] + 2 * x->nbins : nullptr;
            d.uniform = (b->store == PV_STORE_U8 && x->cfg.rfi_active && x->cfg.zero_dming) ? 1 : 0;
        }
        const int variant = (flags & PV_BATCH_TUNE) ? -1 : PV_BATCH_VARIANT_OF(flags);
        rc = pv::dd_batch_create(&b->dd, db.data(), nbeams, variant, b->store, s0);
        if (rc != PV_OK) return fail(rc);
    }
    {
        long long cap = 0;
        std::vector<ExportJob> ej(nbeams);
        for (int i = 0; i < nbeams; ++i) {
            pv_beam* x = b->beams[i];
            ej[i] = ExportJob{x->d_events, x->d_total, x->cap};
            cap = std::max(cap, x->cap);
        }
        b->host_cap = std::min<long long>(cap, PV_BATCH_HOST_EVENTS);
        const size_t counts = sizeof(long long) * 2 * nbeams, masks = sizeof(int) * 2 * nbeams;
        const size_t status = 16, head = 2 * counts + ((masks + 15) & ~(size_t)15) + status;
        const size_t bytes = head + sizeof(pv_event) * 2 * (size_t)nbeams * b->host_cap;
        if (cudaMalloc(&b->d_step, sizeof(long long)) != cudaSuccess ||
            cudaMemset(b->d_step, 0, sizeof(long long)) != cudaSuccess ||
            cudaMalloc(&b->d_export, sizeof(ExportJob) * nbeams) != cudaSuccess ||
            cudaMemcpy(b->d_export, ej.data(), sizeof(ExportJob) * nbeams, cudaMemcpyHostToDevice) !=
                cudaSuccess ||
            cudaHostAlloc(&b->h_mapped, bytes, cudaHostAllocMapped) != cudaSuccess) {
            pv::set_error("pv_batch_create: cannot allocate the step counter and event slots");
            return fail(PV_ERR_NOMEM);
        }
        std::memset(b->h_mapped, 0, bytes);
        char* h = static_cast<char*>(b->h_mapped);
        b->h_counts = reinterpret_cast<long long*>(h);
        b->h_windows = reinterpret_cast<long long*>(h + counts);
        b->h_mask = reinterpret_cast<int*>(h + 2 * counts);
        b->h_status = reinterpret_cast<int*>(h + 2 * counts + ((masks + 15) & ~(size_t)15));
        b->h_events = reinterpret_cast<pv_event*>(h + head);
        int lowest = 0, highest = 0;
        if (cudaStreamCreateWithFlags(&b->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaDeviceGetStreamPriorityRange(&lowest, &highest) != cudaSuccess ||
            cudaStreamCreateWithPriority(&b->side, cudaStreamNonBlocking, lowest) != cudaSuccess ||
            cudaStreamCreateWithPriority(&b->branch_a, cudaStreamNonBlocking, highest) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->join_ev, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->join_a, cudaEventDisableTiming) != cudaSuccess) {
            pv::set_error("pv_batch_create: cannot create streams");
            return fail(PV_ERR_CUDA);
        }
        const int nk = b->rfi ? pv::rfi_batch_launches(b->rfi) : 0;
        for (int k = 1; k < nk; ++k) {
            b->rfi_side.push_back(nullptr);
            b->rfi_join.push_back(nullptr);
            b->rfi_tail.push_back(nullptr);
            if (cudaStreamCreateWithPriority(&b->rfi_side.back(), cudaStreamNonBlocking, highest) != cudaSuccess ||
                cudaEventCreateWithFlags(&b->rfi_join.back(), cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&b->rfi_tail.back(), cudaEventDisableTiming) != cudaSuccess) {
                pv::set_error("pv_batch_create: cannot create streams");
                return fail(PV_ERR_CUDA);
            }
        }
        for (int i = 0; i < 2; ++i)
            if (cudaEventCreateWithFlags(&b->done[i], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&b->copied[i], cudaEventDisableTiming) != cudaSuccess) {
                pv::set_error("pv_batch_create: cudaEventCreate failed");
                return fail(PV_ERR_CUDA);
            }
    }
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
    // the buffer the beam's next chunk is read from (a beam's chunks alternate between two)
    if (d_voltages) *d_voltages = b->d_in[(size_t)(b->processed[beam] & 1) * b->n + beam];
    if (bytes) *bytes = b->in_bytes[beam];
    return PV_OK;
}

extern "C" int pv_batch_input_parity(pv_batch* b, int beam, int parity, void** d_voltages, long long* bytes) {
    if (!b || beam < 0 || beam >= b->n || (parity != 0 && parity != 1)) return PV_ERR_ARG;
    if (d_voltages) *d_voltages = b->d_in[(size_t)parity * b->n + beam];
    if (bytes) *bytes = b->in_bytes[beam];
    return PV_OK;
}

namespace {

// Sets this step's mask (all beams when h_active is null) in its host-mapped
// slot, once the step that last read the slot (two back) has finished.
int set_mask(pv_batch* b, const unsigned char* h_active) {
    const int par = (int)(b->step & 1);
    if (b->done_valid[par]) PV_CUDA(cudaEventSynchronize(b->done[par]), "wait for the step two back");
    int* m = b->h_mask + (size_t)par * b->n;
    for (int i = 0; i < b->n; ++i) m[i] = h_active ? (h_active[i] != 0) : 1;
    return PV_OK;
}

int launch_step(pv_batch* b, cudaStream_t s) {
    const int par = (int)(b->step & 1);
    if (b->exec) {
        PV_CUDA(cudaGraphLaunch(b->exec, s), "launch step graph");
        pv::count_launch(b->graph_kernels);
    } else {
        PV_TRY(enqueue_step(b, s, false));
    }
    PV_CUDA(cudaEventRecord(b->done[par], s), "record step completion");
    b->done_valid[par] = true;
    // the host's mirror of plan_kernel and advance_kernel
    const int* m = b->h_mask + (size_t)par * b->n;
    for (int i = 0; i < b->n; ++i) {
        pv::BeamStep& B = b->mirror[i];
        B.active = m[i];
        B.sel = B.done + B.lag + 1 <= B.written + (b->pipelined ? 0 : B.active);
        B.window = B.done;
        B.written += B.active;
        B.done += B.sel;
        b->processed[i] += B.active;
    }
    b->step += 1;
    b->timed = (b->flags & PV_BATCH_TIMING) != 0;
    return PV_OK;
}

}  // namespace

extern "C" int pv_batch_reset_beam(pv_batch* b, int beam, void* stream) {
    if (!b || beam < 0 || beam >= b->n) return PV_ERR_ARG;
    cudaStream_t s = pv::as_stream(stream);
    // every issued step has finished with this beam's buffers
    for (int i = 0; i < 2; ++i)
        if (b->done_valid[i]) PV_CUDA(cudaEventSynchronize(b->done[i]), "wait for the issued steps");
    pv_beam* x = b->beams[beam];
    const int elem = b->store == PV_STORE_F32 ? 4 : (b->store == PV_STORE_F16 ? 2 : 1);
    PV_CUDA(cudaMemsetAsync(x->d_ring, elem == 1 ? 0x80 : 0, (size_t)elem * x->nbins * (size_t)x->row_stride, s),
            "clear ring");
    const size_t hist = sizeof(float2) * (size_t)x->cfg.nsub * 2 * 7 * x->cfg.nchan_sub;
    for (int h = 0; h < 2; ++h) PV_CUDA(cudaMemsetAsync(b->d_hist[2 * beam + h], 0, hist, s), "clear PPF history");
    PV_CUDA(cudaMemsetAsync(x->d_out, 0, sizeof(float) * (size_t)x->cfg.tdms * x->cfg.chunk, s), "clear window");
    PV_TRY(pv::rfi_reset(x->rfi, s));
    if (b->store == PV_STORE_U8 && b->d_scale[beam]) {
        std::vector<float> so(2 * (size_t)x->nbins + 1, 0.0f);
        if (x->cfg.rfi_active && x->cfg.zero_dming) std::fill(so.begin(), so.begin() + x->nbins, 6.0f / 127.0f);
        PV_CUDA(cudaStreamSynchronize(s), "synchronise");
        PV_CUDA(cudaMemcpy(b->d_scale[beam], so.data(), sizeof(float) * so.size(), cudaMemcpyHostToDevice),
                "reset ring calibration");
    }
    pv::BeamStep& m = b->mirror[beam];
    const long long base = m.base;
    const int lag = m.lag;
    m = pv::BeamStep{};
    m.base = base;
    m.written = base;
    m.lag = lag;
    b->processed[beam] = 0;
    PV_CUDA(cudaStreamSynchronize(s), "synchronise");
    PV_CUDA(cudaMemcpy(b->d_bs + beam, &m, sizeof(m), cudaMemcpyHostToDevice), "reset beam progress");
    return PV_OK;
}

extern "C" int pv_batch_run(pv_batch* b, const unsigned char* h_active, void* stream) {
    if (!b) return PV_ERR_ARG;
    PV_TRY(set_mask(b, h_active));
    return launch_step(b, pv::as_stream(stream));
}

extern "C" int pv_batch_run_host(pv_batch* b, const void* const* h_voltages,
                                 const unsigned char* h_active, void* stream) {
    if (!b || !h_voltages) return PV_ERR_ARG;
    cudaStream_t s = pv::as_stream(stream);
    const int par = (int)(b->step & 1);
    for (int i = 0; i < b->n; ++i)
        if ((!h_active || h_active[i]) && !h_voltages[i]) {
            pv::set_error("pv_batch_run_host: no voltages for beam %d", i);
            return PV_ERR_ARG;
        }
    PV_TRY(set_mask(b, h_active));
    // a beam's input buffer was last read by its step before last, at the
    // latest the batch step two back
    if (b->done_valid[par]) PV_CUDA(cudaStreamWaitEvent(b->copy_stream, b->done[par], 0), "wait");
    for (int i = 0; i < b->n; ++i) {
        if (h_active && !h_active[i]) continue;
        PV_CUDA(cudaMemcpyAsync(b->d_in[(size_t)(b->processed[i] & 1) * b->n + i], h_voltages[i],
                                b->in_bytes[i], cudaMemcpyHostToDevice, b->copy_stream),
                "copy voltages to the device");
    }
    PV_CUDA(cudaEventRecord(b->copied[par], b->copy_stream), "record copy");
    PV_CUDA(cudaStreamWaitEvent(s, b->copied[par], 0), "wait for the copy");
    return launch_step(b, s);
}

extern "C" int pv_batch_events(pv_batch* b, int beam, long long step, pv_event* h_events,
                               long long cap, long long* h_count, long long* h_first_sample) {
    if (!b || beam < 0 || beam >= b->n || !h_count) return PV_ERR_ARG;
    if (step < 0) step = b->step + step;  // -1: the last step issued, -2: the one before
    if (step < 0 || step >= b->step || step < b->step - 2) {
        pv::set_error("pv_batch_events: step %lld is not one of the last two issued (%lld)", step,
                      b->step);
        return PV_ERR_ARG;
    }
    const int par = (int)(step & 1);
    PV_CUDA(cudaEventSynchronize(b->done[par]), "wait for the step");
    const int status = ((volatile int*)b->h_status)[par];
    if (status != PV_OK) {
        pv::set_error("pv_batch_events: a dedispersion pipeline wait gave up (status %d)", status);
        return status;
    }
    const size_t slot = (size_t)par * b->n + beam;
    const long long total = ((volatile long long*)b->h_counts)[slot];
    if (total < 0) {  // no window of this beam completed in that step
        *h_count = 0;
        if (h_first_sample) *h_first_sample = -1;
        return PV_OK;
    }
    pv_beam* x = b->beams[beam];
    *h_count = total;
    if (h_first_sample) *h_first_sample = ((volatile long long*)b->h_windows)[slot] * x->cfg.chunk;
    const long long n = std::min(std::min(total, std::min(x->cap, b->host_cap)), cap);
    if (h_events && n > 0)
        std::memcpy(h_events, b->h_events + slot * b->host_cap, sizeof(pv_event) * n);
    return PV_OK;
}

extern "C" int pv_batch_info(const pv_batch* b, int beam, long long* h_info8) {
    if (!b || beam < 0 || beam >= b->n || !h_info8) return PV_ERR_ARG;
    const pv_beam* x = b->beams[beam];
    const pv::BeamStep& B = b->mirror[beam];
    h_info8[0] = x->nbins;
    h_info8[1] = x->max_shift;
    h_info8[2] = x->lag;
    h_info8[3] = x->ring_len;
    h_info8[4] = x->inverted;
    h_info8[5] = B.written;   // logical chunks in the ring after the steps issued
    h_info8[6] = B.done - 1;  // last window dedispersed (-1: none yet)
    const long long elem = b->store == PV_STORE_F32 ? 4 : (b->store == PV_STORE_F16 ? 2 : 1);
    h_info8[7] = (long long)x->nbins * x->row_stride * elem;  // ring bytes
    return PV_OK;
}

extern "C" int pv_batch_tiles(const pv_batch* b, int* h_shape8, int* h_dms, float* h_tune_ms,
                              long long* h_graph_kernels) {
    if (!b) return PV_ERR_ARG;
    if (h_shape8) PV_TRY(pv::dd_batch_shape(b->dd, h_shape8));
    if (h_dms) {
        const auto& d = pv::dd_batch_dms(b->dd);
        std::copy(d.begin(), d.end(), h_dms);
    }
    if (h_tune_ms) {
        const auto& t = pv::dd_batch_tune_ms(b->dd);
        for (int i = 0; i < PV_BATCH_VARIANTS; ++i) h_tune_ms[i] = i < (int)t.size() ? t[i] : -1.0f;
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
    const int from[5] = {0, 1, 2, 6, 4}, to[5] = {1, 2, 3, 4, 5};
    for (int i = 0; i < 5; ++i) {
        PV_CUDA(cudaEventSynchronize(b->ev[to[i]]), "synchronise stage event");
        PV_CUDA(cudaEventElapsedTime(&h_ms5[i], b->ev[from[i]], b->ev[to[i]]), "stage time");
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

extern "C" int pv_batch_step_done(const pv_batch* b, long long step) {
    if (!b || step < 0 || step >= b->step) return PV_ERR_ARG;
    if (step < b->step - 2) return 1;  // older steps finished before the step two back was issued
    const cudaError_t e = cudaEventQuery(b->done[step & 1]);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return pv::cuda_status(e, "pv_batch_step_done");
}

extern "C" long long pv_batch_footprint(const pv_beam_config* c, int flags) {
    if (!c || c->nsub <= 0 || c->nchan_sub <= 0 || c->int_chan <= 0 || c->chunk <= 0 ||
        c->tdms <= 0 || c->tsamp <= 0.0) {
        pv::set_error("pv_batch_footprint: invalid beam configuration");
        return PV_ERR_ARG;
    }
    const int nchan_fb = c->nchan_sub / c->int_chan;
    const int nbins = c->nsub * nchan_fb;
    std::vector<float> k(nbins);
    int inverted = 0;
    if (pv_dm_shifts(c->fch1, c->foff, nbins, k.data(), &inverted) != PV_OK) return PV_ERR_ARG;
    // the dedispersion plan's maximum delay and the beam's ring
    const float ts = (float)c->tsamp;
    const float start = (c->dm_low < 0.0f ? 0.0f : c->dm_low) / ts, step = c->dm_step / ts;
    const float vmax = std::fmaf((float)(c->tdms - 1), step, start);
    int max_shift = 0;
    for (float kc : k) max_shift = std::max(max_shift, (int)(kc * vmax));
    const long long lag = (max_shift + c->chunk - 1) / c->chunk;
    const long long ring_len = (lag + 1 + ((flags & PV_BATCH_PIPELINED) ? 1 : 0)) * c->chunk;
    const long long row_stride = (ring_len + 31) / 32 * 32;
    const long long cap = c->event_capacity > 0 ? c->event_capacity : (1LL << 20);
    const long long elem = (flags & PV_BATCH_STORE_U8) ? 1 : ((flags & PV_BATCH_STORE_F16) ? 2 : 4);
    long long bytes = elem * nbins * row_stride;                      // ring
    if (flags & PV_BATCH_STORE_U8) bytes += 8LL * nbins + 4;          // row scales and offsets
    bytes += 4LL * c->chunk * nbins;                                   // filterbank
    bytes += 4LL * c->tdms * c->chunk;                                 // dedispersed window
    bytes += (long long)sizeof(pv_event) * cap;                        // events
    bytes += (long long)pv::analyse_scratch_bytes(c->tdms, c->chunk, c->bin_pow2) + 256;
    if (c->udp_packet_bytes > 0 && c->udp_subbands > 0)  // two input buffers of packet streams
        bytes += 2LL * (c->nsub / c->udp_subbands) * c->chunk * c->int_time * (c->nchan_sub / 16) *
                 c->udp_packet_bytes;
    else
        bytes += 2LL * c->nsub * 2 * c->chunk * c->int_time * c->nchan_sub * 4;  // two input buffers
    bytes += 2LL * 2 * (long long)sizeof(float2) * c->nsub * 7 * c->nchan_sub;  // two PPF histories
    bytes += 16LL * c->history + 12LL * nbins;                        // clipper state, bandpass
    return bytes;
}
