// One beam's device-resident hot path (the DedispersionPipeline call order,
// src/pipelines/udpstream/src/DedispersionPipeline.cpp:96-174, with the
// StokesIntegrator of UdpBFPipeline.cpp:80-92):
//
//   int16 voltages -> K1 fused PPF + Stokes I + integration -> K2/K3 RFI clip
//   (in place) -> transposed write into the per-channel ring -> K4
//   dedispersion of the window whose delays are complete -> K5 analyser.
//
// Everything runs on the caller's stream with buffers allocated once, so a
// chunk costs no host synchronisation until its events are read.  The ring
// holds (L+1) chunks, L = ceil(max delay / chunk): chunk k completes the
// delays of output window k-L (overlap-save), which is dedispersed and
// searched as soon as chunk k lands.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pv_internal.cuh"

namespace {

void destroy(pv_beam* b) {
    if (b->ppf) pv_ppf_destroy(b->ppf);
    if (b->rfi) pv_rfi_destroy(b->rfi);
    if (b->plan) pv_dedisp_plan_destroy(b->plan);
    for (void* p : {(void*)b->d_ring, (void*)b->d_fb, (void*)b->d_fb_raw, (void*)b->d_out,
                    (void*)b->d_events, b->d_scratch, b->d_in})
        if (p) cudaFree(p);
    if (b->h_total) cudaFreeHost(b->h_total);
    for (auto e : b->ev)
        if (e) cudaEventDestroy(e);
    delete b;
}

}  // namespace

namespace pv {

// pv_beam_create with `extra` more chunks of ring than the delays need (the
// batch's pipelined mode writes chunk k while window k-lag-1 is read).
int beam_create(pv_beam** out, const pv_beam_config* c, int extra, int elem) {
    if (!out || !c || extra < 0 || (elem != 4 && elem != 2 && elem != 1)) return PV_ERR_ARG;
    *out = nullptr;
    if (c->nsub <= 0 || c->nchan_sub <= 0 || c->int_time <= 0 || c->int_chan <= 0 ||
        c->nchan_sub % c->int_chan != 0 || c->chunk <= 0 || c->tdms <= 0 || c->tsamp <= 0.0) {
        pv::set_error("pv_beam_create: invalid beam configuration");
        return PV_ERR_CONFIG;
    }
    if (c->udp_packet_bytes > 0 &&
        (c->udp_subbands <= 0 || c->nsub % c->udp_subbands != 0 || c->udp_packet_bytes % 4 != 0 ||
         c->udp_packet_bytes < 16 + c->udp_subbands * 16 * 2 * 4 ||
         (c->nchan_sub != 16 && c->nchan_sub != 32 && c->nchan_sub != 64) || c->ntaps != 8)) {
        pv::set_error("pv_beam_create: packet input needs 16, 32 or 64 channels, 8 taps, subbands per packet "
                      "dividing nsub and a packet size that is a multiple of 4 holding them");
        return PV_ERR_CONFIG;
    }
    auto* b = new pv_beam;
    b->cfg = *c;
    b->cfg.bp_text = nullptr;
    b->nchan_fb = c->nchan_sub / c->int_chan;
    b->nbins = c->nsub * b->nchan_fb;
    int rc = pv_ppf_create(&b->ppf, c->nchan_sub, c->ntaps, c->window, nullptr);
    if (rc == PV_OK)
        rc = pv_rfi_create(&b->rfi, c->bp_text, c->cr, c->sr, c->history, c->zero_dming,
                           c->rms_from_mean, c->band_matching, c->rfi_active);
    std::vector<float> k(b->nbins);
    if (rc == PV_OK) rc = pv_dm_shifts(c->fch1, c->foff, b->nbins, k.data(), &b->inverted);
    const float start = (c->dm_low < 0.0f ? 0.0f : c->dm_low) / (float)c->tsamp;
    const float step = c->dm_step / (float)c->tsamp;
    if (rc == PV_OK) rc = pv_dedisp_plan_create(&b->plan, k.data(), b->nbins, c->tdms, start, step);
    if (rc != PV_OK) {
        destroy(b);
        return rc;
    }
    b->max_shift = pv_dedisp_plan_max_shift(b->plan);
    b->lag = (b->max_shift + c->chunk - 1) / c->chunk;
    b->ring_len = (long long)(b->lag + 1 + extra) * c->chunk;
    b->row_stride = (b->ring_len + 31) / 32 * 32;
    b->cap = c->event_capacity > 0 ? c->event_capacity : (1LL << 20);
    b->rms = std::sqrt((float)b->nchan_fb * (float)c->nsub);  // DedispersionAnalyser.cpp:38
    const size_t scratch = pv::analyse_scratch_bytes(c->tdms, c->chunk, c->bin_pow2);
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    alloc((void**)&b->d_ring, (size_t)elem * b->nbins * (size_t)b->row_stride);
    alloc((void**)&b->d_fb, sizeof(float) * (size_t)c->chunk * b->nbins);
    if (c->debug_taps) alloc((void**)&b->d_fb_raw, sizeof(float) * (size_t)c->chunk * b->nbins);
    alloc((void**)&b->d_out, sizeof(float) * (size_t)c->tdms * c->chunk);
    alloc((void**)&b->d_events, sizeof(pv_event) * (size_t)b->cap);
    alloc(&b->d_scratch, scratch + 256);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->h_total, sizeof(long long));
    if (e == cudaSuccess)
        e = cudaMemset(b->d_ring, elem == 1 ? 0x80 : 0, (size_t)elem * b->nbins * (size_t)b->row_stride);
    if (e != cudaSuccess) {
        pv::set_error("pv_beam_create: %s (ring of %lld x %lld samples)", cudaGetErrorString(e),
                      (long long)b->nbins, b->row_stride);
        destroy(b);
        return PV_ERR_NOMEM;
    }
    b->d_total = reinterpret_cast<long long*>(static_cast<char*>(b->d_scratch) + scratch);
    if (c->prefilled) b->chunks = b->lag;  // the ring already holds lag chunks of zeros
    if (c->timing) {
        for (auto& ev : b->ev) {
            if (cudaEventCreate(&ev) != cudaSuccess) {
                pv::set_error("pv_beam_create: cudaEventCreate failed");
                destroy(b);
                return PV_ERR_CUDA;
            }
        }
    }
    *out = b;
    return PV_OK;
}

}  // namespace pv

extern "C" int pv_beam_create(pv_beam** out, const pv_beam_config* c) {
    return pv::beam_create(out, c, 0);
}

extern "C" void pv_beam_destroy(pv_beam* b) {
    if (b) destroy(b);
}

extern "C" int pv_beam_info(const pv_beam* b, long long* h_info8) {
    if (!b || !h_info8) return PV_ERR_ARG;
    h_info8[0] = b->nbins;
    h_info8[1] = b->max_shift;
    h_info8[2] = b->lag;
    h_info8[3] = b->ring_len;
    h_info8[4] = b->inverted;
    h_info8[5] = b->chunks;
    h_info8[6] = b->window;
    h_info8[7] = (long long)b->nbins * b->row_stride * (long long)sizeof(float);
    return PV_OK;
}

extern "C" long long pv_beam_input_bytes(const pv_beam* b, int in_int16) {
    if (!b) return -1;
    const pv_beam_config& c = b->cfg;
    if (c.udp_packet_bytes > 0)  // the packet streams of one chunk
        return (long long)(c.nsub / c.udp_subbands) * c.chunk * c.int_time * (c.nchan_sub / 16) *
               c.udp_packet_bytes;
    return (long long)c.nsub * 2 * c.chunk * c.int_time * c.nchan_sub * (in_int16 ? 4 : 8);
}

extern "C" int pv_beam_process(pv_beam* b, const void* d_voltages, int in_int16, void* stream) {
    if (!b || !d_voltages) {
        pv::set_error("pv_beam_process: invalid arguments");
        return PV_ERR_ARG;
    }
    const pv_beam_config& c = b->cfg;
    cudaStream_t s = pv::as_stream(stream);
    const int nblocks = c.chunk * c.int_time;
    auto mark = [&](int i) {
        if (c.timing) cudaEventRecord(b->ev[i], s);
    };
    int nu = 0;
    mark(0);
    if (c.udp_packet_bytes > 0) {  // the chunk is packets: in_int16 does not apply
        PV_TRY(pv::channelise_stokes_i(b->ppf, d_voltages, c.nsub, nblocks, c.int_time, c.int_chan, b->d_fb, &nu,
                                       c.udp_packet_bytes, c.udp_subbands, s));
    } else {
        PV_TRY(pv_channelise(b->ppf, d_voltages, in_int16, c.nsub, nblocks, 1, c.int_time, c.int_chan,
                             b->d_fb, &nu, stream));
    }
    if (nu != c.chunk) {
        pv::set_error("pv_beam_process: integration produced %d of %d samples", nu, c.chunk);
        return PV_ERR_STATE;
    }
    if (b->d_fb_raw)
        PV_CUDA(cudaMemcpyAsync(b->d_fb_raw, b->d_fb, sizeof(float) * (size_t)c.chunk * b->nbins,
                                cudaMemcpyDeviceToDevice, s), "copy filterbank tap");
    mark(1);
    PV_TRY(pv_rfi_run(b->rfi, b->d_fb, c.chunk, c.nsub, 1, b->nchan_fb, nullptr, stream));
    mark(2);
    PV_TRY(pv::ring_write_device(b->d_ring, b->row_stride, b->ring_len, b->chunks * c.chunk, b->d_fb,
                                 c.chunk, c.nsub, 1, b->nchan_fb, b->inverted, s));
    mark(3);
    b->chunks += 1;
    b->timed = false;
    if (b->chunks > b->lag) {
        const long long w = b->chunks - 1 - b->lag;
        PV_TRY(pv_dedisp_plan_run(b->plan, b->d_out, c.chunk, b->d_ring, b->row_stride, 0,
                                  b->ring_len, (w * c.chunk) % b->ring_len, c.chunk, stream));
        mark(4);
        PV_TRY(pv::analyse_launch(b->d_out, c.chunk, c.tdms, c.chunk, c.threshold, b->rms,
                                  c.bin_pow2, b->d_events, b->cap, b->d_total, b->d_scratch, s));
        mark(5);
        PV_CUDA(cudaMemcpyAsync(b->h_total, b->d_total, sizeof(long long), cudaMemcpyDeviceToHost, s),
                "read event count");
        b->window = w;
        b->timed = c.timing != 0;
    }
    return PV_OK;
}

extern "C" int pv_beam_stage_ms(pv_beam* b, float* h_ms5) {
    if (!b || !h_ms5) return PV_ERR_ARG;
    if (!b->timed) {
        pv::set_error("pv_beam_stage_ms: timing is off or no window was dedispersed yet");
        return PV_ERR_STATE;
    }
    for (int i = 0; i < 5; ++i) {
        PV_CUDA(cudaEventSynchronize(b->ev[i + 1]), "synchronise stage event");
        PV_CUDA(cudaEventElapsedTime(&h_ms5[i], b->ev[i], b->ev[i + 1]), "stage time");
    }
    return PV_OK;
}

extern "C" int pv_beam_process_host(pv_beam* b, const void* h_voltages, int in_int16, void* stream) {
    if (!b || !h_voltages) return PV_ERR_ARG;
    const size_t bytes = (size_t)pv_beam_input_bytes(b, in_int16);
    if (b->in_bytes < bytes) {
        if (b->d_in) cudaFree(b->d_in);
        b->d_in = nullptr;
        b->in_bytes = 0;
        PV_CUDA(cudaMalloc(&b->d_in, bytes), "allocate input staging");
        b->in_bytes = bytes;
    }
    PV_CUDA(cudaMemcpyAsync(b->d_in, h_voltages, bytes, cudaMemcpyHostToDevice, pv::as_stream(stream)),
            "copy voltages to the device");
    return pv_beam_process(b, b->d_in, in_int16, stream);
}

extern "C" int pv_beam_events(pv_beam* b, pv_event* h_events, long long cap, long long* h_count,
                              long long* h_first_sample, void* stream) {
    if (!b || !h_count) return PV_ERR_ARG;
    cudaStream_t s = pv::as_stream(stream);
    PV_CUDA(cudaStreamSynchronize(s), "synchronise");
    if (b->window < 0) {
        *h_count = 0;
        if (h_first_sample) *h_first_sample = -1;
        return PV_OK;
    }
    int status = PV_OK;
    PV_TRY(pv_dedisp_plan_status(b->plan, &status));
    if (status != PV_OK) {
        pv::set_error("pv_beam_events: a dedispersion pipeline wait gave up (status %d)", status);
        return status;
    }
    *h_count = *b->h_total;
    if (h_first_sample) *h_first_sample = b->window * b->cfg.chunk;
    const long long n = std::min(std::min(*b->h_total, b->cap), cap);
    if (h_events && n > 0)
        PV_CUDA(cudaMemcpy(h_events, b->d_events, sizeof(pv_event) * n, cudaMemcpyDeviceToHost),
                "copy events");
    return PV_OK;
}

// ---------------------------------------------------------------------------
// Saved state: a header naming the configuration and the stream position,
// then the PPF tap history, the clipper's running state and the ring's
// ring_len columns of every channel row.
// ---------------------------------------------------------------------------
namespace {

struct BeamStateHeader {
    char magic[8];
    long long version, bytes;
    long long nbins, nsub, nchan_sub, ntaps, int_time, int_chan, chunk, tdms, history, lag, ring_len;
    long long chunks;  // chunks in the ring (prefilled silence included)
    long long ppf_bytes, rfi_bytes, ring_bytes;
    double fch1, foff, tsamp, dm_low, dm_step;
};
constexpr char kStateMagic[8] = {'P', 'V', 'B', 'E', 'A', 'M', 'S', '1'};

BeamStateHeader state_header(const pv_beam* b) {
    const pv_beam_config& c = b->cfg;
    BeamStateHeader h{};
    std::memcpy(h.magic, kStateMagic, 8);
    h.version = 1;
    h.nbins = b->nbins;
    h.nsub = c.nsub;
    h.nchan_sub = c.nchan_sub;
    h.ntaps = c.ntaps;
    h.int_time = c.int_time;
    h.int_chan = c.int_chan;
    h.chunk = c.chunk;
    h.tdms = c.tdms;
    h.history = c.history;
    h.lag = b->lag;
    h.ring_len = b->ring_len;
    h.chunks = b->chunks;
    h.ppf_bytes = pv::ppf_state_bytes(b->ppf, c.nsub, 2);
    h.rfi_bytes = pv::rfi_state_bytes(b->rfi, b->nbins);
    h.ring_bytes = (long long)b->nbins * b->ring_len * (long long)sizeof(float);
    h.fch1 = c.fch1;
    h.foff = c.foff;
    h.tsamp = c.tsamp;
    h.dm_low = c.dm_low;
    h.dm_step = c.dm_step;
    h.bytes = (long long)sizeof(BeamStateHeader) + h.ppf_bytes + h.rfi_bytes + h.ring_bytes;
    return h;
}

}  // namespace

extern "C" long long pv_beam_state_size(const pv_beam* b) {
    if (!b) return -1;
    return state_header(b).bytes;
}

extern "C" int pv_beam_state_save(pv_beam* b, void* h_buf, long long cap, void* stream) {
    if (!b || !h_buf) return PV_ERR_ARG;
    const BeamStateHeader h = state_header(b);
    if (cap < h.bytes) {
        pv::set_error("pv_beam_state_save: %lld bytes needed, %lld given", h.bytes, cap);
        return PV_ERR_ARG;
    }
    cudaStream_t s = pv::as_stream(stream);
    char* p = static_cast<char*>(h_buf);
    std::memcpy(p, &h, sizeof(h));
    p += sizeof(h);
    PV_TRY(pv::ppf_state_io(b->ppf, b->cfg.nsub, 2, p, true, s));
    p += h.ppf_bytes;
    PV_TRY(pv::rfi_state_io(b->rfi, b->nbins, p, true, s));
    p += h.rfi_bytes;
    PV_CUDA(cudaMemcpy2DAsync(p, sizeof(float) * (size_t)b->ring_len, b->d_ring, sizeof(float) * (size_t)b->row_stride,
                              sizeof(float) * (size_t)b->ring_len, (size_t)b->nbins, cudaMemcpyDeviceToHost, s),
            "save ring");
    PV_CUDA(cudaStreamSynchronize(s), "synchronise state save");
    return PV_OK;
}

extern "C" int pv_beam_state_load(pv_beam* b, const void* h_buf, long long bytes, void* stream) {
    if (!b || !h_buf) return PV_ERR_ARG;
    const BeamStateHeader want = state_header(b);
    BeamStateHeader h{};
    if (bytes < (long long)sizeof(h)) {
        pv::set_error("pv_beam_state_load: %lld bytes are not a beam state", bytes);
        return PV_ERR_ARG;
    }
    std::memcpy(&h, h_buf, sizeof(h));
    if (std::memcmp(h.magic, kStateMagic, 8) != 0 || h.version != 1) {
        pv::set_error("pv_beam_state_load: not a beam state of this library version");
        return PV_ERR_ARG;
    }
    if (h.bytes != bytes || h.nbins != want.nbins || h.nsub != want.nsub || h.nchan_sub != want.nchan_sub ||
        h.ntaps != want.ntaps || h.int_time != want.int_time || h.int_chan != want.int_chan ||
        h.chunk != want.chunk || h.tdms != want.tdms || h.history != want.history || h.lag != want.lag ||
        h.ring_len != want.ring_len || h.ppf_bytes != want.ppf_bytes || h.rfi_bytes != want.rfi_bytes ||
        h.ring_bytes != want.ring_bytes || h.fch1 != want.fch1 || h.foff != want.foff || h.tsamp != want.tsamp ||
        h.dm_low != want.dm_low || h.dm_step != want.dm_step) {
        pv::set_error("pv_beam_state_load: the state was saved from a beam of another configuration");
        return PV_ERR_CONFIG;
    }
    cudaStream_t s = pv::as_stream(stream);
    const char* p = static_cast<const char*>(h_buf) + sizeof(h);
    PV_TRY(pv::ppf_state_io(b->ppf, b->cfg.nsub, 2, const_cast<char*>(p), false, s));
    p += h.ppf_bytes;
    PV_TRY(pv::rfi_state_io(b->rfi, b->nbins, const_cast<char*>(p), false, s));
    p += h.rfi_bytes;
    PV_CUDA(cudaMemcpy2DAsync(b->d_ring, sizeof(float) * (size_t)b->row_stride, p, sizeof(float) * (size_t)b->ring_len,
                              sizeof(float) * (size_t)b->ring_len, (size_t)b->nbins, cudaMemcpyHostToDevice, s),
            "load ring");
    PV_CUDA(cudaStreamSynchronize(s), "synchronise state load");
    b->chunks = h.chunks;
    b->window = -1;  // no window of this stream has been dedispersed since the load
    b->timed = false;
    return PV_OK;
}

extern "C" int pv_beam_buffers(const pv_beam* b, float** d_filterbank, float** d_filterbank_raw,
                               float** d_dedispersed, float** d_ring) {
    if (!b) return PV_ERR_ARG;
    if (d_filterbank) *d_filterbank = b->d_fb;
    if (d_filterbank_raw) *d_filterbank_raw = b->d_fb_raw;
    if (d_dedispersed) *d_dedispersed = b->d_out;
    if (d_ring) *d_ring = b->d_ring;
    return PV_OK;
}
