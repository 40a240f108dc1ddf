// Serving loop: many beams streaming chunks into the batched engine on one
// GPU (pv_serve).  No counterpart in the reference, whose pipelines run one
// beam per process and take chunks as DedispersionPipeline::run does
// (pipelines/udpstream/src/DedispersionPipeline.cpp:96-174).
//
// A stream is one beam: a pv_beam_config, the arrival times of its chunks
// and their sizes (spectra, multiples of the engine's step chunk).  A chunk
// is queued as sub-chunks of one step each.  Streams are admitted under an
// HBM budget (the device footprint pv_batch_footprint computes): a stream
// that arrives takes, at once, the slot of a drained stream of the same
// configuration in a running cohort; the others are admitted first fit every
// admit_every seconds as a new cohort (one pv_batch on its own CUDA stream,
// so the steps of all cohorts overlap on the device).  Every step of a
// cohort takes one sub-chunk of each of its beams that has one queued
// (continuous batching: a chunk that arrives while a step runs joins the
// next one).  A cohort whose streams have all drained is released, and its
// memory returned to the budget, as soon as a waiting stream needs the
// memory, else after it has lingered idle for `linger` seconds, kept for a
// stream of its configuration.  The chunk latency is the time from a chunk's arrival to the end
// of the step that processed its last sub-chunk.
//
// The FIFO1 policy is the plain per-chunk path: one pv_beam per stream, the
// oldest queued sub-chunk of any admitted stream processed alone, copied in,
// dedispersed and its events read back before the next (the reference's job
// per buffer).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "pv_internal.cuh"

namespace {

// --------------------------------------------------------------------------
// Engines over the library (the default hooks)
// --------------------------------------------------------------------------
struct GpuCtx {
    int policy = PV_SERVE_BATCH;
    int flags = 0;
    std::vector<const void*> volts;  // per stream: one sub-chunk of page-locked voltages
};

struct GpuCohort {
    pv_batch* batch = nullptr;
    std::vector<pv_beam*> beams;     // FIFO1: one beam per slot
    std::vector<int> streams;        // the stream of each slot
    std::vector<const pv_beam_config*> cfgs;
    cudaStream_t stream = nullptr;
    long long steps = 0;
};

long long gpu_footprint(void* ctx, const pv_beam_config* c) {
    const GpuCtx* g = static_cast<GpuCtx*>(ctx);
    return pv_batch_footprint(c, g->policy == PV_SERVE_FIFO1 ? 0 : g->flags);
}

void gpu_close(void* ctx, void* h) {
    (void)ctx;
    auto* c = static_cast<GpuCohort*>(h);
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->batch) pv_batch_destroy(c->batch);
    for (pv_beam* b : c->beams) pv_beam_destroy(b);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

void* gpu_open(void* ctx, const pv_beam_config* cfgs, const int* ids, int n) {
    const GpuCtx* g = static_cast<GpuCtx*>(ctx);
    auto* c = new GpuCohort;
    c->streams.assign(ids, ids + n);
    int rc = pv::cuda_status(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "create cohort stream");
    if (rc == PV_OK && g->policy == PV_SERVE_FIFO1) {
        c->beams.assign(n, nullptr);
        for (int i = 0; i < n && rc == PV_OK; ++i) rc = pv_beam_create(&c->beams[i], &cfgs[i]);
    } else if (rc == PV_OK) {
        rc = pv_batch_create(&c->batch, cfgs, n, g->flags);
    }
    if (rc != PV_OK) {
        gpu_close(ctx, c);
        return nullptr;
    }
    return c;
}

long long gpu_step(void* ctx, void* h, const unsigned char* active, int n) {
    const GpuCtx* g = static_cast<GpuCtx*>(ctx);
    auto* c = static_cast<GpuCohort*>(h);
    if (g->policy == PV_SERVE_FIFO1) {
        for (int i = 0; i < n; ++i) {
            if (!active[i]) continue;
            if (pv_beam_process_host(c->beams[i], g->volts[c->streams[i]], 1, c->stream) != PV_OK) return -1;
            long long count = 0, first = 0;
            if (pv_beam_events(c->beams[i], nullptr, 0, &count, &first, c->stream) != PV_OK) return -1;
        }
        return c->steps++;
    }
    std::vector<const void*> v(n);
    for (int i = 0; i < n; ++i) v[i] = g->volts[c->streams[i]];
    if (pv_batch_run_host(c->batch, v.data(), active, c->stream) != PV_OK) return -1;
    return c->steps++;
}

int gpu_done(void* ctx, void* h, long long step) {
    (void)ctx;
    auto* c = static_cast<GpuCohort*>(h);
    if (!c->batch) return 1;  // FIFO1 steps complete before step() returns
    return pv_batch_step_done(c->batch, step) == 1 ? 1 : 0;
}

long long gpu_events(void* ctx, void* h, long long step, int slot, pv_event* out, long long cap,
                     long long* first) {
    const GpuCtx* g = static_cast<GpuCtx*>(ctx);
    auto* c = static_cast<GpuCohort*>(h);
    long long count = 0;
    *first = -1;
    if (g->policy == PV_SERVE_FIFO1) {
        if (pv_beam_events(c->beams[slot], out, cap, &count, first, c->stream) != PV_OK) return -1;
        return count;
    }
    if (pv_batch_events(c->batch, slot, step, out, cap, &count, first) != PV_OK) return -1;
    return count;
}

int gpu_reset_slot(void* ctx, void* h, int slot, int stream) {
    const GpuCtx* g = static_cast<GpuCtx*>(ctx);
    auto* c = static_cast<GpuCohort*>(h);
    if (g->policy == PV_SERVE_FIFO1) return PV_ERR_STATE;  // the plain path does not reuse slots
    c->streams[slot] = stream;
    return pv_batch_reset_beam(c->batch, slot, c->stream);
}

double wall_clock(void*) {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}
void wall_sleep(void*, double s) {
    std::this_thread::sleep_for(std::chrono::duration<double>(std::max(s, 0.0)));
}

// --------------------------------------------------------------------------
// The loop
// --------------------------------------------------------------------------
bool same_config(const pv_beam_config& a, const pv_beam_config& b) {
    pv_beam_config x = a, y = b;
    const bool same_bp = (!a.bp_text && !b.bp_text) ||
                         (a.bp_text && b.bp_text && std::strcmp(a.bp_text, b.bp_text) == 0);
    x.bp_text = y.bp_text = nullptr;
    return same_bp && std::memcmp(&x, &y, sizeof(x)) == 0;
}

struct Cohort {
    void* handle = nullptr;
    std::vector<int> slot_stream;   // stream served by each slot (-1: free)
    double footprint = 0.0;
    double idle_since = -1.0;       // time since which every stream has drained (-1: busy)
    std::deque<std::pair<long long, std::vector<std::pair<int, int>>>> inflight;  // step, (stream, chunk)
};

struct Sub {
    int chunk;
};

double percentile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    std::sort(v.begin(), v.end());
    // linear interpolation between closest ranks (numpy's default)
    const double pos = q / 100.0 * (double)(v.size() - 1);
    const size_t i = (size_t)pos;
    const double f = pos - (double)i;
    return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

}  // namespace

extern "C" int pv_serve(const pv_serve_config* cfg, const pv_beam_config* beams, const pv_serve_stream* streams,
                        int nstreams, const pv_serve_engine* engine_in, const pv_serve_output* output,
                        pv_serve_stats* out) {
    if (!cfg || !beams || !streams || nstreams <= 0 || !out) {
        pv::set_error("pv_serve: invalid arguments");
        return PV_ERR_ARG;
    }
    if (cfg->policy != PV_SERVE_BATCH && cfg->policy != PV_SERVE_FIFO1) {
        pv::set_error("pv_serve: unknown policy %d", cfg->policy);
        return PV_ERR_ARG;
    }
    for (int i = 0; i < nstreams; ++i) {
        const pv_serve_stream& s = streams[i];
        for (int k = 0; k < s.nchunks; ++k)
            if (s.sizes[k] <= 0 || s.sizes[k] % beams[i].chunk != 0 || (k > 0 && s.arrivals[k] < s.arrivals[k - 1])) {
                pv::set_error("pv_serve: stream %d chunk %d: sizes must be positive multiples of the chunk (%d) "
                              "and arrivals ascending", i, k, beams[i].chunk);
                return PV_ERR_ARG;
            }
        if (!engine_in && !s.h_voltages) {
            pv::set_error("pv_serve: stream %d has no voltages", i);
            return PV_ERR_ARG;
        }
    }
    GpuCtx gctx;
    pv_serve_engine eng{};
    if (engine_in) {
        eng = *engine_in;
    } else {
        gctx.policy = cfg->policy;
        gctx.flags = cfg->batch_flags;
        for (int i = 0; i < nstreams; ++i) gctx.volts.push_back(streams[i].h_voltages);
        eng.ctx = &gctx;
        eng.footprint = gpu_footprint;
        eng.open = gpu_open;
        eng.step = gpu_step;
        eng.done = gpu_done;
        eng.reset_slot = gpu_reset_slot;
        eng.close = gpu_close;
        eng.events = gpu_events;
    }
    if (!eng.clock) eng.clock = wall_clock;
    if (!eng.sleep) eng.sleep = wall_sleep;
    const bool batch = cfg->policy == PV_SERVE_BATCH;
    const int max_inflight = batch ? std::max(1, std::min(cfg->max_inflight > 0 ? cfg->max_inflight : 2, 2)) : 1;
    const bool reuse = batch && cfg->reuse_slots;

    std::vector<double> foot(nstreams);
    for (int i = 0; i < nstreams; ++i) {
        const long long f = eng.footprint(eng.ctx, &beams[i]);
        if (f < 0) return PV_ERR_CONFIG;
        foot[i] = (double)f;
    }
    // every arrival in time order
    struct Arrival {
        double t;
        int stream, chunk;
    };
    std::vector<Arrival> arrivals;
    for (int i = 0; i < nstreams; ++i)
        for (int k = 0; k < streams[i].nchunks; ++k) arrivals.push_back({streams[i].arrivals[k], i, k});
    std::stable_sort(arrivals.begin(), arrivals.end(), [](const Arrival& a, const Arrival& b) { return a.t < b.t; });
    std::vector<long long> last_arrival(nstreams, -1);  // index of each stream's last arrival
    for (size_t a = 0; a < arrivals.size(); ++a) last_arrival[arrivals[a].stream] = (long long)a;

    std::vector<std::deque<Sub>> queues(nstreams);
    std::vector<int> owner_cohort(nstreams, -1), owner_slot(nstreams, -1);
    std::vector<std::vector<int>> sub_left(nstreams);
    for (int i = 0; i < nstreams; ++i) sub_left[i].assign(streams[i].nchunks, 0);
    std::vector<int> left(nstreams);
    for (int i = 0; i < nstreams; ++i) left[i] = streams[i].nchunks;
    std::vector<double> admitted_at(nstreams, -1.0);
    std::vector<char> waiting_flag(nstreams, 0);
    std::deque<int> waiting;
    std::vector<Cohort*> cohorts;
    double used = 0.0, peak = 0.0, last_admit = -1e300, units = 0.0;
    std::vector<double> lat, lat_adm, ratio, waits;
    std::vector<pv_event> evbuf(output && output->events ? (size_t)PV_BATCH_HOST_EVENTS : 0);
    long long reused = 0, opened = 0, steps_issued = 0;
    int max_beams = 0;
    size_t nxt = 0;
    int rc = PV_OK;
    const double t0 = eng.clock(eng.ctx);
    auto served_beams = [&]() {
        int n = 0;
        for (Cohort* c : cohorts)
            for (int s : c->slot_stream) n += s >= 0;
        return n;
    };
    auto drained = [&](int i) { return left[i] == 0 && queues[i].empty(); };
    auto all_arrived = [&](int i) { return (long long)nxt > last_arrival[i]; };
    while (rc == PV_OK) {
        const double now = eng.clock(eng.ctx) - t0;
        bool busy = false;
        // arrivals
        while (nxt < arrivals.size() && arrivals[nxt].t <= now) {
            const Arrival& a = arrivals[nxt++];
            const int nsub = streams[a.stream].sizes[a.chunk] / beams[a.stream].chunk;
            sub_left[a.stream][a.chunk] = nsub;
            for (int j = 0; j < nsub; ++j) queues[a.stream].push_back(Sub{a.chunk});
            if (owner_cohort[a.stream] < 0 && !waiting_flag[a.stream]) {
                waiting.push_back(a.stream);
                waiting_flag[a.stream] = 1;
            }
        }
        // a waiting stream takes the free slot of a drained stream of its configuration
        if (reuse && !waiting.empty()) {
            for (auto it = waiting.begin(); it != waiting.end();) {
                const int i = *it;
                bool placed = false;
                for (size_t ci = 0; ci < cohorts.size() && !placed; ++ci) {
                    Cohort* c = cohorts[ci];
                    if (!c->inflight.empty()) continue;  // a reset waits for the cohort's steps
                    for (size_t sl = 0; sl < c->slot_stream.size() && !placed; ++sl) {
                        const int j = c->slot_stream[sl];
                        if (j < 0 || !drained(j) || !all_arrived(j) || !same_config(beams[i], beams[j])) continue;
                        if (eng.reset_slot(eng.ctx, c->handle, (int)sl, i) != PV_OK) continue;
                        c->slot_stream[sl] = i;
                        owner_cohort[j] = -2;  // j is finished: it holds no slot
                        owner_cohort[i] = (int)ci;
                        owner_slot[i] = (int)sl;
                        admitted_at[i] = eng.clock(eng.ctx) - t0;
                        waits.push_back(admitted_at[i] - streams[i].arrivals[0]);
                        ++reused;
                        placed = true;
                    }
                }
                if (placed) {
                    waiting_flag[i] = 0;
                    it = waiting.erase(it);
                    busy = true;
                } else {
                    ++it;
                }
            }
        }
        // admission of waiting streams as a new cohort, first fit in arrival order
        if (!waiting.empty() && now - last_admit >= cfg->admit_every) {
            std::vector<int> take;
            for (auto it = waiting.begin(); it != waiting.end();) {
                if (used + foot[*it] <= cfg->budget_bytes) {
                    take.push_back(*it);
                    used += foot[*it];
                    waiting_flag[*it] = 0;
                    it = waiting.erase(it);
                } else {
                    ++it;
                }
            }
            if (!take.empty()) {
                std::vector<pv_beam_config> cf;
                for (int i : take) cf.push_back(beams[i]);
                void* h = eng.open(eng.ctx, cf.data(), take.data(), (int)take.size());
                if (!h) {
                    rc = PV_ERR_NOMEM;
                    break;
                }
                ++opened;
                auto* c = new Cohort;
                c->handle = h;
                c->slot_stream = take;
                for (int i : take) c->footprint += foot[i];
                for (size_t sl = 0; sl < take.size(); ++sl) {
                    owner_cohort[take[sl]] = (int)cohorts.size();
                    owner_slot[take[sl]] = (int)sl;
                    admitted_at[take[sl]] = eng.clock(eng.ctx) - t0;
                    waits.push_back(admitted_at[take[sl]] - streams[take[sl]].arrivals[0]);
                }
                cohorts.push_back(c);
                peak = std::max(peak, used);
                last_admit = now;
                busy = true;
            }
        }
        max_beams = std::max(max_beams, served_beams());
        // completions
        for (Cohort* c : cohorts) {
            while (!c->inflight.empty() && eng.done(eng.ctx, c->handle, c->inflight.front().first)) {
                const long long step_id = c->inflight.front().first;
                const auto work = c->inflight.front().second;
                c->inflight.pop_front();
                const double tnow = eng.clock(eng.ctx) - t0;
                // the windows this step dedispersed, to the output (every slot: pipelined,
                // a window comes in the step after its last chunk)
                if (output && output->events && eng.events) {
                    for (size_t sl = 0; sl < c->slot_stream.size(); ++sl) {
                        const int i = c->slot_stream[sl];
                        if (i < 0) continue;
                        long long first = -1;
                        const long long n = eng.events(eng.ctx, c->handle, step_id, (int)sl, evbuf.data(),
                                                       (long long)evbuf.size(), &first);
                        if (n < 0) {
                            rc = PV_ERR_CUDA;
                            break;
                        }
                        if (first >= 0)
                            output->events(output->ctx, i, first, evbuf.data(), std::min(n, (long long)evbuf.size()),
                                           n);
                    }
                }
                for (const auto& w : work) {
                    const int i = w.first, k = w.second;
                    units += streams[i].units_per_spectrum * beams[i].chunk;
                    if (--sub_left[i][k] == 0) {
                        const double a = streams[i].arrivals[k];
                        lat.push_back(tnow - a);
                        if (a >= admitted_at[i]) lat_adm.push_back(tnow - a);
                        ratio.push_back((tnow - a) / (streams[i].sizes[k] * beams[i].tsamp));
                        left[i] -= 1;
                    }
                }
                busy = true;
            }
        }
        // steps
        if (batch) {
            for (Cohort* c : cohorts) {
                if ((int)c->inflight.size() >= max_inflight) continue;
                const int n = (int)c->slot_stream.size();
                std::vector<unsigned char> active(n, 0);
                std::vector<std::pair<int, int>> work;
                for (int sl = 0; sl < n; ++sl) {
                    const int i = c->slot_stream[sl];
                    if (i >= 0 && owner_cohort[i] >= 0 && !queues[i].empty()) {
                        active[sl] = 1;
                        work.push_back({i, queues[i].front().chunk});
                        queues[i].pop_front();
                    }
                }
                if (work.empty()) continue;
                const long long id = eng.step(eng.ctx, c->handle, active.data(), n);
                if (id < 0) {
                    rc = PV_ERR_CUDA;
                    break;
                }
                ++steps_issued;
                c->inflight.push_back({id, work});
                busy = true;
            }
        } else {
            bool any_inflight = false;
            for (Cohort* c : cohorts) any_inflight = any_inflight || !c->inflight.empty();
            if (!any_inflight) {
                double best_t = 1e300;
                int best_c = -1, best_s = -1, best_i = -1;
                for (size_t ci = 0; ci < cohorts.size(); ++ci)
                    for (size_t sl = 0; sl < cohorts[ci]->slot_stream.size(); ++sl) {
                        const int i = cohorts[ci]->slot_stream[sl];
                        if (i < 0 || queues[i].empty()) continue;
                        const double t = streams[i].arrivals[queues[i].front().chunk];
                        if (t < best_t || (t == best_t && i < best_i)) {
                            best_t = t;
                            best_c = (int)ci;
                            best_s = (int)sl;
                            best_i = i;
                        }
                    }
                if (best_c >= 0) {
                    Cohort* c = cohorts[best_c];
                    std::vector<unsigned char> active(c->slot_stream.size(), 0);
                    active[best_s] = 1;
                    const std::pair<int, int> w{best_i, queues[best_i].front().chunk};
                    queues[best_i].pop_front();
                    const long long id = eng.step(eng.ctx, c->handle, active.data(), (int)active.size());
                    if (id < 0) {
                        rc = PV_ERR_CUDA;
                        break;
                    }
                    ++steps_issued;
                    c->inflight.push_back({id, {w}});
                    busy = true;
                }
            }
        }
        if (rc != PV_OK) break;
        // Release cohorts whose streams have drained: at once when a waiting
        // stream needs the memory (no slot here suits it) or no stream will
        // arrive any more, else after they have lingered idle (kept for a
        // stream of their configuration).
        for (size_t ci = 0; ci < cohorts.size();) {
            Cohort* c = cohorts[ci];
            bool idle = c->inflight.empty();
            for (int i : c->slot_stream) idle = idle && (i < 0 || (drained(i) && all_arrived(i)));
            if (!idle) {
                c->idle_since = -1.0;
                ++ci;
                continue;
            }
            if (c->idle_since < 0.0) c->idle_since = now;
            bool needed = nxt >= arrivals.size() || !reuse || now - c->idle_since >= cfg->linger;
            for (int w : waiting) {
                bool suits = false;
                for (int i : c->slot_stream) suits = suits || (i >= 0 && same_config(beams[w], beams[i]));
                needed = needed || !suits;
            }
            if (needed) {
                eng.close(eng.ctx, c->handle);
                used -= c->footprint;
                for (int i : c->slot_stream)
                    if (i >= 0) owner_cohort[i] = -2;
                delete c;
                cohorts.erase(cohorts.begin() + (long long)ci);
                // keep the owners' cohort indices in step with the vector
                for (int i = 0; i < nstreams; ++i)
                    if (owner_cohort[i] > (int)ci) owner_cohort[i] -= 1;
                busy = true;
            } else {
                ++ci;
            }
        }
        if (nxt >= arrivals.size() && cohorts.empty() && waiting.empty()) break;
        if (cfg->horizon > 0.0 && now > cfg->horizon) break;
        if (!busy) {
            double pause = 0.001;
            if (nxt < arrivals.size()) pause = std::min(std::max(arrivals[nxt].t - now, 0.0), 0.001);
            eng.sleep(eng.ctx, pause);
        }
    }
    const double wall = eng.clock(eng.ctx) - t0;
    for (Cohort* c : cohorts) {
        eng.close(eng.ctx, c->handle);
        delete c;
    }
    if (rc != PV_OK) return rc;
    std::memset(out, 0, sizeof(*out));
    long long chunks = 0, done_chunks = 0;
    for (int i = 0; i < nstreams; ++i) {
        chunks += streams[i].nchunks;
        done_chunks += streams[i].nchunks - left[i];
    }
    out->chunks = chunks;
    out->chunks_done = done_chunks;
    out->wall_s = wall;
    out->units = units;
    out->throughput = wall > 0.0 ? units / wall : 0.0;
    out->latency_p50 = percentile(lat, 50);
    out->latency_p99 = percentile(lat, 99);
    out->latency_max = lat.empty() ? 0.0 : *std::max_element(lat.begin(), lat.end());
    out->latency_admitted_p50 = percentile(lat_adm, 50);
    out->latency_admitted_p99 = percentile(lat_adm, 99);
    out->latency_over_duration_p50 = percentile(ratio, 50);
    out->latency_over_duration_p99 = percentile(ratio, 99);
    out->within_real_time =
        ratio.empty() ? 1.0 : (double)std::count_if(ratio.begin(), ratio.end(), [](double r) { return r < 1.0; }) /
                                  (double)ratio.size();
    out->admission_wait_p50 = percentile(waits, 50);
    out->admission_wait_p99 = percentile(waits, 99);
    out->max_concurrent_beams = max_beams;
    out->peak_footprint_bytes = peak;
    out->cohorts = opened;
    out->slot_reuses = reused;
    out->steps = steps_issued;
    return PV_OK;
}
