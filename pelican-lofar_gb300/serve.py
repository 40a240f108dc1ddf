"""Serving loop: many beams streaming chunks into the batched engine on one GPU.

A stream is one beam: a ``pv_beam_config`` and the arrival times and sizes
(spectra) of its chunks.  Chunks are cut into sub-chunks of the engine's step
size (4096 spectra) and queued per beam.  Beams are admitted under an HBM
budget (each beam's device footprint from ``pv_batch_footprint``) in cohorts:
every admission creates one batch over the beams admitted together, on its
own CUDA stream, so the steps of all cohorts overlap on the device.  In every
step of a cohort, exactly the beams with a queued sub-chunk are active
(continuous batching at sub-chunk granularity: a chunk that arrives while a
step runs joins the next one).  A cohort is released, and its memory returned
to the budget, once every stream in it has ended and drained; waiting beams
are then admitted.

Latency of a chunk: from its arrival to the end of the step that processed
its last sub-chunk (the dedispersed window that covers its last sample comes
``lag`` chunks later, as in any streaming dedisperser).

The comparison path ("plain") serves the same streams with one ``pv_beam``
per beam and one sub-chunk at a time, oldest first, each copied in, processed
and its events read back before the next (the reference's job-per-buffer
style).

Engines implement ``footprint(cfg)``, optionally ``prepare(cfgs)`` (called
before the clock starts) and ``open(cfgs, ids) -> cohort`` with
``step(active) -> id``, ``done(id)``, ``close()``; the tests drive the loop
with a fake engine on the CPU.
"""
import collections
import time

import numpy as np

SUB_CHUNK = 4096


class Stream:
    """One beam's stream: its configuration, chunk arrival times (s, from the
    start of the run) and chunk sizes (spectra, multiples of SUB_CHUNK)."""

    def __init__(self, cfg, arrivals, sizes, units_per_spectrum, tsamp=1.0):
        self.cfg = cfg
        self.arrivals = list(arrivals)
        self.sizes = list(sizes)
        self.units_per_spectrum = units_per_spectrum  # trials x channels
        self.tsamp = tsamp  # seconds per spectrum

    @property
    def end(self):
        return self.arrivals[-1] if self.arrivals else 0.0


def poisson_streams(beams, duration, seed, start_spread=0.5, min_life=0.3):
    """Streams for beam dicts with keys cfg, tsamp, tdms, nchan: each starts
    at a uniform time in [0, start_spread*duration), lives for a uniform share
    of the rest (at least min_life of the run), has a fixed chunk size drawn
    from 1..8 sub-chunks and Poisson arrivals at one chunk per chunk
    duration."""
    rng = np.random.default_rng(seed)
    out = []
    for b in beams:
        size = SUB_CHUNK * int(rng.integers(1, 9))
        mean = size * b["tsamp"]
        t0 = rng.uniform(0, start_spread * duration)
        t1 = min(duration, t0 + max(min_life * duration, rng.uniform(0, duration - t0)))
        t, arr = t0, []
        while True:
            t += rng.exponential(mean)
            if t >= t1:
                break
            arr.append(t)
        if not arr:
            arr = [min(t0 + mean, duration)]
        out.append(Stream(b["cfg"], arr, [size] * len(arr), b["tdms"] * b["nchan"], b["tsamp"]))
    return out


class _Cohort:
    def __init__(self, handle, ids, footprint, t_admit):
        self.handle = handle
        self.ids = ids
        self.footprint = footprint
        self.inflight = collections.deque()  # (step id, [(stream, chunk, last)])
        self.t_admit = t_admit


class Server:
    """Runs streams through an engine under an HBM budget (bytes).

    policy "batch": every step of a cohort takes one sub-chunk of every beam
    that has one (continuous batching); "fifo1": one sub-chunk per step, the
    oldest queued one, and each step completes before the next is issued."""

    def __init__(self, engine, streams, budget, policy="batch", admit_every=0.5, max_inflight=2):
        self.engine = engine
        self.streams = streams
        self.budget = budget
        self.policy = policy
        self.admit_every = admit_every
        self.max_inflight = max_inflight if policy == "batch" else 1

    def run(self, clock=time.perf_counter, sleep=time.sleep, horizon=None):
        streams = self.streams
        n = len(streams)
        foot = [self.engine.footprint(s.cfg) for s in streams]
        prepare = getattr(self.engine, "prepare", None)
        if prepare:  # receive buffers exist before the streams start
            prepare([s.cfg for s in streams])
        events = sorted((t, i, k) for i, s in enumerate(streams) for k, t in enumerate(s.arrivals))
        nxt = 0
        queues = [collections.deque() for _ in range(n)]  # (chunk, sub index, last)
        owner = [None] * n  # (cohort, slot) once admitted
        waiting = []
        admitted_at = [None] * n
        first_arrival = [s.arrivals[0] if s.arrivals else None for s in streams]
        cohorts = []
        used = peak = 0
        last_admit = -1e9
        lat, lat_adm, ratio, waits, units = [], [], [], [], 0.0
        left = [len(s.arrivals) for s in streams]  # chunks not yet completed
        sub_left = {}  # (stream, chunk) -> sub-chunks not yet completed
        max_beams = 0
        t0 = clock()
        while True:
            now = clock() - t0
            busy = False
            # arrivals
            while nxt < len(events) and events[nxt][0] <= now:
                t, i, k = events[nxt]
                nxt += 1
                nsub = streams[i].sizes[k] // SUB_CHUNK
                sub_left[(i, k)] = nsub
                for j in range(nsub):
                    queues[i].append((k, j, j == nsub - 1))
                if owner[i] is None and i not in waiting:
                    waiting.append(i)
            # admission of waiting beams, first fit in arrival order
            if waiting and now - last_admit >= self.admit_every:
                take = []
                for i in list(waiting):
                    if used + foot[i] <= self.budget:
                        take.append(i)
                        used += foot[i]
                        waiting.remove(i)
                if take:
                    handle = self.engine.open([streams[i].cfg for i in take], take)
                    c = _Cohort(handle, take, sum(foot[i] for i in take), now)
                    for slot, i in enumerate(take):
                        owner[i] = (c, slot)
                        admitted_at[i] = clock() - t0
                        waits.append(admitted_at[i] - first_arrival[i])
                    cohorts.append(c)
                    peak = max(peak, used)
                    last_admit = now
                    busy = True
                max_beams = max(max_beams, sum(len(c.ids) for c in cohorts))
            # completions
            for c in cohorts:
                while c.inflight and c.handle.done(c.inflight[0][0]):
                    _, work = c.inflight.popleft()
                    tnow = clock() - t0
                    for i, k, last in work:
                        units += streams[i].units_per_spectrum * SUB_CHUNK
                        sub_left[(i, k)] -= 1
                        if sub_left[(i, k)] == 0:
                            a = streams[i].arrivals[k]
                            lat.append(tnow - a)
                            if a >= admitted_at[i]:
                                lat_adm.append(tnow - a)
                            ratio.append((tnow - a) / (streams[i].sizes[k] * streams[i].tsamp))
                            left[i] -= 1
                    busy = True
            # steps
            if self.policy == "batch":
                for c in cohorts:
                    if len(c.inflight) >= self.max_inflight:
                        continue
                    active = np.array([1 if queues[i] else 0 for i in c.ids], np.uint8)
                    if not active.any():
                        continue
                    work = []
                    for slot, i in enumerate(c.ids):
                        if active[slot]:
                            k, j, last = queues[i].popleft()
                            work.append((i, k, last))
                    c.inflight.append((c.handle.step(active), work))
                    busy = True
            else:  # fifo1: the oldest queued sub-chunk of any admitted beam, one at a time
                if not any(c.inflight for c in cohorts):
                    best = None
                    for c in cohorts:
                        for slot, i in enumerate(c.ids):
                            if queues[i]:
                                k = queues[i][0][0]
                                key = (streams[i].arrivals[k], i)
                                if best is None or key < best[0]:
                                    best = (key, c, slot, i)
                    if best is not None:
                        _, c, slot, i = best
                        active = np.zeros(len(c.ids), np.uint8)
                        active[slot] = 1
                        k, j, last = queues[i].popleft()
                        c.inflight.append((c.handle.step(active), [(i, k, last)]))
                        busy = True
            # release cohorts whose streams have all ended and drained
            for c in list(cohorts):
                if not c.inflight and all(left[i] == 0 and not queues[i] for i in c.ids):
                    c.handle.close()
                    cohorts.remove(c)
                    used -= c.footprint
                    busy = True
            if nxt >= len(events) and not cohorts and not waiting:
                break
            if horizon is not None and now > horizon:
                break
            if not busy:
                pause = 0.001
                if nxt < len(events):
                    pause = min(max(events[nxt][0] - now, 0.0), 0.001)
                sleep(pause)
        wall = clock() - t0

        def pct(x):
            x = np.array(x) if x else np.zeros(1)
            return {"p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99)),
                    "max": float(x.max())}
        within = float(np.mean(np.array(ratio) < 1.0)) if ratio else 1.0
        done_chunks = sum(len(s.arrivals) - left[i] for i, s in enumerate(streams))
        return {"policy": self.policy, "beams": n, "chunks": int(sum(len(s.arrivals) for s in streams)),
                "chunks_done": int(done_chunks), "wall_s": wall,
                "throughput": units / wall, "units": units,
                "latency_s": pct(lat),
                "latency_after_admission_s": pct(lat_adm),
                "latency_over_chunk_duration": pct(ratio),
                "chunks_within_real_time": within,
                "admission_wait_s": pct(waits),
                "max_concurrent_beams": max_beams, "peak_footprint_gb": peak / 1e9,
                "budget_gb": self.budget / 1e9}


# ---------------------------------------------------------------------------
# engines on the GPU
# ---------------------------------------------------------------------------

class BatchEngine:
    """Cohorts are pv.Batch objects (graph, pipelined) fed from page-locked,
    page-locked staging buffers holding one synthetic sub-chunk per beam."""

    def __init__(self, pv, make_voltages, stream_factory, pipelined=True, tune=False, variant=3, store="f32"):
        self.pv = pv
        self.make_voltages = make_voltages  # cfg -> int16 device tensor of one sub-chunk
        self.stream_factory = stream_factory
        self.pipelined = pipelined
        self.tune = tune
        self.variant = variant
        self.store = store  # delay-ring storage: "f32", "f16" or "u8"

    def footprint(self, cfg):
        return self.pv.batch_footprint(cfg, self.pipelined, self.store)

    def prepare(self, cfgs):
        self.staging = _staging(self.pv, self.make_voltages, cfgs)

    def open(self, cfgs, ids):
        return _BatchCohort(self, cfgs, [self.staging[i] for i in ids])


def _staging(pv, make_voltages, cfgs):
    """One page-locked receive buffer per stream, holding a
    synthetic sub-chunk of voltages."""
    out = []
    for c in cfgs:
        v = make_voltages(c)
        hb = pv.HostBuffer(v.numel() * v.element_size())
        hb.fill_from(v)
        out.append(hb)
        del v
    return out


class _BatchCohort:
    def __init__(self, eng, cfgs, staging):
        pv = eng.pv
        self.batch = pv.Batch(cfgs, tune=eng.tune, graph=True, variant=eng.variant,
                              pipelined=eng.pipelined, store=eng.store)
        self.stream = eng.stream_factory()
        self.staging = staging
        self.steps = 0

    def step(self, active):
        self.batch.run_host(self.staging, active=active, stream=self.stream)
        self.steps += 1
        return self.steps - 1

    def done(self, step_id):
        return self.batch.step_done(step_id)

    def close(self):
        self.stream.synchronize()
        self.batch = None
        self.staging = []


class PlainEngine:
    """The plain per-chunk path: one pv_beam per beam, a sub-chunk copied in,
    processed and its events read back before the next."""

    def __init__(self, pv, make_voltages, stream_factory):
        self.pv = pv
        self.make_voltages = make_voltages
        self.stream_factory = stream_factory

    def footprint(self, cfg):
        return self.pv.batch_footprint(cfg, False)

    def prepare(self, cfgs):
        self.staging = _staging(self.pv, self.make_voltages, cfgs)

    def open(self, cfgs, ids):
        return _PlainCohort(self, cfgs, [self.staging[i] for i in ids])


class _PlainCohort:
    def __init__(self, eng, cfgs, staging):
        pv = eng.pv
        self.beams = [pv.Beam(c) for c in cfgs]
        self.stream = eng.stream_factory()
        self.staging = staging
        self.steps = 0

    def step(self, active):
        for slot in np.flatnonzero(active):
            self.beams[slot].process_host(self.staging[slot], stream=self.stream)
            self.beams[slot].events(cap=1 << 16, stream=self.stream)  # synchronises
        self.steps += 1
        return self.steps - 1

    def done(self, step_id):
        return True

    def close(self):
        self.beams = []
        self.staging = []
