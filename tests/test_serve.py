"""The serving loop (pv_serve, C++ in the library) on the CPU with a fake
engine and a fake clock through its hooks: admission under the HBM budget,
continuous batching of queued sub-chunks, a drained stream's slot given to a
waiting stream of the same configuration, release of drained cohorts, the
plain one-at-a-time policy, and latency accounting (no GPU)."""
import numpy as np
import pytest

import pv as pvmod
import serve

SUB = 4096  # spectra per step


class FakeEngine:
    """A step takes per_step seconds of the fake clock plus per_beam per active
    beam; a configuration's footprint is its tdms field (bytes)."""

    def __init__(self, per_step=0.01, per_beam=0.002):
        self.t = 0.0
        self.per_step, self.per_beam = per_step, per_beam
        self.opened, self.steps, self.resets = [], [], []

    def clock(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-4)

    def footprint(self, cfg):
        return cfg.tdms

    def open(self, cfgs, ids):
        eng = self

        class Cohort:
            def __init__(self):
                self.ends, self.closed, self.ids = [], False, list(ids)

        c = Cohort()
        self.opened.append(c)
        return c

    def step(self, c, active):
        self.steps.append(active.copy())
        start = max(self.t, c.ends[-1] if c.ends else 0.0)
        c.ends.append(start + self.per_step + self.per_beam * int(active.sum()))
        return len(c.ends) - 1

    def done(self, c, i):
        return self.t >= c.ends[i]

    def reset_slot(self, c, slot, stream):
        self.resets.append((slot, c.ids[slot], stream))
        c.ids[slot] = stream
        return 0

    def close(self, c):
        c.closed = True


def _cfg(pv, tdms, tsamp=327.68e-6):
    return pv.beam_config(nsub=4, nchan_sub=16, fch1=140.0, foff=0.01, tsamp=tsamp, tdms=tdms, dm_step=0.1,
                          chunk=SUB, bp_text=None, rfi_active=0)


def _streams(n, rng, duration=2.0, tdms=10):
    cfgs, streams = [], []
    for i in range(n):
        arr = np.sort(rng.uniform(0, duration, size=rng.integers(1, 5)))
        sizes = [SUB * int(rng.integers(1, 4)) for _ in arr]
        cfgs.append(tdms)
        streams.append({"arrivals": arr, "sizes": sizes, "units_per_spectrum": 100})
    return cfgs, streams


def _serve(pv, tdms_list, streams, budget, **kw):
    eng = kw.pop("engine", None) or FakeEngine()
    rep = pv.serve([_cfg(pv, t) for t in tdms_list], streams, budget, engine=eng, **kw)
    return rep, eng


def test_every_chunk_is_served_and_counted(pv):
    rng = np.random.default_rng(1)
    tdms, streams = _streams(12, rng)
    rep, eng = _serve(pv, tdms, streams, 10 ** 9)
    assert rep["chunks_done"] == rep["chunks"] == sum(len(s["arrivals"]) for s in streams)
    subs = sum(sz // SUB for s in streams for sz in s["sizes"])
    assert rep["units"] == subs * SUB * 100
    assert all(c.closed for c in eng.opened)
    assert rep["latency_p99"] >= rep["latency_p50"] > 0
    assert rep["steps"] == len(eng.steps)


def test_admission_respects_the_budget_and_frees_memory(pv):
    rng = np.random.default_rng(2)
    tdms, streams = _streams(10, rng, tdms=30)
    rep, eng = _serve(pv, tdms, streams, 100, admit_every=0.0, reuse_slots=False)
    assert rep["peak_footprint_bytes"] <= 100
    assert rep["max_concurrent_beams"] <= 3
    assert rep["chunks_done"] == rep["chunks"]  # later beams were admitted as cohorts retired
    assert len(eng.opened) >= 4 and rep["cohorts"] == len(eng.opened)


def test_batching_takes_every_beam_with_queued_work(pv):
    streams = [{"arrivals": [0.0, 0.0, 0.0], "sizes": [SUB] * 3, "units_per_spectrum": 1} for _ in range(5)]
    rep, eng = _serve(pv, [1] * 5, streams, 10 ** 9, admit_every=0.0)
    # one cohort of 5 beams, each with 3 sub-chunks: three full steps
    assert len(eng.opened) == 1
    assert [int(a.sum()) for a in eng.steps] == [5, 5, 5]


def test_a_drained_streams_slot_goes_to_the_next_stream_of_its_configuration(pv):
    """The budget holds one beam.  Three streams of one configuration follow
    each other: the drained cohort lingers and each stream takes the previous
    one's slot (one cohort, no admission wait)."""
    streams = [{"arrivals": [0.1 + 1.0 * k, 0.2 + 1.0 * k], "sizes": [SUB, 2 * SUB], "units_per_spectrum": 1}
               for k in range(3)]
    rep, eng = _serve(pv, [10, 10, 10], streams, 10, admit_every=0.0, linger=5.0)
    assert rep["chunks_done"] == rep["chunks"] == 6
    assert rep["slot_reuses"] == 2 and [r[1:] for r in eng.resets] == [(0, 1), (1, 2)]
    assert rep["cohorts"] == 1 and rep["admission_wait_p99"] < 1e-3
    assert rep["peak_footprint_bytes"] <= 10


def test_a_waiting_stream_that_needs_the_memory_releases_a_drained_cohort(pv):
    """Another configuration arrives while the first stream's cohort lingers:
    the cohort is released at once and the new stream admitted."""
    streams = [{"arrivals": [0.1], "sizes": [SUB], "units_per_spectrum": 1},
               {"arrivals": [1.0], "sizes": [SUB], "units_per_spectrum": 1}]
    rep, eng = _serve(pv, [10, 7], streams, 10, admit_every=0.0, linger=100.0)
    assert rep["cohorts"] == 2 and rep["slot_reuses"] == 0 and eng.opened[0].closed
    assert rep["admission_wait_p99"] < 0.01


def test_different_configurations_do_not_share_slots(pv):
    streams = [{"arrivals": [0.1], "sizes": [SUB], "units_per_spectrum": 1},
               {"arrivals": [1.0], "sizes": [SUB], "units_per_spectrum": 1}]
    rep, eng = _serve(pv, [10, 11], streams, 100, admit_every=0.0)
    assert rep["slot_reuses"] == 0 and rep["cohorts"] == 2


def test_fifo_policy_serves_one_sub_chunk_at_a_time_oldest_first(pv):
    streams = [{"arrivals": [0.2], "sizes": [SUB], "units_per_spectrum": 1},
               {"arrivals": [0.1], "sizes": [2 * SUB], "units_per_spectrum": 1}]
    rep, eng = _serve(pv, [1, 1], streams, 10 ** 9, policy="fifo1", admit_every=0.0)
    assert all(int(a.sum()) == 1 for a in eng.steps)
    assert rep["chunks_done"] == 2 and len(eng.steps) == 3


def test_latency_is_arrival_to_the_step_that_finishes_the_chunk(pv):
    """One stream, one chunk of two sub-chunks arriving at 0.5 s, steps of
    0.012 s: the chunk completes two steps after its arrival."""
    streams = [{"arrivals": [0.5], "sizes": [2 * SUB], "units_per_spectrum": 1}]
    rep, eng = _serve(pv, [1], streams, 10 ** 9, admit_every=0.0, max_inflight=1)
    assert rep["latency_p50"] == pytest.approx(0.024, abs=2e-3)
    assert rep["latency_over_duration_p50"] == pytest.approx(rep["latency_p50"] / (2 * SUB * 327.68e-6))
    assert rep["within_real_time"] == 1.0


def test_sizes_must_be_whole_steps(pv):
    streams = [{"arrivals": [0.0], "sizes": [SUB + 1], "units_per_spectrum": 1}]
    with pytest.raises(pvmod.PvError, match="multiples of the chunk"):
        _serve(pv, [1], streams, 10 ** 9)


def test_poisson_streams_have_the_chunk_rate_of_real_time():
    beams = [{"cfg": None, "tsamp": 327.68e-6, "tdms": 1024, "nchan": 512} for _ in range(200)]
    st = serve.poisson_streams(beams, duration=600.0, seed=5)
    rates = []
    for s in st:
        life = s.arrivals[-1] - s.arrivals[0]
        if len(s.arrivals) > 20 and life > 0:
            rates.append((len(s.arrivals) - 1) / life * s.sizes[0] * 327.68e-6)
    assert abs(np.median(rates) - 1.0) < 0.15  # about one chunk per chunk duration
