"""The serving loop's scheduling on the CPU, with a fake engine: admission
under the HBM budget, continuous batching of queued sub-chunks, release of
finished cohorts, and latency accounting (no GPU)."""
import numpy as np

import serve


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-4)


class FakeEngine:
    """A step takes `per_step` seconds of the fake clock plus `per_beam` per
    active beam; footprints come from the config dicts."""

    def __init__(self, clock, per_step=0.01, per_beam=0.002):
        self.clock, self.per_step, self.per_beam = clock, per_step, per_beam
        self.opened, self.steps = [], []

    def footprint(self, cfg):
        return cfg["bytes"]

    def open(self, cfgs, ids):
        eng = self

        class Cohort:
            def __init__(self):
                self.ends = []
                self.closed = False
                self.cfgs = cfgs

            def step(self, active):
                eng.steps.append(active.copy())
                start = max(eng.clock.t, self.ends[-1] if self.ends else 0.0)
                self.ends.append(start + eng.per_step + eng.per_beam * int(active.sum()))
                return len(self.ends) - 1

            def done(self, i):
                return eng.clock.t >= self.ends[i]

            def close(self):
                self.closed = True

        c = Cohort()
        self.opened.append(c)
        return c


def _streams(n, rng, duration=2.0, nbytes=10):
    out = []
    for i in range(n):
        arr = np.sort(rng.uniform(0, duration, size=rng.integers(1, 5)))
        sizes = [serve.SUB_CHUNK * int(rng.integers(1, 4)) for _ in arr]
        out.append(serve.Stream({"bytes": nbytes, "id": i}, arr, sizes, units_per_spectrum=100))
    return out


def test_every_chunk_is_served_and_counted():
    rng = np.random.default_rng(1)
    clock = FakeClock()
    streams = _streams(12, rng)
    eng = FakeEngine(clock)
    rep = serve.Server(eng, streams, budget=10**9).run(clock=clock, sleep=clock.sleep)
    assert rep["chunks_done"] == rep["chunks"] == sum(len(s.arrivals) for s in streams)
    subs = sum(sz // serve.SUB_CHUNK for s in streams for sz in s.sizes)
    assert rep["units"] == subs * serve.SUB_CHUNK * 100
    assert all(c.closed for c in eng.opened)
    assert rep["latency_s"]["p99"] >= rep["latency_s"]["p50"] > 0


def test_admission_respects_the_budget_and_frees_memory():
    rng = np.random.default_rng(2)
    clock = FakeClock()
    streams = _streams(10, rng, nbytes=30)
    eng = FakeEngine(clock)
    rep = serve.Server(eng, streams, budget=100, admit_every=0.0).run(clock=clock, sleep=clock.sleep)
    assert rep["peak_footprint_gb"] * 1e9 <= 100
    assert rep["max_concurrent_beams"] <= 3
    assert rep["chunks_done"] == rep["chunks"]  # later beams were admitted as cohorts retired
    assert len(eng.opened) >= 4


def test_batching_takes_every_beam_with_queued_work():
    rng = np.random.default_rng(3)
    clock = FakeClock()
    streams = [serve.Stream({"bytes": 1}, [0.0, 0.0, 0.0], [serve.SUB_CHUNK] * 3, 1) for _ in range(5)]
    eng = FakeEngine(clock)
    serve.Server(eng, streams, budget=10**9, admit_every=0.0).run(clock=clock, sleep=clock.sleep)
    # one cohort of 5 beams, each with 3 sub-chunks: three full steps
    assert len(eng.opened) == 1
    assert [int(a.sum()) for a in eng.steps] == [5, 5, 5]


def test_fifo_policy_serves_one_sub_chunk_at_a_time_oldest_first():
    clock = FakeClock()
    streams = [serve.Stream({"bytes": 1}, [0.2], [serve.SUB_CHUNK], 1),
               serve.Stream({"bytes": 1}, [0.1], [2 * serve.SUB_CHUNK], 1)]
    eng = FakeEngine(clock)
    rep = serve.Server(eng, streams, budget=10**9, policy="fifo1", admit_every=0.0).run(
        clock=clock, sleep=clock.sleep)
    assert all(int(a.sum()) == 1 for a in eng.steps)
    assert rep["chunks_done"] == 2
    order = [int(np.flatnonzero(a)[0]) for a in eng.steps]
    assert len(order) == 3


def test_poisson_streams_have_the_chunk_rate_of_real_time():
    beams = [{"cfg": None, "tsamp": 327.68e-6, "tdms": 1024, "nchan": 512} for _ in range(200)]
    st = serve.poisson_streams(beams, duration=600.0, seed=5)
    rates = []
    for s in st:
        life = s.arrivals[-1] - s.arrivals[0]
        if len(s.arrivals) > 20 and life > 0:
            rates.append((len(s.arrivals) - 1) / life * s.sizes[0] * 327.68e-6)
    assert abs(np.median(rates) - 1.0) < 0.15  # about one chunk per chunk duration
