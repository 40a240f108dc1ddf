"""Streams for the serving loop.

The loop itself is ``pv_serve`` in the library (C++, ``csrc/serve.cu``;
Python entry ``pv.serve``): admission under an HBM budget, continuous
batching of queued sub-chunks, a drained stream's slot given to the next
stream of its configuration, release of drained cohorts and latency
accounting.  This module describes the streams it serves: one beam each, a
``pv_beam_config`` with the arrival times and sizes (spectra) of its chunks,
and draws Poisson streams at one chunk per chunk duration.
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
