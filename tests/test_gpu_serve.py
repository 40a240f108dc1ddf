"""The serving loop (pv_serve) on the GPU: every window a served stream
delivers equals the same stream run alone through pv_beam, in the mix of
cohorts, continuous batching and a drained stream's slot taken over by the
next stream of its configuration."""
import numpy as np
import pytest

from gen import make_bp_text, voltages

pytestmark = pytest.mark.gpu

CHUNK = 512


def _cfg(pv, nsub, tdms, dm_max):
    nch = 16
    foff = 0.1953125 / nch
    fch1 = 140.0 - (nch // 2) * foff
    bp = make_bp_text(nsub * nch, fch1, foff, 245.0, 245.0 / np.sqrt(8.0))
    return pv.beam_config(nsub=nsub, nchan_sub=nch, window="hamming", fch1=fch1, foff=foff,
                          tsamp=5.12e-6 * nch * 4, tdms=tdms, dm_step=dm_max / (tdms - 1), chunk=CHUNK,
                          threshold=4.0, bp_text=bp, cr=5.0, sr=4.0, history=1000, zero_dming=1, prefilled=1)


def test_served_streams_equal_each_stream_alone(pv, cuda):
    import torch
    a, b = _cfg(pv, 8, 64, 20.0), _cfg(pv, 12, 48, 10.0)
    cfgs = [a, b, a]
    rng = np.random.default_rng(77)
    hosts = []
    for c in cfgs:
        v16, _ = voltages(rng, c.nsub, 2, CHUNK * 4 * c.nchan_sub)
        hb = pv.HostBuffer(v16.nbytes)
        hb.fill_from(torch.from_numpy(v16.reshape(c.nsub, 2, -1)))
        hosts.append(hb)
    streams = [
        {"arrivals": [0.0, 0.05, 0.1, 0.15], "sizes": [CHUNK, 2 * CHUNK, CHUNK, 3 * CHUNK]},
        {"arrivals": [0.02, 0.3, 0.4], "sizes": [CHUNK, CHUNK, 2 * CHUNK]},
        {"arrivals": [1.5, 1.55], "sizes": [2 * CHUNK, 2 * CHUNK]},  # after stream 0 has drained
    ]
    for s, h, c in zip(streams, hosts, cfgs):
        s["voltages"] = h
        s["units_per_spectrum"] = c.tdms * c.nsub * c.nchan_sub
    foot = [pv.batch_footprint(c, True) for c in cfgs]
    budget = foot[0] + foot[1]  # no room for a second cohort of the first configuration
    got = {}

    def on_events(stream, first, ev, total):
        assert (stream, first) not in got
        got[(stream, first)] = (ev.copy(), total)

    rep = pv.serve(cfgs, streams, budget, admit_every=0.0, linger=10.0, on_events=on_events)
    assert rep["chunks_done"] == rep["chunks"] == 9
    assert rep["slot_reuses"] == 1 and rep["peak_footprint_bytes"] <= budget
    # each stream alone: one pv_beam per stream, its sub-chunks in order
    want = {}
    for i, (s, c) in enumerate(zip(streams, cfgs)):
        beam = pv.Beam(c)
        for size in s["sizes"]:
            for _ in range(size // CHUNK):
                beam.process_host(s["voltages"])
                ev, n, first = beam.events()
                if first >= 0:
                    want[(i, first)] = (ev, n)
    assert len(got) >= 6
    events = 0
    for key, (ev, total) in got.items():
        assert key in want, key
        w_ev, w_n = want[key]
        assert total == w_n and np.array_equal(ev, w_ev[:len(ev)])
        events += total - 1
    assert events > 0
    assert {k[0] for k in got} == {0, 1, 2}
