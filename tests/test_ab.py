"""ALFABURST spectrometer ingest (ABDataAdapter, lib/src/ABDataAdapter.cpp:14-173):
the header pass on the host and the spectra on the GPU against the oracle's
packet-by-packet restatement, pinned by the reference emulator's known answer
(lib/test/src/ABEmulator.cpp:49-98)."""
import numpy as np
import pytest

from gen import ab_emulator_packets

NCH = 16
PSIZE = 8 + 8 * NCH


def _state():
    return {"seen": 0, "count0": 0, "last_time": 0.0}


def test_emulator_packets_decode_to_the_known_answer(oracle):
    """The emulator writes 42, 43, 44, 45 in host (little-endian) order and the
    adapter swaps them as network order: XX + YY = 0x2A00 + 0x2B00 = 21760."""
    pk = ab_emulator_packets(64, NCH, counter0=1000)
    spec, t, gaps, n = oracle.ab_deserialise(pk, 4, NCH, 0, 0.000128, _state())
    assert spec.shape == (16, NCH) and n == 16 and gaps == 0
    assert np.all(spec == 21760.0)
    assert t == 15 * float(np.float32(0.000128))  # timed from the first packet's count


CASES = [
    dict(quarter0=0, skip=(), samples=0),
    dict(quarter0=2, skip=(), samples=0),       # chunks not aligned to a spectrum
    dict(quarter0=0, skip=(9,) + tuple(range(30, 38)), samples=0),  # lost packets: a gap, missing spectra
    dict(quarter0=1, skip=(), samples=2),       # <packet samples> sizes the blob only
]


def _chunks(rng, case, nchunks=3, npk=40):
    pk = ab_emulator_packets(nchunks * npk + len(case["skip"]), NCH, counter0=77, quarter0=case["quarter0"],
                             records=rng.integers(0, 65536, (nchunks * npk + len(case["skip"]), NCH, 4)),
                             skip=case["skip"])
    return [pk[k * npk * PSIZE:(k + 1) * npk * PSIZE] for k in range(nchunks)]


@pytest.mark.parametrize("case", CASES)
def test_header_pass_equals_the_oracle(pv, oracle, case):
    import ctypes as C
    rng = np.random.default_rng(len(case["skip"]) + 10 * case["quarter0"])
    cfg = pv.AbConfig(4, NCH, case["samples"], 0.000128)
    st, ost = pv.AbState(), _state()
    total_gaps = 0
    for chunk in _chunks(rng, case):
        want, t, gaps, n = oracle.ab_deserialise(chunk, 4, NCH, case["samples"], 0.000128, ost)
        total_gaps += gaps
        idx = np.zeros(64, np.int32)
        nsp, nbl, ts, g = C.c_longlong(0), C.c_longlong(0), C.c_double(0), C.c_longlong(0)
        pv.check(pv.load().pv_ab_headers(C.byref(cfg), C.byref(st), chunk.ctypes.data, len(chunk),
                                         idx.ctypes.data, len(idx), C.byref(nsp), C.byref(nbl), C.byref(ts),
                                         C.byref(g)))
        assert (nsp.value, nbl.value, ts.value, g.value) == (n, len(want), t, gaps)
        assert np.all(np.frombuffer(chunk, np.uint8).reshape(-1, PSIZE)[idx[:n], 6] == 1)
    assert st.seen == ost["seen"] and st.count0 == ost["count0"]
    assert total_gaps == (1 if case["skip"] else 0)  # 8 packets lost: two counts apart


def test_header_pass_rejects_a_short_index(pv):
    import ctypes as C
    cfg = pv.AbConfig(4, NCH, 0, 0.000128)
    pk = ab_emulator_packets(16, NCH)
    idx = np.zeros(2, np.int32)
    nsp, nbl, ts, g = C.c_longlong(0), C.c_longlong(0), C.c_double(0), C.c_longlong(0)
    rc = pv.load().pv_ab_headers(C.byref(cfg), C.byref(pv.AbState()), pk.ctypes.data, len(pk), idx.ctypes.data,
                                 len(idx), C.byref(nsp), C.byref(nbl), C.byref(ts), C.byref(g))
    assert rc < 0 and b"index capacity" in pv.load().pv_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_gpu_spectra_equal_the_oracle(pv, oracle, cuda, case):
    rng = np.random.default_rng(5 + len(case["skip"]))
    ad = pv.ABDataAdapter(packets=4, channels=NCH, samples=case["samples"], seconds=0.000128)
    ost = _state()
    for chunk in _chunks(rng, case):
        got = ad.deserialise(chunk).cpu().numpy()
        want, t, gaps, n = oracle.ab_deserialise(chunk, 4, NCH, case["samples"], 0.000128, ost)
        assert got.shape == (len(want), 1, 1, NCH)
        assert np.array_equal(got.reshape(want.shape), want)
        assert (ad.timestamp, ad.gaps) == (t, gaps)


@pytest.mark.gpu
def test_gpu_emulator_packets_decode_to_the_known_answer(pv, cuda):
    ad = pv.ABDataAdapter(packets=4, channels=1024, seconds=0.000128)
    got = ad.deserialise(ab_emulator_packets(1024, 1024)).cpu().numpy()  # the reference XML's chunk
    assert got.shape == (256, 1, 1, 1024) and np.all(got == 21760.0)


@pytest.mark.parametrize("pps,tail", [(2, 0), (1, 0), (4, 100), (5, 7)])
def test_header_pass_edge_cases_equal_the_oracle(pv, oracle, pps, tail):
    """Fewer than 3 packets per spectrum (the quarter to keep, pps - 3, wraps
    as an unsigned number, so no packet fills a spectrum) and chunks ending in
    part of a packet (ignored)."""
    import ctypes as C
    rng = np.random.default_rng(pps * 100 + tail)
    pk = ab_emulator_packets(24, NCH, counter0=3, records=rng.integers(0, 65536, (24, NCH, 4)))
    chunk = np.concatenate([pk, rng.integers(0, 256, tail).astype(np.uint8)])
    want, t, gaps, n = oracle.ab_deserialise(chunk, pps, NCH, 0, 0.001, _state())
    cfg = pv.AbConfig(pps, NCH, 0, 0.001)
    idx = np.zeros(32, np.int32)
    nsp, nbl, ts, g = C.c_longlong(0), C.c_longlong(0), C.c_double(0), C.c_longlong(0)
    pv.check(pv.load().pv_ab_headers(C.byref(cfg), C.byref(pv.AbState()), chunk.ctypes.data, len(chunk),
                                     idx.ctypes.data, len(idx), C.byref(nsp), C.byref(nbl), C.byref(ts),
                                     C.byref(g)))
    assert (nsp.value, nbl.value, ts.value, g.value) == (n, len(want), t, gaps)
    assert nbl.value == 24 // pps
    if pps < 3:
        assert n == 0
