"""The oracle pinned against the reference's own tests and golden values
(CPU only)."""
import numpy as np
import pytest

from gen import GEN_FCH1, GEN_FOFF, GEN_NCHAN, GEN_NSUB, GEN_TSAMP, dm_index, generator_pulse


def test_known_answer_dm10(oracle):
    # DedispersionModuleTest::test_method (lib/test/src/DedispersionModuleTest.cpp:346-406):
    # the generator pulse at DM 10, 200 trials of 0.1, gives dmAmplitude(0, 10.0)
    # == nSubbands*nChannels.
    blobs = generator_pulse(8192, 10.0)
    m = oracle.DedispersionModule(8192, 200, 0.0, 0.1, GEN_FCH1, GEN_FOFF)
    outs = m.add(blobs[0], GEN_TSAMP)
    assert len(outs) == 1
    data, first = outs[0]
    maxshift, remaining, nout, nchan, inverted = m.params()
    assert nchan == GEN_NSUB * GEN_NCHAN and not inverted
    assert data.shape == (200, 8192 - maxshift - remaining)
    assert first == 0
    assert data[dm_index(10.0, 0.0, 0.1), 0] == np.float32(GEN_NSUB * GEN_NCHAN)


def test_analyser_finds_more_events_than_trials(oracle):
    # DedispersionAnalyserTest::test_singleEvent (lib/test/src/DedispersionAnalyserTest.cpp:54-71)
    blobs = generator_pulse(8192, 10.0)
    m = oracle.DedispersionModule(8192, 200, 0.0, 0.1, GEN_FCH1, GEN_FOFF)
    data, _ = m.add(blobs[0], GEN_TSAMP)[0]
    rms = float(np.sqrt(np.float32(GEN_NCHAN) * np.float32(GEN_NSUB)))
    ev = oracle.analyse(data, 6.0, rms)
    assert len(ev) > 200
    assert tuple(ev[0]) == (0, 0, 1.0, 0.0)


def test_binmap(oracle):
    # BinMapTest::test_bin (lib/test/src/BinMapTest.cpp:41-61)
    start, width = 142.779541, 0.006104
    assert oracle.lib().or_binmap_index(start, width, start) == 0
    assert oracle.lib().or_binmap_index(start, width, start + width) == 1


def test_bandpass_rebin(oracle):
    # BandPassTest::test_reBin (lib/test/src/BandPassTest.cpp:35-70)
    L = oracle.lib()
    start, width = np.float32(137.304688), np.float32(-0.0007628)
    params = np.array([4460.84130843, -24.8135957376], np.float32)
    bp = L.or_bandpass_create(7936, float(start), float(width),
                              params.ctypes.data_as(oracle.C.POINTER(oracle.C.c_float)), 2)
    rms, median = np.float32(44.3413175435), np.float32(1128.9281113)
    L.or_bandpass_set_rms(bp, float(rms))
    L.or_bandpass_set_median(bp, float(median))
    kill_start, kill_end = np.float32(start + 3 * width), np.float32(start + 15 * width)
    L.or_bandpass_kill_band(bp, float(kill_start), float(kill_end))
    a = L.or_bandpass_intensity_of_bin(bp, 0)
    L.or_bandpass_rebin(bp, 7936 * 2, float(start), float(width) / 2.0)
    assert L.or_bandpass_intensity(bp, float(kill_start)) < 0.00001
    assert L.or_bandpass_intensity(bp, float(kill_end)) < 0.00001
    assert L.or_bandpass_intensity_of_bin(bp, 15 * 2) < 0.00001
    assert abs(median / 2.0 - L.or_bandpass_median(bp)) < 0.000001
    assert abs(rms * np.sqrt(2.0) - L.or_bandpass_rms(bp)) < 0.000001
    assert abs(a / 2.0 - L.or_bandpass_intensity_of_bin(bp, 0)) < 0.001
    L.or_bandpass_destroy(bp)


def test_dedispersion_spectra_dm_index():
    # DedispersionSpectraTest::test_dmIndex (lib/test/src/DedispersionSpectraTest.cpp:40-62)
    start, width, bins = 0.1, 0.2, 100
    mx = float(np.float32(np.float32(start) + np.float32(width) * np.float32(bins - 1)))
    assert dm_index(mx, start, width) == bins - 1


def test_dm_shift_table_formula(oracle):
    # DedispersionModule.cpp:153-157 restated in numpy (double, then float)
    n = 512
    fch1, foff = 146.0, -6.25 / n
    k, inv = oracle.dm_shifts(fch1, foff, n)
    f = fch1 + foff * np.arange(n)
    ref = (4148.741601 * ((1.0 / f / f) - (1.0 / fch1 / fch1))).astype(np.float32)
    assert not inv and np.array_equal(k, ref)
    # an ascending band is the same band read from the top
    k2, inv2 = oracle.dm_shifts(fch1 + foff * (n - 1), -foff, n)
    assert inv2 and np.allclose(k2, k, rtol=0, atol=1e-6)
    assert np.all(k2 >= 0)


def test_dedisperse_sequential_order(oracle):
    # The FP32 sum runs over channels in order (DedispersionKernel.cu:32-43).
    rng = np.random.default_rng(1)
    nchan, nout, tdms = 37, 50, 9
    k, _ = oracle.dm_shifts(150.0, -0.05, nchan)
    start, step = np.float32(0.0), np.float32(2.0)
    sh = oracle.shift_table(k, tdms, start, step)
    buf = (rng.standard_normal((nchan, nout + sh.max() + 4)) * 1000).astype(np.float32)
    out = oracle.dedisperse(buf, nout, tdms, k, start, step)
    for d in range(tdms):
        for t in range(0, nout, 7):
            acc = np.float32(0)
            for c in range(nchan):
                acc = np.float32(acc + buf[c, t + sh[d, c]])
            assert out[d, t] == acc


def test_shift_table_matches_float_formula(oracle):
    n, tdms = 64, 40
    k, _ = oracle.dm_shifts(150.0, -0.1, n)
    start, step = np.float32(0.3), np.float32(7.25)
    sh = oracle.shift_table(k, tdms, start, step)
    for d in range(tdms):
        dv = np.float32(np.float64(d) * np.float64(step) + np.float64(start))  # fmaf
        assert np.array_equal(sh[d], (k * dv).astype(np.float32).astype(np.int32))


def test_analyser_order_and_values(oracle):
    rng = np.random.default_rng(2)
    data = rng.standard_normal((5, 64 * 3 + 17)).astype(np.float32) * 3
    ev = oracle.analyse(data, 2.0, 1.0, 6)
    thr = oracle.thresholds(2.0, 1.0, 6)
    expect = [(0, 0, 1.0, 0.0)]
    for dm in range(5):
        for i in range(3):
            b = data[dm, i * 64:(i + 1) * 64].copy()
            for j in range(64):
                if b[j] >= thr[0]:
                    expect.append((dm, i * 64 + j, 1.0, b[j]))
            for n in range(1, 7):
                b = (b[0::2] + b[1::2]).astype(np.float32)
                for j in range(len(b)):
                    if b[j] >= thr[n]:
                        expect.append((dm, i * 64 + (1 << n) * j, float(1 << n), b[j]))
    assert [tuple(e) for e in ev] == [tuple(np.float32(x) if isinstance(x, float) else x for x in e)
                                      for e in expect]
