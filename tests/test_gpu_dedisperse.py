"""K0 delay table, K4 dedispersion and K5 analyser on the GPU against the
oracle, through the C ABI."""
import numpy as np
import pytest

from gen import GEN_FCH1, GEN_FOFF, GEN_NCHAN, GEN_NSUB, GEN_TSAMP, dm_index, generator_pulse

pytestmark = pytest.mark.gpu

# (fch1, foff, nchan, tdms, dm_low, dm_step, tsamp)
DELAY_CASES = [
    (150.0, -6.0 / 2048, 2048, 200, 0.0, 0.1, GEN_TSAMP),               # reference test fixture
    (146.25, 0.01220703125, 512, 512, 0.0, 100.0 / 511, 327.68e-6),      # 32 subbands from 140 MHz
    (110.0, 0.0122070312, 3904, 2048, 0.0, 500.0 / 2047, 327.68e-6),     # 244 subbands from 110 MHz
    (150.0, -0.05, 97, 37, 1.5, 0.37, 1e-3),                              # ragged, dmLow > 0
]


@pytest.mark.parametrize("case", DELAY_CASES)
def test_delay_table_bit_exact(pv, oracle, cuda, case):
    import torch
    fch1, foff, n, tdms, lo, step, tsamp = case
    k, _ = pv.dm_shifts(fch1, foff, n)
    start = np.float32(np.float32(lo) / np.float32(tsamp))
    stp = np.float32(np.float32(step) / np.float32(tsamp))
    got = pv.delay_table(torch.from_numpy(k).to(cuda), tdms, float(start), float(stp)).cpu().numpy()
    want = oracle.shift_table(k, tdms, start, stp)
    assert np.array_equal(got, want)
    # FP64 delay table: report how many entries differ (documented deviation)
    f64 = oracle.shift_table_f64(fch1, foff, n, tdms, lo, step, tsamp)
    frac = np.mean(f64 != want)
    assert frac < 0.05


def _shift_bounds(oracle, k, tdms, start, step):
    return int(oracle.shift_table(k, tdms, start, step).max())


# (nchan, nout, tdms, fch1, foff, dm_step, tsamp)
DD_CASES = [
    (64, 300, 40, 150.0, -0.1, 0.5, 327.68e-6),
    (512, 1024, 512, 146.25, -0.01220703125, 100.0 / 511, 327.68e-6),
    (97, 777, 37, 150.0, -0.05, 0.37, 1e-3),
    (3904, 256, 48, 157.6, -0.0122070312, 500.0 / 2047, 327.68e-6),
    (16, 64, 1, 150.0, -1.0, 1.0, 1e-3),
]


@pytest.mark.parametrize("case", DD_CASES)
def test_dedisperse_bit_exact(pv, oracle, cuda, case):
    import torch
    nchan, nout, tdms, fch1, foff, step, tsamp = case
    rng = np.random.default_rng(nchan + tdms)
    k, _ = pv.dm_shifts(fch1, foff, nchan)
    start = np.float32(0.0)
    stp = np.float32(np.float32(step) / np.float32(tsamp))
    ms = _shift_bounds(oracle, k, tdms, start, stp)
    buf = (rng.standard_normal((nchan, nout + ms + 3)) * 4).astype(np.float32)
    want = oracle.dedisperse(buf, nout, tdms, k, start, stp)
    d_buf = torch.from_numpy(buf).to(cuda)
    got = pv.dedisperse(d_buf, nout, tdms, torch.from_numpy(k).to(cuda), float(start), float(stp))
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), want)
    f64 = oracle.dedisperse(buf, nout, tdms, k, start, stp, f64=True)
    scale = np.sqrt(nchan) * 4
    assert np.max(np.abs(got.cpu().numpy() - f64)) / scale < 1e-5


def test_reference_entry_point_known_answer(pv, oracle, cuda):
    """cacheDedisperseLoop-shaped call on the DedispersionModuleTest fixture:
    dmAmplitude(0, 10.0) == nSubbands*nChannels."""
    import torch
    B = 8192
    blob = generator_pulse(B, 10.0)[0]
    n = GEN_NSUB * GEN_NCHAN
    k, inv = pv.dm_shifts(GEN_FCH1, GEN_FOFF, n)
    ms, rem = pv.maxshift(0.0, 0.1, 200, k, GEN_TSAMP, B)
    buf = np.ascontiguousarray(blob[:, :, 0, :].reshape(B, n).T)  # [chan][t]
    start = np.float32(0.0) / np.float32(GEN_TSAMP)
    stp = np.float32(0.1) / np.float32(GEN_TSAMP)
    nout = B - ms - rem
    out = torch.zeros((200, nout), dtype=torch.float32, device=cuda)
    pv.dedisperse_ref_api(out, torch.from_numpy(buf).to(cuda), float(start), float(stp), 200, B,
                          torch.from_numpy(k).to(cuda), ms + rem, n)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert got[dm_index(10.0, 0.0, 0.1), 0] == np.float32(n)
    m = oracle.DedispersionModule(B, 200, 0.0, 0.1, GEN_FCH1, GEN_FOFF)
    want, _ = m.add(blob, GEN_TSAMP)[0]
    assert np.array_equal(got, want)


@pytest.mark.parametrize("bin_pow2", [6, 3, 0, 8])
def test_analyser_bit_exact(pv, oracle, cuda, bin_pow2):
    import torch
    rng = np.random.default_rng(bin_pow2)
    tdms, nsamp = 33, 64 * 20 + 13
    data = rng.standard_normal((tdms, nsamp)).astype(np.float32) * 3.0
    data[5, 100:120] += 6
    thr, rms = 2.5, 1.0
    want = oracle.analyse(data, thr, rms, bin_pow2)
    got, n = pv.analyse(torch.from_numpy(data).to(cuda), thr, rms, bin_pow2)
    assert n == len(want)
    assert np.array_equal(got, want.astype(got.dtype))


def test_analyser_known_answer_and_empty(pv, oracle, cuda):
    import torch
    B = 8192
    blob = generator_pulse(B, 10.0)[0]
    m = oracle.DedispersionModule(B, 200, 0.0, 0.1, GEN_FCH1, GEN_FOFF)
    data, _ = m.add(blob, GEN_TSAMP)[0]
    rms = float(np.sqrt(np.float32(GEN_NCHAN) * np.float32(GEN_NSUB)))
    got, n = pv.analyse(torch.from_numpy(data).to(cuda), 6.0, rms)
    want = oracle.analyse(data, 6.0, rms)
    assert n > 200 and np.array_equal(got, want.astype(got.dtype))
    # empty and shorter-than-a-block inputs give only the dummy event
    for shape in [(0, 0), (4, 63)]:
        got, n = pv.analyse(torch.zeros(shape, dtype=torch.float32, device=cuda), 6.0, rms)
        assert n == 1 and tuple(got[0]) == (0, 0, 1.0, 0.0)


def test_analyser_capacity_truncates(pv, oracle, cuda):
    import torch
    data = np.full((2, 128), 10.0, np.float32)
    want = oracle.analyse(data, 1.0, 1.0, 6)
    got, n = pv.analyse(torch.from_numpy(data).to(cuda), 1.0, 1.0, 6, cap=50)
    assert n == len(want) and len(got) == 50
    assert np.array_equal(got, want[:50].astype(got.dtype))


def test_ring_write_transposes_and_wraps(pv, cuda):
    import ctypes as C
    import torch
    L = pv.load()
    L.pv_ring_write.argtypes = [C.c_void_p, C.c_longlong, C.c_longlong, C.c_longlong, C.c_void_p,
                                C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    rng = np.random.default_rng(3)
    nt, nsub, npol, nchan = 70, 5, 2, 8
    nbins = nsub * nchan
    stokes = rng.standard_normal((nt, nsub, npol, nchan)).astype(np.float32)
    ring_len, stride, pos = 100, 104, 61
    for inverted in (0, 1):
        ring = torch.full((nbins, stride), -7.0, device=cuda)
        pv.check(L.pv_ring_write(C.c_void_p(ring.data_ptr()), stride, ring_len, pos,
                                 C.c_void_p(torch.from_numpy(stokes).to(cuda).data_ptr()), nt, nsub,
                                 npol, nchan, inverted, C.c_void_p(0)))
        torch.cuda.synchronize()
        got = ring.cpu().numpy()
        want = np.full((nbins, stride), -7.0, np.float32)
        bins = stokes[:, :, 0, :].reshape(nt, nbins)
        if inverted:
            bins = bins[:, ::-1]
        for t in range(nt):
            want[:, (pos + t) % ring_len] = bins[t]
        assert np.array_equal(got, want)


def test_ring_mode_equals_linear(pv, oracle, cuda):
    import ctypes as C
    import torch
    L = pv.load()
    L.pv_dedisp_plan_create.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_float), C.c_int,
                                        C.c_int, C.c_float, C.c_float]
    L.pv_dedisp_plan_run.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p,
                                     C.c_longlong, C.c_longlong, C.c_longlong, C.c_longlong,
                                     C.c_int, C.c_void_p]
    L.pv_dedisp_plan_max_shift.argtypes = [C.c_void_p]
    rng = np.random.default_rng(4)
    nchan, nout, tdms = 300, 1000, 70
    k, _ = pv.dm_shifts(150.0, -0.03, nchan)
    start, step = np.float32(0.0), np.float32(3.7)
    plan = C.c_void_p()
    pv.check(L.pv_dedisp_plan_create(C.byref(plan), k.ctypes.data_as(C.POINTER(C.c_float)), nchan,
                                     tdms, float(start), float(step)))
    ms = L.pv_dedisp_plan_max_shift(plan)
    assert ms == oracle.shift_table(k, tdms, start, step).max()
    ring_len = nout + ms
    lin = rng.standard_normal((nchan, ring_len)).astype(np.float32)
    want = oracle.dedisperse(np.concatenate([lin, np.zeros((nchan, 4), np.float32)], 1), nout, tdms,
                             k, start, step)
    for t_base in (0, 1, ring_len // 2, ring_len - 1):
        stride = ring_len + 5
        ring = np.zeros((nchan, stride), np.float32)
        for t in range(ring_len):
            ring[:, (t_base + t) % ring_len] = lin[:, t]
        d_ring = torch.from_numpy(ring).to(cuda)
        out = torch.empty((tdms, nout), device=cuda)
        pv.check(L.pv_dedisp_plan_run(plan, C.c_void_p(out.data_ptr()), nout,
                                      C.c_void_p(d_ring.data_ptr()), stride, 0, ring_len, t_base,
                                      nout, C.c_void_p(0)))
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), want)
    L.pv_dedisp_plan_destroy(plan)


@pytest.mark.parametrize("nchan,nout,tdms", [(301, 2500, 37), (64, 100, 16), (1000, 4096, 48)])
def test_ring_pipeline_kernel_bit_exact(pv, oracle, cuda, nchan, nout, tdms):
    """Ring rows aligned to 16 bytes take the TMA/mbarrier pipeline: bit-exact
    against the oracle for every ring rotation, ragged channel stages, partial
    trial and time tiles, and identical to the cp.async kernel."""
    import ctypes as C
    import os
    import torch
    L = pv.load()
    rng = np.random.default_rng(nchan + nout)
    k, _ = pv.dm_shifts(150.0, -0.02, nchan)
    start, step = np.float32(0.0), np.float32(2.3)
    plan = C.c_void_p()
    pv.check(L.pv_dedisp_plan_create(C.byref(plan), k.ctypes.data_as(C.POINTER(C.c_float)), nchan,
                                     tdms, float(start), float(step)))
    ms = L.pv_dedisp_plan_max_shift(plan)
    ring_len = (nout + ms + 8 + 3) // 4 * 4
    lin = rng.standard_normal((nchan, ring_len)).astype(np.float32)
    want = oracle.dedisperse(np.concatenate([lin, np.zeros((nchan, 4), np.float32)], 1), nout, tdms,
                             k, start, step)
    stride = ring_len + 4
    for t_base in (0, 4, ring_len // 2 + 1, ring_len - 3):
        ring = np.zeros((nchan, stride), np.float32)
        for t in range(ring_len):
            ring[:, (t_base + t) % ring_len] = lin[:, t]
        d_ring = torch.from_numpy(ring).to(cuda)
        outs = []
        for v1 in (False, True):
            if v1:
                os.environ["PV_DEDISP_V1"] = "1"
            try:
                out = torch.full((tdms, nout), float("nan"), device=cuda)
                pv.check(L.pv_dedisp_plan_run(plan, C.c_void_p(out.data_ptr()), nout,
                                              C.c_void_p(d_ring.data_ptr()), stride, 0, ring_len,
                                              t_base, nout, C.c_void_p(0)))
                torch.cuda.synchronize()
                outs.append(out.cpu().numpy())
            finally:
                os.environ.pop("PV_DEDISP_V1", None)
        assert np.array_equal(outs[0], want)
        assert np.array_equal(outs[1], want)
    status = C.c_int(-99)
    L.pv_dedisp_plan_status.argtypes = [C.c_void_p, C.POINTER(C.c_int)]
    pv.check(L.pv_dedisp_plan_status(plan, C.byref(status)))
    assert status.value == 0
    L.pv_dedisp_plan_destroy(plan)
