"""pv_analyse_noalloc: the analyser for callers that cannot allocate device
memory (a real-time pipeline running under a fixed HBM budget, or a host whose
device allocator belongs to another framework).

Its results must equal pv_analyse's on the same input, on consecutive calls
that reuse its fixed scratch array.  This file is collected last, so a failure
here stops a -x run only after every other test has run; it also passes when
run on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ARGS = [C.c_void_p, C.c_longlong, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, C.c_void_p,
        C.c_longlong, C.POINTER(C.c_longlong), C.c_void_p]


def _run(pv, fn, d_data, threshold, rms, bin_pow2, cap):
    import torch
    tdms, nsamp = d_data.shape
    ev = torch.zeros(cap * 4, dtype=torch.int32, device=d_data.device)
    n = C.c_longlong(-1)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ld = d_data.stride(0) if tdms > 0 else nsamp  # an empty tensor reports stride 0
    pv.check(fn(C.c_void_p(d_data.data_ptr()), ld, tdms, nsamp, threshold, rms,
                bin_pow2, C.c_void_p(ev.data_ptr()), cap, C.byref(n), stream))
    k = min(n.value, cap)
    return ev[: 4 * k].cpu().numpy().view(pv.EVENT_DTYPE).copy(), n.value


@pytest.mark.parametrize("tdms,nsamp,bin_pow2", [(200, 4096, 6), (37, 64 * 20 + 13, 3), (512, 2048, 8)])
def test_no_alloc_matches_pv_analyse_on_two_calls(pv, cuda, tdms, nsamp, bin_pow2):
    import torch
    L = pv.load()
    for name in ("pv_analyse", "pv_analyse_noalloc"):
        getattr(L, name).restype = C.c_int
        getattr(L, name).argtypes = ARGS
    rng = np.random.default_rng(tdms + nsamp)
    data = (rng.standard_normal((tdms, nsamp)) * 2.0).astype(np.float32)
    data[tdms // 3, 100:160] += 6.0
    d = torch.from_numpy(data).to(cuda)
    thr, rms, cap = 2.5, 1.0, 1 + tdms * nsamp * 2
    want, n_want = _run(pv, L.pv_analyse, d, thr, rms, bin_pow2, cap)
    assert n_want > 1
    for _ in range(2):  # the second call reuses the array the first one left behind
        got, n_got = _run(pv, L.pv_analyse_noalloc, d, thr, rms, bin_pow2, cap)
        assert n_got == n_want
        assert np.array_equal(got, want)


@pytest.mark.parametrize("tdms,nsamp,bin_pow2,cap", [(200, 4096, 6, 5), (8, 40, 6, 16), (0, 256, 6, 4),
                                                     (37, 64 * 20 + 13, 3, 1)])
def test_no_alloc_matches_pv_analyse_when_truncated_or_empty(pv, cuda, tdms, nsamp, bin_pow2, cap):
    """Fewer event slots than events (the total still counts them all), and
    calls with no (trial, block) pair (no trials, or fewer samples than one
    2^bin_pow2 block: only the dummy event)."""
    import torch
    L = pv.load()
    for name in ("pv_analyse", "pv_analyse_noalloc"):
        getattr(L, name).restype = C.c_int
        getattr(L, name).argtypes = ARGS
    rng = np.random.default_rng(tdms + nsamp + cap)
    data = (rng.standard_normal((tdms, nsamp)) * 2.0).astype(np.float32)
    d = torch.from_numpy(data).to(cuda)
    want, n_want = _run(pv, L.pv_analyse, d, 2.5, 1.0, bin_pow2, cap)
    if tdms == 0 or nsamp < (1 << bin_pow2):
        assert n_want == 1
    else:
        assert n_want > cap
    for _ in range(2):
        got, n_got = _run(pv, L.pv_analyse_noalloc, d, 2.5, 1.0, bin_pow2, cap)
        assert n_got == n_want
        assert np.array_equal(got, want)


def test_no_alloc_rejects_calls_beyond_its_limit(pv, cuda):
    import torch
    L = pv.load()
    L.pv_analyse_noalloc.restype = C.c_int
    L.pv_analyse_noalloc.argtypes = ARGS
    tdms, nsamp = 4096, 64 * 512  # 2^21 (trial, block) pairs > the 2^20 limit
    d = torch.zeros((tdms, nsamp), dtype=torch.float32, device=cuda)
    ev = torch.zeros(16, dtype=torch.int32, device=cuda)
    n = C.c_longlong(-1)
    rc = L.pv_analyse_noalloc(C.c_void_p(d.data_ptr()), nsamp, tdms, nsamp, 6.0, 1.0, 6,
                              C.c_void_p(ev.data_ptr()), 4, C.byref(n), C.c_void_p(0))
    assert rc == -1
    assert b"limit" in L.pv_last_error()
