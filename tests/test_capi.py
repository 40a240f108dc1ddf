"""The C ABI library loads and exports every symbol include/*.h declares
(no compute calls; runs without a GPU)."""
import ctypes as C
import glob
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"\b(pv_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(pv):
    lib = C.CDLL(pv.LIB_PATH)
    names = _declared()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_host_functions_match_oracle(pv, oracle):
    # Host-side parts of the boundary (no device needed).
    for fch1, foff, n in [(150.0, -6.0 / 2048, 2048), (140.0, 0.01220703125, 512),
                          (110.0, 195.3125e-3 / 16, 3904)]:
        a, inv_a = pv.dm_shifts(fch1, foff, n)
        b, inv_b = oracle.dm_shifts(fch1, foff, n)
        assert inv_a == inv_b and np.array_equal(a, b)
        for tdms, lo, step, tsamp, B in [(512, 0.0, 100.0 / 511, 327.68e-6, 8192),
                                         (200, 0.0, 0.1, 327.68e-6, 8192)]:
            try:
                got = pv.maxshift(lo, step, tdms, a, tsamp, B)
            except pv.PvError:
                got = None
            want = oracle.maxshift(lo, step, tdms, b, tsamp, B)
            if got is not None:
                assert got == want
            else:
                assert want[0] >= B
    for thr, rms, p in [(6.0, 22.627417, 6), (6.0, 62.48, 8), (5.5, 45.254833, 3)]:
        assert np.array_equal(pv.thresholds(thr, rms, p), oracle.thresholds(thr, rms, p))


def test_errors_are_reported_not_thrown(pv):
    L = pv.load()
    out = np.zeros(4, np.float32)
    inv = C.c_int()
    rc = L.pv_dm_shifts(0.0, -1.0, 4, out.ctypes.data_as(C.POINTER(C.c_float)), C.byref(inv))
    assert rc == -3
    assert b"frequencyChannel1" in L.pv_last_error()


def test_rfi_config_errors(pv):
    """Configuration errors surface as status codes with the reference's text."""
    import pytest
    with pytest.raises(pv.PvError, match="BandPassData"):
        pv.RFI("", cr=5.0)
    with pytest.raises(pv.PvError, match="at least 6"):
        pv.RFI("1\n2\n3\n")
    inactive = pv.RFI("", active=False)
    assert inactive is not None
