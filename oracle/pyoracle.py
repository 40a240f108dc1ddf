"""ctypes binding of the CPU oracle (test infrastructure only).

Loaded by the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py``.  The product library never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

EVENT_DTYPE = np.dtype([("dm", "<i4"), ("t", "<i4"), ("bin_factor", "<f4"), ("value", "<f4")])

_lib = None


def build(force=False):
    """Compile the oracle with its Makefile (g++, OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or (
        os.path.getmtime(LIB_PATH) < max(os.path.getmtime(os.path.join(HERE, f))
                                         for f in ("oracle.cpp", "oracle.h"))):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def _f32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _f64p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i32p(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, i, f, d, ll = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_longlong
        P = C.POINTER
        sigs = {
            "or_dm_shifts": (i, [d, d, i, P(C.c_float)]),
            "or_maxshift": (None, [f, f, i, P(C.c_float), i, d, i, P(i), P(i)]),
            "or_shift_table": (None, [P(C.c_float), i, i, f, f, P(i)]),
            "or_shift_table_f64": (None, [d, d, i, i, d, d, d, P(i)]),
            "or_dedisperse": (None, [P(C.c_float), i, ll, i, i, P(C.c_float), f, f, P(C.c_float), i]),
            "or_dedisperse_f64": (None, [P(C.c_float), i, ll, i, i, P(C.c_float), f, f, P(C.c_double), i]),
            "or_thresholds": (None, [f, f, i, P(C.c_float)]),
            "or_analyse": (ll, [P(C.c_float), i, i, f, f, i, vp, ll]),
            "or_fir_coefficients": (i, [i, i, i, P(C.c_double)]),
            "or_ppf_create": (vp, [i, i, P(C.c_float)]),
            "or_ppf_destroy": (None, [vp]),
            "or_ppf_run": (i, [vp, P(C.c_float), i, i, i, P(C.c_float)]),
            "or_stokes": (None, [P(C.c_float), i, i, i, i, P(C.c_float)]),
            "or_integrate": (i, [P(C.c_float), i, i, i, i, i, i, P(C.c_float)]),
            "or_rfi_create": (vp, [C.c_char_p, f, f, i, i, i, i, i, i, C.c_char_p, i]),
            "or_rfi_destroy": (None, [vp]),
            "or_rfi_run": (i, [vp, P(C.c_float), P(C.c_float), i, i, i, i, vp]),
            "or_rfi_state": (None, [vp, P(C.c_double)]),
            "or_rfi_bandpass": (i, [vp, P(C.c_float), i]),
            "or_sum_canonical": (d, [P(C.c_float), i, i]),
            "or_bandpass_create": (vp, [i, d, d, P(C.c_float), i]),
            "or_bandpass_destroy": (None, [vp]),
            "or_bandpass_set_rms": (None, [vp, f]),
            "or_bandpass_set_median": (None, [vp, f]),
            "or_bandpass_set_mean": (None, [vp, f]),
            "or_bandpass_kill_band": (None, [vp, f, f]),
            "or_bandpass_rebin": (None, [vp, i, d, d]),
            "or_bandpass_intensity": (f, [vp, f]),
            "or_bandpass_intensity_of_bin": (f, [vp, i]),
            "or_bandpass_median": (f, [vp]),
            "or_bandpass_rms": (f, [vp]),
            "or_bandpass_mean": (f, [vp]),
            "or_binmap_index": (i, [d, d, d]),
            "or_ddmod_create": (vp, [i, i, f, f, d, d]),
            "or_ddmod_destroy": (None, [vp]),
            "or_ddmod_add": (i, [vp, P(C.c_float), i, i, i, i, d]),
            "or_ddmod_pop": (i, [vp, P(C.c_float), ll, P(ll)]),
            "or_ddmod_params": (None, [vp, P(i), P(i), P(i), P(i), P(i)]),
            "or_num_threads": (i, []),
            "or_udp_check": (i, [i, i, i, i, i, i, i, ll, P(ll), P(i)]),
            "or_udp_unpack": (i, [vp, ll, i, i, i, i, i, P(C.c_float)]),
            "or_udp_time": (None, [vp, i, P(C.c_double), P(C.c_double)]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


# --------------------------------------------------------------------------
# numpy-level helpers
# --------------------------------------------------------------------------

def dm_shifts(fch1, foff, nchan):
    out = np.zeros(nchan, np.float32)
    inv = lib().or_dm_shifts(fch1, foff, nchan, _f32p(out))
    return out, bool(inv)


def maxshift(dm_low, dm_step, tdms, dmshift, tsamp, buffer_samples):
    ms, rem = C.c_int(), C.c_int()
    lib().or_maxshift(dm_low, dm_step, tdms, _f32p(dmshift), len(dmshift), tsamp,
                      buffer_samples, C.byref(ms), C.byref(rem))
    return ms.value, rem.value


def shift_table(dmshift, tdms, start_over_tsamp, step_over_tsamp):
    out = np.zeros((tdms, len(dmshift)), np.int32)
    lib().or_shift_table(_f32p(dmshift), len(dmshift), tdms, start_over_tsamp,
                         step_over_tsamp, _i32p(out))
    return out


def shift_table_f64(fch1, foff, nchan, tdms, dm_low, dm_step, tsamp):
    out = np.zeros((tdms, nchan), np.int32)
    lib().or_shift_table_f64(fch1, foff, nchan, tdms, dm_low, dm_step, tsamp, _i32p(out))
    return out


def dedisperse(buf, nout, tdms, dmshift, start_over_tsamp, step_over_tsamp, nthreads=0,
               f64=False):
    buf = np.ascontiguousarray(buf, np.float32)
    nchan, ld = buf.shape
    if f64:
        out = np.zeros((tdms, nout), np.float64)
        lib().or_dedisperse_f64(_f32p(buf), nchan, ld, nout, tdms, _f32p(dmshift),
                                start_over_tsamp, step_over_tsamp, _f64p(out), nthreads)
    else:
        out = np.zeros((tdms, nout), np.float32)
        lib().or_dedisperse(_f32p(buf), nchan, ld, nout, tdms, _f32p(dmshift),
                            start_over_tsamp, step_over_tsamp, _f32p(out), nthreads)
    return out


def thresholds(thr, rms, bin_pow2):
    out = np.zeros(bin_pow2 + 1, np.float32)
    lib().or_thresholds(thr, rms, bin_pow2, _f32p(out))
    return out


def analyse(data, thr, rms, bin_pow2=6):
    data = np.ascontiguousarray(data, np.float32)
    tdms, nsamp = data.shape
    n = lib().or_analyse(_f32p(data), tdms, nsamp, thr, rms, bin_pow2, None, 0)
    ev = np.zeros(n, EVENT_DTYPE)
    lib().or_analyse(_f32p(data), tdms, nsamp, thr, rms, bin_pow2, ev.ctypes.data, n)
    return ev


def fir_coefficients(ntaps, nchan, window="kaiser"):
    w = {"hamming": 0, "blackman": 1, "gaussian": 2, "kaiser": 3}[window]
    out = np.zeros((ntaps, nchan), np.float64)
    if lib().or_fir_coefficients(ntaps, nchan, w, _f64p(out)) != 0:
        raise ValueError("bad coefficient shape")
    return out


class PPF:
    def __init__(self, nchan, ntaps, coeffs):
        self._c = np.ascontiguousarray(coeffs, np.float32)
        self.nchan, self.ntaps = nchan, ntaps
        self.h = lib().or_ppf_create(nchan, ntaps, _f32p(self._c))

    def run(self, x):
        """x: complex64 [sub][pol][block][nchan] -> complex64 [block][sub][pol][nchan]."""
        x = np.ascontiguousarray(x, np.complex64)
        nsub, npol, nblk, nch = x.shape
        assert nch == self.nchan
        out = np.zeros((nblk, nsub, npol, nch), np.complex64)
        rc = lib().or_ppf_run(self.h, x.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)),
                              nsub, npol, nblk,
                              out.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)))
        if rc != 0:
            raise RuntimeError("or_ppf_run failed")
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_ppf_destroy(self.h)
            self.h = None


def stokes(spectra, nstokes=1):
    """spectra complex64 [t][sub][2][nchan] -> float32 [t][sub][nstokes][nchan]."""
    s = np.ascontiguousarray(spectra, np.complex64)
    nt, nsub, npol, nchan = s.shape
    assert npol == 2
    out = np.zeros((nt, nsub, nstokes, nchan), np.float32)
    lib().or_stokes(s.view(np.float32).ctypes.data_as(C.POINTER(C.c_float)), nt, nsub, nchan,
                    nstokes, _f32p(out))
    return out


def integrate(x, window, bin_chans=1):
    x = np.ascontiguousarray(x, np.float32)
    nt, nsub, npol, nchan = x.shape
    w = min(window, nt)
    out = np.zeros((nt // w, nsub, npol, nchan // bin_chans), np.float32)
    lib().or_integrate(_f32p(x), nt, nsub, npol, nchan, window, bin_chans, _f32p(out))
    return out


class RFI:
    """RFI_Clipper restatement; mode 0 = reference FP32, mode 1 = FP64 variant."""

    def __init__(self, bp_text, cr=10.0, sr=4.0, history=10, zero_dming=False,
                 mean_over_rms=True, band_matching=True, mode=0, parts=256):
        err = C.create_string_buffer(512)
        self.h = lib().or_rfi_create(bp_text.encode(), cr, sr, history, int(zero_dming),
                                     int(mean_over_rms), int(band_matching), mode, parts, err, 512)
        if not self.h:
            raise ValueError(err.value.decode())

    def run(self, data, weights=None, flags=False):
        """In place on float32 [t][sub][pol][nchan]; returns flags if asked."""
        assert data.dtype == np.float32 and data.flags.c_contiguous
        nt, nsub, npol, nchan = data.shape
        if weights is None:
            weights = np.ones_like(data)
        fl = np.zeros((nt, nsub * nchan), np.uint8) if flags else None
        rc = lib().or_rfi_run(self.h, _f32p(data), _f32p(weights), nt, nsub, npol, nchan,
                              fl.ctypes.data if fl is not None else None)
        if rc != 0:
            raise RuntimeError("or_rfi_run failed %d" % rc)
        return fl

    def state(self):
        out = np.zeros(10, np.float64)
        lib().or_rfi_state(self.h, _f64p(out))
        return out

    def bandpass(self, nbins):
        out = np.zeros(nbins, np.float32)
        lib().or_rfi_bandpass(self.h, _f32p(out), nbins)
        return out

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_rfi_destroy(self.h)
            self.h = None


class DedispersionModule:
    """DedispersionModule + DedispersionBuffer streaming restatement."""

    def __init__(self, buffer_samples, tdms, dm_low, dm_step, fch1, foff):
        self.tdms = tdms
        self.h = lib().or_ddmod_create(buffer_samples, tdms, dm_low, dm_step, fch1, foff)

    def add(self, stokes, tsamp):
        s = np.ascontiguousarray(stokes, np.float32)
        nt, nsub, npol, nchan = s.shape
        n = lib().or_ddmod_add(self.h, _f32p(s), nt, nsub, npol, nchan, tsamp)
        if n < 0:
            raise ValueError("maxshift requirements are bigger than the number of samples")
        outs = []
        for _ in range(n):
            ms, rem, nout = self.params()[:3]
            buf = np.zeros((self.tdms, nout), np.float32)
            first = C.c_longlong()
            lib().or_ddmod_pop(self.h, _f32p(buf), buf.size, C.byref(first))
            outs.append((buf, first.value))
        return outs

    def params(self):
        v = [C.c_int() for _ in range(5)]
        lib().or_ddmod_params(self.h, *[C.byref(x) for x in v])
        return tuple(x.value for x in v)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_ddmod_destroy(self.h)
            self.h = None


def sum_canonical(x, parts=256):
    x = np.ascontiguousarray(x, np.float32)
    return lib().or_sum_canonical(_f32p(x), len(x), parts)


def rfi_parts(nbins):
    """Partial-sum count (the GPU clipper's thread count) for a band of nbins."""
    return 256 if nbins <= 1024 else (512 if nbins <= 4096 else 1024)


def num_threads():
    return lib().or_num_threads()


# --------------------------------------------------------------------------
# F1 LOFAR UDP packets
# --------------------------------------------------------------------------

def udp_check(fixed, bits, npackets, spp, nchan, nsub, npol, chunk_bytes):
    """(code, packet_bytes, nblocks); code 0 when AdapterTimeSeriesDataSet's checks pass."""
    pb, nb = C.c_longlong(0), C.c_int(0)
    rc = lib().or_udp_check(int(fixed), bits, npackets, spp, nchan, nsub, npol, chunk_bytes,
                            C.byref(pb), C.byref(nb))
    return rc, pb.value, nb.value


def udp_unpack(chunk, packet_bytes, npackets, bits, nsub, npol, spp):
    """complex64 [nsub][npol][npackets*spp] from a chunk of packets (bytes or uint8 array)."""
    buf = np.frombuffer(chunk, np.uint8) if not isinstance(chunk, np.ndarray) else chunk
    buf = np.ascontiguousarray(buf, np.uint8)
    out = np.zeros((nsub, npol, npackets * spp), np.complex64)
    rc = lib().or_udp_unpack(buf.ctypes.data, packet_bytes, npackets, bits, nsub, npol, spp,
                             out.ctypes.data_as(C.POINTER(C.c_float)))
    if rc:
        raise ValueError("16-bit packets carry two polarisations")
    return out


def udp_time(packet, clock_mhz=200):
    buf = np.ascontiguousarray(np.frombuffer(bytes(packet[:16]), np.uint8))
    ts, rate = C.c_double(0), C.c_double(0)
    lib().or_udp_time(buf.ctypes.data, clock_mhz, C.byref(ts), C.byref(rate))
    return ts.value, rate.value
