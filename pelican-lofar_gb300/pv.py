"""ctypes binding of libpv.so, the GB300 beam-processing library.

Device buffers are torch CUDA tensors (PyTorch provides device memory and
streams only; all compute runs in libpv's own kernels).  Every call raises
PvError with the library's message on a non-zero status.  The library must
be built (``build.py``); nothing here falls back to a CPU path.
"""
import ctypes as C
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "libpv.so")
HEADER = os.path.join(ROOT, "include", "pv.h")

EVENT_DTYPE = np.dtype([("dm", "<i4"), ("t", "<i4"), ("bin_factor", "<f4"), ("value", "<f4")])


class PvError(RuntimeError):
    pass


class pv_event(C.Structure):
    _fields_ = [("dm", C.c_int32), ("t", C.c_int32), ("bin_factor", C.c_float), ("value", C.c_float)]


_lib = None


def header_symbols():
    """Function names declared in include/pv.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pv_[a-z0-9_]+)\s*\(", text)))


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PvError("libpv.so is not built; run pelican-lofar_gb300/build.py")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L):
    vp, i, f, d, ll = C.c_void_p, C.c_int, C.c_float, C.c_double, C.c_longlong
    P = C.POINTER
    sigs = {
        "pv_last_error": (C.c_char_p, []),
        "pv_version": (i, []),
        "pv_kernel_launches": (ll, []),
        "pv_dm_shifts": (i, [d, d, i, P(C.c_float), P(i)]),
        "pv_maxshift": (i, [f, f, i, P(C.c_float), i, d, i, P(i), P(i)]),
        "pv_delay_table": (i, [vp, vp, i, i, f, f, vp]),
        "pv_dedisperse": (i, [vp, ll, vp, f, f, i, i, vp, i, i, vp]),
        "pv_dedisperse_ex": (i, [vp, ll, vp, ll, ll, i, i, i, vp, f, f, vp]),
        "pv_dedisp_plan_create": (i, [P(vp), P(C.c_float), i, i, f, f]),
        "pv_dedisp_plan_destroy": (None, [vp]),
        "pv_dedisp_plan_max_shift": (i, [vp]),
        "pv_dedisp_plan_run": (i, [vp, vp, ll, vp, ll, ll, ll, ll, i, vp]),
        "pv_ring_write": (i, [vp, ll, ll, ll, vp, i, i, i, i, i, vp]),
        "pv_window_from_name": (i, [C.c_char_p]),
        "pv_fir_coefficients": (i, [i, i, i, P(C.c_double)]),
        "pv_ppf_create": (i, [P(vp), i, i, i, vp]),
        "pv_ppf_destroy": (None, [vp]),
        "pv_ppf_coefficients": (i, [vp, P(C.c_float)]),
        "pv_ppf_reset": (i, [vp]),
        "pv_ppf_run": (i, [vp, vp, i, i, i, vp, vp]),
        "pv_channelise": (i, [vp, vp, i, i, i, i, i, i, vp, P(i), vp]),
        "pv_stokes": (i, [vp, i, i, i, i, vp, vp]),
        "pv_integrate": (i, [vp, i, i, i, i, i, i, vp, P(i), vp]),
        "pv_rfi_create": (i, [P(vp), C.c_char_p, f, f, i, i, i, i, i]),
        "pv_rfi_destroy": (None, [vp]),
        "pv_rfi_run": (i, [vp, vp, i, i, i, i, vp, vp]),
        "pv_rfi_state": (i, [vp, P(C.c_double)]),
        "pv_rfi_bandpass": (i, [vp, P(C.c_float), i]),
        "pv_rfi_bandpass_current": (i, [vp, P(C.c_float), i, P(C.c_float)]),
        "pv_rfi_parts": (i, [i]),
        "pv_beam_create": (i, [P(vp), vp]),
        "pv_beam_destroy": (None, [vp]),
        "pv_beam_input_bytes": (ll, [vp, i]),
        "pv_beam_process": (i, [vp, vp, i, vp]),
        "pv_beam_process_host": (i, [vp, vp, i, vp]),
        "pv_beam_events": (i, [vp, vp, ll, P(ll), P(ll), vp]),
        "pv_beam_info": (i, [vp, P(ll)]),
        "pv_beam_buffers": (i, [vp, P(vp), P(vp), P(vp), P(vp)]),
        "pv_beam_stage_ms": (i, [vp, P(C.c_float)]),
        "pv_beam_state_size": (ll, [vp]),
        "pv_beam_state_save": (i, [vp, vp, ll, vp]),
        "pv_beam_state_load": (i, [vp, vp, ll, vp]),
        "pv_host_alloc": (i, [P(vp), ll, i]),
        "pv_host_free": (None, [vp]),
        "pv_batch_create": (i, [P(vp), vp, i, i]),
        "pv_batch_destroy": (None, [vp]),
        "pv_batch_input": (i, [vp, i, P(vp), P(ll)]),
        "pv_batch_input_parity": (i, [vp, i, i, P(vp), P(ll)]),
        "pv_batch_run": (i, [vp, vp, vp]),
        "pv_batch_run_host": (i, [vp, P(vp), vp, vp]),
        "pv_batch_events": (i, [vp, i, ll, vp, ll, P(ll), P(ll)]),
        "pv_batch_info": (i, [vp, i, P(ll)]),
        "pv_batch_tiles": (i, [vp, P(i), P(i), P(C.c_float), P(ll)]),
        "pv_batch_stage_ms": (i, [vp, P(C.c_float)]),
        "pv_batch_buffers": (i, [vp, i, P(vp), P(vp), P(vp)]),
        "pv_batch_step_done": (i, [vp, ll]),
        "pv_batch_footprint": (ll, [vp, i]),
        "pv_batch_reset_beam": (i, [vp, i, vp]),
        "pv_serve": (i, [vp, vp, vp, i, vp, vp, vp]),
        "pv_udp_check": (i, [vp, ll, P(ll), P(i)]),
        "pv_udp_unpack": (i, [vp, vp, ll, vp, i, vp]),
        "pv_udp_time": (i, [vp, vp, P(d), P(d)]),
        "pv_ab_headers": (i, [vp, vp, vp, ll, vp, ll, P(ll), P(ll), P(d), P(ll)]),
        "pv_ab_unpack": (i, [vp, vp, ll, vp, ll, ll, vp, vp]),
        "pv_sigproc_header": (i, [vp, vp, ll, P(ll)]),
        "pv_sigproc_mjd": (d, [d]),
        "pv_sigproc_pack": (i, [vp, i, i, i, i, i, i, f, f, vp, vp]),
        "pv_events_text": (i, [vp, ll, d, d, ll, d, d, f, i, vp, ll, P(ll)]),
        "pv_trigger_message": (i, [vp, ll, d, d, ll, d, d, f, i, f, C.c_char_p, C.c_char_p, i, C.c_char_p,
                                   C.c_char_p, C.c_char_p, vp, ll, P(ll)]),
        "pv_bandpass_recorder_create": (i, [P(vp), ll, i, f, f]),
        "pv_bandpass_recorder_destroy": (None, [vp]),
        "pv_bandpass_recorder_add": (i, [vp, vp, i, i, i, i, vp]),
        "pv_bandpass_recorder_result": (i, [vp, P(f), P(f), P(i), vp, ll, P(ll)]),
        "pv_device_copy": (i, [vp, vp, ll, vp]),
        "pv_ddmod_create": (i, [P(vp), i, i, f, f, d, d]),
        "pv_ddmod_destroy": (None, [vp]),
        "pv_ddmod_add": (i, [vp, vp, i, i, i, i, d, P(i), vp]),
        "pv_ddmod_pop": (i, [vp, vp, ll, P(i), P(ll), vp]),
        "pv_ddmod_params": (i, [vp, P(i)]),
        "pv_dedisp_plan_status": (i, [vp, P(i)]),
        "pv_dedisp_plan_clear_status": (i, [vp, vp]),
        "pv_set_wait_limit": (ll, [ll]),
        "pv_stall_next_launches": (i, [i]),
        "pv_analyser_thresholds": (i, [f, f, i, P(C.c_float)]),
        "pv_analyse": (i, [vp, ll, i, i, f, f, i, vp, ll, P(ll), vp]),
    }
    for name, (res, args) in sigs.items():
        if hasattr(L, name):
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args


def check(rc):
    if rc != 0:
        raise PvError("libpv error %d: %s" % (rc, load().pv_last_error().decode()))
    return rc


def launches():
    return load().pv_kernel_launches()


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


# ---------------------------------------------------------------------------
# host helpers
# ---------------------------------------------------------------------------

def dm_shifts(fch1, foff, nchan):
    out = np.zeros(nchan, np.float32)
    inv = C.c_int()
    check(load().pv_dm_shifts(fch1, foff, nchan, out.ctypes.data_as(C.POINTER(C.c_float)),
                              C.byref(inv)))
    return out, bool(inv.value)


def maxshift(dm_low, dm_step, tdms, dmshift, tsamp, buffer_samples):
    dmshift = np.ascontiguousarray(dmshift, np.float32)
    ms, rem = C.c_int(), C.c_int()
    check(load().pv_maxshift(dm_low, dm_step, tdms, dmshift.ctypes.data_as(C.POINTER(C.c_float)),
                             len(dmshift), tsamp, buffer_samples, C.byref(ms), C.byref(rem)))
    return ms.value, rem.value


def thresholds(threshold, rms, bin_pow2):
    out = np.zeros(bin_pow2 + 1, np.float32)
    check(load().pv_analyser_thresholds(threshold, rms, bin_pow2,
                                        out.ctypes.data_as(C.POINTER(C.c_float))))
    return out


# ---------------------------------------------------------------------------
# device calls (torch CUDA tensors)
# ---------------------------------------------------------------------------

def delay_table(d_dmshift, tdms, start_over_tsamp, step_over_tsamp, stream=None):
    import torch
    nchan = d_dmshift.numel()
    out = torch.empty((tdms, nchan), dtype=torch.int32, device=d_dmshift.device)
    check(load().pv_delay_table(_ptr(out), _ptr(d_dmshift), nchan, tdms, start_over_tsamp,
                                step_over_tsamp, _stream(stream)))
    return out


def dedisperse(d_in, nout, tdms, d_dmshift, start_over_tsamp, step_over_tsamp, out=None,
               row_len=None, stream=None):
    """d_in: float32 [nchan][row_stride] CUDA tensor -> [tdms][nout]."""
    import torch
    assert d_in.dtype == torch.float32 and d_in.is_contiguous()
    nchan, stride = d_in.shape
    if out is None:
        out = torch.empty((tdms, nout), dtype=torch.float32, device=d_in.device)
    check(load().pv_dedisperse_ex(_ptr(out), out.stride(0), _ptr(d_in), stride,
                                  stride if row_len is None else row_len, nchan, nout, tdms,
                                  _ptr(d_dmshift), start_over_tsamp, step_over_tsamp,
                                  _stream(stream)))
    return out


class DedispPlan:
    """A dedispersion plan (pv_dedisp_plan_*): delay constants and tile choice
    for one channel set and trial grid; runs on linear or ring rows."""

    def __init__(self, dmshift, tdms, start_over_tsamp, step_over_tsamp):
        k = np.ascontiguousarray(dmshift, np.float32)
        self.nchan, self.tdms = len(k), tdms
        self.h = C.c_void_p()
        check(load().pv_dedisp_plan_create(C.byref(self.h), k.ctypes.data_as(C.POINTER(C.c_float)),
                                           len(k), tdms, start_over_tsamp, step_over_tsamp))

    def max_shift(self):
        return load().pv_dedisp_plan_max_shift(self.h)

    def run(self, d_in, nout, out=None, ring_len=0, t_base=0, row_len=None, stream=None):
        """d_in: float32 [nchan][row_stride] -> out [tdms][nout] (ring rows
        when ring_len > 0: output t reads column (t_base + t + shift) mod ring_len)."""
        import torch
        assert d_in.dtype == torch.float32 and d_in.is_contiguous() and d_in.shape[0] == self.nchan
        stride = d_in.shape[1]
        if out is None:
            out = torch.empty((self.tdms, nout), dtype=torch.float32, device=d_in.device)
        check(load().pv_dedisp_plan_run(self.h, _ptr(out), out.stride(0), _ptr(d_in), stride,
                                        stride if row_len is None else row_len, ring_len, t_base, nout,
                                        _stream(stream)))
        return out

    def status(self):
        st = C.c_int()
        check(load().pv_dedisp_plan_status(self.h, C.byref(st)))
        return st.value

    def clear_status(self, stream=None):
        check(load().pv_dedisp_plan_clear_status(self.h, _stream(stream)))

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.pv_dedisp_plan_destroy(self.h)
            self.h = C.c_void_p()


def stall_next_launches(n):
    """Failure-path test hook: the next n pipelined dedispersion launches
    withhold their first stage's copies, so a wait there runs out."""
    return load().pv_stall_next_launches(int(n))


def set_wait_limit(ns):
    """Limit (ns) of the pipelined kernels' bounded device waits from now on
    (<= 0: the default 0.5 s); returns the previous limit."""
    return load().pv_set_wait_limit(int(ns))


def dedisperse_ref_api(d_out, d_in, start_over_tsamp, step_over_tsamp, tdms, num_samples,
                       d_dmshift, maxshift_total, nchans, stream=None):
    """The cacheDedisperseLoop-shaped entry point."""
    check(load().pv_dedisperse(_ptr(d_out), d_out.numel() * 4, _ptr(d_in), start_over_tsamp,
                               step_over_tsamp, tdms, num_samples, _ptr(d_dmshift),
                               maxshift_total, nchans, _stream(stream)))
    return d_out


def analyse(d_data, threshold, rms, bin_pow2=6, cap=None, stream=None):
    """Returns a numpy structured array of events (dummy first)."""
    import torch
    tdms, nsamp = d_data.shape
    if cap is None:
        cap = 1 + tdms * nsamp * 2
    cap = max(int(cap), 1)
    ev = torch.empty(cap * 4, dtype=torch.int32, device=d_data.device)
    n = C.c_longlong()
    check(load().pv_analyse(_ptr(d_data), d_data.stride(0), tdms, nsamp, threshold, rms, bin_pow2,
                            _ptr(ev), cap, C.byref(n), _stream(stream)))
    k = min(n.value, cap)
    host = ev[: 4 * k].cpu().numpy().view(EVENT_DTYPE)
    return host.copy(), n.value


# ---------------------------------------------------------------------------
# channeliser chain and RFI clipper
# ---------------------------------------------------------------------------

WINDOWS = {"hamming": 0, "blackman": 1, "gaussian": 2, "kaiser": 3}


def fir_coefficients(ntaps, nchan, window="kaiser"):
    out = np.zeros((ntaps, nchan), np.float64)
    check(load().pv_fir_coefficients(ntaps, nchan, WINDOWS[window],
                                     out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


class PPF:
    """Device channeliser with its tap history (PPFChanneliser)."""

    def __init__(self, nchan, ntaps=8, window="kaiser", coeffs=None):
        self.nchan, self.ntaps = nchan, (1 if nchan == 1 else ntaps)  # one channel: no filter
        self.h = C.c_void_p()
        c = None
        if coeffs is not None:
            self._c = np.ascontiguousarray(coeffs, np.float32)
            c = self._c.ctypes.data_as(C.c_void_p)
        check(load().pv_ppf_create(C.byref(self.h), nchan, ntaps, WINDOWS[window], c))

    def coefficients(self):
        out = np.zeros((self.ntaps, self.nchan), np.float32)
        check(load().pv_ppf_coefficients(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out

    def run(self, d_in, stream=None):
        """d_in complex64 CUDA tensor [sub][pol][block*nchan] -> [block][sub][pol][nchan]."""
        import torch
        nsub, npol, n = d_in.shape
        nblocks = n // self.nchan
        out = torch.empty((nblocks, nsub, npol, self.nchan), dtype=torch.complex64, device=d_in.device)
        check(load().pv_ppf_run(self.h, _ptr(d_in), nsub, npol, nblocks, _ptr(out), _stream(stream)))
        return out

    def channelise(self, d_in, nstokes=1, window=4, bin=1, stream=None):
        """Fused PPF+Stokes+integration; d_in complex64 or int16 [sub][2][n(*2)]."""
        import torch
        int16 = d_in.dtype == torch.int16
        nsub = d_in.shape[0]
        n = d_in.shape[2] // (2 if int16 else 1)
        nblocks = n // self.nchan
        w = min(window, nblocks)
        nu = nblocks // w
        out = torch.empty((nu, nsub, nstokes, self.nchan // bin), dtype=torch.float32, device=d_in.device)
        got = C.c_int()
        check(load().pv_channelise(self.h, _ptr(d_in), int(int16), nsub, nblocks, nstokes, window, bin,
                                   _ptr(out), C.byref(got), _stream(stream)))
        assert got.value == nu
        return out

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.pv_ppf_destroy(self.h)
            self.h = C.c_void_p()


def stokes(d_spectra, nstokes=1, stream=None):
    import torch
    nt, nsub, npol, nchan = d_spectra.shape
    out = torch.empty((nt, nsub, nstokes, nchan), dtype=torch.float32, device=d_spectra.device)
    check(load().pv_stokes(_ptr(d_spectra), nt, nsub, nchan, nstokes, _ptr(out), _stream(stream)))
    return out


def integrate(d_in, window, bin=1, stream=None):
    import torch
    nt, nsub, npol, nchan = d_in.shape
    w = min(window, max(nt, 1))
    out = torch.empty((nt // w, nsub, npol, nchan // bin), dtype=torch.float32, device=d_in.device)
    nu = C.c_int()
    check(load().pv_integrate(_ptr(d_in), nt, nsub, npol, nchan, window, bin, _ptr(out), C.byref(nu),
                              _stream(stream)))
    return out


class RFI:
    """Device RFI_Clipper."""

    def __init__(self, bp_text, cr=10.0, sr=4.0, history=10, zero_dming=False, mean_over_rms=True,
                 band_matching=True, active=True, split=None):
        self.h = C.c_void_p()
        check(load().pv_rfi_create(C.byref(self.h), bp_text.encode() if bp_text else None, cr, sr,
                                   history, int(zero_dming), int(mean_over_rms), int(band_matching),
                                   int(active)))
        if split is not None:  # 0 one CTA, 1 wide bands over 4 CTAs, 2 over clusters of 128-thread CTAs
            check(load().pv_rfi_set_split(self.h, int(split)))

    def run(self, d_data, flags=False, stream=None):
        import torch
        nt, nsub, npol, nchan = d_data.shape
        fl = torch.zeros((nt, nsub * nchan), dtype=torch.uint8, device=d_data.device) if flags else None
        check(load().pv_rfi_run(self.h, _ptr(d_data), nt, nsub, npol, nchan,
                                _ptr(fl) if fl is not None else None, _stream(stream)))
        return fl

    def state(self):
        out = np.zeros(10, np.float64)
        check(load().pv_rfi_state(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.pv_rfi_destroy(self.h)
            self.h = C.c_void_p()


# ---------------------------------------------------------------------------
# beam pipeline
# ---------------------------------------------------------------------------

class BeamConfig(C.Structure):
    _fields_ = [("nsub", C.c_int), ("nchan_sub", C.c_int), ("ntaps", C.c_int), ("window", C.c_int),
                ("int_time", C.c_int), ("int_chan", C.c_int), ("fch1", C.c_double),
                ("foff", C.c_double), ("tsamp", C.c_double), ("tdms", C.c_int),
                ("dm_low", C.c_float), ("dm_step", C.c_float), ("chunk", C.c_int),
                ("threshold", C.c_float), ("bin_pow2", C.c_int), ("event_capacity", C.c_longlong),
                ("bp_text", C.c_char_p), ("cr", C.c_float), ("sr", C.c_float),
                ("history", C.c_int), ("zero_dming", C.c_int), ("rms_from_mean", C.c_int),
                ("band_matching", C.c_int), ("rfi_active", C.c_int), ("debug_taps", C.c_int),
                ("timing", C.c_int), ("prefilled", C.c_int), ("udp_packet_bytes", C.c_int),
                ("udp_subbands", C.c_int)]


def beam_config(**kw):
    d = dict(ntaps=8, window=WINDOWS["kaiser"], int_time=4, int_chan=1, dm_low=0.0, threshold=6.0,
             bin_pow2=6, event_capacity=0, cr=10.0, sr=4.0, history=10, zero_dming=0,
             rms_from_mean=1, band_matching=1, rfi_active=1, debug_taps=0, timing=0, prefilled=0,
             udp_packet_bytes=0, udp_subbands=0)
    d.update(kw)
    if isinstance(d.get("window"), str):
        d["window"] = WINDOWS[d["window"]]
    bp = d.pop("bp_text", None)
    cfg = BeamConfig(**d)
    cfg._bp = bp.encode() if isinstance(bp, str) else bp
    cfg.bp_text = cfg._bp
    return cfg


class Beam:
    """One beam's device-resident chain (PPF..analyser) through the C ABI."""

    def __init__(self, cfg):
        self.cfg = cfg
        self.h = C.c_void_p()
        check(load().pv_beam_create(C.byref(self.h), C.byref(cfg)))

    def info(self):
        out = (C.c_longlong * 8)()
        check(load().pv_beam_info(self.h, out))
        keys = ["nbins", "max_shift", "lag", "ring_len", "inverted", "chunks", "window", "ring_bytes"]
        return dict(zip(keys, list(out)))

    def input_bytes(self, int16=True):
        return load().pv_beam_input_bytes(self.h, int(int16))

    def process(self, d_voltages, stream=None):
        import torch
        int16 = d_voltages.dtype == torch.int16
        check(load().pv_beam_process(self.h, _ptr(d_voltages), int(int16), _stream(stream)))

    def process_host(self, h_voltages, stream=None):
        """h_voltages: numpy int16 [sub][2][n][2] or complex64 (pinned torch tensor also works)."""
        if hasattr(h_voltages, "data_ptr"):
            import torch
            ptr, int16 = h_voltages.data_ptr(), h_voltages.dtype == torch.int16
        else:
            ptr, int16 = h_voltages.ctypes.data, h_voltages.dtype == np.int16
        check(load().pv_beam_process_host(self.h, C.c_void_p(ptr), int(int16), _stream(stream)))

    def events(self, cap=1 << 20, stream=None):
        n, first = C.c_longlong(), C.c_longlong()
        check(load().pv_beam_events(self.h, None, 0, C.byref(n), C.byref(first), _stream(stream)))
        k = min(n.value, cap)
        ev = np.zeros(k, EVENT_DTYPE)
        if k:
            check(load().pv_beam_events(self.h, C.c_void_p(ev.ctypes.data), k, C.byref(n),
                                        C.byref(first), _stream(stream)))
        return ev, n.value, first.value

    def stage_ms(self):
        out = (C.c_float * 5)()
        check(load().pv_beam_stage_ms(self.h, out))
        return dict(zip(["channelise", "rfi", "ring_write", "dedisperse", "analyse"], list(out)))

    def buffers(self):
        p = [C.c_void_p() for _ in range(4)]
        check(load().pv_beam_buffers(self.h, *[C.byref(x) for x in p]))
        return [x.value for x in p]

    def save_state(self, stream=None):
        """The stream state (tap history, clipper state, ring) as bytes."""
        n = load().pv_beam_state_size(self.h)
        buf = np.empty(n, np.uint8)
        check(load().pv_beam_state_save(self.h, C.c_void_p(buf.ctypes.data), n, _stream(stream)))
        return buf

    def load_state(self, state, stream=None):
        state = np.ascontiguousarray(state, np.uint8)
        check(load().pv_beam_state_load(self.h, C.c_void_p(state.ctypes.data), state.nbytes, _stream(stream)))

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.pv_beam_destroy(self.h)
            self.h = C.c_void_p()


BATCH_TUNE, BATCH_GRAPH, BATCH_TIMING, BATCH_PIPELINED = 1, 2, 4, 8
BATCH_VARIANTS = 9  # PV_BATCH_VARIANTS: dedispersion tile variants
BATCH_RFI_ONE_CTA = 64  # PV_BATCH_RFI_ONE_CTA: every clipper on one CTA
BATCH_RFI_CLUSTER8 = 128  # PV_BATCH_RFI_CLUSTER8: clusters of 128-thread CTAs
BATCH_RFI_CLUSTER4 = 0x10000  # PV_BATCH_RFI_CLUSTER4: beams of 1024 partials on 4 CTAs

class UdpConfig(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("fixed_size_packets", "sample_bits", "packets_per_chunk",
                                       "samples_per_packet", "nchan", "nsub", "npol", "clock_mhz")]


UDP_OUT = {"c32": 0, "i16": 1}


class UdpAdapter:
    """AdapterTimeSeriesDataSet (lib/src/AdapterTimeSeriesDataSet.cpp:35-293)
    on the GPU.  Keyword names are the adapter's XML options.  deserialise()
    takes one chunk of packets (a device uint8 tensor, or host bytes / numpy
    uint8, copied in first) and returns the TimeSeriesDataSetC32 on the
    device: complex64 [sub][pol][block][nchan] ("c32"), or the same samples
    as int16 [sub][pol][block*nchan][2] ("i16", the station format the
    channeliser takes).  The chunk's LOFAR time stamp and block rate are
    kept as attributes, and out_of_sequence is set as the reference warns
    (:113-116)."""

    def __init__(self, fixedSizePackets=True, dataBitSize=0, udpPacketsPerIteration=0,
                 samplesPerPacket=0, outputChannelsPerSubband=0, subbandsPerPacket=0,
                 nRawPolarisations=0, clock=200):
        self.cfg = UdpConfig(int(bool(fixedSizePackets)), dataBitSize, udpPacketsPerIteration,
                             samplesPerPacket, outputChannelsPerSubband, subbandsPerPacket,
                             nRawPolarisations, clock)
        self.timestamp = self.block_rate = None
        self.out_of_sequence = False
        self._last = 0.0

    def check(self, chunk_bytes):
        """(packet_bytes, time blocks) of a chunk; PvError with the reference's message."""
        pb, nb = C.c_longlong(0), C.c_int(0)
        check(load().pv_udp_check(C.byref(self.cfg), chunk_bytes, C.byref(pb), C.byref(nb)))
        return pb.value, nb.value

    def deserialise(self, chunk, out="c32", stream=None):
        import torch
        import numpy as np
        c = self.cfg
        if isinstance(chunk, torch.Tensor) and chunk.is_cuda:
            d_chunk, head = chunk, chunk[:16].cpu().numpy()
        else:
            host = np.frombuffer(chunk, np.uint8) if not isinstance(chunk, np.ndarray) else chunk
            head = np.ascontiguousarray(host[:16])
            d_chunk = torch.from_numpy(np.ascontiguousarray(host, np.uint8)).cuda()
        nbytes = d_chunk.numel()
        _, nblocks = self.check(nbytes)
        if out == "c32":
            res = torch.empty((c.nsub, c.npol, nblocks, c.nchan), dtype=torch.complex64, device=d_chunk.device)
        else:
            res = torch.empty((c.nsub, c.npol, nblocks * c.nchan, 2), dtype=torch.int16, device=d_chunk.device)
        check(load().pv_udp_unpack(C.byref(c), _ptr(d_chunk), nbytes, _ptr(res), UDP_OUT[out], _stream(stream)))
        ts, rate = C.c_double(0), C.c_double(0)
        check(load().pv_udp_time(C.byref(c), head.ctypes.data, C.byref(ts), C.byref(rate)))
        self.timestamp, self.block_rate = ts.value, rate.value
        self.out_of_sequence = self.timestamp - self._last > self.block_rate
        self._last = self.timestamp + nblocks * c.nchan * self.block_rate
        return res


class AbConfig(C.Structure):
    _fields_ = [("packets_per_spectrum", C.c_int), ("channels", C.c_int), ("samples_per_packet", C.c_int),
                ("tsamp", C.c_float)]


class AbState(C.Structure):
    _fields_ = [("seen", C.c_longlong), ("count0", C.c_ulonglong), ("last_time", C.c_double)]


class ABDataAdapter:
    """ABDataAdapter (lib/src/ABDataAdapter.cpp:14-173), the input of
    ABPipeline: chunks of ALFABURST spectrometer packets -> a device
    SpectrumDataSetStokes float32 [block][1][1][channels] of Stokes I.
    Keyword names follow the XML options (<spectrum packets>, <packet
    channels>, <packet samples>, <samplingTime seconds>).  The headers are
    read on the host; timestamp (the chunk's last packet), block_rate and gaps
    (the reference's "FATAL!" packets) are kept as attributes."""

    def __init__(self, packets=4, channels=1024, samples=0, seconds=0.0):
        self.cfg = AbConfig(packets, channels, samples, seconds)
        self.state = AbState()
        self.timestamp, self.block_rate, self.gaps = 0.0, float(np.float32(seconds)), 0

    def deserialise(self, chunk, stream=None):
        import torch
        host = np.ascontiguousarray(np.frombuffer(chunk, np.uint8) if not isinstance(chunk, np.ndarray)
                                    else chunk.view(np.uint8).reshape(-1))
        npk = len(host) // (8 + 8 * self.cfg.channels)
        idx = np.zeros(max(1, npk), np.int32)
        nsp, nbl, ts, gaps = C.c_longlong(0), C.c_longlong(0), C.c_double(0), C.c_longlong(0)
        check(load().pv_ab_headers(C.byref(self.cfg), C.byref(self.state), host.ctypes.data, len(host),
                                   idx.ctypes.data, len(idx), C.byref(nsp), C.byref(nbl), C.byref(ts),
                                   C.byref(gaps)))
        d_chunk = torch.from_numpy(host).cuda()
        d_idx = torch.from_numpy(idx[:max(1, nsp.value)]).cuda()
        out = torch.empty((nbl.value, 1, 1, self.cfg.channels), dtype=torch.float32, device=d_chunk.device)
        check(load().pv_ab_unpack(C.byref(self.cfg), _ptr(d_chunk), len(host), _ptr(d_idx), nsp.value,
                                  nbl.value, _ptr(out), _stream(stream)))
        self.timestamp, self.gaps = ts.value, gaps.value
        return out


class SigprocParams(C.Structure):
    _fields_ = [("machine_id", C.c_int), ("telescope_id", C.c_int), ("nchans", C.c_int), ("nbits", C.c_int),
                ("nifs", C.c_int), ("src_raj", C.c_double), ("src_dej", C.c_double), ("fch1", C.c_double),
                ("foff", C.c_double), ("tsamp", C.c_double), ("tstart", C.c_double),
                ("source_name", C.c_char * 80)]


def sigproc_header(params, tstart):
    """SigprocStokesWriter's header bytes (lib/src/SigprocStokesWriter.cpp:129-146)
    from its values (a dict with SigprocParams' fields but tstart)."""
    p = SigprocParams(**{k: (v.encode() if k == "source_name" else v) for k, v in params.items()})
    p.tstart = tstart
    n = C.c_longlong(0)
    load().pv_sigproc_header(C.byref(p), None, 0, C.byref(n))
    buf = C.create_string_buffer(n.value)
    check(load().pv_sigproc_header(C.byref(p), buf, n.value, C.byref(n)))
    return buf.raw[:n.value]


def sigproc_mjd(lofar_timestamp):
    return load().pv_sigproc_mjd(lofar_timestamp)


def sigproc_pack(d_stokes, npols_write=1, nbits=32, crop_min=0.0, crop_max=255.0, stream=None):
    """The filterbank data block of float32 [t][sub][pol][chan] on the device
    (:195-234, 288-293): a device uint8 tensor of the bytes the writer emits."""
    import torch
    nt, nsub, npol, nchan = d_stokes.shape
    out = torch.empty(nt * npols_write * nsub * nchan * (nbits // 8), dtype=torch.uint8, device=d_stokes.device)
    check(load().pv_sigproc_pack(_ptr(d_stokes), nt, nsub, npol, nchan, npols_write, nbits, crop_min, crop_max,
                                 _ptr(out), _stream(stream)))
    return out


EVENTS_TEXT_HEADER = ("# Generated by DedispersionDataAnalysisOutput\n# Events\n# ------\n"
                      "# Time|Dm|Amplitude|BinFactor\n# ------\n")


def events_text(events, start_timestamp, block_rate, first_sample, dm_low, dm_step, rms, dump_index):
    """The text DedispersionDataAnalysisOutput::sendStream writes for one
    analysed buffer (lib/src/DedispersionDataAnalysisOutput.cpp:80-112)."""
    import numpy as np
    ev = np.ascontiguousarray(events)
    n = C.c_longlong(0)
    args = (ev.ctypes.data if len(ev) else None, len(ev), start_timestamp, block_rate, first_sample, dm_low,
            dm_step, rms, dump_index)
    load().pv_events_text(*args, None, 0, C.byref(n))
    buf = C.create_string_buffer(n.value + 1)
    check(load().pv_events_text(*args, buf, n.value, C.byref(n)))
    return buf.raw[:n.value].decode()


def trigger_message(events, start_timestamp, block_rate, first_sample, dm_low, dm_step, rms, min_events,
                    snr_threshold, station, id_root, message_number, cfreq_mhz, beam_ra, beam_dec):
    """The FRATS trigger TriggerOutput sends for one analysed buffer
    (lib/src/TriggerOutput.cpp:151-183), or None when the buffer raises none."""
    import numpy as np
    ev = np.ascontiguousarray(events)
    n = C.c_longlong(0)
    args = (ev.ctypes.data if len(ev) else None, len(ev), start_timestamp, block_rate, first_sample, dm_low,
            dm_step, rms, min_events, snr_threshold, station.encode(), id_root.encode(), message_number,
            cfreq_mhz.encode(), beam_ra.encode(), beam_dec.encode())
    check(load().pv_trigger_message(*args, None, 0, C.byref(n)))
    if n.value == 0:
        return None
    buf = C.create_string_buffer(n.value + 1)
    check(load().pv_trigger_message(*args, buf, n.value, C.byref(n)))
    return buf.raw[:n.value].decode()


class TriggerOutput:
    """TriggerOutput (lib/src/TriggerOutput.cpp:33-204): each analysed buffer
    that raises a FRATS trigger sends it as one UDP datagram to every receiver
    and appends it, with a newline, to the log file.  The identifier root is
    the construction time (yyyyMMddhhmm, local) and the beam id to two digits."""

    def __init__(self, station="", beamID="", rajd="", decjd="", cfreq_mhz="", snr=0.0, events=0,
                 receiver=None, logfile=None, format="FRATS"):
        import socket
        import time
        self.format = format
        self.station, self.ra, self.dec, self.cfreq = station, rajd, decjd, cfreq_mhz
        self.snr, self.min_events = float(snr), int(events)
        self.id_root = "%s-%s" % (time.strftime("%Y%m%d%H%M"), beamID.rjust(2, "0"))
        self.counter = 0
        self.receivers = []
        if receiver and receiver[0] and receiver[1]:
            s = socket.socket(socket.AF_INET, socket.SOCK_DGRAM)
            self.receivers.append((s, (receiver[0], int(receiver[1]))))
        self.log = None
        if logfile:
            try:
                self.log = open(logfile, "ab")
            except OSError:
                print("unable to open file for writing: " + logfile, file=sys.stderr)

    def send_stream(self, events, start_timestamp, block_rate, first_sample, dm_low, dm_step, rms):
        """Returns the message sent, or None."""
        if self.format != "FRATS":
            print("Trigger format not recognized / implemented", file=sys.stderr)
            return None
        msg = trigger_message(events, start_timestamp, block_rate, first_sample, dm_low, dm_step, rms,
                              self.min_events, self.snr, self.station, self.id_root, self.counter + 1,
                              self.cfreq, self.ra, self.dec)
        if msg is None:
            return None
        self.counter += 1
        if not self.ra:
            print("No RA/Dec found, conversion not yet implemented", file=sys.stderr)
        for s, addr in self.receivers:
            s.sendto(msg.encode(), addr)
        if self.log:
            self.log.write(msg.encode() + b"\n")
            self.log.flush()
        return msg

    def close(self):
        for s, _ in self.receivers:
            s.close()
        self.receivers = []
        if self.log:
            self.log.close()
            self.log = None


class BandPassRecorder:
    """BandPassRecorder (lib/src/BandPassRecorder.cpp:22-190): run() adds a
    device Stokes set [t][sub][pol][chan] and returns True once the fit of
    requiredSamples spectra is ready; result() gives (coefficients, rms,
    channels trimmed, .bp text)."""

    def __init__(self, requiredSamples=20000, coefficients=3, startFrequency=None, endFrequency=None):
        if startFrequency is None:
            raise PvError("BandPassRecorder: <Band startFrequency=?> not defined")
        if endFrequency is None:
            raise PvError("BandPassRecorder: <Band endFrequency=?> not defined")
        self.n = coefficients
        self.h = C.c_void_p()
        check(load().pv_bandpass_recorder_create(C.byref(self.h), requiredSamples, coefficients,
                                                 startFrequency, endFrequency))

    def run(self, d_stokes, stream=None):
        nt, nsub, npol, nchan = d_stokes.shape
        rc = load().pv_bandpass_recorder_add(self.h, _ptr(d_stokes), nt, nsub, npol, nchan, _stream(stream))
        if rc < 0:
            check(rc)
        return rc == 1

    def result(self):
        import numpy as np
        co = (C.c_float * self.n)()
        rms, trimmed, n = C.c_float(0), C.c_int(0), C.c_longlong(0)
        check(load().pv_bandpass_recorder_result(self.h, co, C.byref(rms), C.byref(trimmed), None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value + 1)
        check(load().pv_bandpass_recorder_result(self.h, co, C.byref(rms), C.byref(trimmed), buf, n.value,
                                                 C.byref(n)))
        return np.array(co[:], np.float32), rms.value, trimmed.value, buf.raw[:n.value].decode()

    def __del__(self):
        if getattr(self, "h", None):
            load().pv_bandpass_recorder_destroy(self.h)
            self.h = None


BATCH_STORE = {"f32": 0, "f16": 16, "u8": 32}
HOST_EVENTS = 65536  # PV_BATCH_HOST_EVENTS


def batch_footprint(cfg, pipelined=True, store="f32"):
    """Device bytes of one beam of this configuration in a batch."""
    n = load().pv_batch_footprint(C.byref(cfg), (BATCH_PIPELINED if pipelined else 0) | BATCH_STORE[store])
    if n < 0:
        check(int(n))
    return int(n)


class Batch:
    """Many beams advanced one chunk per step by batched launches (pv_batch)."""

    def __init__(self, cfgs, tune=True, graph=True, timing=False, variant=0, pipelined=False, store="f32",
                 rfi_one_cta=False, rfi_cluster8=False, rfi_cluster4=False):
        self.cfgs = list(cfgs)
        self.pipelined = pipelined
        self.store = store
        self._arr = (BeamConfig * len(self.cfgs))(*self.cfgs)
        flags = (BATCH_TUNE if tune else (variant << 8)) | (BATCH_GRAPH if graph else 0) | \
            (BATCH_TIMING if timing else 0) | (BATCH_PIPELINED if pipelined else 0) | BATCH_STORE[store] | \
            (BATCH_RFI_ONE_CTA if rfi_one_cta else 0) | (BATCH_RFI_CLUSTER8 if rfi_cluster8 else 0) | \
            (BATCH_RFI_CLUSTER4 if rfi_cluster4 else 0)
        self.h = C.c_void_p()
        check(load().pv_batch_create(C.byref(self.h), self._arr, len(self.cfgs), flags))

    def __len__(self):
        return len(self.cfgs)

    def input(self, beam):
        p, n = C.c_void_p(), C.c_longlong()
        check(load().pv_batch_input(self.h, beam, C.byref(p), C.byref(n)))
        return p.value, n.value

    def set_input(self, beam, d_voltages, stream=None, both=False):
        """Device-to-device copy of one beam's int16 voltages into the input
        buffer of its next chunk, or (both) of its chunks of either parity:
        the same chunk at every step."""
        bufs = []
        if both:
            for par in (0, 1):
                p, n = C.c_void_p(), C.c_longlong()
                check(load().pv_batch_input_parity(self.h, beam, par, C.byref(p), C.byref(n)))
                bufs.append((p.value, n.value))
        else:
            bufs.append(self.input(beam))
        for p, n in bufs:
            assert d_voltages.numel() * d_voltages.element_size() == n
            check(load().pv_device_copy(C.c_void_p(p), _ptr(d_voltages), n, _stream(stream)))

    def _mask(self, active):
        if active is None:
            return None
        m = np.ascontiguousarray(np.asarray(active, dtype=np.uint8))
        assert m.shape == (len(self.cfgs),)
        return m

    def run(self, active=None, stream=None):
        """One step; active: per-beam flags of the beams that have a chunk (None: all)."""
        m = self._mask(active)
        check(load().pv_batch_run(self.h, None if m is None else C.c_void_p(m.ctypes.data),
                                  _stream(stream)))

    def run_host(self, h_voltages, active=None, stream=None):
        m = self._mask(active)
        ptrs = (C.c_void_p * len(h_voltages))(
            *[C.c_void_p(None if v is None else (v.data_ptr() if hasattr(v, "data_ptr") else v.ctypes.data))
              for v in h_voltages])
        check(load().pv_batch_run_host(self.h, ptrs, None if m is None else C.c_void_p(m.ctypes.data),
                                       _stream(stream)))

    def events(self, beam, step=-1, cap=1 << 16):
        """(events, total count, first sample) of one beam at one of the last
        two issued steps (-1: the last, -2: the one before, or the step's
        index); waits for that step only."""
        n, first = C.c_longlong(), C.c_longlong()
        check(load().pv_batch_events(self.h, beam, step, None, 0, C.byref(n), C.byref(first)))
        k = min(n.value, cap, HOST_EVENTS)
        ev = np.zeros(k, EVENT_DTYPE)
        if k:
            check(load().pv_batch_events(self.h, beam, step, C.c_void_p(ev.ctypes.data), k, C.byref(n),
                                         C.byref(first)))
        return ev, n.value, first.value

    def info(self, beam):
        out = (C.c_longlong * 8)()
        check(load().pv_batch_info(self.h, beam, out))
        keys = ["nbins", "max_shift", "lag", "ring_len", "inverted", "written", "window", "ring_bytes"]
        return dict(zip(keys, list(out)))

    def tiles(self):
        shape, dms = (C.c_int * 8)(), (C.c_int * len(self.cfgs))()
        tune, nk = (C.c_float * BATCH_VARIANTS)(), C.c_longlong()
        check(load().pv_batch_tiles(self.h, shape, dms, tune, C.byref(nk)))
        keys = ["variant", "time_tile", "chan_per_stage", "stages", "slot", "tiles", "ctas", "smem"]
        d = dict(zip(keys, list(shape)))
        d["dms"] = list(dms)
        d["tune_ms"] = list(tune)
        d["graph_kernels"] = nk.value
        return d

    def stage_ms(self):
        out = (C.c_float * 5)()
        check(load().pv_batch_stage_ms(self.h, out))
        return dict(zip(["channelise", "rfi", "ring_write", "dedisperse", "analyse"], list(out)))

    def buffers(self, beam):
        p = [C.c_void_p() for _ in range(3)]
        check(load().pv_batch_buffers(self.h, beam, *[C.byref(x) for x in p]))
        return [x.value for x in p]

    def step_done(self, step):
        rc = load().pv_batch_step_done(self.h, step)
        if rc < 0:
            check(rc)
        return rc == 1

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.pv_batch_destroy(self.h)
            self.h = C.c_void_p()


class HostBuffer:
    """Page-locked host memory from the library (optionally write-combined)."""

    def __init__(self, nbytes, write_combined=False, int16=True):
        self.nbytes = int(nbytes)
        self.int16 = int16
        p = C.c_void_p()
        check(load().pv_host_alloc(C.byref(p), self.nbytes, int(write_combined)))
        self.ptr = p.value

    def data_ptr(self):
        return self.ptr

    @property
    def dtype(self):
        import torch
        return torch.int16 if self.int16 else torch.complex64

    def fill_from(self, tensor, stream=None):
        """Copies a device (or host) tensor of the same size into the buffer and waits."""
        assert tensor.numel() * tensor.element_size() == self.nbytes
        check(load().pv_device_copy(C.c_void_p(self.ptr), _ptr(tensor), self.nbytes, _stream(stream)))
        import torch
        torch.cuda.synchronize()

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.pv_host_free(C.c_void_p(self.ptr))
            self.ptr = None


def device_array(ptr, shape, device=None, dtype="float32"):
    """A torch copy (float32, float16 or uint8) of library-owned device memory."""
    import torch
    tt = {"float32": torch.float32, "float16": torch.float16, "uint8": torch.uint8}[dtype]
    t = torch.empty(shape, dtype=tt, device=device or "cuda")
    check(load().pv_device_copy(_ptr(t), C.c_void_p(ptr), t.numel() * t.element_size(), _stream(None)))
    return t


class DedispersionModule:
    """DedispersionModule with the reference's buffering (host numpy blobs in,
    host DedispersionSpectra out)."""

    def __init__(self, buffer_samples, tdms, dm_low, dm_step, fch1, foff):
        self.tdms = tdms
        self.h = C.c_void_p()
        check(load().pv_ddmod_create(C.byref(self.h), buffer_samples, tdms, dm_low, dm_step, fch1,
                                     foff))

    def add(self, stokes, tsamp, stream=None):
        s = np.ascontiguousarray(stokes, np.float32)
        nt, nsub, npol, nchan = s.shape
        done = C.c_int()
        check(load().pv_ddmod_add(self.h, C.c_void_p(s.ctypes.data), nt, nsub, npol, nchan, tsamp,
                                  C.byref(done), _stream(stream)))
        outs = []
        for _ in range(done.value):
            p = self.params()
            buf = np.empty((self.tdms, p["nout"]), np.float32)
            n, first = C.c_int(), C.c_longlong()
            check(load().pv_ddmod_pop(self.h, C.c_void_p(buf.ctypes.data), buf.size, C.byref(n),
                                      C.byref(first), _stream(stream)))
            outs.append((buf, first.value))
        return outs

    def params(self):
        out = (C.c_int * 6)()
        check(load().pv_ddmod_params(self.h, out))
        return dict(zip(["maxshift", "remaining", "nout", "nchan", "inverted", "queued"], list(out)))

    def __del__(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.pv_ddmod_destroy(self.h)
            self.h = C.c_void_p()


# ---------------------------------------------------------------------------
# serving loop (pv_serve)
# ---------------------------------------------------------------------------

SERVE_BATCH, SERVE_FIFO1 = 0, 1


class ServeConfig(C.Structure):
    _fields_ = [("budget_bytes", C.c_double), ("policy", C.c_int), ("batch_flags", C.c_int),
                ("max_inflight", C.c_int), ("admit_every", C.c_double), ("horizon", C.c_double),
                ("reuse_slots", C.c_int), ("linger", C.c_double)]


class ServeStream(C.Structure):
    _fields_ = [("nchunks", C.c_int), ("arrivals", C.POINTER(C.c_double)), ("sizes", C.POINTER(C.c_int)),
                ("h_voltages", C.c_void_p), ("units_per_spectrum", C.c_double)]


class ServeStats(C.Structure):
    _fields_ = [(n, C.c_longlong) for n in ("chunks", "chunks_done", "cohorts", "slot_reuses", "steps")] + \
               [("max_concurrent_beams", C.c_int)] + \
               [(n, C.c_double) for n in ("wall_s", "units", "throughput", "latency_p50", "latency_p99",
                                          "latency_max", "latency_admitted_p50", "latency_admitted_p99",
                                          "latency_over_duration_p50", "latency_over_duration_p99",
                                          "within_real_time", "admission_wait_p50", "admission_wait_p99",
                                          "peak_footprint_bytes")]


_FOOT = C.CFUNCTYPE(C.c_longlong, C.c_void_p, C.c_void_p)
_OPEN = C.CFUNCTYPE(C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.c_int)
_STEP = C.CFUNCTYPE(C.c_longlong, C.c_void_p, C.c_void_p, C.POINTER(C.c_ubyte), C.c_int)
_DONE = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_longlong)
_RESET = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int)
_CLOSE = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p)
_CLOCK = C.CFUNCTYPE(C.c_double, C.c_void_p)
_SLEEP = C.CFUNCTYPE(None, C.c_void_p, C.c_double)
_EVENTS = C.CFUNCTYPE(C.c_longlong, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p, C.c_longlong,
                      C.POINTER(C.c_longlong))
_OUTPUT = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_longlong, C.c_void_p, C.c_longlong, C.c_longlong)


class ServeEngine(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("footprint", _FOOT), ("open", _OPEN), ("step", _STEP), ("done", _DONE),
                ("reset_slot", _RESET), ("close", _CLOSE), ("clock", _CLOCK), ("sleep", _SLEEP),
                ("events", _EVENTS)]


class ServeOutput(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("events", _OUTPUT)]


def _engine_hooks(eng):
    """C hooks over a Python engine with footprint(cfg), open(cfgs, ids) ->
    cohort, step(cohort, active) -> id, done(cohort, id), reset_slot(cohort,
    slot, stream), close(cohort), clock() and sleep(s); cohorts are kept by
    handle number."""
    cohorts, nxt = {}, [1]

    def foot(ctx, cfg):
        return int(eng.footprint(C.cast(cfg, C.POINTER(BeamConfig)).contents))

    def open_(ctx, cfgs, ids, n):
        arr = C.cast(cfgs, C.POINTER(BeamConfig))
        c = eng.open([arr[k] for k in range(n)], [ids[k] for k in range(n)])
        if c is None:
            return None
        h = nxt[0]
        nxt[0] += 1
        cohorts[h] = c
        return h

    def step(ctx, h, active, n):
        return int(eng.step(cohorts[h], np.ctypeslib.as_array(active, (n,)).copy()))

    def done(ctx, h, i):
        return 1 if eng.done(cohorts[h], i) else 0

    def reset(ctx, h, slot, stream):
        return int(eng.reset_slot(cohorts[h], slot, stream))

    def close(ctx, h):
        eng.close(cohorts.pop(h))

    hooks = ServeEngine(None, _FOOT(foot), _OPEN(open_), _STEP(step), _DONE(done), _RESET(reset), _CLOSE(close),
                        _CLOCK(lambda ctx: float(eng.clock())), _SLEEP(lambda ctx, dt: eng.sleep(dt)), _EVENTS(0))
    return hooks


def serve(configs, streams, budget_bytes, policy="batch", batch_flags=None, max_inflight=2, admit_every=0.5,
          horizon=0.0, reuse_slots=True, linger=2.0, engine=None, on_events=None):
    """pv_serve: configs[i] (BeamConfig) is stream i's beam; streams[i] a dict
    with arrivals (s), sizes (spectra), voltages (a HostBuffer with one
    sub-chunk, or None with an engine) and units_per_spectrum.  engine (for
    tests) replaces the GPU and the clock.  Returns the statistics as a dict."""
    n = len(configs)
    cfg_arr = (BeamConfig * n)(*configs)
    keep = []
    st_arr = (ServeStream * n)()
    for i, s in enumerate(streams):
        a = np.ascontiguousarray(s["arrivals"], np.float64)
        z = np.ascontiguousarray(s["sizes"], np.int32)
        keep += [a, z]
        v = s.get("voltages")
        st_arr[i] = ServeStream(len(a), a.ctypes.data_as(C.POINTER(C.c_double)), z.ctypes.data_as(C.POINTER(C.c_int)),
                                C.c_void_p(v.ptr) if v is not None else None, float(s["units_per_spectrum"]))
    if batch_flags is None:
        batch_flags = BATCH_GRAPH | BATCH_PIPELINED
    sc = ServeConfig(float(budget_bytes), SERVE_BATCH if policy == "batch" else SERVE_FIFO1, int(batch_flags),
                     int(max_inflight), float(admit_every), float(horizon), int(bool(reuse_slots)), float(linger))
    out = ServeStats()
    hooks = _engine_hooks(engine) if engine is not None else None
    output = None
    if on_events is not None:  # on_events(stream, first_sample, events array, total)
        def _out(ctx, stream, first, ev, nev, total):
            arr = np.ctypeslib.as_array(C.cast(ev, C.POINTER(C.c_int32)), (int(nev) * 4,)).view(EVENT_DTYPE).copy()
            on_events(int(stream), int(first), arr, int(total))
        output = ServeOutput(None, _OUTPUT(_out))
    check(load().pv_serve(C.byref(sc), cfg_arr, st_arr, n, C.byref(hooks) if hooks is not None else None,
                          C.byref(output) if output is not None else None, C.byref(out)))
    return {f: getattr(out, f) for f, _ in ServeStats._fields_}
