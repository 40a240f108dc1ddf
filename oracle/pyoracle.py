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
            "or_rfi_run_guided": (i, [vp, P(C.c_float), P(C.c_float), i, i, i, i, vp, C.c_double,
                                      C.c_double, vp, P(C.c_double)]),
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
            "or_sigproc_pack": (ll, [P(C.c_float), i, i, i, i, i, i, f, f, vp]),
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

    def run_guided(self, data, hint, eps_chan, eps_spec):
        """run() following another implementation's flags where this run's
        decision statistic lies within eps of its threshold (or_rfi_run_guided).
        Returns (flags, report) with report a dict of counts and statistics."""
        assert data.dtype == np.float32 and data.flags.c_contiguous
        nt, nsub, npol, nchan = data.shape
        hint = np.ascontiguousarray(hint, dtype=np.uint8).reshape(nt, nsub * nchan)
        weights = np.ones_like(data)
        fl = np.zeros((nt, nsub * nchan), np.uint8)
        rep = np.zeros(12, np.float64)
        rc = lib().or_rfi_run_guided(self.h, _f32p(data), _f32p(weights), nt, nsub, npol, nchan,
                                     hint.ctypes.data, eps_chan, eps_spec, fl.ctypes.data, _f64p(rep))
        if rc != 0:
            raise RuntimeError("or_rfi_run_guided failed %d" % rc)
        keys = ("chan_decisions", "chan_near", "chan_mismatch", "chan_near_max", "spec_decisions",
                "spec_near", "spec_mismatch", "spec_near_max", "chan_closest", "spec_closest",
                "first_difference")
        return fl, {k: float(v) for k, v in zip(keys, rep)}

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


def ab_deserialise(chunk, packets_per_spectrum, channels, samples_per_packet, tsamp, state):
    """ABDataAdapter::deserialise (ABDataAdapter.cpp:44-173), packet by packet
    in Python.  Header bytes 0-5 are the integration count, most significant
    first (the reference reads 8 bytes little-endian, masks 48 bits and swaps
    them back); a packet's time is (count - start) * tsamp in double with
    tsamp a float, start being 0 for the very first packet and that packet's
    count afterwards; a time more than tsamp after the previous packet's is a
    gap.  Packets of quarter packets_per_spectrum - 3 (compared as unsigned)
    fill the next block with float(ntohs(XX) + ntohs(YY)) per channel.  The
    blob has (packets // packets_per_spectrum) * samples blocks (samples 0
    counts as 1); spectra past it are dropped, blocks not filled are 0.
    state: dict with seen, count0, last_time, updated in place.  Returns
    (spectra float32 [blocks][channels], timestamp, gaps, blocks filled)."""
    psize = 8 + 8 * channels
    raw = np.frombuffer(bytes(chunk), np.uint8)
    npk = len(raw) // psize
    nblocks = npk // packets_per_spectrum * (samples_per_packet if samples_per_packet > 0 else 1)
    out = np.zeros((nblocks, channels), np.float32)
    keep = (packets_per_spectrum - 3) & 0xFFFFFFFF
    ts = float(np.float32(tsamp))
    block, gaps, t = 0, 0, 0.0
    for p in range(npk):
        h = raw[p * psize:p * psize + 8]
        count = int.from_bytes(bytes(h[:6]), "big")
        start = state["count0"] if state["seen"] else 0
        t = float((count - start) & 0xFFFFFFFFFFFFFFFF) * ts
        if state["seen"]:
            if t - state["last_time"] > ts:
                gaps += 1
        else:
            state["count0"] = count
        if int(h[6]) == keep and block < nblocks:
            rec = raw[p * psize + 8:(p + 1) * psize].view(">u2").reshape(channels, 4)
            out[block] = (rec[:, 0].astype(np.int64) + rec[:, 1].astype(np.int64)).astype(np.float32)
            block += 1
        state["last_time"] = t
        state["seen"] += 1
    return out, t, gaps, block


# --------------------------------------------------------------------------
# F2 outputs: SigprocStokesWriter and DedispersionDataAnalysisOutput
# --------------------------------------------------------------------------

def sigproc_pack(stokes, npols_write, nbits, crop_min=0.0, crop_max=255.0):
    """Data block bytes of float32 [t][sub][pol][chan] (SigprocStokesWriter.cpp:187-236)."""
    x = np.ascontiguousarray(stokes, np.float32)
    nt, nsub, npol, nchan = x.shape
    out = np.zeros(nt * npols_write * nsub * nchan * (nbits // 8), np.uint8)
    n = lib().or_sigproc_pack(_f32p(x), nt, nsub, npol, nchan, npols_write, nbits, crop_min, crop_max,
                              out.ctypes.data)
    assert n == out.size
    return out


def sigproc_params(opts):
    """The header values SigprocStokesWriter's constructor derives from its XML
    options (SigprocStokesWriter.cpp:15-111), with the C++ expression types:
    float members, unsigned integer options, a double 0.5 and 1e6."""
    f32 = np.float32
    get = opts.get
    n_total = int(get("totalComplexSubbands", 1))
    clock = f32(get("clock", 200))
    integ = int(get("integrateTimeBins", 1))
    integ_f = int(get("integrateFrequencyChannels", 1))
    nchan = int(get("outputChannelsPerSubband", 128)) // integ_f
    nraw = int(get("nRawPolarisations", 2))
    top = int(f32(get("topSubbandIndex", 150)))      # float option into an unsigned member
    lbahba = int(f32(get("LBA_0_or_HBA_1", 1)))
    sbw = f32(clock / f32(nraw * n_total))
    cw = f32(sbw / f32(nchan))
    if get("fch1") is None:
        base = f32(sbw * f32(top))
        if lbahba == 0:
            fch1 = f32(float(base) + 0.5 * float(sbw) - 0.5 * float(cw))
        elif clock == 200:
            fch1 = f32(float(f32(f32(100) + base)) + 0.5 * float(sbw) - 0.5 * float(cw))
        else:
            fch1 = f32(float(f32(f32(160) + base)) + 0.5 * float(sbw) - 0.5 * float(cw))
    else:
        fch1 = f32(get("fch1"))
    foff = -cw if get("foff") is None else f32(get("foff"))
    if get("tsamp") is None:
        prod = (nraw * n_total * nchan * integ_f * integ) & 0xFFFFFFFF  # unsigned arithmetic
        tsamp = f32(float(f32(f32(prod) / clock)) / 1e6)
    else:
        tsamp = f32(get("tsamp"))
    ra_s, dec_s = str(get("RAJ", "000000.0")), str(get("DecJ", "000000.0"))
    name = ra_s[:4] + ("+" + dec_s[:4] if f32(dec_s) > 0 else dec_s[:5])
    nsub = int(get("subbandsPerPacket", 1))
    return dict(machine_id=int(get("MachineID", 9)), telescope_id=int(get("TelescopeID", 0)),
                nchans=nchan * nsub, nbits=int(get("dataBits", 32)), nifs=int(get("nPolsToWrite", 1)),
                src_raj=float(f32(ra_s)), src_dej=float(f32(dec_s)), fch1=float(fch1), foff=float(foff),
                tsamp=float(tsamp), source_name=name)


def sigproc_header(p, tstart):
    """Header bytes (SigprocStokesWriter.cpp:115-146)."""
    import struct

    def s(x):
        b = x.encode()
        return struct.pack("<i", len(b)) + b
    out = s("HEADER_START") + s("machine_id") + struct.pack("<i", p["machine_id"])
    out += s("telescope_id") + struct.pack("<i", p["telescope_id"]) + s("data_type") + struct.pack("<i", 1)
    out += s("source_name") + s(p["source_name"])
    for k in ("src_raj", "src_dej", "fch1", "foff"):
        out += s(k) + struct.pack("<d", p[k])
    out += s("nchans") + struct.pack("<i", p["nchans"]) + s("tsamp") + struct.pack("<d", p["tsamp"])
    out += s("nbits") + struct.pack("<i", p["nbits"]) + s("tstart") + struct.pack("<d", tstart)
    out += s("nifs") + struct.pack("<i", p["nifs"]) + s("HEADER_END")
    return out


EVENTS_TEXT_HEADER = ("# Generated by DedispersionDataAnalysisOutput\n# Events\n# ------\n"
                      "# Time|Dm|Amplitude|BinFactor\n# ------\n")


def events_text(events, start_timestamp, block_rate, first_sample, dm_low, dm_step, rms, dump_index):
    """DedispersionDataAnalysisOutput::sendStream for one buffer
    (DedispersionDataAnalysisOutput.cpp:80-112): QTextStream at precision 14
    prints reals like %.14g; SNR is value / (rms * sqrt(binFactor)) in double,
    stored as float."""
    f32 = np.float32
    lines, snr_max, dm_best = [], f32(0), f32(0)

    def t_of(t):
        return start_timestamp + float((int(t) + int(first_sample)) & 0xFFFFFFFF) * block_rate
    for e in events[1:]:
        mjd = t_of(e["t"]) / 86400
        dm = f32(dm_low + dm_step * int(e["dm"]))
        snr = f32(float(e["value"]) / (float(f32(rms)) * np.sqrt(float(e["bin_factor"]))))
        if snr > snr_max:
            dm_best, snr_max = dm, snr
        lines.append("%.14g,   %.14g, %.14g, %d\n" % (mjd, float(dm), float(snr), int(e["bin_factor"])))
    mjd0 = t_of(events[0]["t"] if len(events) else 0) / 86400
    lines.append("# Written buffer :%d | MJDstart: %.14g | Best DM: %.14g | Max SNR: %.14g  Done\n"
                 % (dump_index, mjd0, float(dm_best), float(snr_max)))
    return "".join(lines)


def trigger_message(events, start_timestamp, block_rate, first_sample, dm_low, dm_step, rms, min_events,
                    snr_threshold, station, id_root, message_number, cfreq_mhz, beam_ra, beam_dec):
    """TriggerOutput::_convertToTrigger_FRATS (TriggerOutput.cpp:151-183):
    with at least min_events events (the first, dummy one counts), the event
    of largest float SNR value / (rms * sqrt(binFactor)) wins (the running
    maximum starts at 0 with no event, since the reference leaves it unset;
    ties keep the first); at SNR >= threshold the message is built field by
    field with QString::arg(s, width, '0'), i.e. left-padded with '0'."""
    f32 = np.float32
    if len(events) < min_events:
        return None
    best, snr_max = None, f32(0)
    for e in events:
        snr = f32(e["value"]) / (f32(rms) * np.sqrt(f32(e["bin_factor"])))
        if snr > snr_max:
            best, snr_max = e, snr
    if best is None or not snr_max >= f32(snr_threshold):
        return None
    t = start_timestamp + float((int(best["t"]) + int(first_sample)) & 0xFFFFFFFF) * block_rate
    dm = f32(dm_low + dm_step * int(best["dm"]))
    return ("artemis:%s##ID:%s%s##cFreqMHz:%s##beamRA:%s##beamDec:%s##eTime:%s##eDM:%s##eSNR:%s"
            % (station, id_root, str(message_number).rjust(4, "0"), cfreq_mhz.rjust(10, "0"),
               beam_ra.rjust(10, "0"), beam_dec.rjust(9, "0"), ("%.9f" % t).rjust(20, "0"),
               ("%.3f" % float(dm)).rjust(9, "0"), ("%.2f" % float(snr_max)).rjust(6, "0")))


# --------------------------------------------------------------------------
# F3 BandPassRecorder
# --------------------------------------------------------------------------

def bandpass_record(chunks, required, ncoeffs, start, end, seg=256):
    """BandPassRecorder (BandPassRecorder.cpp:22-190) as it is meant to work:
    polarisation 0 of each float32 [t][sub][pol][chan] chunk is summed per
    channel (FP32 in time order within 256-spectrum segments of each call,
    the segments added in FP64) until `required` spectra; the mean spectrum
    is fitted by least squares in f^0..f^(n-1) (numpy lstsq), channels more
    than 2 residual RMS above the fit are set to the fit and the fit is
    repeated until none is.  Returns (coefficients, rms of the cleaned mean
    spectrum, channels trimmed) or None while more spectra are needed."""
    total, acc = 0, None
    for x in chunks:
        nt, nsub, npol, nchan = x.shape
        i = np.ascontiguousarray(x[:, :, 0, :].reshape(nt, nsub * nchan), np.float32)
        if acc is None:
            acc = np.zeros(nsub * nchan, np.float64)
        for t0 in range(0, nt, seg):
            part = np.cumsum(i[t0:t0 + seg], axis=0, dtype=np.float32)[-1]
            acc = acc + part.astype(np.float64)
        total += nt
        if total >= required and total > 0:
            break
    if acc is None or total < required:
        return None
    n = acc.size
    width = (float(np.float32(end)) - float(np.float32(start))) / n
    f = (float(np.float32(start)) + width * np.arange(n)).astype(np.float32).astype(np.float64)
    y = acc / total
    V = np.vander(f, ncoeffs, increasing=True)
    trimmed = 0
    for _ in range(1000):
        coef = np.linalg.lstsq(V, y, rcond=None)[0]
        res = y - V @ coef
        margin = 2.0 * np.sqrt(max(0.0, np.mean(res ** 2) - np.mean(res) ** 2))
        cut = res > margin
        trimmed += int(cut.sum())
        if not cut.any():
            break
        y = np.where(cut, V @ coef, y)
    rms = np.sqrt(max(0.0, np.mean(y ** 2) - np.mean(y) ** 2))
    return coef, float(rms), trimmed

