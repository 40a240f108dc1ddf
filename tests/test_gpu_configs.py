"""Parity at the workloads' own sizes.

* Plain single beam: 32 LOFAR subbands from 140 MHz, dual-polarisation
  complex int16 at 5.12 us, 65536 samples per subband per chunk, an 8-tap
  Hamming PPF to 16 channels (512 channels, 81.92 us), Stokes I, x4
  integration (1024 spectra of 327.68 us per chunk), RFI_Clipper at 5 sigma,
  512 trials over DM 0-100, events at 6 sigma; seeded noise (sigma 16) and
  one dispersed pulse at DM 56.8, 1 ms wide, peak S/N about 15.  Ten chunks
  stream through pv_beam (the first window comes out after the sixth).
* Full band: 244 subbands from 110 MHz (3904 channels), 16384 spectra per
  chunk, 2048 trials over DM 0-500; 3 % of the channels carry narrowband
  sinusoids at 20 sigma, broadband bursts arrive about once per 10^4 spectra
  and ten dispersed pulses (DM 10-500, 0.5-5 ms) are injected.  Two chunks
  stream through a prefilled pv_beam; the full 2048 x 3904 x 16384 window is
  dedispersed and analysed.  A third test dedisperses a full window of a
  synthetic normalised filterbank holding ten dispersed pulses.

Every stage is checked against the oracle:
  - channeliser: within 1e-4 of the mean power (FFT rounding is free);
  - clipper: bit-exact (data and flags) against the oracle's FP64-baseline
    restatement, the library's arithmetic; and against the reference's own
    FP32 arithmetic (RFI_Clipper.cpp:315-342,415-438) every channel and
    spectrum decision is equal except where the reference's decision
    statistic lies within EPS_CHAN (channel: |(I - dataModel - bp) -
    margin| in units of rmsRunAve) or EPS_SPEC (spectrum: |(mean -
    meanRunAve) - tolerance| in units of bandpass rms / sqrt(nBins)) of its
    threshold; the oracle follows the library's decision at such points so
    that every later decision is still compared; normalised values agree to
    1e-4 except those within EPS_NORM of crFactor, which the final clip
    (I > crFactor => 0) may zero in one run only;
  - dedispersion: bit-exact against the oracle's FP32 sum of the library's
    filterbank, and within MAX_REL_FP64 of the FP64 sum (relative to
    max(|x|, sqrt(nchan)), the noise of a sum of nchan unit-variance
    channels);
  - analyser: events bit-exact against the oracle on the same spectra; events
    of the reference-arithmetic chain equal except those within EPS_EVENT
    (relative) of their width's threshold;
  - the injected pulses are found at their trial and sample.
"""
import numpy as np
import pytest

from gen import lofar_band, lofar_stream, make_bp_text

pytestmark = pytest.mark.gpu

EPS_CHAN = 1e-3     # channel clip statistic, units of rmsRunAve
EPS_SPEC = 1e-2     # spectrum rejection statistic, units of bandpass rms / sqrt(nBins)
EPS_EVENT = 1e-4    # event value, relative to its threshold
EPS_NORM = 1e-4     # normalised value against crFactor (the final clip), relative
MAX_REL_FP64 = 1e-3  # dedispersed power against the FP64 sum
K_DM = 4148.741601


def _events_map(ev):
    return {(int(e["dm"]), int(e["t"]), float(e["bin_factor"])): float(e["value"]) for e in ev[1:]}


def events_match_except_near(got, want, thr, eps=EPS_EVENT):
    """Events present in one list only must lie within eps (relative) of the
    threshold of their width; common events agree to 1e-3 of it.  Returns
    the number of near-threshold differences."""
    g, w = _events_map(got), _events_map(want)
    near = 0
    for k in set(g) ^ set(w):
        v = g.get(k, w.get(k))
        t = float(thr[int(round(np.log2(k[2])))])
        assert abs(v - t) <= eps * t, ("event beyond epsilon of its threshold", k, v, t)
        near += 1
    for k in set(g) & set(w):
        t = float(thr[int(round(np.log2(k[2])))])
        assert abs(g[k] - w[k]) <= 1e-3 * t, (k, g[k], w[k])
    return near


def fp64_rel_error(got, f64, nchan):
    fin = np.isfinite(f64)
    assert np.array_equal(fin, np.isfinite(got))
    scale = np.maximum(np.abs(f64[fin]), np.sqrt(nchan))
    return float(np.max(np.abs(got[fin] - f64[fin]) / scale)) if fin.any() else 0.0


class Stream:
    """One beam streamed through pv_beam and, beside it, through the oracle:
    the library's arithmetic (FP64-baseline clipper, bit-exact) and the
    reference's (FP32 clipper guided within epsilon)."""

    def __init__(self, pv, oracle, cuda, nsub, nch, f_sub0, chunk, tdms, dm_max, window, bp,
                 cr=5.0, sr=4.0, history=10000, prefilled=0):
        self.pv, self.oracle, self.cuda = pv, oracle, cuda
        self.nsub, self.nch, self.chunk, self.tdms = nsub, nch, chunk, tdms
        self.nbins = nsub * nch
        self.fch1, self.foff = lofar_band(f_sub0, nsub, nch)
        self.tsamp = 5.12e-6 * nch * 4
        kw = dict(nsub=nsub, nchan_sub=nch, window=window, fch1=self.fch1, foff=self.foff, tsamp=self.tsamp,
                  tdms=tdms, dm_step=dm_max / (tdms - 1), chunk=chunk, threshold=6.0, bp_text=bp, cr=cr,
                  sr=sr, history=history, zero_dming=1, debug_taps=1, prefilled=prefilled)
        self.beam = pv.Beam(pv.beam_config(**kw))
        info = self.beam.info()
        self.lag, self.max_shift = info["lag"], info["max_shift"]
        self.prefilled = prefilled
        self.k, inv = oracle.dm_shifts(self.fch1, self.foff, self.nbins)
        assert inv and info["inverted"] == 1
        self.start = np.float32(0.0) / np.float32(self.tsamp)
        self.step = np.float32(np.float32(dm_max / (tdms - 1))) / np.float32(self.tsamp)
        assert self.max_shift == oracle.shift_table(self.k, tdms, self.start, self.step).max()
        coeffs = oracle.fir_coefficients(8, nch, window).astype(np.float32)
        self.ppf = oracle.PPF(nch, 8, coeffs)
        parts = pv.load().pv_rfi_parts(self.nbins)
        rk = dict(cr=cr, sr=sr, history=history, zero_dming=True)
        self.g_rfi = pv.RFI(bp, **rk)                   # the library's clipper, standalone, for its flags
        self.o_rfi1 = oracle.RFI(bp, mode=1, parts=parts, **rk)
        self.o_rfi0 = oracle.RFI(bp, mode=0, **rk)      # the reference's arithmetic
        self.rms = float(np.sqrt(np.float32(nch) * np.float32(nsub)))
        self.thr = oracle.thresholds(6.0, self.rms, 6)
        self.cr = cr
        self.post, self.ref0 = [], []                   # clipped filterbanks [t][nbins]
        self.flags = []                                 # the library's clipper flags [t][nbins]
        self.report = {"chan_decisions": 0, "chan_near": 0, "chan_mismatch": 0, "chan_near_max": 0.0,
                       "spec_decisions": 0, "spec_near": 0, "spec_mismatch": 0, "spec_near_max": 0.0,
                       "chan_closest": np.inf, "spec_closest": np.inf}
        self.windows, self.events, self.max_fp64, self.near_events = 0, [], 0.0, 0

    def feed(self, v16):
        """One chunk of int16 voltages [sub][2][n][2]."""
        import torch
        pv, o = self.pv, self.oracle
        nsub, nch, chunk = self.nsub, self.nch, self.chunk
        self.beam.process(torch.from_numpy(v16).to(self.cuda))
        torch.cuda.synchronize()
        fb_p, raw_p, out_p, _ = self.beam.buffers()
        raw = pv.device_array(raw_p, (chunk, nsub, 1, nch)).cpu().numpy()
        post = pv.device_array(fb_p, (chunk, nsub, 1, nch)).cpu().numpy()
        # channeliser against the oracle (FP32 FFT against the oracle's FP64 FFT): tolerance
        vc = (v16[..., 0].astype(np.float32) + 1j * v16[..., 1].astype(np.float32)).astype(np.complex64)
        want_raw = o.integrate(o.stokes(self.ppf.run(vc.reshape(nsub, 2, chunk * 4, nch)), 1), 4, 1)
        del vc
        assert np.max(np.abs(raw - want_raw)) <= 1e-4 * float(want_raw.mean())
        # the standalone clipper equals the beam's, and gives the flags
        x = torch.from_numpy(raw.copy()).to(self.cuda)
        gflags = self.g_rfi.run(x, flags=True).cpu().numpy()
        assert np.array_equal(x.cpu().numpy(), post)
        # library arithmetic: bit-exact data and flags
        d1 = raw.copy()
        f1 = self.o_rfi1.run(d1, flags=True)
        assert np.array_equal(d1, post)
        assert np.array_equal(f1, gflags)
        # reference arithmetic, guided within epsilon
        d0 = raw.copy()
        _, rep = self.o_rfi0.run_guided(d0, gflags, EPS_CHAN, EPS_SPEC)
        for key in ("chan_decisions", "chan_near", "chan_mismatch", "spec_decisions", "spec_near",
                    "spec_mismatch"):
            self.report[key] += int(rep[key])
        for key in ("chan_near_max", "spec_near_max"):
            self.report[key] = max(self.report[key], rep[key])
        for key in ("chan_closest", "spec_closest"):
            self.report[key] = min(self.report[key], rep[key])
        assert rep["chan_mismatch"] == 0 and rep["spec_mismatch"] == 0, rep
        fin = np.isfinite(post)
        assert np.array_equal(fin, np.isfinite(d0))
        # the last clip of a kept spectrum, I > crFactor => 0 (RFI_Clipper.cpp:528-530), is a
        # threshold too: a value within EPS_NORM of crFactor may be 0 in one run only
        a, b = d0[fin], post[fin]
        near_cr = ((a == 0) & (np.abs(b - self.cr) <= EPS_NORM * self.cr)) | \
                  ((b == 0) & (np.abs(a - self.cr) <= EPS_NORM * self.cr))
        self.report["norm_clip_near"] = self.report.get("norm_clip_near", 0) + int(near_cr.sum())
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1.0)
        assert np.max(rel[~near_cr], initial=0.0) <= 1e-4
        self.flags.append(gflags)
        self.post.append(post.reshape(chunk, -1))
        self.ref0.append(d0.reshape(chunk, -1))
        # a window comes out once the ring holds its delays
        ck = len(self.post) - 1
        if ck >= (0 if self.prefilled else self.lag):
            w = ck if self.prefilled else ck - self.lag
            got = pv.device_array(out_p, (self.tdms, chunk)).cpu().numpy()
            ev, n, first = self.beam.events()
            assert first == w * chunk
            self._check_window(w, got, ev, n)

    def _buffer(self, hist, w):
        """Band-inverted [nbins][chunk + max_shift + 1] buffer of window w."""
        base = self.lag * self.chunk if self.prefilled else 0
        lo, hi = w * self.chunk, (w + 1) * self.chunk + self.max_shift + 1
        buf = np.zeros((hi - lo, self.nbins), np.float32)
        data = np.concatenate(hist, axis=0)
        a, b = max(lo, base), min(hi, base + data.shape[0])
        if b > a:
            buf[a - lo:b - lo] = data[a - base:b - base]
        return np.ascontiguousarray(buf[:, ::-1].T)

    def _check_window(self, w, got, ev, n):
        o = self.oracle
        buf = self._buffer(self.post, w)
        want = o.dedisperse(buf, self.chunk, self.tdms, self.k, self.start, self.step)
        assert np.array_equal(got, want, equal_nan=True)
        f64 = o.dedisperse(buf, self.chunk, self.tdms, self.k, self.start, self.step, f64=True)
        self.max_fp64 = max(self.max_fp64, fp64_rel_error(got, f64, self.nbins))
        assert self.max_fp64 <= MAX_REL_FP64
        want_ev = o.analyse(want, 6.0, self.rms, 6)
        assert n == len(want_ev) and np.array_equal(ev, want_ev.astype(ev.dtype))
        # the reference-arithmetic chain
        ref = o.dedisperse(self._buffer(self.ref0, w), self.chunk, self.tdms, self.k, self.start, self.step)
        self.near_events += events_match_except_near(ev, o.analyse(ref, 6.0, self.rms, 6), self.thr)
        self.events.append((w * self.chunk, ev))
        self.windows += 1

    def best_event(self):
        """(S/N, dm index, absolute sample) of the strongest event."""
        best = (-np.inf, -1, -1)
        for first, ev in self.events:
            for e in ev[1:]:
                snr = float(e["value"]) / (self.rms * np.sqrt(float(e["bin_factor"])))
                if np.isfinite(snr) and snr > best[0]:
                    best = (snr, int(e["dm"]), first + int(e["t"]))
        return best


def test_plain_single_beam_stream_full_size(pv, oracle, cuda):
    """32 subbands x 65536 samples per chunk, ten chunks, the DM 56.8 pulse."""
    nsub, nch, chunk, tdms, dm_max = 32, 16, 1024, 512, 100.0
    raw = chunk * 4 * nch
    nchunks = 10
    t0, dm = 0.9, 56.8  # the pulse reaches the top channel 0.9 s into the stream
    rng = np.random.default_rng(20260514)
    v = lofar_stream(rng, nsub, raw * nchunks, 140.0, nch, pulses=[(dm, t0, 1e-3, 0.52)])
    fch1, foff = lofar_band(140.0, nsub, nch)
    level = 245.0  # mean Stokes-I power of one channel of this chain at sigma 16
    bp = make_bp_text(nsub * nch, fch1, foff, level, level / np.sqrt(8.0))
    s = Stream(pv, oracle, cuda, nsub, nch, 140.0, chunk, tdms, dm_max, "hamming", bp)
    assert s.lag == 6
    for ck in range(nchunks):
        s.feed(np.ascontiguousarray(v[:, :, ck * raw:(ck + 1) * raw]))
    assert s.windows == nchunks - s.lag
    r = s.report
    assert r["chan_decisions"] == nchunks * chunk * nsub * nch and r["spec_decisions"] == nchunks * chunk
    assert r["chan_mismatch"] == 0 and r["spec_mismatch"] == 0
    snr, d_best, t_best = s.best_event()
    step = dm_max / (tdms - 1)
    assert abs(d_best - dm / step) <= 2.0, (d_best, dm / step)
    assert abs(t_best - t0 / s.tsamp) <= 16, (t_best, t0 / s.tsamp)
    assert 10.0 <= snr <= 25.0, snr
    print("plain single beam: clipper vs reference arithmetic", r, "fp64 max rel", s.max_fp64,
          "near-threshold events", s.near_events, "best event S/N %.2f dm %d t %d" % (snr, d_best, t_best))


def fullband_chunk(gen, nsub, nch, n, chans, ck, pulses, device):
    """Chunk ck of the full-band stream as int16 voltages [sub][2][n][2],
    generated on the device from the seeded generator gen and copied to the
    host: Gaussian noise (sigma 16), sinusoids at the centres of the
    narrowband channels `chans` at 20 sigma of integrated power, broadband
    bursts (4x the noise power for one spectrum) about once per 10^4 spectra,
    and pulses (dm, t0 at the top channel in stream seconds, FWHM width,
    scale): complex noise of scale x the noise variance under a Gaussian
    envelope centred at each subband's delay, widened by the subband's own
    dispersion sweep."""
    import torch
    sigma, tsr, sub_bw = 16.0, 5.12e-6, 0.1953125
    v = torch.randn((nsub, 2, n, 2), generator=gen, device=device, dtype=torch.float32) * sigma
    t_off = ck * n * tsr
    t = t_off + torch.arange(n, device=device, dtype=torch.float64) * tsr
    # a tone of amplitude a * sigma in both polarisations adds a^2 * 2 sigma^2 of power to its channel;
    # 20 sigma of a 16-degree-of-freedom chi-square power is 20 / sqrt(8) = 7.1 times its mean
    amp = float(np.sqrt(20.0 / np.sqrt(8.0))) * sigma
    for g in chans:
        sb, c = divmod(int(g), nch)
        nu = (c - nch // 2) * (sub_bw / nch) * 1e6
        ph = 2 * np.pi * nu * t + (int(g) * 0.7548776662 % 1.0) * 2 * np.pi
        v[sb, :, :, 0] += (amp * torch.cos(ph)).float()
        v[sb, :, :, 1] += (amp * torch.sin(ph)).float()
    spectra = n // (4 * nch)
    nb = max(1, int(round(spectra / 1e4)))
    starts = torch.randint(0, n - 4 * nch, (nb,), generator=gen, device=device).tolist()
    for b0 in starts:
        v[:, :, b0:b0 + 4 * nch, :] *= 2.0
    f_top = lofar_band(110.0, nsub, nch)[0] + (sub_bw / nch) * (nsub * nch - 1)
    for dm, t0, width, scale in pulses:
        for sb in range(nsub):
            fc = 110.0 + sb * sub_bw
            tc = t0 + K_DM * dm * (1 / fc ** 2 - 1 / f_top ** 2) - t_off
            sweep = K_DM * dm * (1 / (fc - sub_bw / 2) ** 2 - 1 / (fc + sub_bw / 2) ** 2)
            sig = np.hypot(width, sweep) / 2.3548
            lo, hi = int((tc - 4 * sig) / tsr), int((tc + 4 * sig) / tsr) + 1
            lo, hi = max(lo, 0), min(hi, n)
            if hi <= lo:
                continue
            tt = torch.arange(lo, hi, device=device, dtype=torch.float32) * tsr
            env = torch.exp(-0.5 * ((tt - tc) / sig) ** 2) * float(np.sqrt(scale) * sigma)
            v[sb, :, lo:hi, :] += torch.randn((2, hi - lo, 2), generator=gen, device=device) * env[None, :, None]
    return torch.clamp(torch.round(v), -32768, 32767).to(torch.int16).cpu().numpy()


def test_fullband_beam_two_chunks_full_size(pv, oracle, cuda):
    """244 subbands, 16384 spectra per chunk, 2048 trials; narrowband RFI,
    bursts and pulses; two chunks into a prefilled ring."""
    nsub, nch, chunk, tdms, dm_max = 244, 16, 16384, 2048, 500.0
    n = chunk * 4 * nch
    nbins = nsub * nch
    fch1, foff = lofar_band(110.0, nsub, nch)
    level = 245.0
    bp = make_bp_text(nbins, fch1, foff, level, level / np.sqrt(8.0))
    s = Stream(pv, oracle, cuda, nsub, nch, 110.0, chunk, tdms, dm_max, "kaiser", bp, prefilled=1)
    import torch
    rng = np.random.default_rng(244)
    chans = np.sort(rng.choice(nbins, size=int(0.03 * nbins), replace=False))
    pulses = [(float(rng.uniform(10, 500)), float(rng.uniform(0.05, 10.0)), float(rng.uniform(0.5e-3, 5e-3)),
               0.5) for _ in range(10)]
    gen = torch.Generator(device=cuda)
    gen.manual_seed(244)
    for ck in range(2):
        v = fullband_chunk(gen, nsub, nch, n, chans, ck, pulses, cuda)
        s.feed(v)
        del v
    r = s.report
    assert s.windows == 2
    assert r["chan_mismatch"] == 0 and r["spec_mismatch"] == 0
    # the narrowband channels are clipped in the spectra the clipper keeps after its warm-up
    fl = np.concatenate(s.flags, axis=0)[1000:]
    kept = (fl[:, 0] & 2) == 0
    clipped = (fl[kept] & 1) != 0
    rfi = np.zeros(nbins, bool)
    rfi[chans] = True
    per_channel = clipped[:, rfi].mean(axis=0)
    print("narrowband channels: clipped in %.3f of kept spectra (median over channels %.3f, lowest %.3f); "
          "other channels %.5f" % (clipped[:, rfi].mean(), np.median(per_channel), per_channel.min(),
                                   clipped[:, ~rfi].mean()))
    # (measured: 0.885 of the kept spectra for every narrowband channel, none for the others)
    assert kept.mean() > 0.9
    assert np.median(per_channel) > 0.8 and clipped[:, ~rfi].mean() < 0.01
    print("full band: clipper vs reference arithmetic", r, "fp64 max rel", s.max_fp64,
          "near-threshold events", s.near_events)


def test_fullband_window_dedispersion_finds_pulses(pv, oracle, cuda):
    """A full 2048-trial window of 3904 channels x 16384 samples (ring
    rows, the pv_beam path's kernel) over a normalised filterbank with ten
    dispersed pulses: bit-exact against the FP32 oracle, within 1e-3 of
    FP64, events bit-exact, every pulse found at its trial and sample."""
    import torch
    nsub, nch, nout, tdms, dm_max = 244, 16, 16384, 2048, 500.0
    nbins = nsub * nch
    fch1, foff = lofar_band(110.0, nsub, nch)
    tsamp = 5.12e-6 * nch * 4
    k, inv = oracle.dm_shifts(fch1, foff, nbins)  # highest channel first
    start = np.float32(0.0) / np.float32(tsamp)
    step = np.float32(np.float32(dm_max / (tdms - 1))) / np.float32(tsamp)
    plan = pv.DedispPlan(k, tdms, start, step)
    ms = plan.max_shift()
    ld = (nout + ms + 8 + 3) & ~3  # 16-byte rows: the TMA pipeline kernel
    rng = np.random.default_rng(3904)
    buf = rng.standard_normal((nbins, ld), dtype=np.float32)
    table = oracle.shift_table(k, tdms, start, step)
    pulses = []
    for j in range(10):
        d = int(rng.integers(40, tdms - 40))
        t = int(rng.integers(64, nout - 64))
        width = int(rng.integers(2, 16))
        amp = np.float32(15.0 / np.sqrt(nbins * width))  # S/N about 15 in a box of the pulse's width
        for c in range(nbins):
            p = t + table[d, c]
            buf[c, p:p + width] += amp
        pulses.append((d, t, width))
    # ring rows: the same samples rotated so that output 0 reads from column t_base
    ring_len = ld
    t_base = 12345
    ring = np.roll(buf, t_base, axis=1)
    d_ring = torch.from_numpy(ring).to(cuda)
    got = plan.run(d_ring, nout, ring_len=ring_len, t_base=t_base).cpu().numpy()
    assert plan.status() == 0
    want = oracle.dedisperse(buf, nout, tdms, k, start, step)
    assert np.array_equal(got, want)
    f64 = oracle.dedisperse(buf, nout, tdms, k, start, step, f64=True)
    err = fp64_rel_error(got, f64, nbins)
    assert err <= MAX_REL_FP64
    rms = float(np.sqrt(np.float32(nch) * np.float32(nsub)))
    ev, n = pv.analyse(torch.from_numpy(got).to(cuda), 6.0, rms, 6)
    want_ev = oracle.analyse(want, 6.0, rms, 6)
    assert n == len(want_ev) and np.array_equal(ev, want_ev.astype(ev.dtype))
    evm = _events_map(ev)
    for d, t, width in pulses:
        near = [(v / (rms * np.sqrt(key[2])), key) for key, v in evm.items()
                if abs(key[0] - d) <= 1 and key[1] <= t + width and key[1] + key[2] >= t]
        assert near, (d, t, width)
        assert max(near)[0] >= 8.0, (d, t, width, max(near))
    print("full-band window: fp64 max rel %.2e, %d events" % (err, n))
