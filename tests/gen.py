"""Seeded synthetic inputs shared by the tests.

``generator_pulse`` restates the reference's test fixture
DedispersionDataGenerator::generate (lib/test/src/DedispersionDataGenerator.cpp:26-81):
32 subbands x 64 channels from 150 MHz with foff = -6/2048 MHz, 327.68 us
samples, value 1.0 inside a 10-sample dispersed track and 0 elsewhere.
"""
import numpy as np

GEN_NSUB, GEN_NCHAN = 32, 64
GEN_FCH1 = 150.0
GEN_FOFF = -6.0 / (GEN_NSUB * GEN_NCHAN)
GEN_TSAMP = 0.00032768
GEN_WIDTH = 10


def generator_pulse(nsamples, dm, nblocks=1, nsub=GEN_NSUB, nchan=GEN_NCHAN, fch1=GEN_FCH1,
                    foff=None, tsamp=GEN_TSAMP, width=GEN_WIDTH, start_bin=0):
    """Blobs [t][sub][1][chan] float32, as the reference generator builds them."""
    if foff is None:
        foff = -6.0 / (nsub * nchan)
    dm = float(np.float32(dm))
    blobs = []
    for i in range(nblocks):
        I = np.zeros((nsamples, nsub, 1, nchan), np.float32)
        offset = i * nsamples
        for ac in range(nsub * nchan):
            f = fch1 + foff * ac
            index = int(dm * (4148.741601 * ((1.0 / f / f) - (1.0 / fch1 / fch1)) / tsamp)) + start_bin
            sample = index - offset
            s, c = divmod(ac, nchan)
            lo, hi = max(sample, 0), min(sample + width, nsamples)
            if hi > lo:
                I[lo:hi, s, 0, c] = 1.0
        blobs.append(I)
    return blobs


def dm_index(dm, dm_low, dm_step):
    """BinMap::binIndex with the float start/width of DedispersionSpectra::resize."""
    return int(0.5 + ((dm - float(np.float32(dm_low))) / float(np.float32(dm_step))))


def buffer_with_padding(rng, nchan, nout, max_shift, dist="normal"):
    """A [nchan][nout+max_shift+pad] float32 buffer of noise."""
    ld = nout + max_shift + 8
    if dist == "normal":
        return rng.standard_normal((nchan, ld), dtype=np.float32)
    return rng.random((nchan, ld), dtype=np.float32)


def make_bp_text(nbins, start, width, median, rms, coeffs=()):
    """A bandpass file in the BandPassAdapter format (BandPassAdapter.cpp:30-108):
    nChan, start, end, channel width, rms, then the polynomial coefficients
    starting with the median."""
    end = start + width * nbins
    lines = ["# synthetic bandpass", "%d" % nbins, repr(float(start)), repr(float(end)),
             repr(float(width)), repr(float(rms)), repr(float(median))]
    lines += [repr(float(c)) for c in coeffs]
    return "\n".join(lines) + "\n"


def voltages(rng, nsub, npol, nsamp, sigma=16.0):
    """Complex int16 dual-pol station voltages [sub][pol][nsamp][2] (Gaussian,
    rounded and saturated) and the same values as complex64."""
    v = rng.normal(0.0, sigma, size=(nsub, npol, nsamp, 2))
    v = np.clip(np.rint(v), -32768, 32767).astype(np.int16)
    c = (v[..., 0].astype(np.float32) + 1j * v[..., 1].astype(np.float32)).astype(np.complex64)
    return v, c


def stokes_filterbank(rng, nt, nsub, nchan, level=1000.0, dof=8, rfi_channels=0.03, burst_rate=2e-3,
                      shape=None):
    """Positive Stokes-I spectra [t][sub][1][chan]: level * chi^2_dof/dof noise,
    a fraction of channels with persistent narrowband RFI and occasional
    broadband bursts."""
    nbins = nsub * nchan
    base = np.full(nbins, level, np.float64) if shape is None else np.asarray(shape, np.float64)
    x = rng.gamma(dof / 2.0, 2.0 / dof, size=(nt, nbins)) * base
    bad = rng.random(nbins) < rfi_channels
    x[:, bad] *= 4.0
    bursts = rng.random(nt) < burst_rate
    x[bursts] *= 1.5
    return x.astype(np.float32).reshape(nt, nsub, 1, nchan)


def inject_dispersed_pulse(vc, sub_freq0, sub_bw, tsamp_raw, dm, t0, width, snr_scale, rng,
                           f_ref=None):
    """Adds a dispersed broadband burst to complex voltages vc [sub][pol][n]
    (in place, complex64).  The burst is complex Gaussian noise under a
    Gaussian envelope of FWHM `width` seconds arriving at t0 (seconds) at
    frequency f_ref and at t0 + k*DM*(f^-2 - f_ref^-2) at frequency f
    (k = 4148.741601).  In each subband the envelope is centred at the delay
    of the subband centre fc, and the rest of the delay,
    k*DM*(f^-2 - fc^-2), is applied in the Fourier domain as the group delay
    of a phase over the subband's baseband frequencies.  snr_scale is the
    burst's voltage variance relative to the noise at the envelope peak."""
    nsub, npol, n = vc.shape
    sigma_env = width / 2.3548
    if f_ref is None:
        f_ref = sub_freq0 + (nsub - 0.5) * sub_bw  # top of the band
    k_dm = 4148.741601
    noise_var = float(np.mean(np.abs(vc[:, :, : min(n, 4096)]) ** 2)) / 2.0
    for s in range(nsub):
        fc = sub_freq0 + s * sub_bw
        tc = t0 + k_dm * dm * (1 / fc ** 2 - 1 / f_ref ** 2)
        # in-subband delays relative to the centre: positive below fc, negative above
        lo_d = k_dm * dm * (1 / (fc + sub_bw / 2) ** 2 - 1 / fc ** 2)
        hi_d = k_dm * dm * (1 / (fc - sub_bw / 2) ** 2 - 1 / fc ** 2)
        a = tc + lo_d - 6 * sigma_env
        b = tc + hi_d + 6 * sigma_env
        if b / tsamp_raw <= 0 or a / tsamp_raw >= n:
            continue
        L = 1 << int(np.ceil(np.log2(max((b - a) / tsamp_raw, 16) * 2)))
        start = int(np.floor(a / tsamp_raw)) - L // 4
        t = (start + np.arange(L)) * tsamp_raw
        env = np.exp(-0.5 * ((t - tc) / sigma_env) ** 2)
        nu = np.fft.fftfreq(L, d=tsamp_raw) / 1e6  # MHz, baseband
        order = np.argsort(nu)
        f = fc + nu[order]
        delay = k_dm * dm * (1 / f ** 2 - 1 / fc ** 2)  # seconds, relative to the centre
        # phase whose frequency derivative gives the group delay
        dnu = (nu[1] - nu[0]) * 1e6
        phase = np.empty(L)
        phase[order] = -2 * np.pi * np.cumsum(delay) * dnu
        for p in range(npol):
            burst = (rng.standard_normal(L) + 1j * rng.standard_normal(L)) * np.sqrt(snr_scale * noise_var) * env
            disp = np.fft.ifft(np.fft.fft(burst) * np.exp(1j * phase))
            lo, hi = max(start, 0), min(start + L, n)
            if hi > lo:
                vc[s, p, lo:hi] += disp[lo - start:hi - start].astype(np.complex64)
    return vc


def ab_emulator_packets(npackets, channels, counter0=0, quarter0=0, beam=0, records=None, skip=()):
    """Packets as the reference's ABEmulator writes them (lib/test/src/ABEmulator.cpp:
    49-98): the header counter big-endian in bytes 0-5, the spectral quarter in
    byte 6 (0..3, the counter advancing after quarter 3), the beam in byte 7,
    then per channel four 16-bit values in host (little-endian) order: 42, 43,
    44, 45.  records (uint16 [npackets][channels][4]) replaces those values,
    written big-endian as the spectrometer sends them; packets whose index is
    in skip are left out (lost packets)."""
    psize = 8 + 8 * channels
    chunks = []
    counter, quarter = counter0, quarter0
    emu = np.tile(np.array((42, 43, 44, 45), "<i2"), channels).view(np.uint8)
    for p in range(npackets):
        if p not in skip:
            pk = np.zeros(psize, np.uint8)
            pk[:6] = np.frombuffer(counter.to_bytes(6, "big"), np.uint8)
            pk[6], pk[7] = quarter, beam
            pk[8:] = emu if records is None else np.asarray(records[p], ">u2").reshape(-1).view(np.uint8)
            chunks.append(pk)
        quarter = (quarter + 1) % 4
        if quarter == 0:
            counter += 1
    return np.concatenate(chunks) if chunks else np.zeros(0, np.uint8)


def lofar_band(f_sub0, nsub, nchan_sub, sub_bw=0.1953125):
    """Filterbank channel 0 frequency and channel width (MHz) of nsub LOFAR
    subbands from centre frequency f_sub0, channelised into nchan_sub
    channels each (the PPF puts the subband centre at channel nchan_sub/2)."""
    foff = sub_bw / nchan_sub
    return f_sub0 - (nchan_sub // 2) * foff, foff


def top_channel_freq(f_sub0, nsub, nchan_sub, sub_bw=0.1953125):
    """Frequency of the highest filterbank channel: the reference frequency
    of the dedispersion delays (the band is handled highest channel first)."""
    fch1, foff = lofar_band(f_sub0, nsub, nchan_sub, sub_bw)
    return fch1 + foff * (nsub * nchan_sub - 1)


def lofar_stream(rng, nsub, nsamp, f_sub0, nchan_sub, pulses=(), rfi_channels=(), rfi_amp=0.0,
                 bursts=(), burst_gain=0.0, burst_len=0, sigma=16.0, sub_bw=0.1953125,
                 tsamp_raw=5.12e-6, t_offset=0.0):
    """Dual-polarisation complex int16 station voltages [sub][pol][nsamp][2]:
    Gaussian noise (sigma per component), persistent narrowband sinusoids at
    the centre of the filterbank channels listed in rfi_channels (global
    channel index sub*nchan_sub + c, amplitude rfi_amp * sigma), broadband
    bursts (noise power raised by burst_gain over burst_len raw samples from
    each start in bursts) and dispersed pulses (dm, t0 at the top channel in
    seconds, FWHM width in seconds, snr_scale; see inject_dispersed_pulse),
    rounded and saturated to int16.  t_offset (seconds) is the stream time of
    sample 0: the sinusoids keep their phase across consecutive chunks."""
    v = rng.standard_normal((nsub, 2, nsamp, 2), dtype=np.float32) * np.float32(sigma)
    vc = (v[..., 0] + 1j * v[..., 1]).astype(np.complex64)
    del v
    f_ref = top_channel_freq(f_sub0, nsub, nchan_sub, sub_bw)
    for dm, t0, width, scale in pulses:  # before the RFI, which would raise the noise estimate
        inject_dispersed_pulse(vc, f_sub0, sub_bw, tsamp_raw, dm, t0, width, scale, rng, f_ref=f_ref)
    if len(rfi_channels):
        t = t_offset + np.arange(nsamp) * tsamp_raw
        for g in rfi_channels:
            s, c = divmod(int(g), nchan_sub)
            nu = (c - nchan_sub // 2) * (sub_bw / nchan_sub) * 1e6  # Hz from the subband centre
            phase = (int(g) * 0.7548776662 % 1.0) * 2 * np.pi + np.array([0.0, 1.0])  # fixed per channel
            for p in range(2):
                vc[s, p] += (rfi_amp * sigma * np.exp(1j * (2 * np.pi * nu * t + phase[p]))).astype(np.complex64)
    for b in bursts:
        lo, hi = int(b), min(int(b) + burst_len, nsamp)
        if hi > lo:
            extra = rng.standard_normal((nsub, 2, hi - lo, 2), dtype=np.float32) * np.float32(
                sigma * np.sqrt(burst_gain))
            vc[:, :, lo:hi] += (extra[..., 0] + 1j * extra[..., 1]).astype(np.complex64)
    out = np.empty((nsub, 2, nsamp, 2), np.int16)
    out[..., 0] = np.clip(np.rint(vc.real), -32768, 32767)
    out[..., 1] = np.clip(np.rint(vc.imag), -32768, 32767)
    return out


def lofar_packets(v16, ts0=1300000000, seq0=1000, spp=16, packet_bytes=8148):
    """Station voltages [sub][2][n][2] int16 as fixed-size 16-bit LOFAR UDP
    packets (16-byte header, data [subband][time][pol] complex int16,
    padding to packet_bytes; lib/LofarUdpHeader.h:25-35): n/spp packets."""
    nsub, npol, n, _ = v16.shape
    npk = n // spp
    data = np.ascontiguousarray(v16[:, :, :npk * spp].reshape(nsub, npol, npk, spp, 2).transpose(2, 0, 3, 1, 4))
    useful = nsub * spp * npol * 4
    chunk = np.zeros((npk, packet_bytes), np.uint8)
    hdr = np.zeros(npk, dtype=[("version", "u1"), ("source", "u1"), ("config", "<u2"), ("station", "<u2"),
                               ("beamlets", "u1"), ("blocks", "u1"), ("ts", "<u4"), ("seq", "<u4")])
    hdr["version"] = 3
    hdr["config"] = 16
    hdr["beamlets"] = nsub
    hdr["blocks"] = spp
    hdr["ts"] = ts0
    hdr["seq"] = seq0 + spp * np.arange(npk)
    chunk[:, :16] = hdr.view(np.uint8).reshape(npk, 16)
    chunk[:, 16:16 + useful] = data.reshape(npk, -1).view(np.uint8)
    return chunk.reshape(-1)
