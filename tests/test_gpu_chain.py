"""K1 channeliser chain and K2/K3 RFI clipper on the GPU against the oracle,
through the C ABI."""
import numpy as np
import pytest

from gen import make_bp_text, stokes_filterbank, voltages

pytestmark = pytest.mark.gpu


def _ppf_pair(pv, oracle, nchan, ntaps, window):
    coeffs = oracle.fir_coefficients(ntaps, nchan, window).astype(np.float32)
    return pv.PPF(nchan, ntaps, coeffs=coeffs), oracle.PPF(nchan, ntaps, coeffs), coeffs


@pytest.mark.parametrize("nchan,ntaps,window", [(16, 8, "hamming"), (64, 8, "kaiser"),
                                                (512, 8, "kaiser"), (32, 4, "blackman")])
def test_ppf_matches_oracle(pv, oracle, cuda, nchan, ntaps, window):
    import torch
    rng = np.random.default_rng(nchan)
    nsub, npol, nblk = 5, 2, 48
    _, x = voltages(rng, nsub, npol, nblk * nchan)
    g, o, _ = _ppf_pair(pv, oracle, nchan, ntaps, window)
    got = g.run(torch.from_numpy(x).to(cuda)).cpu().numpy()
    want = o.run(x.reshape(nsub, npol, nblk, nchan))
    # FIR sums are bit-identical; the FFT is FP32 against the oracle's FP64,
    # so compare powers relative to the mean channel power.
    p_got, p_want = np.abs(got) ** 2, np.abs(want.astype(np.complex128)) ** 2
    assert np.max(np.abs(p_got - p_want)) <= 2e-5 * p_want.mean()
    assert np.max(np.abs(got - want)) <= 2e-5 * np.sqrt(p_want.mean())


@pytest.mark.parametrize("nchan,ntaps,window", [(24, 8, "kaiser"), (6, 4, "hamming"), (96, 8, "blackman")])
def test_ppf_even_channel_counts_match_oracle(pv, oracle, cuda, nchan, ntaps, window):
    """Even channel counts that are not powers of two (PPFChanneliser.cpp:42-44):
    the FIR as for the others, the transform a direct FP32 DFT against the
    oracle's FP64 one; spectra and Stokes I over two chunks (the tap history
    carried on the device)."""
    import torch
    rng = np.random.default_rng(nchan)
    nsub, npol, nblk = 3, 2, 40
    g, o, _ = _ppf_pair(pv, oracle, nchan, ntaps, window)
    for _ in range(2):
        _, x = voltages(rng, nsub, npol, nblk * nchan)
        got = g.run(torch.from_numpy(x).to(cuda)).cpu().numpy()
        want = o.run(x.reshape(nsub, npol, nblk, nchan))
        p_want = np.abs(want.astype(np.complex128)) ** 2
        assert np.max(np.abs(np.abs(got) ** 2 - p_want)) <= 2e-5 * p_want.mean()
        assert np.max(np.abs(got - want)) <= 2e-5 * np.sqrt(p_want.mean())


def test_ppf_single_channel_is_the_time_series(pv, oracle, cuda):
    """One channel: the spectra are the time samples, bit for bit."""
    import torch
    rng = np.random.default_rng(3)
    nsub, npol, nblk = 4, 2, 33
    _, x = voltages(rng, nsub, npol, nblk)
    g = pv.PPF(1, 8)
    got = g.run(torch.from_numpy(x).to(cuda)).cpu().numpy()
    want = oracle.PPF(1, 8, np.ones((8, 1), np.float32)).run(x.reshape(nsub, npol, nblk, 1))
    assert np.array_equal(got, want)


def test_ppf_history_is_continuous(pv, oracle, cuda):
    """Two calls carry the tap history: identical to one call over both."""
    import torch
    rng = np.random.default_rng(5)
    nchan, nsub, nblk = 16, 4, 40
    _, x = voltages(rng, nsub, 2, nblk * nchan)
    a, _, c = _ppf_pair(pv, oracle, nchan, 8, "hamming")
    b = pv.PPF(nchan, 8, coeffs=c)
    whole = a.run(torch.from_numpy(x).to(cuda)).cpu().numpy()
    first = b.run(torch.from_numpy(np.ascontiguousarray(x[:, :, :13 * nchan])).to(cuda)).cpu().numpy()
    second = b.run(torch.from_numpy(np.ascontiguousarray(x[:, :, 13 * nchan:])).to(cuda)).cpu().numpy()
    assert np.array_equal(np.concatenate([first, second]), whole)


def test_stokes_and_integrator_bit_exact(pv, oracle, cuda):
    import torch
    rng = np.random.default_rng(6)
    nt, nsub, nchan = 37, 6, 16
    spec = (rng.standard_normal((nt, nsub, 2, nchan)) + 1j * rng.standard_normal((nt, nsub, 2, nchan))).astype(np.complex64) * 40
    for nstokes in (1, 4):
        got = pv.stokes(torch.from_numpy(spec).to(cuda), nstokes).cpu().numpy()
        want = oracle.stokes(spec, nstokes)
        assert np.array_equal(got, want)
        for window, binc in [(4, 1), (3, 2), (50, 4), (1, 16)]:
            gi = pv.integrate(torch.from_numpy(want).to(cuda), window, binc).cpu().numpy()
            wi = oracle.integrate(want, window, binc)
            assert np.array_equal(gi, wi)


@pytest.mark.parametrize("nchan,nstokes,window,binc", [(16, 1, 4, 1), (64, 4, 4, 2), (16, 1, 16, 1)])
def test_fused_channeliser_bit_exact(pv, oracle, cuda, nchan, nstokes, window, binc):
    """int16 voltages -> PPF -> Stokes -> integration in one kernel equals the
    reference's Stokes and integrator applied to the GPU channeliser output."""
    import torch
    rng = np.random.default_rng(nchan + window)
    nsub, nblk = 7, 4 * 19 + 3
    v16, x = voltages(rng, nsub, 2, nblk * nchan)
    f, _, c = _ppf_pair(pv, oracle, nchan, 8, "kaiser")
    u = pv.PPF(nchan, 8, coeffs=c)
    for chunk in range(2):  # the history carries across calls in both paths
        fused = f.channelise(torch.from_numpy(v16.reshape(nsub, 2, -1)).to(cuda), nstokes, window,
                             binc).cpu().numpy()
        spec = u.run(torch.from_numpy(x).to(cuda)).cpu().numpy()
        want = oracle.integrate(oracle.stokes(spec, nstokes), window, binc)
        assert np.array_equal(fused, want)


@pytest.mark.parametrize("nchan,window,nblk,int16", [(16, 4, 4 * 150 + 3, True), (32, 8, 517, True),
                                                     (64, 4, 4 * 70, True), (16, 16, 300, False),
                                                     (64, 1, 9, True)])
def test_register_channeliser_equals_shared_memory_kernel(pv, oracle, cuda, monkeypatch, nchan, window,
                                                          nblk, int16):
    """The register/shuffle Stokes-I kernel (N = 16, 32, 64; 8 taps) and the
    shared-memory kernel agree bit for bit, over several block ranges per
    subband, ragged ends and two calls that carry the tap history."""
    import torch
    rng = np.random.default_rng(nchan * 7 + nblk)
    nsub = 5
    v16, x = voltages(rng, nsub, 2, nblk * nchan)
    coeffs = oracle.fir_coefficients(8, nchan, "kaiser").astype(np.float32)
    d_in = torch.from_numpy(v16.reshape(nsub, 2, -1) if int16 else x).to(cuda)
    outs = {}
    for mode in ("fast", "generic"):
        if mode == "generic":
            monkeypatch.setenv("PV_CHAN_GENERIC", "1")
        f = pv.PPF(nchan, 8, coeffs=coeffs)
        outs[mode] = [f.channelise(d_in, 1, window, 1).cpu().numpy() for _ in range(2)]
    for a, b in zip(outs["fast"], outs["generic"]):
        assert a.shape == (nblk // window, nsub, 1, nchan)
        assert np.array_equal(a, b)


BP_START, BP_WIDTH = 140.0, 0.01220703125


@pytest.mark.parametrize("case", [
    dict(coeffs=(), nbins_file=512, zero_dm=False, history=1200),
    dict(coeffs=(0.3, -0.0011), nbins_file=512, zero_dm=True, history=1100),
    dict(coeffs=(), nbins_file=256, zero_dm=False, history=1024),
])
def test_rfi_bit_exact_fp64_variant(pv, oracle, cuda, case):
    """GPU clipper == the oracle's FP64 variant: data, channel flags and
    spectrum flags, over two chunks (state carried on the device)."""
    import torch
    rng = np.random.default_rng(21)
    nt, nsub, nchan = 2300, 32, 16
    shape = None
    if case["coeffs"]:
        f = BP_START + BP_WIDTH * np.arange(512)
        shape = 1000.0 + 0.3 * f - 0.0011 * f * f
    data = stokes_filterbank(rng, nt, nsub, nchan, shape=shape)
    bp = make_bp_text(case["nbins_file"], BP_START, BP_WIDTH * 512 / case["nbins_file"], 1000.0, 50.0,
                      case["coeffs"])
    kw = dict(cr=5.0, sr=4.0, history=case["history"], zero_dming=case["zero_dm"])
    g = pv.RFI(bp, **kw)
    o = oracle.RFI(bp, mode=1, parts=pv.load().pv_rfi_parts(nsub * nchan), **kw)
    for sl in (slice(0, 1100), slice(1100, nt)):
        d = np.ascontiguousarray(data[sl])
        dd = torch.from_numpy(d).to(cuda)
        gf = g.run(dd, flags=True).cpu().numpy()
        of = o.run(d, flags=True)
        assert np.array_equal(gf, of)
        assert np.array_equal(dd.cpu().numpy(), d)
    assert np.array_equal(g.state()[[0, 1, 5, 6, 7, 8, 9]], o.state()[[0, 1, 5, 6, 7, 8, 9]])


def test_rfi_four_stokes_clips_all_polarisations(pv, oracle, cuda):
    import torch
    rng = np.random.default_rng(3)
    nt, nsub, nchan = 1300, 16, 16
    I = stokes_filterbank(rng, nt, nsub, nchan)
    data = np.concatenate([I, I * 0.1, I * 0.2, I * -0.3], axis=2)  # [t][sub][4][chan]
    bp = make_bp_text(256, BP_START, BP_WIDTH, 1000.0, 50.0)
    g = pv.RFI(bp, cr=5.0, history=1050)
    o = oracle.RFI(bp, cr=5.0, history=1050, mode=1)
    dd = torch.from_numpy(np.ascontiguousarray(data)).to(cuda)
    gf = g.run(dd, flags=True).cpu().numpy()
    d = np.ascontiguousarray(data)
    of = o.run(d, flags=True)
    assert np.array_equal(gf, of) and np.array_equal(dd.cpu().numpy(), d)



@pytest.mark.parametrize("split", [0, 1, 2])
@pytest.mark.parametrize("nsub,nchan", [(128, 16), (96, 64)])
def test_rfi_wide_bands_bit_exact(pv, oracle, cuda, nsub, nchan, split):
    """2048 and 6144 channels: 512 and 1024 partial sums per reduction, on
    one CTA (split 0) or spread over a cluster of CTAs (1: 4 x 256 threads
    for 1024 partials; 2: 4 or 8 x 128 threads)."""
    import torch
    rng = np.random.default_rng(nsub)
    nt = 1250
    nbins = nsub * nchan
    data = stokes_filterbank(rng, nt, nsub, nchan)
    bp = make_bp_text(nbins, BP_START, BP_WIDTH, 1000.0, 50.0)
    parts = pv.load().pv_rfi_parts(nbins)
    assert parts == (512 if nbins <= 4096 else 1024)
    g = pv.RFI(bp, cr=5.0, history=1100, split=split)
    o = oracle.RFI(bp, cr=5.0, history=1100, mode=1, parts=parts)
    dd = torch.from_numpy(np.ascontiguousarray(data)).to(cuda)
    gf = g.run(dd, flags=True).cpu().numpy()
    d = np.ascontiguousarray(data)
    of = o.run(d, flags=True)
    assert np.array_equal(gf, of) and np.array_equal(dd.cpu().numpy(), d)


def test_rfi_cluster_four_stokes_bit_exact(pv, oracle, cuda):
    """6144 channels of four Stokes parameters over a cluster of 8 CTAs: every
    polarisation of a clipped channel and spectrum is replaced."""
    import torch
    rng = np.random.default_rng(5)
    nt, nsub, nchan = 1100, 96, 64
    I = stokes_filterbank(rng, nt, nsub, nchan)
    data = np.ascontiguousarray(np.concatenate([I, I * 0.1, I * 0.2, I * -0.3], axis=2))
    bp = make_bp_text(nsub * nchan, BP_START, BP_WIDTH, 1000.0, 50.0)
    parts = pv.load().pv_rfi_parts(nsub * nchan)
    g = pv.RFI(bp, cr=5.0, history=1050, split=2)
    o = oracle.RFI(bp, cr=5.0, history=1050, mode=1, parts=parts)
    dd = torch.from_numpy(data).to(cuda)
    gf = g.run(dd, flags=True).cpu().numpy()
    of = o.run(data, flags=True)
    assert np.array_equal(gf, of) and np.array_equal(dd.cpu().numpy(), data)


@pytest.mark.parametrize("split", [1, 2])
def test_rfi_cluster_chunks_in_steady_state_bit_exact(pv, oracle, cuda, split):
    """6144 channels over a cluster, four chunks with a 300-spectrum history:
    from the second chunk on a launch starts in the steady state, whose first
    update overwrites the oldest history entry every CTA has just read."""
    import torch
    rng = np.random.default_rng(17)
    nsub, nchan, per = 96, 64, 400
    data = stokes_filterbank(rng, 4 * per, nsub, nchan)
    bp = make_bp_text(nsub * nchan, BP_START, BP_WIDTH, 1000.0, 50.0)
    parts = pv.load().pv_rfi_parts(nsub * nchan)
    g = pv.RFI(bp, cr=5.0, history=300, split=split)
    o = oracle.RFI(bp, cr=5.0, history=300, mode=1, parts=parts)
    for k in range(4):
        d = np.ascontiguousarray(data[k * per:(k + 1) * per])
        dd = torch.from_numpy(d).to(cuda)
        gf = g.run(dd, flags=True).cpu().numpy()
        of = o.run(d, flags=True)
        assert np.array_equal(gf, of) and np.array_equal(dd.cpu().numpy(), d), k
    assert np.array_equal(g.state()[[0, 1, 5, 6, 7, 8, 9]], o.state()[[0, 1, 5, 6, 7, 8, 9]])
