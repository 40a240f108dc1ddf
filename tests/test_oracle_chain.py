"""CPU checks of the channeliser-chain and RFI restatements."""
import numpy as np
import pytest

from gen import make_bp_text, stokes_filterbank


@pytest.mark.parametrize("window", ["kaiser", "hamming", "blackman", "gaussian"])
@pytest.mark.parametrize("nchan,ntaps", [(16, 8), (64, 8), (512, 8), (32, 4), (24, 8), (6, 4)])
def test_fir_coefficients_product_vs_oracle(pv, oracle, window, nchan, ntaps):
    """The library's host coefficient design against the oracle's
    (PolyphaseCoefficients.cpp:308-364), two independent restatements."""
    a = pv.fir_coefficients(ntaps, nchan, window)
    b = oracle.fir_coefficients(ntaps, nchan, window)
    assert np.max(np.abs(a - b)) <= 1e-6 * np.max(np.abs(b))
    # the centre tap normalises the prototype to 1 before the 1/nchan scale
    centre = (ntaps * nchan - 1) // 2
    t, c = divmod(centre, nchan)
    assert abs(abs(a[t, c]) * nchan - 1.0) < 1e-12


def test_ppf_oracle_against_numpy(oracle):
    """FIR in float, FFT as numpy.fft (FFTW_FORWARD convention)."""
    rng = np.random.default_rng(0)
    N, T, nsub, npol, nblk = 16, 8, 3, 2, 40
    coeffs = oracle.fir_coefficients(T, N, "hamming").astype(np.float32)
    x = (rng.standard_normal((nsub, npol, nblk, N)) + 1j * rng.standard_normal((nsub, npol, nblk, N))).astype(np.complex64)
    ppf = oracle.PPF(N, T, coeffs)
    got = ppf.run(x)
    pad = np.concatenate([np.zeros((nsub, npol, T - 1, N), np.complex64), x], axis=2)
    for b in range(nblk):
        y = np.zeros((nsub, npol, N), np.complex64)
        for t in range(T):
            y = (y + (pad[:, :, b + t, :] * coeffs[t]).astype(np.complex64)).astype(np.complex64)
        want = np.fft.fft(y.astype(np.complex128), axis=-1)
        assert np.allclose(got[b], want, rtol=1e-5, atol=1e-4 * np.abs(want).max())


BP_START, BP_WIDTH = 140.0, 0.01220703125


def _rfi_case(deg, nbins_file=512):
    coeffs = {0: (), 2: (0.0,)}[deg] if deg == 0 else (0.3, -0.001)
    median = 1000.0
    return make_bp_text(nbins_file, BP_START, BP_WIDTH * 512 / nbins_file, median, 50.0, coeffs)


@pytest.mark.parametrize("deg,zero_dm,history", [(0, False, 1200), (2, True, 1100), (0, True, 3000)])
def test_rfi_fp64_variant_flags_match_reference_arithmetic(oracle, deg, zero_dm, history):
    """The FP64 variant's flags, given to the reference-arithmetic run as a
    guide, differ from its own decisions only within 1e-3 rmsRunAve (channel)
    or 1e-2 bandpass rms / sqrt(nBins) (spectrum) of the thresholds; the
    normalised outputs then agree to 1e-4 relative."""
    rng = np.random.default_rng(11)
    nt, nsub, nchan = 3600, 32, 16
    data = stokes_filterbank(rng, nt, nsub, nchan)
    bp = _rfi_case(deg)
    r1 = oracle.RFI(bp, cr=5.0, sr=4.0, history=history, zero_dming=zero_dm, mode=1)
    d1 = data.copy()
    f1 = r1.run(d1, flags=True)
    r0 = oracle.RFI(bp, cr=5.0, sr=4.0, history=history, zero_dming=zero_dm, mode=0)
    d0 = data.copy()
    f0, rep = r0.run_guided(d0, f1, 1e-3, 1e-2)
    assert rep["chan_decisions"] == nt * nsub * nchan and rep["spec_decisions"] == nt
    assert rep["chan_mismatch"] == 0 and rep["spec_mismatch"] == 0, rep
    assert np.array_equal(f0, f1)
    fin = np.isfinite(d1)
    assert np.array_equal(fin, np.isfinite(d0))
    assert np.max(np.abs(d0[fin] - d1[fin]) / np.maximum(np.abs(d1[fin]), 1.0)) <= 1e-4
    # unguided, the reference arithmetic reaches the same flags on these data
    r0b = oracle.RFI(bp, cr=5.0, sr=4.0, history=history, zero_dming=zero_dm, mode=0)
    assert np.array_equal(r0b.run(data.copy(), flags=True), f1)


def test_guided_run_counts_a_planted_difference(oracle):
    """A flag flipped in the guide far from its threshold is a mismatch; the
    run still follows the guide, so nothing else differs."""
    rng = np.random.default_rng(12)
    nt, nsub, nchan = 1500, 16, 16
    data = stokes_filterbank(rng, nt, nsub, nchan)
    bp = _rfi_case(0, nbins_file=256)
    r1 = oracle.RFI(bp, cr=5.0, sr=4.0, history=1100, mode=1)
    f1 = r1.run(data.copy(), flags=True)
    hint = f1.copy()
    hint[1300, 17] ^= 1  # a channel decision well inside the kept data
    r0 = oracle.RFI(bp, cr=5.0, sr=4.0, history=1100, mode=0)
    f0, rep = r0.run_guided(data.copy(), hint, 1e-3, 1e-2)
    assert rep["chan_mismatch"] == 1 and rep["chan_near"] == 0 and rep["first_difference"] == 1300
    assert np.array_equal(f0, hint)


@pytest.mark.parametrize("N", [24, 6])
def test_ppf_oracle_dft_against_numpy(oracle, N):
    """Channel counts that are not powers of two (the reference takes any even
    count, PPFChanneliser.cpp:42-44): the oracle's DFT as numpy.fft."""
    rng = np.random.default_rng(N)
    T, nsub, npol, nblk = 8, 2, 2, 20
    coeffs = oracle.fir_coefficients(T, N, "kaiser").astype(np.float32)
    x = (rng.standard_normal((nsub, npol, nblk, N)) + 1j * rng.standard_normal((nsub, npol, nblk, N))).astype(np.complex64)
    got = oracle.PPF(N, T, coeffs).run(x)
    pad = np.concatenate([np.zeros((nsub, npol, T - 1, N), np.complex64), x], axis=2)
    y = np.zeros((nsub, npol, nblk, N), np.complex128)
    for t in range(T):
        y += pad[:, :, t:t + nblk, :].astype(np.complex128) * coeffs[t][None, None, None, :]
    want = np.fft.fft(y, axis=-1).transpose(2, 0, 1, 3)
    assert np.max(np.abs(got - want)) <= 1e-4 * np.sqrt(np.mean(np.abs(want) ** 2))


def test_ppf_oracle_single_channel_is_the_time_series(oracle):
    """One channel: the spectra are the time samples (PPFChanneliser.cpp:108-131)."""
    rng = np.random.default_rng(1)
    x = (rng.standard_normal((3, 2, 17, 1)) + 1j * rng.standard_normal((3, 2, 17, 1))).astype(np.complex64)
    got = oracle.PPF(1, 8, np.ones((8, 1), np.float32)).run(x)
    assert np.array_equal(got, x.transpose(2, 0, 1, 3))
