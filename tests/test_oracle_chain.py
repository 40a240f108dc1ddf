"""CPU checks of the channeliser-chain and RFI restatements."""
import numpy as np
import pytest

from gen import make_bp_text, stokes_filterbank


@pytest.mark.parametrize("window", ["kaiser", "hamming", "blackman", "gaussian"])
@pytest.mark.parametrize("nchan,ntaps", [(16, 8), (64, 8), (512, 8), (32, 4)])
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


def test_rfi_fp64_variant_flags_match_reference_arithmetic(oracle):
    """The FP64 variant changes clip decisions only near their thresholds."""
    rng = np.random.default_rng(11)
    nt, nsub, nchan = 2400, 32, 16
    data = stokes_filterbank(rng, nt, nsub, nchan)
    bp = _rfi_case(0)
    runs = []
    for mode in (0, 1):
        r = oracle.RFI(bp, cr=5.0, sr=4.0, history=1200, mode=mode)
        d = data.copy()
        fl = r.run(d, flags=True)
        runs.append((d, fl))
    (d0, f0), (d1, f1) = runs
    spec0, spec1 = (f0 & 2) != 0, (f1 & 2) != 0
    assert np.mean(spec0[:, 0] != spec1[:, 0]) < 0.01
    both = ~spec0[:, 0] & ~spec1[:, 0]
    chan_diff = (f0[both] & 1) != (f1[both] & 1)
    assert chan_diff.mean() < 1e-3
    # normalised output agrees closely where both kept the spectrum
    assert np.allclose(d0[both], d1[both], rtol=1e-3, atol=1e-3)
