"""BandPassRecorder: the integrated spectrum on the GPU and the polynomial
fit with 2-sigma trimming against the oracle, and the .bp text it writes
loading into the RFI clipper."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _filterbank(rng, nt, nsub=31, npol=1, nchan=16, start=110.0, end=116.0546875, spikes=()):
    n = nsub * nchan
    f = (start + (end - start) / n * np.arange(n)).astype(np.float32)
    model = 1000.0 + 30.0 * (f - 113.0) - 4.0 * (f - 113.0) ** 2
    x = model[None, :] + rng.normal(0.0, 20.0, (nt, n))
    for ch in spikes:
        x[:, ch] += 400.0  # persistent narrowband RFI
    x = x.astype(np.float32).reshape(nt, nsub, 1, nchan)
    if npol > 1:
        x = np.concatenate([x] + [x * 0.5] * (npol - 1), axis=2)
    return np.ascontiguousarray(x)


@pytest.mark.parametrize("npol", [1, 4])
def test_recorder_fit_equals_the_oracle(pv, oracle, cuda, npol):
    import torch
    rng = np.random.default_rng(npol)
    chunks = [_filterbank(rng, nt, npol=npol, spikes=(7, 100, 300)) for nt in (700, 1200, 517)]
    rec = pv.BandPassRecorder(requiredSamples=2000, coefficients=3, startFrequency=110.0,
                              endFrequency=116.0546875)
    ready = [rec.run(torch.from_numpy(c).to(cuda)) for c in chunks]
    assert ready == [False, False, True]
    coef, rms, trimmed, bp = rec.result()
    want = oracle.bandpass_record(chunks, 2000, 3, 110.0, 116.0546875)
    assert want is not None
    f = np.linspace(110.0, 116.0, 50)
    got_v = np.polynomial.polynomial.polyval(f, coef.astype(np.float64))
    want_v = np.polynomial.polynomial.polyval(f, want[0])
    # float coefficients of raw frequency powers: terms of ~1e5 cancel to ~1e3
    assert np.max(np.abs(got_v - want_v) / np.abs(want_v)) < 1e-4
    assert trimmed == want[2] >= 3  # the RFI channels at least
    assert abs(rms - want[1]) <= 1e-5 * want[1]
    lines = [ln for ln in bp.splitlines() if not ln.startswith("#")]
    assert int(lines[0]) == 31 * 16 and len(lines) == 5 + 3
    assert np.allclose([float(v) for v in lines[5:]], coef, rtol=1e-7)
    # the clipper loads the recorded bandpass
    pv.RFI(bp, cr=5.0, sr=4.0, history=1000, zero_dming=True)
    assert oracle.RFI(bp, 5.0, 4.0, 1000, True).bandpass(31 * 16).size == 31 * 16


def test_recorder_starts_a_new_integration_after_a_fit(pv, cuda):
    import torch
    rng = np.random.default_rng(9)
    rec = pv.BandPassRecorder(requiredSamples=100, coefficients=2, startFrequency=110.0,
                              endFrequency=116.0546875)
    a = _filterbank(rng, 150)
    assert rec.run(torch.from_numpy(a).to(cuda))
    assert not pv.BandPassRecorder(requiredSamples=1000, coefficients=2, startFrequency=110.0,
                                   endFrequency=116.0546875).run(torch.from_numpy(a).to(cuda))
    assert not rec.run(torch.from_numpy(a[:50]).to(cuda))  # 50 of 100 spectra of the new integration
    with pytest.raises(pv.PvError, match="startFrequency"):
        pv.BandPassRecorder(requiredSamples=10, coefficients=2, endFrequency=1.0)
