"""Reduced-precision delay rings (FP16, and uint8 with a per-channel scale and
offset) against the FP32 batch and an FP64 dedispersion of the same
filterbank: dedispersed-power error and event agreement."""
import numpy as np
import pytest

from gen import voltages
from test_gpu_batch import MIX, beam_kw, calibrated

pytestmark = pytest.mark.gpu


def _rel_rms(a, b):
    b = np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a.astype(np.float64) - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def _near_threshold(ev, thr, rms, eps):
    """Events whose value lies within eps (relative) of their level's threshold."""
    level = thr * rms * np.sqrt(ev["bin_factor"].astype(np.float64))
    return np.abs(ev["value"] - level) <= eps * level


@pytest.fixture(scope="module")
def runs(pv, oracle, cuda):
    import torch
    rng = np.random.default_rng(2024)
    cfgs = [calibrated(pv, cuda, beam_kw(**m), rng) for m in MIX]
    batches = {st: pv.Batch(cfgs, tune=False, graph=True, store=st) for st in ("f32", "f16", "u8")}
    lags = [batches["f32"].info(i)["lag"] for i in range(len(cfgs))]
    rng = np.random.default_rng(77)
    for step in range(max(lags) + 3):
        for i, c in enumerate(cfgs):
            v16, _ = voltages(rng, c.nsub, 2, c.chunk * 4 * c.nchan_sub)
            x = torch.from_numpy(v16.reshape(c.nsub, 2, -1)).to(cuda)
            for b in batches.values():
                b.set_input(i, x)
        for b in batches.values():
            b.run()
        torch.cuda.synchronize()
    res = {st: [] for st in batches}
    for st, b in batches.items():
        for i, c in enumerate(cfgs):
            ev, n, first = b.events(i)
            out = pv.device_array(b.buffers(i)[1], (c.tdms, c.chunk)).cpu().numpy()
            res[st].append((ev, n, first, out))
    # FP64 dedispersion of each beam's last window from the FP32 ring, and of
    # the same ring clipped to the u8 code range (+-6 sigma, sigma = 1 after the
    # zero-DMing clipper): spectra the clipper rejects (-0.2 minus the
    # bandpass) saturate there
    ref, ref_sat, ref_codes = [], [], []
    for i, c in enumerate(cfgs):
        info = batches["f32"].info(i)
        nbins = info["nbins"]
        stride = info["ring_bytes"] // (4 * nbins)
        ring = pv.device_array(batches["f32"].buffers(i)[2], (nbins, stride)).cpu().numpy()
        w = info["window"]
        cols = (w * c.chunk + np.arange(c.chunk + info["max_shift"] + 1)) % info["ring_len"]
        k, _ = oracle.dm_shifts(c.fch1, c.foff, nbins)
        start = np.float32(0.0) / np.float32(c.tsamp)
        step = np.float32(c.dm_step) / np.float32(c.tsamp)
        ref.append(oracle.dedisperse(ring[:, cols], c.chunk, c.tdms, k, start, step, f64=True))
        lim = 6.0 / 127.0
        sat = np.clip(ring[:, cols], -128 * lim, 127 * lim)
        ref_sat.append(oracle.dedisperse(sat, c.chunk, c.tdms, k, start, step, f64=True))
        # the u8 ring's codes, centred: their FP64 sums are the exact integer sums
        info8 = batches["u8"].info(i)
        stride8 = info8["ring_bytes"] // nbins
        codes = pv.device_array(batches["u8"].buffers(i)[2], (nbins, stride8), dtype="uint8").cpu().numpy()
        ref_codes.append(oracle.dedisperse(codes[:, cols].astype(np.float32) - 128.0, c.chunk, c.tdms, k,
                                           start, step, f64=True))
    return cfgs, res, ref, ref_sat, ref_codes


def test_fp32_ring_equals_fp64_within_1e5(runs):
    cfgs, res, ref, _, _ = runs
    for (ev, n, first, out), r in zip(res["f32"], ref):
        assert first >= 0
        assert _rel_rms(out, r) < 1e-5  # FP32 sums of ~10^2-10^3 channels


def test_fp16_ring_dedispersed_power_within_1e3_of_fp64(runs):
    cfgs, res, ref, _, _ = runs
    for (ev, n, first, out), r in zip(res["f16"], ref):
        assert _rel_rms(out, r) < 1e-3


def test_u8_ring_quantisation_error_is_bounded(runs):
    """Against the FP64 sum of the same samples clipped to the code range, the
    u8 error is the quantisation noise: steps of 6/127 sigma."""
    cfgs, res, ref, ref_sat, _ = runs
    for (ev, n, first, out), r in zip(res["u8"], ref_sat):
        assert _rel_rms(out, r) < 0.05


def test_u8_codes_of_uniform_scale_beams_are_summed_exactly(runs):
    """With the clipper and zero-DMing every row has the scale 6/127: the
    kernel sums the codes as integers, so each output is the FP32 product of
    the scale and the exact sum."""
    cfgs, res, _, _, ref_codes = runs
    sc = np.float64(np.float32(6.0 / 127.0))
    for (ev, n, first, out), r in zip(res["u8"], ref_codes):
        assert np.array_equal(out, (sc * r).astype(np.float32))


def test_fp16_events_agree_with_fp32_but_near_the_threshold(runs):
    cfgs, res, ref, _, _ = runs
    compared = 0
    for c, (e32, n32, f32, _), (e16, n16, f16, _) in zip(cfgs, res["f32"], res["f16"]):
        assert f32 == f16
        rms = np.sqrt(np.float32(c.nsub * c.nchan_sub))

        def key(e):
            return set(zip(e["dm"].tolist(), e["t"].tolist(), e["bin_factor"].tolist()))
        only32 = key(e32) - key(e16)
        only16 = key(e16) - key(e32)
        for only, ev in ((only32, e32), (only16, e16)):
            if not only:
                continue
            sel = np.array([(a, b, f) in only for a, b, f in zip(ev["dm"], ev["t"], ev["bin_factor"])])
            assert _near_threshold(ev[sel], c.threshold, rms, 5e-3).all()
        compared += len(e32)
    assert compared > 0


def test_u8_rows_calibrate_from_data_without_a_clipper(pv, cuda):
    """Beams without a clipper take each channel's offset (median) and scale
    (median absolute deviation) from its first varying chunk: the dedispersed
    fluctuations then stay at the quantisation level."""
    import torch
    rng = np.random.default_rng(5)
    kw = dict(beam_kw(4, 16, 32, 0.5), rfi_active=0, bp_text=None)
    cfg = pv.beam_config(**kw)
    b32 = pv.Batch([cfg], tune=False, graph=False, store="f32")
    b8 = pv.Batch([cfg], tune=False, graph=False, store="u8")
    lag = b32.info(0)["lag"]
    for _ in range(lag + 2):
        v16, _ = voltages(rng, cfg.nsub, 2, cfg.chunk * 4 * cfg.nchan_sub)
        x = torch.from_numpy(v16.reshape(cfg.nsub, 2, -1)).to(cuda)
        for b in (b32, b8):
            b.set_input(0, x)
            b.run()
    torch.cuda.synchronize()
    o32 = pv.device_array(b32.buffers(0)[1], (cfg.tdms, cfg.chunk)).cpu().numpy()
    o8 = pv.device_array(b8.buffers(0)[1], (cfg.tdms, cfg.chunk)).cpu().numpy()
    m = o32.mean(axis=1, keepdims=True)
    assert _rel_rms(o8 - m, o32 - m) < 0.05  # unclipped Stokes I: compare the fluctuations
