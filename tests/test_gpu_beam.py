"""One beam's device-resident chain (PPF -> Stokes -> integrate -> RFI -> ring ->
dedisperse -> analyse) checked stage by stage against the oracle over a
stream of chunks."""
import numpy as np
import pytest

from gen import make_bp_text, voltages

pytestmark = pytest.mark.gpu

SUB_BW = 0.1953125  # MHz, LOFAR subband width at the 200 MHz clock


def lofar_band(f_sub0, nsub, nchan_sub):
    """Filterbank channel 0 frequency and width for nsub subbands starting at
    f_sub0 channelised into nchan_sub channels each (the PPF's DC channel is
    nchan_sub/2)."""
    foff = SUB_BW / nchan_sub
    return f_sub0 - (nchan_sub // 2) * foff, foff


def _setup(pv, oracle, nsub=8, nchan_sub=16, chunk=512, tdms=64, dm_max=30.0, history=1000):
    fch1, foff = lofar_band(140.0, nsub, nchan_sub)
    tsamp = 5.12e-6 * nchan_sub * 4
    nbins = nsub * nchan_sub
    bp = make_bp_text(nbins, fch1, foff, 1000.0, 50.0)
    kw = dict(nsub=nsub, nchan_sub=nchan_sub, window="hamming", fch1=fch1, foff=foff, tsamp=tsamp,
              tdms=tdms, dm_step=dm_max / (tdms - 1), chunk=chunk, threshold=6.0, bp_text=bp, cr=5.0,
              sr=4.0, history=history, debug_taps=1)
    beam = pv.Beam(pv.beam_config(**kw))
    return beam, kw, bp


def test_beam_chain_matches_oracle_stage_by_stage(pv, oracle, cuda):
    import torch
    beam, kw, bp = _setup(pv, oracle)
    info = beam.info()
    nsub, nch, chunk, tdms = kw["nsub"], kw["nchan_sub"], kw["chunk"], kw["tdms"]
    nbins = nsub * nch
    assert info["inverted"] == 1 and info["nbins"] == nbins
    lag = info["lag"]
    k, inv = oracle.dm_shifts(kw["fch1"], kw["foff"], nbins)
    start = np.float32(0.0) / np.float32(kw["tsamp"])
    step = np.float32(kw["dm_step"]) / np.float32(kw["tsamp"])
    assert info["max_shift"] == oracle.shift_table(k, tdms, start, step).max()
    coeffs = oracle.fir_coefficients(8, nch, "hamming").astype(np.float32)
    o_ppf = oracle.PPF(nch, 8, coeffs)
    o_rfi = oracle.RFI(bp, cr=5.0, sr=4.0, history=kw["history"], mode=1)
    fb_raw_p, _, out_p, _ = beam.buffers()[1], None, beam.buffers()[2], None
    fb_p = beam.buffers()[0]
    rng = np.random.default_rng(99)
    history_fb = []
    n_chunks = lag + 4
    windows = 0
    for ck in range(n_chunks):
        v16, vc = voltages(rng, nsub, 2, chunk * 4 * nch)
        beam.process(torch.from_numpy(v16.reshape(nsub, 2, -1)).to(cuda))
        torch.cuda.synchronize()
        raw = pv.device_array(fb_raw_p, (chunk, nsub, 1, nch)).cpu().numpy()
        post = pv.device_array(fb_p, (chunk, nsub, 1, nch)).cpu().numpy()
        # K1 against the oracle channeliser (FP32 FFT vs FP64): tolerance
        spec = o_ppf.run(vc.reshape(nsub, 2, chunk * 4, nch))
        want_raw = oracle.integrate(oracle.stokes(spec, 1), 4, 1)
        assert np.max(np.abs(raw - want_raw)) <= 1e-4 * want_raw.mean()
        # RFI on identical input: bit-exact
        d = raw.copy()
        o_rfi.run(d)
        assert np.array_equal(post, d)
        history_fb.append(post)
        if ck >= lag:
            w = ck - lag
            block = np.concatenate(history_fb[w:ck + 1], axis=0).reshape(-1, nbins)
            buf = np.ascontiguousarray(block[:, ::-1].T)  # inverted band: highest frequency first
            want = oracle.dedisperse(buf, chunk, tdms, k, start, step)
            got = pv.device_array(out_p, (tdms, chunk)).cpu().numpy()
            assert np.array_equal(got, want)
            ev, n, first = beam.events()
            assert first == w * chunk
            rms = float(np.sqrt(np.float32(nch) * np.float32(nsub)))
            want_ev = oracle.analyse(want, 6.0, rms, 6)
            assert n == len(want_ev) and np.array_equal(ev, want_ev.astype(ev.dtype))
            windows += 1
    assert windows == n_chunks - lag


def test_beam_host_input_equals_device_input(pv, oracle, cuda):
    import torch
    a, kw, _ = _setup(pv, oracle, chunk=256)
    b, _, _ = _setup(pv, oracle, chunk=256)
    rng = np.random.default_rng(5)
    lag = a.info()["lag"]
    for _ in range(lag + 2):
        v16, _ = voltages(rng, kw["nsub"], 2, 256 * 4 * kw["nchan_sub"])
        a.process(torch.from_numpy(v16.reshape(kw["nsub"], 2, -1)).to(cuda))
        b.process_host(np.ascontiguousarray(v16))
        ea, na, fa = a.events()
        eb, nb, fb = b.events()
        assert na == nb and fa == fb and np.array_equal(ea, eb)
        if fa < 0:
            continue  # no window yet: the output buffers hold nothing
        oa = pv.device_array(a.buffers()[2], (kw["tdms"], 256)).cpu().numpy()
        ob = pv.device_array(b.buffers()[2], (kw["tdms"], 256)).cpu().numpy()
        assert np.array_equal(oa, ob)


def test_beam_state_saved_and_loaded_continues_bit_for_bit(pv, oracle, cuda):
    """A beam that loads another beam's state after chunk k gives, from chunk
    k+1 on, the same filterbanks, windows and events as the beam that ran
    continuously; the state of the loaded beam saves back to the same bytes;
    a beam of another configuration refuses it."""
    import torch
    a, kw, _ = _setup(pv, oracle, chunk=256, history=1000)
    nsub, nch, chunk, tdms = kw["nsub"], kw["nchan_sub"], kw["chunk"], kw["tdms"]
    rng = np.random.default_rng(31)
    chunks = [torch.from_numpy(voltages(rng, nsub, 2, chunk * 4 * nch)[0].reshape(nsub, 2, -1)).to(cuda)
              for _ in range(12)]
    fresh = pv.Beam(pv.beam_config(**kw))
    s0 = fresh.save_state()
    k = 8  # past the clipper's 1000-spectrum warm-up and the ring's lag
    assert a.info()["lag"] < k
    for c in chunks[:k]:
        a.process(c)
    state = a.save_state()
    assert state.nbytes == pv.load().pv_beam_state_size(a.h) > s0.nbytes // 2
    assert not np.array_equal(state, s0)
    b = pv.Beam(pv.beam_config(**kw))
    b.load_state(state)
    assert np.array_equal(b.save_state(), state)
    assert b.events()[2] == -1  # no window since the load
    for c in chunks[k:]:
        a.process(c)
        b.process(c)
        ea, na, fa = a.events()
        eb, nb, fb = b.events()
        assert na == nb and fa == fb >= 0 and np.array_equal(ea, eb)
        for i in (0, 2):
            shape = (chunk, nsub, 1, nch) if i == 0 else (tdms, chunk)
            assert np.array_equal(pv.device_array(a.buffers()[i], shape).cpu().numpy(),
                                  pv.device_array(b.buffers()[i], shape).cpu().numpy())
    other = pv.Beam(pv.beam_config(**dict(kw, tdms=tdms + 1)))
    with pytest.raises(pv.PvError, match="another configuration"):
        other.load_state(state)
