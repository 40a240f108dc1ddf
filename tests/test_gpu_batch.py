"""The batched engine (pv_batch) against the same beams run alone through the
single-beam chain (pv_beam, itself checked stage by stage against the
oracle): every beam's filterbank, dedispersed window and event list are
bit-identical in the batch, with and without graph capture, for every
dedispersion tile variant."""
import numpy as np
import pytest

from gen import make_bp_text, voltages

pytestmark = pytest.mark.gpu

SUB_BW = 0.1953125  # MHz


def beam_kw(nsub, nch, tdms, dm_step, f0=140.0, descending=False, chunk=512, threshold=4.0, **extra):
    foff = SUB_BW / nch
    fch1 = f0 - (nch // 2) * foff
    if descending:
        fch1, foff = fch1 + foff * (nsub * nch - 1), -foff
    tsamp = 5.12e-6 * nch * 4
    kw = dict(nsub=nsub, nchan_sub=nch, window="kaiser", fch1=fch1, foff=foff, tsamp=tsamp,
              tdms=tdms, dm_step=dm_step, chunk=chunk, threshold=threshold, cr=5.0, sr=4.0,
              history=1000, bin_pow2=4, zero_dming=1)  # zero-DMing as every reference pipeline XML
    kw.update(extra)
    return kw


def calibrated(pv, cuda, kw, rng):
    """The beam config with a flat bandpass at the filterbank's own mean and rms."""
    import torch
    nbins = kw["nsub"] * kw["nchan_sub"]
    probe = pv.Beam(pv.beam_config(**dict(kw, rfi_active=0, bp_text=None, tdms=8)))
    v16, _ = voltages(rng, kw["nsub"], 2, kw["chunk"] * 4 * kw["nchan_sub"])
    probe.process(torch.from_numpy(v16.reshape(kw["nsub"], 2, -1)).to(cuda))
    torch.cuda.synchronize()
    fb = pv.device_array(probe.buffers()[0], (kw["chunk"], nbins)).cpu().numpy()
    lo = min(kw["fch1"], kw["fch1"] + kw["foff"] * (nbins - 1))
    bp = make_bp_text(nbins, lo, abs(kw["foff"]), float(fb.mean()), float(fb.std()))
    return pv.beam_config(**dict(kw, bp_text=bp))


MIX = [
    dict(nsub=6, nch=16, tdms=40, dm_step=0.5),
    dict(nsub=4, nch=64, tdms=64, dm_step=1.0),
    dict(nsub=12, nch=16, tdms=64, dm_step=10.0),           # wide delay spread: short DM tiles
    dict(nsub=3, nch=32, tdms=100, dm_step=0.4, descending=True),
    dict(nsub=8, nch=16, tdms=33, dm_step=0.9, threshold=5.0),
]


@pytest.fixture(scope="module")
def mix_configs(pv, cuda):
    rng = np.random.default_rng(2024)
    return [calibrated(pv, cuda, beam_kw(**m), rng) for m in MIX]


@pytest.mark.parametrize("tune,graph,variant,prefilled,pipelined",
                         [(True, True, 0, False, False), (False, False, 1, False, False),
                          (False, True, 3, True, False), (False, True, 0, False, True),
                          (True, True, 0, True, True), (False, True, 4, True, False),
                          (False, False, 5, False, True), (False, True, 4, False, True),
                          (False, True, 6, True, False), (False, False, 7, False, True),
                          (False, True, 8, False, False), (False, True, 6, False, True)])
def test_batch_equals_beams_alone(pv, cuda, mix_configs, tune, graph, variant, prefilled, pipelined):
    """Filterbank, event list and dedispersed window of every beam equal the
    single-beam chain's; pipelined, a window arrives one step later."""
    _compare_with_beams_alone(pv, cuda, mix_configs, tune, graph, variant, prefilled, pipelined,
                              wide_spread=True)


@pytest.mark.parametrize("pipelined", [False, True])
def test_batch_with_two_clipper_classes_equals_beams_alone(pv, cuda, mix_configs, pipelined):
    """A beam of more than 1024 channels puts its clipper in a second CTA-size
    class; pipelined, that class runs on its own stream and a dedispersion
    launch on the same queue follows it."""
    rng = np.random.default_rng(99)
    big = calibrated(pv, cuda, beam_kw(40, 32, 24, 0.05), rng)  # 1280 channels
    assert pv.load().pv_rfi_parts(1280) != pv.load().pv_rfi_parts(256)
    _compare_with_beams_alone(pv, cuda, mix_configs[:2] + [big], False, True, 0, False, pipelined)


def _compare_with_beams_alone(pv, cuda, mix, tune, graph, variant, prefilled, pipelined, wide_spread=False,
                              rfi_one_cta=False, rfi_cluster8=False, rfi_cluster4=False):
    import torch
    cfgs = mix
    if prefilled:  # rings start as lag chunks of silence: windows from the first chunk on
        cfgs = [type(c).from_buffer_copy(c) for c in cfgs]
        for c, o in zip(cfgs, mix):
            c._bp, c.bp_text, c.prefilled = o._bp, o._bp, 1
    batch = pv.Batch(cfgs, tune=tune, graph=graph, variant=variant, pipelined=pipelined, rfi_one_cta=rfi_one_cta,
                     rfi_cluster8=rfi_cluster8, rfi_cluster4=rfi_cluster4)
    alone = [pv.Beam(c) for c in cfgs]
    lags = [batch.info(i)["lag"] for i in range(len(cfgs))]
    assert lags == [b.info()["lag"] for b in alone]
    shape = batch.tiles()
    assert shape["tiles"] > 0 and all(1 <= d <= 16 for d in shape["dms"])
    if wide_spread and not tune and variant in (0, 3):  # 16 channel slots of ~3.5k samples
        assert min(shape["dms"]) < 16  # the wide-spread beam needs a short DM tile
    if graph:
        assert shape["graph_kernels"] >= len(cfgs)
    delay = 1 if pipelined else 0
    rng = np.random.default_rng(7)
    history = []  # per step: per beam (events, count, first, dedispersed or None)
    compared = events_seen = 0
    for step in range(max(lags) + 3 + delay):
        ins = []
        for c in cfgs:
            v16, _ = voltages(rng, c.nsub, 2, c.chunk * 4 * c.nchan_sub)
            ins.append(torch.from_numpy(v16.reshape(c.nsub, 2, -1)).to(cuda))
        for i, x in enumerate(ins):
            batch.set_input(i, x)
            alone[i].process(x)
        batch.run()
        torch.cuda.synchronize()
        rec = []
        for i, (c, b) in enumerate(zip(cfgs, alone)):
            nbins = c.nsub * c.nchan_sub
            fb_b, out_b, _ = batch.buffers(i)
            fb_a, _, out_a, _ = b.buffers()
            assert np.array_equal(pv.device_array(fb_b, (c.chunk, nbins)).cpu().numpy(),
                                  pv.device_array(fb_a, (c.chunk, nbins)).cpu().numpy())
            ea, na, firsta = b.events()
            da = pv.device_array(out_a, (c.tdms, c.chunk)).cpu().numpy() if firsta >= 0 else None
            rec.append((ea, na, firsta, da))
            eb, nb, firstb = batch.events(i)
            if step < delay:
                assert firstb == -1
                continue
            ea, na, firsta, da = history[step - delay][i] if delay else rec[i]
            assert (nb, firstb) == (na, firsta)
            assert np.array_equal(eb, ea)
            if firsta >= 0:
                assert np.array_equal(pv.device_array(out_b, (c.tdms, c.chunk)).cpu().numpy(), da)
                compared += 1
                events_seen += na - 1
        history.append(rec)
    assert compared >= len(cfgs) * 3
    if prefilled:
        assert compared == len(cfgs) * (max(lags) + 3)
    assert events_seen > 0


@pytest.mark.parametrize("pipelined,one_cta,cluster8,cluster4", [(False, True, False, False),
                                                                (True, False, True, False),
                                                                (False, False, False, False),
                                                                (True, False, False, True)])
def test_batch_clipper_shapes_equal_beams_alone(pv, cuda, mix_configs, pipelined, one_cta, cluster8, cluster4):
    """Beams of 1280 and 5120 channels (512 and 1024 partial sums): their
    batched clippers on one CTA each, on clusters of 128-thread CTAs, or the
    5120-channel beam on 4 CTAs give the same filterbanks, windows and events
    as the beams alone (the same partial sums in the same order whatever the
    CTAs)."""
    rng = np.random.default_rng(98)
    big = calibrated(pv, cuda, beam_kw(40, 32, 24, 0.05), rng)    # 1280 channels
    wide = calibrated(pv, cuda, beam_kw(80, 64, 16, 0.02), rng)   # 5120 channels
    assert pv.load().pv_rfi_parts(5120) == 1024 and pv.load().pv_rfi_parts(1280) == 512
    _compare_with_beams_alone(pv, cuda, mix_configs[:1] + [big, wide], False, True, 0, False, pipelined,
                              rfi_one_cta=one_cta, rfi_cluster8=cluster8, rfi_cluster4=cluster4)


def test_batch_autotuner_times_the_variants(pv, cuda, mix_configs):
    batch = pv.Batch(mix_configs[:2], tune=True, graph=False)
    t = batch.tiles()
    timed = [x for x in t["tune_ms"] if x > 0]
    assert len(timed) >= 2
    assert t["tune_ms"][t["variant"]] == min(timed)


def test_batch_rejects_unsupported_beams(pv, cuda, mix_configs):
    bad = pv.beam_config(**dict(beam_kw(4, 8, 16, 1.0), bp_text=None, rfi_active=0))
    with pytest.raises(pv.PvError, match="batched channeliser"):
        pv.Batch([mix_configs[0], bad])
    other_chunk = pv.beam_config(**dict(beam_kw(4, 16, 16, 1.0, chunk=256), bp_text=None, rfi_active=0))
    with pytest.raises(pv.PvError, match="same chunk"):
        pv.Batch([mix_configs[0], other_chunk])


def test_batch_host_steps_overlap_and_events_of_previous_step(pv, cuda, mix_configs):
    """run_host returns before its step finishes; the events of step k are read
    while step k+1 runs and equal those of the beams run alone."""
    import torch
    cfgs = mix_configs[:3]
    batch = pv.Batch(cfgs, tune=False, graph=True)
    alone = [pv.Beam(c) for c in cfgs]
    rng = np.random.default_rng(11)
    want = []
    nsteps = max(batch.info(i)["lag"] for i in range(len(cfgs))) + 3
    hosts_prev = None
    for step in range(nsteps):
        hosts = []
        for c in cfgs:
            v16, _ = voltages(rng, c.nsub, 2, c.chunk * 4 * c.nchan_sub)
            hosts.append(torch.from_numpy(v16.reshape(c.nsub, 2, -1)).pin_memory())
        want.append([b.events()[:2] if b.process_host(h) is None else None for b, h in zip(alone, hosts)])
        batch.run_host(hosts)
        if step:
            for i in range(len(cfgs)):
                ev, n, _ = batch.events(i, step=step - 1)
                assert n == want[step - 1][i][1] and np.array_equal(ev, want[step - 1][i][0])
                ev2, n2, _ = batch.events(i, step=-2)  # counted back from the last issued step
                assert n2 == n and np.array_equal(ev2, ev)
        hosts_prev = hosts  # pinned sources stay alive until their copies are done
    for i in range(len(cfgs)):
        ev, n, _ = batch.events(i)
        assert n == want[-1][i][1] and np.array_equal(ev, want[-1][i][0])
    with pytest.raises(pv.PvError, match="last two"):
        batch.events(0, step=0)
    del hosts_prev


def test_a_later_batch_with_smaller_beams_leaves_an_earlier_batch_runnable(pv, cuda, mix_configs):
    """Kernel attributes are global to the process: a batch created after
    another, with smaller beams, must not shrink the shared memory that the
    first batch's captured launches use."""
    import torch
    big = pv.Batch(mix_configs, tune=False, graph=True)
    small = pv.Batch(mix_configs[:1], tune=False, graph=True)
    rng = np.random.default_rng(5)
    for b, cfgs in ((big, mix_configs), (small, mix_configs[:1]), (big, mix_configs)):
        for i, c in enumerate(cfgs):
            v16, _ = voltages(rng, c.nsub, 2, c.chunk * 4 * c.nchan_sub)
            b.set_input(i, torch.from_numpy(v16.reshape(c.nsub, 2, -1)).to(cuda))
        b.run()
        for i in range(len(cfgs)):
            b.events(i)  # waits for the step and raises if it failed
    torch.cuda.synchronize()


@pytest.mark.parametrize("pipelined", [False, True])
def test_batch_with_idle_beams_equals_beams_alone(pv, cuda, mix_configs, pipelined):
    """Continuous batching: in every step only some beams have a chunk.  Each
    beam's windows (events and dedispersed data) equal those of the beam run
    alone on its own chunks, whatever the other beams do."""
    import torch
    cfgs = mix_configs
    n = len(cfgs)
    batch = pv.Batch(cfgs, tune=False, graph=True, pipelined=pipelined)
    alone = [pv.Beam(c) for c in cfgs]
    lags = [b.info()["lag"] for b in alone]
    rng = np.random.default_rng(23)
    want = [dict() for _ in range(n)]  # window -> (events, count, dedispersed)
    seen = [0] * n
    steps = 2 * max(lags) + 8
    for step in range(steps):
        active = rng.random(n) < 0.6
        if step == steps - 1:
            active[:] = False  # a step with no chunk at all still completes pipelined windows
        for i, c in enumerate(cfgs):
            if not active[i]:
                continue
            v16, _ = voltages(rng, c.nsub, 2, c.chunk * 4 * c.nchan_sub)
            x = torch.from_numpy(v16.reshape(c.nsub, 2, -1)).to(cuda)
            batch.set_input(i, x)
            alone[i].process(x)
            ev, cnt, first = alone[i].events()
            if first >= 0:
                out = pv.device_array(alone[i].buffers()[2], (c.tdms, c.chunk)).cpu().numpy()
                want[i][first // c.chunk] = (ev, cnt, out)
        batch.run(active=active.astype(np.uint8))
        torch.cuda.synchronize()
        for i, c in enumerate(cfgs):
            ev, cnt, first = batch.events(i)
            if first < 0:
                continue
            w = first // c.chunk
            assert w in want[i], (i, w)
            wev, wcnt, wout = want[i][w]
            assert cnt == wcnt and np.array_equal(ev, wev)
            assert np.array_equal(pv.device_array(batch.buffers(i)[1], (c.tdms, c.chunk)).cpu().numpy(), wout)
            seen[i] += 1
    for i in range(n):
        assert seen[i] == len(want[i]) > 0  # every window the beam completed alone came out once


def test_batch_of_twelve_beams_in_three_clipper_classes_equals_beams_alone(pv, cuda):
    """Twelve beams whose clippers use all three CTA sizes (up to 1024, 4096 and more channels;
    one launch per channel count, several sharing a CTA size), pipelined under one graph: every
    window and event list equals the beam's alone."""
    rng = np.random.default_rng(121)
    shapes = [(4, 16), (6, 32), (3, 64), (8, 16),       # 256-thread class
              (40, 32), (20, 64), (96, 16), (50, 32),   # 512-thread class
              (70, 64), (300, 16), (140, 32), (80, 64)]  # 1024-thread class
    mix = [calibrated(pv, cuda, beam_kw(ns, nc, 16 + 4 * i, 0.05 + 0.02 * i, chunk=256), rng)
           for i, (ns, nc) in enumerate(shapes)]
    parts = {pv.load().pv_rfi_parts(ns * nc) for ns, nc in shapes}
    assert len(parts) == 3
    _compare_with_beams_alone(pv, cuda, mix, False, True, 0, True, True)
