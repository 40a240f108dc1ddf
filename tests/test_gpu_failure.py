"""Failure detection without a GPU fault.  The pipelined dedispersion kernels
bound every device-side wait.  A launch whose first stage's copies are
withheld (pv_stall_next_launches: a barrier that nothing completes) waits
there until a short limit runs out, records PV_ERR_TIMEOUT, waits for its
own copies in flight and returns.  The error reaches the caller through the plan status and
pv_beam_events, and the context stays usable: the next launch with the
default limit is bit-exact.  (The reference reports a failed GPU job as
GPU_Job::Failed and cancels its export, lib/src/DedispersionModule.cpp:299-311.)"""
import numpy as np
import pytest

from gen import make_bp_text, voltages

pytestmark = pytest.mark.gpu

PV_ERR_TIMEOUT = -6


def _ring_case(pv, oracle, rng, nchan=2048, nout=4096, tdms=64):
    k, _ = pv.dm_shifts(150.0, -0.01, nchan)
    start, step = np.float32(0.0), np.float32(2.5)
    plan = pv.DedispPlan(k, tdms, start, step)
    ms = plan.max_shift()
    ring_len = (nout + ms + 8 + 3) & ~3
    lin = rng.standard_normal((nchan, ring_len), dtype=np.float32)
    want = oracle.dedisperse(lin, nout, tdms, k, start, step)
    return plan, lin, ring_len, want


def test_plan_wait_runs_out_then_recovers(pv, oracle, cuda):
    import torch
    rng = np.random.default_rng(66)
    plan, lin, ring_len, want = _ring_case(pv, oracle, rng)
    d_ring = torch.from_numpy(lin).to(cuda)
    nout = want.shape[1]
    prev = pv.set_wait_limit(1000000)  # 1 ms
    try:
        pv.stall_next_launches(1)
        plan.run(d_ring, nout, ring_len=ring_len, t_base=0)
        torch.cuda.synchronize()
        assert plan.status() == PV_ERR_TIMEOUT
        assert pv.stall_next_launches(0) == 0  # the hook was used by that launch
        # later launches stop at their start while the status holds the error
        plan.run(d_ring, nout, ring_len=ring_len, t_base=0)
        torch.cuda.synchronize()
        assert plan.status() == PV_ERR_TIMEOUT
    finally:
        pv.stall_next_launches(0)
        assert pv.set_wait_limit(prev) == 1000000
    plan.clear_status()
    out = plan.run(d_ring, nout, ring_len=ring_len, t_base=0)
    torch.cuda.synchronize()
    assert plan.status() == 0
    assert np.array_equal(out.cpu().numpy(), want)


def test_beam_reports_timeout_and_other_beams_run(pv, oracle, cuda):
    import torch
    nsub, nch, chunk, tdms = 8, 16, 512, 64
    fch1, foff = 140.0 - 8 * 0.1953125 / 16, 0.1953125 / 16
    bp = make_bp_text(nsub * nch, fch1, foff, 1000.0, 50.0)
    kw = dict(nsub=nsub, nchan_sub=nch, window="hamming", fch1=fch1, foff=foff, tsamp=5.12e-6 * nch * 4,
              tdms=tdms, dm_step=30.0 / (tdms - 1), chunk=chunk, threshold=6.0, bp_text=bp, cr=5.0, sr=4.0,
              history=1000, prefilled=1)
    rng = np.random.default_rng(7)
    v16, _ = voltages(rng, nsub, 2, chunk * 4 * nch)
    d_v = torch.from_numpy(v16.reshape(nsub, 2, -1)).to(cuda)
    prev = pv.set_wait_limit(1000000)
    try:
        bad = pv.Beam(pv.beam_config(**kw))
        pv.stall_next_launches(1)
        bad.process(d_v)
        with pytest.raises(pv.PvError) as e:
            bad.events()
        assert "gave up" in str(e.value)
    finally:
        pv.stall_next_launches(0)
        pv.set_wait_limit(prev)
    good = pv.Beam(pv.beam_config(**kw))
    ref = pv.Beam(pv.beam_config(**kw))
    good.process(d_v)
    ref.process(d_v)
    ea, na, fa = good.events()
    eb, nb, fb = ref.events()
    assert na == nb and fa == fb == 0 and np.array_equal(ea, eb)
