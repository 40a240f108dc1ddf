#!/usr/bin/env python3
"""Throughput benchmark of the beam-processing hot path on GB300.

Metric: DM-trial*channel*samples per second (the brute-force dedispersion
work tdms*nchan*nout of every chunk processed), whole job.

Workload "fullband" (default): one beam of 244 LOFAR subbands from 110 MHz
at 16 channels per subband (3904 channels), 327.68 us samples after x4
integration, 16384 output samples per chunk, 2048 DM trials over 0-500
pc/cm^3.  Per step (one chunk): the chunk's RFI-normalised filterbank is
written into the device-resident per-channel ring, dedispersed over every
trial and searched by the analyser.  The ring (3904 x 284,873 samples,
4.45 GB) stays resident, so inputs are larger than L2 and no flush is
needed.

Modes: default ``--impl pv`` runs the library; ``--impl reference`` times the
reference algorithm's CPU restatement (the reference itself cannot be built:
it needs Qt4, Boost, FFTW3 and the pelican core) on the host cores.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "pelican-lofar_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np

K_DISP = 4148.741601


def fullband_config():
    nsub, nchan_sub = 244, 16
    fch1_low = 110.0
    sub_bw = 0.1953125
    foff = sub_bw / nchan_sub
    nchan = nsub * nchan_sub
    tsamp = 5.12e-6 * nchan_sub * 4
    tdms, dm_lo, dm_hi = 2048, 0.0, 500.0
    return dict(workload="fullband-244sub-3904ch-2048dm", nsub=nsub, nchan_sub=nchan_sub,
                nchan=nchan, fch1=fch1_low, foff=foff, tsamp=tsamp, tdms=tdms, dm_low=dm_lo,
                dm_step=(dm_hi - dm_lo) / (tdms - 1), nout=16384, threshold=6.0, bin_pow2=6)


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi sampling during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.samples, self.proc, self.gpu = [], None, gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sms = [float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for i, n in enumerate(names):
                if len(s) > 5 + i and s[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sms)) if sms else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


# ---------------------------------------------------------------------------
# library arm
# ---------------------------------------------------------------------------

class FullbandBeam:
    """One beam: resident ring, dedispersion plan, analyser buffers."""

    def __init__(self, cfg, dev, seed):
        import ctypes as C
        import torch
        import pv
        self.cfg, self.dev, self.pv = cfg, dev, pv
        L = pv.load()
        self.L = L
        k, inv = pv.dm_shifts(cfg["fch1"], cfg["foff"], cfg["nchan"])
        self.inverted = inv
        self.start = float(np.float32(cfg["dm_low"]) / np.float32(cfg["tsamp"]))
        self.step_v = float(np.float32(cfg["dm_step"]) / np.float32(cfg["tsamp"]))
        self.plan = C.c_void_p()
        pv.check(L.pv_dedisp_plan_create(C.byref(self.plan), k.ctypes.data_as(C.POINTER(C.c_float)),
                                         cfg["nchan"], cfg["tdms"], self.start, self.step_v))
        L.pv_dedisp_plan_max_shift.restype = C.c_int
        L.pv_dedisp_plan_max_shift.argtypes = [C.c_void_p]
        L.pv_dedisp_plan_run.restype = C.c_int
        L.pv_dedisp_plan_run.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p,
                                         C.c_longlong, C.c_longlong, C.c_longlong, C.c_longlong,
                                         C.c_int, C.c_void_p]
        L.pv_ring_write.restype = C.c_int
        L.pv_ring_write.argtypes = [C.c_void_p, C.c_longlong, C.c_longlong, C.c_longlong, C.c_void_p,
                                    C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        self.max_shift = L.pv_dedisp_plan_max_shift(self.plan)
        nout, nchan = cfg["nout"], cfg["nchan"]
        self.ring_len = self.max_shift + nout
        self.row_stride = (self.ring_len + 31) // 32 * 32
        g = torch.Generator(device=dev)
        g.manual_seed(seed)
        self.ring = torch.randn((nchan, self.row_stride), generator=g, device=dev, dtype=torch.float32)
        self.out = torch.empty((cfg["tdms"], nout), device=dev, dtype=torch.float32)
        self.chunk_dev = torch.empty((nout, cfg["nsub"], 1, cfg["nchan_sub"]), device=dev,
                                     dtype=torch.float32)
        host = torch.randn((nout, cfg["nsub"], 1, cfg["nchan_sub"]), generator=torch.Generator().manual_seed(seed),
                           dtype=torch.float32)
        self.chunk_host = host.pin_memory()
        self.chunk_dev.copy_(self.chunk_host)
        self.cap = 1 << 20
        self.events = torch.empty(self.cap * 4, dtype=torch.int32, device=dev)
        self.pos = self.max_shift  # logical position of the next new sample
        self.rms = float(np.sqrt(np.float32(cfg["nchan_sub"]) * np.float32(cfg["nsub"])))
        self.n_events = 0

    def units_per_step(self):
        c = self.cfg
        return c["tdms"] * c["nchan"] * c["nout"]

    def step(self, stream, ev_pair=None, e2e=False):
        import ctypes as C
        import torch
        pv, L, c = self.pv, self.L, self.cfg
        s = C.c_void_p(stream.cuda_stream)
        if e2e:
            with torch.cuda.stream(stream):
                self.chunk_dev.copy_(self.chunk_host, non_blocking=True)
        pv.check(L.pv_ring_write(C.c_void_p(self.ring.data_ptr()), self.row_stride, self.ring_len,
                                 self.pos, C.c_void_p(self.chunk_dev.data_ptr()), c["nout"], c["nsub"],
                                 1, c["nchan_sub"], int(self.inverted), s))
        t_base = (self.pos + c["nout"] - self.ring_len) % self.ring_len
        if ev_pair is not None:
            ev_pair[0].record(stream)
        pv.check(L.pv_dedisp_plan_run(self.plan, C.c_void_p(self.out.data_ptr()), c["nout"],
                                      C.c_void_p(self.ring.data_ptr()), self.row_stride, 0,
                                      self.ring_len, t_base, c["nout"], s))
        if ev_pair is not None:
            ev_pair[1].record(stream)
        n = C.c_longlong()
        pv.check(L.pv_analyse(C.c_void_p(self.out.data_ptr()), c["nout"], c["tdms"], c["nout"],
                              c["threshold"], self.rms, c["bin_pow2"], C.c_void_p(self.events.data_ptr()),
                              self.cap, C.byref(n), s))
        self.n_events = n.value
        if e2e:
            k = min(n.value, self.cap)
            host_ev = self.events[: 4 * k].cpu()
            self.last_d2h = host_ev.numel() * 4
        self.pos += c["nout"]


def run_pv(args, cfg):
    import torch
    import torch.distributed as dist
    import pv

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    beam = FullbandBeam(cfg, dev, seed=1234 + rank)
    stream = torch.cuda.Stream(device=dev)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    # device-resident inputs
    for _ in range(args.warmup):
        beam.step(stream)
    barrier()
    launches0 = pv.launches()
    kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    t_start, t_stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    clocks.start()
    t_start.record(stream)
    for i in range(args.steps):
        beam.step(stream, kev[i])
    t_stop.record(stream)
    barrier()
    clk = clocks.stop()
    launches = pv.launches() - launches0
    ms = t_start.elapsed_time(t_stop)
    kernel_ms = [a.elapsed_time(b) for a, b in kev]

    # end to end through host buffers
    for _ in range(max(1, args.warmup // 2)):
        beam.step(stream, e2e=True)
    barrier()
    e_start, e_stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_start.record(stream)
    for _ in range(args.steps):
        beam.step(stream, e2e=True)
    e_stop.record(stream)
    barrier()
    e2e_ms = e_start.elapsed_time(e_stop)

    t = torch.tensor([ms, e2e_ms], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms, e2e_ms = float(t[0]), float(t[1])
    units = beam.units_per_step() * args.steps * world
    value = units / (ms / 1e3)
    e2e_value = units / (e2e_ms / 1e3)

    peaks, peak_src = measured_peaks()
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    fadd_peak = nsm * 128 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    k_avg = float(np.mean(kernel_ms)) / 1e3
    achieved = beam.units_per_step() / k_avg
    roofline = {"kernel": "dedisperse_kernel", "bound": "fp32",
                "achieved": achieved / 1e12, "peak": fadd_peak / 1e12, "unit": "Tadd/s",
                "frac": achieved / fadd_peak, "traffic": None,
                "peak_source": "%d SMs x 128 FP32 lanes x sm_max_mhz of MEASURED_PEAKS.json (%s)"
                               % (nsm, peak_src),
                "kernel_ms": k_avg * 1e3,
                "note": "one FP32 add per DM-trial*channel*sample; shared-memory reads cap the "
                        "FP32-storage kernel at 1/4 of this peak"}
    cpu = cpu_baseline(cfg, args, repeats=3) if (rank == 0 and not args.no_cpu) else None
    h2d = beam.chunk_host.numel() * 4
    line = {"metric": "DM-trial*chan*samples/s", "value": value, "unit": "DM-trial*chan*samples/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian filterbank)",
            "config": {"workload": cfg["workload"], "stage": "ring write + dedisperse + analyse",
                       "nchan": cfg["nchan"], "tdms": cfg["tdms"], "nout": cfg["nout"],
                       "ring_samples": beam.ring_len, "l2": "inputs larger than L2 (4.45 GB ring)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "e2e": {"value": e2e_value, "unit": "DM-trial*chan*samples/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": getattr(beam, "last_d2h", 0)},
            "gpu_launches": launches, "clocks": clk, "roofline": roofline, "cpu_baseline": cpu}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


_CPU_BUF = {}


def cpu_baseline(cfg, args, sample_trials=None, repeats=1):
    """The oracle's OpenMP dedispersion of the same formula (every core) on a
    bounded sample: the lowest trials over the full channel set and chunk."""
    from oracle import pyoracle as po
    po.build()
    k, _ = po.dm_shifts(cfg["fch1"], cfg["foff"], cfg["nchan"])
    start = np.float32(cfg["dm_low"]) / np.float32(cfg["tsamp"])
    step = np.float32(cfg["dm_step"]) / np.float32(cfg["tsamp"])
    tdms = cfg["tdms"]
    nt = min(sample_trials or args.cpu_trials, tdms)
    nout = cfg["nout"]
    key = (cfg["nchan"], nout, nt)
    if key not in _CPU_BUF:
        ms = int(po.shift_table(k, nt, start, step).max())
        rng = np.random.default_rng(5)
        _CPU_BUF.clear()
        _CPU_BUF[key] = rng.random((cfg["nchan"], nout + ms + 1), dtype=np.float32)
    buf = _CPU_BUF[key]
    t0 = time.perf_counter()
    for _ in range(repeats):
        po.dedisperse(buf, nout, nt, k, start, step)
    dt = time.perf_counter() - t0
    units = nt * cfg["nchan"] * nout * repeats
    return {"value": units / dt, "unit": "DM-trial*chan*samples/s", "cores": po.num_threads(),
            "kind": "port",
            "sample": "%d x (%d of %d trials x %d channels x %d samples), %.1f s"
                      % (repeats, nt, tdms, cfg["nchan"], nout, dt)}


def run_reference(args, cfg):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(cfg, args, sample_trials=args.ref_trials)
    t_all = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_baseline(cfg, args, sample_trials=args.ref_trials))
    total = time.perf_counter() - t_all
    value = float(np.mean([v["value"] for v in vals]))
    units_per_step = cfg["tdms"] * cfg["nchan"] * cfg["nout"]
    line = {"impl": "reference", "metric": "DM-trial*chan*samples/s", "value": value,
            "unit": "DM-trial*chan*samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": units_per_step / value * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Gaussian filterbank)",
            "config": {"workload": cfg["workload"], "nchan": cfg["nchan"], "tdms": cfg["tdms"],
                       "nout": cfg["nout"]},
            "cpu_baseline": {"value": value, "unit": "DM-trial*chan*samples/s",
                             "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"] + " per step; the reference needs Qt4, "
                                       "Boost, FFTW3 and pelican, so its algorithm's CPU "
                                       "restatement is timed"},
            "e2e": {"value": value, "unit": "DM-trial*chan*samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "wall_s": total}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="pv", choices=["pv", "reference"])
    ap.add_argument("--cpu-trials", type=int, default=512)
    ap.add_argument("--ref-trials", type=int, default=128)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--tdms", type=int, default=None, help="override (profiling a smaller case)")
    ap.add_argument("--nout", type=int, default=None, help="override (profiling a smaller case)")
    args = ap.parse_args()
    cfg = fullband_config()
    if args.tdms or args.nout:
        tdms = args.tdms or cfg["tdms"]
        cfg.update(tdms=tdms, nout=args.nout or cfg["nout"],
                   dm_step=cfg["dm_step"], workload=cfg["workload"] + "-reduced")
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_pv(args, cfg)


if __name__ == "__main__":
    main()
