#!/usr/bin/env python3
"""Throughput benchmark of the beam-processing hot path on GB300.

Metric: DM-trial*channel*samples per second: the brute-force dedispersion
work (trials x channels x output samples) of every chunk that passes through
the whole chain (PPF, Stokes I, x4 integration, RFI clipper, delay ring,
dedispersion, analyser), divided by wall time on the device.

Workload "batch64" (default): 64 uneven beams advanced one chunk of 4096
integrated spectra per step by the batched engine (pv_batch: every stage of
all beams in a few launches, one persistent dedispersion launch over every
beam's DM x time tiles with autotuned tile shapes, the step replayed from a
captured CUDA graph, pipelined: window k-lag-1 is dedispersed while chunk k is
channelised and clipped).  Beams are drawn with seed 64: subbands from {31, 61,
122, 244} LOFAR subbands of 195.3125 kHz from 110 MHz, 16 or 64 channels per
subband (8-tap Kaiser PPF), x4 integration (327.68 us or 1.31 ms), DM ranges
0-250 or 0-1000 pc/cm^3 in 1024, 2048 or 4096 trials, 5 sigma channel
clipping with zero-DMing and a 10000-spectrum history (the reference's
pipeline XML settings), 6 sigma detection.  Voltages: seeded Gaussian noise
(sigma 16 per component), persistent narrowband sinusoids in 3% of the
channels at 20 sigma, broadband bursts about once per 10^4 samples and 0-5
dispersed pulses per beam.  The same beams also run through the plain
per-beam chain (pv_beam: the same kernels one beam after another, events
read back after every beam), timed in the same run: "plain" and
"batched_over_plain" in the JSON line.  Rings start prefilled (as if each
beam's stream had been preceded by silence) so every beam dedisperses a
window from the first step; the work per step is the steady-state work.
The ring (154 GB) and voltages (45 GB per step) exceed L2, so no flush is
needed between steps.

Workload "fullband": one beam of 244 subbands (3904 channels), 2048 trials of
DM 0-500, chunks of 16384 spectra, through the single-beam chain.

``--impl reference`` times the reference algorithm's CPU restatement (the
reference cannot be built: it needs Qt4, Boost, FFTW3 and the pelican core) on
the host cores: the oracle's OpenMP channeliser, Stokes, integrator and RFI
clipper and its OpenMP brute-force dedispersion of the same formula, on a
bounded sample of the same workload extrapolated to whole chunks.
"""
import argparse
import json
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

SUB_BW = 0.1953125  # MHz
RAW_TSAMP = 5.12e-6  # s
# DRAM bytes per add of the batched dedispersion, measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum) on the mix's first 3 beams: (bytes, adds, the capture)
DD_BATCH_TRAFFIC = {
    ("f32", "pair"): (4.3636e9, 2.04816252928e11, "dedisperse_pair_kernel, tile variant 7, 4096-sample chunks"),
    ("f32", "one"): (1.776e9, 5.1204063232e10, "dedisperse_batch_kernel, FP32 rings, 1024-sample chunks"),
    ("f16", "one"): (0.907e9, 5.1204063232e10, "dedisperse_batch_kernel, FP16 rings, 1024-sample chunks"),
    ("u8", "one"): (0.457e9, 5.1204063232e10, "dedisperse_batch_kernel, u8 rings, 1024-sample chunks"),
}
RING_SAMPLES_PER_WORD = {"f32": 1, "f16": 2, "u8": 4}


def dd_kernel_name(variant):
    """The batched dedispersion kernel of a tile variant."""
    return "dedisperse_batch_kernel" if variant < 4 else "dedisperse_pair_kernel"


PAIR_S = 33       # output samples per lane of the trial-pair kernels
PAIR_LIM = {4: 32, 5: 32, 6: 15, 7: 15, 8: 15}  # largest shift difference read from registers


def shared_words_per_add(cfgs, variant, dms, store="f32", samples=64):
    """Shared-memory words the batched kernel reads per add on these beams:
    for the one-trial variants one sample per add (a 32-bit word holds 1, 2
    or 4 samples of an FP32, FP16 or u8 ring); for the trial-pair variants
    (FP32 rings) a lane reads 33 + delta words for its 66 adds (delta = the
    channel's shift difference between the pair's trials, up to the
    variant's limit) or 66 beyond it.  Evaluated over every channel and a
    sample of the trial pairs of each DM tile, weighted by adds."""
    if variant < 4:
        return 1.0 / RING_SAMPLES_PER_WORD[store]
    lim = PAIR_LIM[variant]
    words = adds = 0.0
    for c, h in zip(cfgs, dms):
        nb = c["nsub"] * c["nchan_sub"]
        f = c["fch1"] + np.arange(nb) * c["foff"]
        k = (4148.741601 * (1.0 / f ** 2 - 1.0 / f.max() ** 2)).astype(np.float32)
        step = np.float32(c["dm_step"]) / np.float32(c["tsamp"])
        ds = np.unique(np.linspace(0, c["tdms"] - 2, samples).astype(np.int64))
        ds = ds[(ds % h) % 2 == 0]  # first trial of a pair within its tile
        if len(ds) == 0:
            continue
        va = ds.astype(np.float32)[:, None] * step
        vb = (ds + 1).astype(np.float32)[:, None] * step
        sa = np.trunc(k[None, :] * va).astype(np.int64)
        sb = np.trunc(k[None, :] * vb).astype(np.int64)
        dl = sb - sa
        w = np.where(dl <= lim, PAIR_S + dl, 2 * PAIR_S).astype(np.float64)
        wt = c["tdms"] * c["chunk"] / len(ds)
        words += w.sum() * wt
        adds += 2 * PAIR_S * dl.size * wt
    return words / adds if adds else 1.0


def beam_dict(nsub, nchan_sub, dm_max, tdms, chunk, **kw):
    int_time = 4
    foff = SUB_BW / nchan_sub
    f_sub0 = 110.0
    d = dict(nsub=nsub, nchan_sub=nchan_sub, int_time=int_time, f_sub0=f_sub0,
             fch1=f_sub0 - (nchan_sub // 2) * foff, foff=foff, tsamp=RAW_TSAMP * nchan_sub * int_time,
             tdms=tdms, dm_low=0.0, dm_max=dm_max, dm_step=dm_max / (tdms - 1), chunk=chunk,
             threshold=6.0, bin_pow2=6, cr=5.0, sr=4.0, history=10000, zero_dming=1, window="kaiser",
             pulses=[])
    d.update(kw)
    return d


def fullband_config():
    d = beam_dict(244, 16, 500.0, 2048, 16384)
    d["workload"] = "fullband-244sub-3904ch-2048dm-16384samp"
    return d


def batch_configs(nbeams=64, chunk=4096, seed=64):
    """The 64-beam mix: uneven subband counts, channel counts, DM ranges and
    trial counts, 0-5 dispersed pulses each (DM uniform in 10..0.9*DM max,
    width 0.5-5 ms, at a uniform time in the chunk)."""
    rng = np.random.default_rng(seed)
    beams = []
    for _ in range(nbeams):
        nsub = int(rng.choice([31, 61, 122, 244]))
        nch = int(rng.choice([16, 64]))
        dm_max = float(rng.choice([250.0, 1000.0]))
        tdms = int(rng.choice([1024, 2048, 4096]))
        npulse = int(rng.integers(0, 6))
        pulses = [(float(rng.uniform(10.0, 0.9 * dm_max)), float(rng.uniform(0.5e-3, 5e-3)),
                   float(rng.uniform(0.1, 0.9))) for _ in range(npulse)]
        beams.append(beam_dict(nsub, nch, dm_max, tdms, chunk, pulses=pulses))
    return beams


def bp_text(cfg, median=1000.0):
    nbins = cfg["nsub"] * cfg["nchan_sub"]
    start, width = cfg["fch1"], cfg["foff"]
    return "\n".join(["# flat bandpass", str(nbins), repr(start), repr(start + width * nbins),
                      repr(width), "50.0", repr(median)]) + "\n"


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi samples taken during the timed region."""
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

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sms = [num(s[1]) for s in self.samples if len(s) > 2 and num(s[1]) is not None]
        mx = [num(s[2]) for s in self.samples if len(s) > 2 and num(s[2]) is not None]
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
# synthetic voltages
# ---------------------------------------------------------------------------

def udp_subbands(cfg):
    """Subbands per LOFAR packet stream for a beam: 61 for 16-bit beamlets, or all of a narrower beam."""
    return 61 if cfg["nsub"] % 61 == 0 else cfg["nsub"]


def to_packets(v, per_packet, ts0=1300000000):
    """int16 voltages [sub][pol][n][2] on the device -> the nsub/per_packet streams of variable-size
    LOFAR packets (16-byte header, [subband][16 samples][pol] complex int16), one after another."""
    import torch
    nsub, _, n, _ = v.shape
    streams, npk = nsub // per_packet, n // 16
    body = v.view(streams, per_packet, 2, npk, 16, 2).permute(0, 3, 1, 4, 2, 5).contiguous()
    body = body.view(torch.uint8).view(streams, npk, per_packet * 16 * 2 * 4)
    hdr = torch.zeros((streams, npk, 4), dtype=torch.int32, device=v.device)
    hdr[:, :, 2] = ts0
    hdr[:, :, 3] = 16 * torch.arange(npk, device=v.device, dtype=torch.int32)
    return torch.cat([hdr.view(torch.uint8).view(streams, npk, 16), body], dim=2).reshape(-1)


def max_over_ranks(times_ms, device, world):
    """Each time (ms) as the maximum over the ranks: the job ends with its slowest replica."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x) for x in times_ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def job_rate(units_per_rank_step, steps, world, ms):
    """Whole-job throughput: the units every rank processed over the slowest rank's time."""
    return units_per_rank_step * steps * world / (ms / 1e3)


def device_voltages(cfg, dev, seed):
    """int16 [sub][pol][n][2] on the device: noise, narrowband RFI, bursts."""
    import torch
    nsub, n = cfg["nsub"], cfg["chunk"] * cfg["int_time"] * cfg["nchan_sub"]
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    v = torch.randn((nsub, 2, n, 2), generator=g, device=dev, dtype=torch.float32) * 16.0
    # persistent narrowband sinusoids in 3% of the channels at 20 sigma
    nbins = nsub * cfg["nchan_sub"]
    rng = np.random.default_rng(seed)
    chans = rng.choice(nbins, size=max(1, int(0.03 * nbins)), replace=False)
    t = torch.arange(n, device=dev, dtype=torch.float64)
    for ch in chans:
        s, c = divmod(int(ch), cfg["nchan_sub"])
        f = (c - cfg["nchan_sub"] // 2) / cfg["nchan_sub"]  # cycles per sample within the subband
        ph = 2 * np.pi * f * t + rng.uniform(0, 2 * np.pi)
        v[s, :, :, 0] += (20 * 16.0 * torch.cos(ph)).float()
        v[s, :, :, 1] += (20 * 16.0 * torch.sin(ph)).float()
    # broadband bursts: 1 per 10^4 samples, 16 samples long, 3x the noise
    nb = max(1, n // 10000)
    for b0 in rng.integers(0, n - 16, size=nb):
        v[:, :, int(b0):int(b0) + 16, :] *= 3.0
    # dispersed pulses (dm, width s, position as a fraction of the chunk): in
    # every subband, complex noise of PULSE_SCALE x the noise variance under a
    # Gaussian envelope centred at the cold-plasma delay of the subband
    # centre, dispersed across the subband in the Fourier domain (the group
    # delay k*DM*(f^-2 - fc^-2) as a phase), so each channel holds the pulse
    # at its own delay.  Every step feeds the same chunk, so the stream is
    # periodic in the chunk duration and the burst is added modulo the chunk:
    # the whole dispersed track is in the stream, a pulse once per chunk.
    # Each channel's power rises by about 0.6 sigma of one integrated sample
    # at the peak, well under the 5-sigma channel clip; dedispersed over
    # hundreds to thousands of channels the pulse stands far above 6 sigma.
    k_dm, tsr = 4148.741601, RAW_TSAMP
    nch = cfg["nchan_sub"]
    f_top = cfg["f_sub0"] + (nsub - 1) * SUB_BW + (nch // 2 - 1) * SUB_BW / nch  # highest channel
    gp = torch.Generator(device=dev)
    gp.manual_seed(seed + 1)
    for dm, width, pos in cfg.get("pulses", []):
        sig = width / 2.3548
        for s in range(nsub):
            fc = cfg["f_sub0"] + s * SUB_BW
            tc = pos * n * tsr + k_dm * dm * (1 / fc ** 2 - 1 / f_top ** 2)
            lo_d = k_dm * dm * (1 / (fc + SUB_BW / 2) ** 2 - 1 / fc ** 2)
            hi_d = k_dm * dm * (1 / (fc - SUB_BW / 2) ** 2 - 1 / fc ** 2)
            L = 1 << int(np.ceil(np.log2(max((hi_d - lo_d + 12 * sig) / tsr, 32) * 2)))
            start = int(np.floor((tc + lo_d - 6 * sig) / tsr)) - L // 4
            t = (start + torch.arange(L, device=dev, dtype=torch.float64)) * tsr
            env = torch.exp(-0.5 * ((t - tc) / sig) ** 2)
            nu = torch.fft.fftfreq(L, d=tsr, device=dev, dtype=torch.float64)
            order = torch.argsort(nu)
            f = fc + nu[order] / 1e6
            delay = k_dm * dm * (1 / f ** 2 - 1 / fc ** 2)
            phase = torch.empty(L, device=dev, dtype=torch.float64)
            phase[order] = -2 * np.pi * torch.cumsum(delay, 0) * (1.0 / (L * tsr))
            rot = torch.polar(torch.ones_like(phase), phase).to(torch.complex64)
            idx = torch.remainder(start + torch.arange(L, device=dev), n)
            envf = (env * float(np.sqrt(PULSE_SCALE * 256.0))).float()
            for p in range(2):
                burst = torch.complex(torch.randn(L, generator=gp, device=dev),
                                      torch.randn(L, generator=gp, device=dev)) * envf
                disp = torch.fft.ifft(torch.fft.fft(burst) * rot)
                # pieces of at most n samples have distinct wrapped indices: the sums are
                # deterministic (index_add_ adds repeated indices atomically, in any order)
                for q in range(0, L, n):
                    v[s, p, :, 0].index_add_(0, idx[q:q + n], disp.real[q:q + n].float())
                    v[s, p, :, 1].index_add_(0, idx[q:q + n], disp.imag[q:q + n].float())
    return torch.clamp(torch.round(v), -32768, 32767).to(torch.int16)


# ---------------------------------------------------------------------------
# library arm
# ---------------------------------------------------------------------------

def pv_config(pv, cfg, **over):
    kw = dict(nsub=cfg["nsub"], nchan_sub=cfg["nchan_sub"], window=cfg["window"],
              int_time=cfg["int_time"], fch1=cfg["fch1"], foff=cfg["foff"], tsamp=cfg["tsamp"],
              tdms=cfg["tdms"], dm_low=cfg["dm_low"], dm_step=cfg["dm_step"], chunk=cfg["chunk"],
              threshold=cfg["threshold"], bin_pow2=cfg["bin_pow2"], bp_text=bp_text(cfg),
              cr=cfg["cr"], sr=cfg["sr"], history=cfg["history"], zero_dming=cfg["zero_dming"])
    kw.update(over)
    return pv.beam_config(**kw)


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
    beam = pv.Beam(pv_config(pv, cfg, timing=1))
    info = beam.info()
    stream = torch.cuda.Stream(device=dev)
    volts = [device_voltages(cfg, dev, 1000 + 7 * rank + i) for i in range(2)]
    host = volts[0].cpu().pin_memory()

    def step(i, e2e=False):
        if e2e:
            beam.process_host(host, stream=stream)
        else:
            beam.process(volts[i % 2], stream=stream)
        ev, n, first = beam.events(cap=1 << 16, stream=stream)
        return ev, n

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    # prime the delay ring (lag chunks) so that every timed chunk dedisperses
    for i in range(info["lag"]):
        step(i)
    for i in range(args.warmup):
        step(i)
    barrier()
    launches0 = pv.launches()
    lat_ms, stage = [], []
    clocks = ClockSampler(local)
    clocks.start()
    t_start, t_stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for i in range(args.steps):
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        ev, n = step(i)
        c1.record(stream)
        c1.synchronize()
        lat_ms.append(c0.elapsed_time(c1))
        stage.append(beam.stage_ms())
    t_stop.record(stream)
    barrier()
    clk = clocks.stop()
    launches = pv.launches() - launches0
    ms = t_start.elapsed_time(t_stop)
    n_events = n

    # end to end: host voltages in pinned memory, events back to the host
    for i in range(max(1, args.warmup)):
        step(i, e2e=True)
    barrier()
    e_start, e_stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_start.record(stream)
    d2h = 0
    for i in range(args.steps):
        ev, n = step(i, e2e=True)
        d2h = 8 + ev.nbytes
    e_stop.record(stream)
    barrier()
    e2e_ms = e_start.elapsed_time(e_stop)

    ms, e2e_ms = max_over_ranks([ms, e2e_ms], dev, world)
    nbins = info["nbins"]
    units_step = cfg["tdms"] * nbins * cfg["chunk"]
    value = job_rate(units_step, args.steps, world, ms)
    e2e_value = job_rate(units_step, args.steps, world, e2e_ms)

    peaks, peak_src = measured_peaks()
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    fadd_peak = nsm * 128 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    st = {k: float(np.mean([s[k] for s in stage])) for k in stage[0]}
    dd_s = st["dedisperse"] / 1e3
    achieved = units_step / dd_s
    in_bytes = beam.input_bytes(True)
    fb_bytes = cfg["chunk"] * nbins * 4
    chan_gbs = (in_bytes + fb_bytes) / (st["channelise"] / 1e3) / 1e9
    roofline = {"kernel": "dedisperse_kernel", "bound": "fp32",
                "achieved": achieved / 1e12, "peak": fadd_peak / 1e12, "unit": "Tadd/s",
                "frac": achieved / fadd_peak, "traffic": None,
                "peak_source": "%d SMs x 128 FP32 lanes x sm_max_mhz of MEASURED_PEAKS.json (%s)"
                               % (nsm, peak_src),
                "per_unit": "one FP32 add per DM-trial*channel*sample (%d per launch)" % units_step,
                "kernel_ms": st["dedisperse"]}
    roofline_chan = {"kernel": "channelise_kernel", "bound": "hbm", "achieved": chan_gbs,
                     "peak": float(peaks.get("hbm_gbs", 6800.0)), "unit": "GB/s",
                     "frac": chan_gbs / float(peaks.get("hbm_gbs", 6800.0)),
                     "per_unit": "int16 voltages in (%d B) + float filterbank out (%d B) per chunk"
                                 % (in_bytes, fb_bytes),
                     "kernel_ms": st["channelise"], "peak_source": peak_src}
    chunk_seconds = cfg["chunk"] * cfg["tsamp"]
    cpu = cpu_baseline(cfg, args) if (rank == 0 and not args.no_cpu) else None
    line = {"metric": "DM-trial*chan*samples/s", "value": value, "unit": "DM-trial*chan*samples/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded Gaussian int16 voltages with narrowband and burst RFI",
            "config": {"workload": cfg["workload"], "nsub": cfg["nsub"], "nchan": nbins,
                       "tdms": cfg["tdms"], "dm_range": [0.0, cfg["dm_max"]], "chunk": cfg["chunk"],
                       "tsamp_s": cfg["tsamp"], "ring_samples": info["ring_len"],
                       "l2": "inputs larger than L2 (2.05 GB voltages per chunk, 4.6 GB ring)",
                       "parallelism": "replicas" if world > 1 else "single beam"},
            "e2e": {"value": e2e_value, "unit": "DM-trial*chan*samples/s",
                    "h2d_bytes_per_step": in_bytes, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_ms / args.steps,
                    "what": "pv_beam_process_host: each chunk's voltages copied from a page-locked "
                            "host buffer, then its events read back to the host"},
            "gpu_launches": launches, "clocks": clk, "roofline": roofline,
            "roofline_channeliser": roofline_chan,
            "stage_ms": st,
            "latency_ms": {"p50": float(np.percentile(lat_ms, 50)),
                           "p99": float(np.percentile(lat_ms, 99)),
                           "chunk_duration": chunk_seconds * 1e3},
            "events_last_chunk": n_events,
            "cpu_baseline": cpu}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def run_batch(args, cfgs, workload):
    """The batched engine over many beams against the plain per-beam chain."""
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
    stream = torch.cuda.Stream(device=dev)
    nb = len(cfgs)
    units = [c["tdms"] * c["nsub"] * c["nchan_sub"] * c["chunk"] for c in cfgs]
    units_step = sum(units)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()

    def seed(i):
        return 5000 + 131 * rank + i

    # ---------------- plain per-beam chain ----------------
    # every beam's chunk resident on the device; host copies for the end-to-end pass
    udp = args.ingest == "udp"

    def beam_cfg(c):
        if not udp:
            return pv_config(pv, c, prefilled=1)
        p = udp_subbands(c)
        return pv_config(pv, c, prefilled=1, udp_packet_bytes=16 + p * 16 * 2 * 4, udp_subbands=p)

    def chunk_input(i, c):  # one step's input of beam i: int16 voltages, or the same as packets
        v = device_voltages(c, dev, seed(i))
        return to_packets(v, udp_subbands(c)) if udp else v

    volts = [chunk_input(i, c) for i, c in enumerate(cfgs)]
    beams = [pv.Beam(beam_cfg(c)) for c in cfgs]
    # page-locked staging, allocated after the arm's device memory: on this host the copy engine
    # read staging allocated first at 60-70 GB/s and staging allocated after the engine at
    # 211 GB/s (write-combined staging: 91 GB/s)
    hosts = []
    for v in volts:
        hosts.append(pv.HostBuffer(v.numel() * v.element_size()))
        hosts[-1].fill_from(v)

    plain_rec = [dict() for _ in range(nb)]  # window index -> (digest, events) of the untimed steps

    def plain_step(e2e=False, record=False):
        d2h = 0
        for i, b in enumerate(beams):
            if e2e:
                b.process_host(hosts[i], stream=stream)
            else:
                b.process(volts[i], stream=stream)
            ev, n, first = b.events(cap=1 << 16, stream=stream)  # synchronises: job per buffer
            d2h += 8 + ev.nbytes
            if record and first >= 0:
                c = cfgs[i]
                plain_rec[i][first // c["chunk"]] = (
                    window_digest(pv, b.buffers()[2], c["tdms"] * c["chunk"], stream), ev[:n].tobytes())
        return d2h

    plain_steps = max(2, args.steps // 2)
    # the warm-up steps are also the parity steps: every window they give is
    # compared with the batched engine's window of the same index
    for _ in range(max(args.warmup, PARITY_STEPS)):
        plain_step(record=True)
    barrier()
    t0 = time.perf_counter()
    for _ in range(plain_steps):
        plain_step()
    barrier()
    plain_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    for _ in range(plain_steps):
        plain_step(e2e=True)
    barrier()
    plain_e2e_ms = (time.perf_counter() - t0) * 1e3
    del beams, volts
    torch.cuda.synchronize()
    torch.cuda.empty_cache()

    # ---------------- batched engine ----------------
    batch = pv.Batch([beam_cfg(c) for c in cfgs], tune=args.variant is None, graph=True, timing=True,
                     variant=args.variant or 0,
                     pipelined=not args.unpipelined, store=args.store, rfi_one_cta=args.rfi_one_cta,
                     rfi_cluster8=args.rfi_cluster8, rfi_cluster4=args.rfi_cluster4)
    # the batch's staging, allocated after the batch (see the plain arm's), holds the plain arm's
    # very bytes: both arms take identical voltages
    bhosts = []
    L = pv.load()
    for i, c in enumerate(cfgs):
        bhosts.append(pv.HostBuffer(hosts[i].nbytes))
        pv.check(L.pv_device_copy(pv.C.c_void_p(bhosts[i].ptr), pv.C.c_void_p(hosts[i].ptr), hosts[i].nbytes,
                                  pv._stream(stream)))
        for par in (0, 1):  # the same chunk at every step: both input buffers
            p, nbytes = pv.C.c_void_p(), pv.C.c_longlong()
            pv.check(L.pv_batch_input_parity(batch.h, i, par, pv.C.byref(p), pv.C.byref(nbytes)))
            assert nbytes.value == bhosts[i].nbytes
            pv.check(L.pv_device_copy(p, pv.C.c_void_p(bhosts[i].ptr), nbytes.value, pv._stream(stream)))
        stream.synchronize()
    del hosts
    torch.cuda.empty_cache()
    infos = [batch.info(i) for i in range(nb)]
    tiles = batch.tiles()
    parity = {"windows_compared": 0, "identical": 0, "events_identical": 0, "events": 0,
              "beams_with_events": 0, "steps": 0}
    with_events = set()
    for _ in range(max(args.warmup, PARITY_STEPS + (0 if args.unpipelined else 1))):
        batch.run(stream=stream)
        stream.synchronize()
        parity["steps"] += 1
        for i in range(nb):
            ev, n, first = batch.events(i, step=-1)
            if first < 0:
                continue
            w = first // cfgs[i]["chunk"]
            if w not in plain_rec[i]:
                continue
            digest = window_digest(pv, batch.buffers(i)[1], cfgs[i]["tdms"] * cfgs[i]["chunk"], stream)
            want_digest, want_ev = plain_rec[i][w]
            parity["windows_compared"] += 1
            parity["identical"] += int(digest == want_digest)
            parity["events_identical"] += int(ev[:n].tobytes() == want_ev)
            parity["events"] += max(0, n - 1)
            if n > 1:
                with_events.add(i)
    parity["beams_with_events"] = len(with_events)
    parity["what"] = ("every beam's dedispersed window (exact digest of its FP32 bits) and event list from the "
                      "batched engine's untimed warm-up steps against the plain per-beam chain's window of "
                      "the same index; events exclude each window's dummy event")
    barrier()
    launches0 = pv.launches()
    lat_ms, stage = [], []
    clocks = ClockSampler(local)
    clocks.start()
    t_start, t_stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for _ in range(args.steps):
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        batch.run(stream=stream)
        c1.record(stream)
        c1.synchronize()
        lat_ms.append(c0.elapsed_time(c1))
        stage.append(batch.stage_ms())
    t_stop.record(stream)
    barrier()
    clk = clocks.stop()
    launches = pv.launches() - launches0
    ms = t_start.elapsed_time(t_stop)
    n_events = sum(batch.events(i, cap=0)[1] - 1 for i in range(nb))

    # end to end: every beam's voltages copied from pinned host memory each
    # step (on the batch's copy stream, overlapping the previous step) and
    # every beam's events of the previous step read back meanwhile
    def read_events(step):
        d2h = 0
        for i in range(nb):
            ev, n, _ = batch.events(i, step=step)
            d2h += 8 + ev.nbytes
        return d2h

    def e2e_run(k):
        d2h = 0
        for j in range(k):
            batch.run_host(bhosts, stream=stream)
            if j:
                d2h = read_events(-2)
        d2h = read_events(-1)
        return d2h

    e2e_run(max(1, args.warmup))
    barrier()
    e2e_steps = max(args.steps, E2E_MIN_STEPS)
    t0 = time.perf_counter()
    d2h = e2e_run(e2e_steps)
    barrier()
    e2e_ms = (time.perf_counter() - t0) * 1e3
    in_bytes = sum(batch.input(i)[1] for i in range(nb))

    # the same host-to-device copies alone (one scratch buffer, the copy engine idle otherwise):
    # the rate that bounds the end-to-end number
    scratch = torch.empty(max(h.nbytes for h in bhosts), dtype=torch.uint8, device=dev)
    h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    h0.record(stream)
    for h in bhosts:
        pv.check(pv.load().pv_device_copy(pv._ptr(scratch), pv.C.c_void_p(h.ptr), h.nbytes, pv._stream(stream)))
    h1.record(stream)
    h1.synchronize()
    h2d_alone_gbs = sum(h.nbytes for h in bhosts) / (h0.elapsed_time(h1) / 1e3) / 1e9
    del scratch
    ring_gb = sum(x["ring_bytes"] for x in infos) / 1e9
    precision = None
    if args.store != "f32" and args.chunk is None:  # reduced profiling cases start in the clipper's warm-up
        del batch
        batch = None
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        few = sorted(range(nb), key=lambda i: cfgs[i]["dm_max"] * cfgs[i]["nsub"])[:PRECISION_BEAMS]
        precision = precision_check(pv, [cfgs[i] for i in few], args.store, dev, seed(0))

    served = None
    if args.serve and args.chunk is None and world == 1:
        del batch, bhosts
        batch = None
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        served = short_serve(pv, cfgs, args.store)
    ms, e2e_ms, plain_ms, plain_e2e_ms = max_over_ranks([ms, e2e_ms, plain_ms, plain_e2e_ms], dev, world)
    value = job_rate(units_step, args.steps, world, ms)
    e2e_value = job_rate(units_step, e2e_steps, world, e2e_ms)
    plain_value = job_rate(units_step, plain_steps, world, plain_ms)
    plain_e2e = job_rate(units_step, plain_steps, world, plain_e2e_ms)

    peaks, peak_src = measured_peaks()
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    fadd_peak = nsm * 128 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    st = {k: float(np.mean([x[k] for x in stage])) for k in stage[0]}
    achieved = units_step / (st["dedisperse"] / 1e3)
    fb_bytes = sum(c["chunk"] * c["nsub"] * c["nchan_sub"] * 4 for c in cfgs)
    chan_gbs = (in_bytes + fb_bytes) / (st["channelise"] / 1e3) / 1e9
    variant = tiles["variant"]
    words = shared_words_per_add(cfgs, variant, tiles["dms"], args.store)
    t_bytes, t_adds, t_what = DD_BATCH_TRAFFIC[(args.store, "pair" if variant >= 4 else "one")]
    roofline = {"kernel": dd_kernel_name(variant), "bound": "fp32",
                "achieved": achieved / 1e12, "peak": fadd_peak / 1e12, "unit": "Tadd/s",
                "frac": achieved / fadd_peak,
                "smem_bound_frac": achieved * words / (fadd_peak / 4),
                "smem_words_per_add": words,
                "smem_bound": "32 four-byte shared-memory words per clock per SM (one 128-byte wavefront); "
                              "the kernel reads smem_words_per_add words per add on this workload",
                "traffic": t_bytes / t_adds * units_step,
                "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture "
                                  "(%s) on the mix's first 3 beams, scaled by adds" % t_what,
                "peak_source": "%d SMs x 128 FP32 lanes x sm_max_mhz of MEASURED_PEAKS.json (%s)"
                               % (nsm, peak_src),
                "per_unit": "one FP32 add per DM-trial*channel*sample (%d per launch)" % units_step,
                "kernel_ms": st["dedisperse"]}
    roofline_chan = {"kernel": "chan_stokes_i_kernel", "bound": "hbm", "achieved": chan_gbs,
                     "peak": hbm, "unit": "GB/s", "frac": chan_gbs / hbm,
                     "per_unit": "int16 voltages in (%d B) + float filterbank out (%d B) per step"
                                 % (in_bytes, fb_bytes),
                     "kernel_ms": st["channelise"], "peak_source": peak_src}
    chunk_s = [c["chunk"] * c["tsamp"] for c in cfgs]
    cpu = cpu_baseline_mix(cfgs) if (rank == 0 and not args.no_cpu) else None
    line = {"metric": "DM-trial*chan*samples/s", "value": value, "unit": "DM-trial*chan*samples/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded Gaussian int16 voltages with narrowband and burst RFI and "
                    "dispersed pulses",
            "config": {"workload": workload, "beams": nb, "chunk": cfgs[0]["chunk"],
                       "ingest": ("LOFAR UDP packets (variable size, 61 or all subbands per stream) "
                                  "read by the channeliser" if udp else "int16 voltages [sub][pol][t]"),
                       "nchan_total": sum(c["nsub"] * c["nchan_sub"] for c in cfgs),
                       "tdms_total": sum(c["tdms"] for c in cfgs), "ring_gb": ring_gb,
                       "ring_storage": args.store,
                       "input_gb_per_step": in_bytes / 1e9, "seed": 64,
                       "l2": "inputs larger than L2 (%.0f GB voltages per step, %.0f GB rings)"
                             % (in_bytes / 1e9, ring_gb),
                       "start": "prefilled rings (silence before each stream)",
                       "mode": ("unpipelined: each step dedisperses the window its chunk completes, in "
                                "one launch after the clippers" if args.unpipelined else
                                "pipelined: window k-lag-1 dedispersed while chunk k is channelised "
                                "and clipped"),
                       "clippers": "one CTA per beam" if args.rfi_one_cta else (
                                   "beams of more than 1024 channels on clusters of 128-thread CTAs"
                                   if args.rfi_cluster8 else (
                                       "one CTA per beam up to 4096 channels, else a cluster of 4 CTAs"
                                       if args.rfi_cluster4 or args.unpipelined else "one CTA per beam")),
                       "parallelism": "replicas" if world > 1 else "one GPU, all beams batched"},
            "e2e": {"value": e2e_value, "unit": "DM-trial*chan*samples/s",
                    "h2d_bytes_per_step": in_bytes, "d2h_bytes_per_step": d2h,
                    "steps": e2e_steps, "ms_per_step": e2e_ms / e2e_steps,
                    "h2d_alone_gbs": h2d_alone_gbs,
                    "h2d_alone_ms_per_step": in_bytes / h2d_alone_gbs / 1e6,
                    "what": "voltages copied from page-locked host buffers on the "
                            "batch's copy stream while the previous step computes; events of the "
                            "previous step read meanwhile; the timed steps start from an idle GPU, "
                            "so the first step's copy overlaps nothing"},
            "plain": {"value": plain_value, "e2e": plain_e2e, "steps": plain_steps,
                      "ms_per_step": plain_ms / plain_steps,
                      "what": "pv_beam per beam, one after another, events read back per beam"},
            "batched_over_plain": value / plain_value,
            "batched_over_plain_e2e": e2e_value / plain_e2e,
            "gpu_launches": launches, "clocks": clk, "roofline": roofline,
            "roofline_channeliser": roofline_chan,
            "stage_wall_ms": {"channelise": st["channelise"], "rfi_wall": st["rfi"],
                              "ring_write_wall": st["ring_write"], "dedisperse": st["dedisperse"],
                              "analyse": st["analyse"],
                              "what": "mean over the timed steps of the CUDA-event intervals at the stage "
                                      "boundaries on each stage's stream; pipelined, rfi_wall and "
                                      "ring_write_wall include the waits of those streams for SMs the "
                                      "concurrent dedispersion holds (the kernels alone: the launch list "
                                      "in profiles/)"},
            "tiles": {k: tiles[k] for k in ("variant", "time_tile", "chan_per_stage", "stages",
                                             "slot", "tiles", "ctas", "tune_ms", "graph_kernels")},
            "latency_ms": {"p50": float(np.percentile(lat_ms, 50)),
                           "p99": float(np.percentile(lat_ms, 99)),
                           "what": "device time of one step; pipelined, a window's events come "
                                   "one step after its last chunk, within 2 x p99",
                           "chunk_duration_min": min(chunk_s) * 1e3,
                           "chunk_duration_max": max(chunk_s) * 1e3},
            "events_last_step": n_events,
            "parity": parity,
            "cpu_baseline": cpu}
    if precision is not None:
        line["precision"] = precision
    if served is not None:
        line["serve"] = served
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


# The short serving run of the default line: the 64 beams of the mix as
# Poisson streams over SERVE_SECONDS under a 160 GB budget, through pv_serve.
SERVE_SECONDS = 20.0


def short_serve(pv, cfgs, store, seed=64):
    """p50/p99 chunk latency of the serving loop (pv_serve) over the batch mix."""
    import torch
    import serve
    dev = torch.device("cuda", 0)
    pcfgs = [pv_config(pv, c) for c in cfgs]
    spec = [{"cfg": pc, "tsamp": c["tsamp"], "tdms": c["tdms"], "nchan": c["nsub"] * c["nchan_sub"]}
            for pc, c in zip(pcfgs, cfgs)]
    streams = serve.poisson_streams(spec, SERVE_SECONDS, seed=seed)
    trace = []
    for i, (pc, st) in enumerate(zip(pcfgs, streams)):
        v = device_voltages(cfgs[i], dev, 7000 + i)
        hb = pv.HostBuffer(v.numel() * v.element_size())
        hb.fill_from(v)
        del v
        trace.append({"arrivals": st.arrivals, "sizes": st.sizes, "voltages": hb,
                      "units_per_spectrum": st.units_per_spectrum})
    flags = pv.BATCH_GRAPH | pv.BATCH_PIPELINED | {"f32": 0, "f16": 16, "u8": 32}[store] | (3 << 8)
    rep = pv.serve(pcfgs, trace, 160e9, policy="batch", batch_flags=flags, admit_every=0.5, linger=2.0,
                   horizon=SERVE_SECONDS + 20.0)
    durations = [s.sizes[0] * c["tsamp"] for s, c in zip(streams, cfgs)]
    return {"streams": len(streams), "seconds": SERVE_SECONDS, "chunks": rep["chunks"],
            "chunks_done": rep["chunks_done"], "latency_p50_ms": rep["latency_p50"] * 1e3,
            "latency_p99_ms": rep["latency_p99"] * 1e3,
            "latency_p99_over_chunk_duration": rep["latency_over_duration_p99"],
            "chunks_within_real_time": rep["within_real_time"],
            "admission_wait_p99_s": rep["admission_wait_p99"], "cohorts": rep["cohorts"],
            "slot_reuses": rep["slot_reuses"], "throughput": rep["throughput"],
            "chunk_duration_s": [min(durations), max(durations)],
            "what": "pv_serve (C++ loop): the mix's 64 beams as Poisson chunk streams (one chunk of 1-8 "
                    "steps per chunk duration), continuous batching under a 160 GB budget; latency from a "
                    "chunk's arrival to the end of the step that processed it"}


PRECISION_BEAMS = 6
# Voltage variance of an injected pulse relative to the noise at its peak.
PULSE_SCALE = 0.2
# Untimed steps of both arms whose windows and events are compared bit for bit.
PARITY_STEPS = 8


def window_digest(pv, ptr, n, stream):
    """Exact digest of n float32 values at a device pointer: the sums of the
    values' bit patterns and of the bit patterns weighted by odd position
    numbers (wrapping 64-bit integer arithmetic)."""
    import torch
    stream.synchronize()
    x = pv.device_array(ptr, (n,))  # copied on the legacy default stream
    torch.cuda.synchronize()
    x = x.view(torch.int32).to(torch.int64)
    w = torch.arange(1, 2 * n, 2, device=x.device, dtype=torch.int64)
    return int(x.sum().item()), int((x * w).sum().item())
# The batched end-to-end run starts from an idle GPU, so its first copy overlaps no compute;
# at least this many steps amortise that fill.
E2E_MIN_STEPS = 30


def precision_check(pv, cfgs, store, dev, seed):
    """The reduced-precision rings against FP32 on a few beams of the workload
    (the smallest delay spans, so that windows complete within a few steps):
    both batches start from silence and take identical voltages; the last
    window's dedispersed power is compared (relative rms over finite samples,
    and again without the outputs that read clipper-rejected spectra) and the
    events by (DM, sample, binning) key (Jaccard index)."""
    import torch
    runs = {st: pv.Batch([pv_config(pv, c) for c in cfgs], tune=False, graph=True, variant=3, store=st)
            for st in ("f32", store)}
    steps = max(runs["f32"].info(i)["lag"] for i in range(len(cfgs))) + 3
    for k in range(steps):
        for i, c in enumerate(cfgs):
            v = device_voltages(c, dev, seed + 7919 * k + i)
            for b in runs.values():
                b.set_input(i, v)
            del v
        for b in runs.values():
            b.run()
        torch.cuda.synchronize()
    errs, inter, union, nonfinite, windows = [], 0, 0, [0, 0], []
    errs_kept, excluded, counted = [], 0, 0
    for i, c in enumerate(cfgs):
        outs, keys = [], []
        for b in (runs["f32"], runs[store]):
            outs.append(pv.device_array(b.buffers(i)[1], (c["tdms"], c["chunk"])).double().cpu().numpy())
            ev, _, first = b.events(i)
            keys.append(set(zip(ev["dm"].tolist(), ev["t"].tolist(), ev["bin_factor"].tolist())))
        windows.append(first // c["chunk"] if first >= 0 else -1)
        ok = np.isfinite(outs[0]) & np.isfinite(outs[1])
        nonfinite[0] += int((~np.isfinite(outs[0])).sum())
        nonfinite[1] += int((~np.isfinite(outs[1])).sum())
        a, b = outs[0][ok], outs[1][ok]
        errs.append(float(np.sqrt(np.mean((b - a) ** 2) / np.mean(a ** 2))))
        # spectra the clipper rejects become -0.2 minus the bandpass (hundreds of sigma below
        # zero after normalisation); the u8 code range (+-6 sigma) saturates them, so the
        # outputs that read one fall far below the noise: leave those out of the second figure
        keep = a >= -8.0 * np.sqrt(c["nsub"] * c["nchan_sub"])
        excluded += int((~keep).sum())
        counted += int(a.size)
        errs_kept.append(float(np.sqrt(np.mean((b[keep] - a[keep]) ** 2) / np.mean(a[keep] ** 2))))
        inter += len(keys[0] & keys[1])
        union += len(keys[0] | keys[1])
    del runs
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return {"beams": len(cfgs), "steps": steps, "windows_compared": len(cfgs),
            "rel_rms_vs_f32_max": max(errs), "rel_rms_vs_f32_mean": float(np.mean(errs)),
            "rel_rms_vs_f32_without_rejected_spectra": {"max": max(errs_kept), "mean": float(np.mean(errs_kept)),
                                                        "outputs_left_out": excluded / max(counted, 1),
                                                        "left_out": "outputs below -8 sigma of the "
                                                                    "dedispersed noise in FP32"},
            "event_jaccard": inter / union if union else None, "events_union": union,
            "windows": windows, "nonfinite_samples": {"f32": nonfinite[0], store: nonfinite[1]},
            "fp32_vs_fp64": "within 1e-5 relative rms (parity tests)"}


# ---------------------------------------------------------------------------
# io workload: the byte-bound kernels before and after the path
# ---------------------------------------------------------------------------

# the reference adapter test's chunk (AdapterTimeSeriesDataSetTest.cpp setUp): 16384 fixed-size
# packets of 61 subbands x 16 samples x 2 polarisations of complex int16
UDP_CHUNK = dict(fixedSizePackets=True, dataBitSize=16, udpPacketsPerIteration=16384, samplesPerPacket=16,
                 outputChannelsPerSubband=16, subbandsPerPacket=61, nRawPolarisations=2)
UDP_PACKET = 8148


def udp_chunk(rng, npk, nsub, spp):
    """npk fixed-size packets with counting headers and random int16 samples."""
    chunk = np.zeros((npk, UDP_PACKET), np.uint8)
    data = rng.integers(-2048, 2048, size=(npk, nsub * spp * 2 * 2), dtype=np.int16)
    chunk[:, 16:16 + data.shape[1] * 2] = data.view(np.uint8)
    hdr = np.zeros((npk, 4), np.uint32)
    hdr[:, 2] = 1300000000
    hdr[:, 3] = 1000 + spp * np.arange(npk)
    chunk[:, :16] = hdr.view(np.uint8)
    return chunk.reshape(-1)


def run_io(args):
    """HBM-bound kernels around the path, each timed alone with CUDA events over
    inputs that rotate through more than L2: the UDP unpack of the reference
    adapter test's chunk (16384 packets, 133 MB) to int16 station order and to
    TimeSeriesDataSetC32; the sigproc pack of a full-band filterbank chunk
    (16384 x 3904) to 8- and 32-bit files; the bandpass recorder's integration
    of the same filterbank; the ALFABURST assembly of 16384 spectrometer
    packets of 1024 channels (134 MB, one packet in four kept)."""
    import torch
    import pv

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    peaks, peak_src = measured_peaks()
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    rng = np.random.default_rng(11)
    nrot = 8  # rotating inputs: 8 x 133 MB of packets, 8 x 256 MB of filterbank
    ad = pv.UdpAdapter(**UDP_CHUNK)
    chunk_bytes = UDP_PACKET * UDP_CHUNK["udpPacketsPerIteration"]
    host_chunk = udp_chunk(rng, UDP_CHUNK["udpPacketsPerIteration"], 61, 16)
    chunks = [torch.from_numpy(host_chunk).to(dev) for _ in range(nrot)]
    nt, nsub, nchan = 16384, 244, 16
    fbs = [torch.randn((nt, nsub, 1, nchan), device=dev) * 50 + 120 for _ in range(nrot)]
    launches0 = pv.launches()
    clocks = ClockSampler(0)
    clocks.start()

    def timed(fn):
        with torch.cuda.stream(stream):
            for k in range(args.warmup):
                fn(k % nrot)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for k in range(args.steps * nrot):
                fn(k % nrot)
            e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / (args.steps * nrot)  # ms per launch

    out_c32 = torch.empty((61, 2, 16384, 16), dtype=torch.complex64, device=dev)
    out_i16 = torch.empty((61, 2, 16384 * 16, 2), dtype=torch.int16, device=dev)
    cfg = ad.cfg
    res = {}

    def udp(out, kind):
        def fn(k):
            pv.check(pv.load().pv_udp_unpack(pv.C.byref(cfg), pv._ptr(chunks[k]), chunk_bytes, pv._ptr(out),
                                             pv.UDP_OUT[kind], pv._stream(stream)))
        return fn
    for kind, out in (("i16", out_i16), ("c32", out_c32)):
        ms = timed(udp(out, kind))
        byts = chunk_bytes + out.numel() * out.element_size()
        res["udp_unpack_" + kind] = {"ms": ms, "bytes": byts, "gbs": byts / ms / 1e6, "frac": byts / ms / 1e6 / hbm}
    for nbits in (8, 32):
        out = torch.empty(nt * nsub * nchan * nbits // 8, dtype=torch.uint8, device=dev)

        def fn(k, out=out, nbits=nbits):
            pv.check(pv.load().pv_sigproc_pack(pv._ptr(fbs[k]), nt, nsub, 1, nchan, 1, nbits, 0.0, 255.0,
                                               pv._ptr(out), pv._stream(stream)))
        ms = timed(fn)
        byts = fbs[0].numel() * 4 + out.numel()
        res["sigproc_pack_%d" % nbits] = {"ms": ms, "bytes": byts, "gbs": byts / ms / 1e6, "frac": byts / ms / 1e6 / hbm}
    rec = pv.BandPassRecorder(requiredSamples=1 << 62, coefficients=3, startFrequency=110.0, endFrequency=157.65625)

    def bp(k):
        pv.check(min(0, pv.load().pv_bandpass_recorder_add(rec.h, pv._ptr(fbs[k]), nt, nsub, 1, nchan,
                                                           pv._stream(stream))))
    ms = timed(bp)
    byts = fbs[0].numel() * 4
    res["bandpass_integrate"] = {"ms": ms, "bytes": byts, "gbs": byts / ms / 1e6, "frac": byts / ms / 1e6 / hbm}
    # ALFABURST spectrometer packets: 8-byte header, 1024 records of four big-endian 16-bit values
    npk_ab, nch_ab = 16384, 1024
    psize = 8 + 8 * nch_ab
    ab_host = np.zeros((npk_ab, psize), np.uint8)
    counts = np.arange(npk_ab, dtype=np.uint64) // 4
    for b in range(6):
        ab_host[:, b] = (counts >> np.uint64(8 * (5 - b))) & np.uint64(0xFF)
    ab_host[:, 6] = np.arange(npk_ab) % 4
    ab_host[:, 8:] = rng.integers(0, 256, (npk_ab, 8 * nch_ab), dtype=np.uint8)
    ab_host = ab_host.reshape(-1)
    abc = pv.AbConfig(4, nch_ab, 0, 0.000128)
    ab_chunks = [torch.from_numpy(ab_host).to(dev) for _ in range(nrot)]
    ab_idx = torch.arange(1, npk_ab, 4, dtype=torch.int32, device=dev)  # the quarter-1 packets
    ab_out = torch.empty((npk_ab // 4, nch_ab), dtype=torch.float32, device=dev)

    def ab(k):
        pv.check(pv.load().pv_ab_unpack(pv.C.byref(abc), pv._ptr(ab_chunks[k]), len(ab_host), pv._ptr(ab_idx),
                                        npk_ab // 4, npk_ab // 4, pv._ptr(ab_out), pv._stream(stream)))
    ms = timed(ab)
    byts = ab_out.numel() * 8 + ab_out.numel() * 4 + ab_idx.numel() * 4  # kept records in, spectra out
    res["ab_unpack"] = {"ms": ms, "bytes": byts, "gbs": byts / ms / 1e6, "frac": byts / ms / 1e6 / hbm}
    clk = clocks.stop()
    launches = pv.launches() - launches0

    # end to end: the chunk from page-locked host memory, unpacked, the voltages read back
    hb = pv.HostBuffer(chunk_bytes)
    hb.fill_from(chunks[0])
    back = torch.empty(out_i16.shape, dtype=torch.int16).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            pv.check(pv.load().pv_device_copy(pv._ptr(chunks[0]), pv.C.c_void_p(hb.ptr), chunk_bytes,
                                              pv._stream(stream)))
            udp(out_i16, "i16")(0)
            back.copy_(out_i16, non_blocking=True)
        stream.synchronize()
    e2e_s = (time.perf_counter() - t0) / args.steps
    u = res["udp_unpack_i16"]
    cpu = None
    if not args.no_cpu:
        from oracle import pyoracle as po
        t0 = time.perf_counter()
        po.udp_unpack(host_chunk, UDP_PACKET, UDP_CHUNK["udpPacketsPerIteration"], 16, 61, 2, 16)
        cs = time.perf_counter() - t0
        cpu = {"value": chunk_bytes / cs / 1e9, "unit": "GB/s of packets", "cores": 1, "kind": "port",
               "sample": "one 16384-packet chunk through the oracle's scalar _readData restatement"}
    line = {"metric": "UDP chunk bytes unpacked per second", "value": chunk_bytes / u["ms"] / 1e6,
            "unit": "GB/s of packets", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": u["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int16", "data": "synthetic: seeded int16 samples in LOFAR packets; seeded Gaussian filterbank",
            "config": {"workload": "io-udp-16384x61sub-sigproc-bandpass-16384x3904",
                       "udp": UDP_CHUNK, "chunk_bytes": chunk_bytes,
                       "l2": "inputs rotate through 8 buffers (1.07 GB of packets, 2.05 GB of filterbank)"},
            "e2e": {"value": chunk_bytes / e2e_s / 1e9, "unit": "GB/s of packets",
                    "h2d_bytes_per_step": chunk_bytes, "d2h_bytes_per_step": out_i16.numel() * 2},
            "gpu_launches": launches, "clocks": clk,
            "roofline": {"kernel": "udp_unpack_kernel<16, false>", "bound": "hbm", "achieved": u["gbs"],
                         "peak": hbm, "unit": "GB/s", "frac": u["frac"], "traffic": None,
                         "per_unit": "chunk bytes read + int16 voltages written per launch",
                         "peak_source": peak_src},
            "kernels": res, "cpu_baseline": cpu}
    print(json.dumps(line))


def serve_beams(nbeams=128, seed=128):
    """The serving mix: channel counts 512-15616 (32, 61, 122 or 244 subbands of
    16 or 64 channels), DM ranges 0-250 or 0-1000 in 1024-4096 trials."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nbeams):
        nsub = int(rng.choice([32, 61, 122, 244]))
        nch = int(rng.choice([16, 64]))
        dm_max = float(rng.choice([250.0, 1000.0]))
        tdms = int(rng.choice([1024, 2048, 4096]))
        out.append(beam_dict(nsub, nch, dm_max, tdms, 4096))
    return out


def run_serve(args, workload):
    """The serving loop (pv_serve, C++ in the library) over 128 streaming
    beams: the batched engine, then the plain per-chunk path, on the same
    Poisson trace."""
    import torch
    import pv
    import serve

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    beams = serve_beams(args.beams)
    cfgs = [pv_config(pv, b) for b in beams]
    spec = [{"cfg": c, "tsamp": b["tsamp"], "tdms": b["tdms"], "nchan": b["nsub"] * b["nchan_sub"]}
            for c, b in zip(cfgs, beams)]
    streams = serve.poisson_streams(spec, args.duration, seed=7)
    budget = int(args.budget_gb * 1e9)

    def staging(cfg):  # one sub-chunk of seeded voltages in page-locked memory: the stream's receive buffer
        g = torch.Generator(device=dev)
        g.manual_seed(int(cfg.nsub) * 1000 + int(cfg.nchan_sub))
        n = serve.SUB_CHUNK * cfg.int_time * cfg.nchan_sub
        v = torch.randn((cfg.nsub, 2, n, 2), generator=g, device=dev) * 16.0
        v = torch.clamp(torch.round(v), -32768, 32767).to(torch.int16)
        hb = pv.HostBuffer(v.numel() * v.element_size())
        hb.fill_from(v)
        return hb

    bufs = [staging(c) for c in cfgs]
    trace = [{"arrivals": s.arrivals, "sizes": s.sizes, "voltages": bufs[i], "units_per_spectrum": s.units_per_spectrum}
             for i, s in enumerate(streams)]
    flags = pv.BATCH_GRAPH | pv.BATCH_PIPELINED | {"f32": 0, "f16": 16, "u8": 32}[args.store] | (3 << 8)
    reports = {}
    clocks = ClockSampler(0)
    clocks.start()
    for name, policy in (("batched", "batch"), ("plain", "fifo1")):
        launches0 = pv.launches()
        rep = pv.serve(cfgs, trace, budget, policy=policy, batch_flags=flags, admit_every=0.5, linger=2.0,
                       horizon=args.duration + args.grace)
        rep["gpu_launches"] = pv.launches() - launches0
        reports[name] = rep
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    clk = clocks.stop()
    b, p = reports["batched"], reports["plain"]
    rt_units = sum(s.units_per_spectrum * sum(s.sizes) for s in streams)
    sub_bytes = [h.nbytes for h in bufs]
    line = {"metric": "DM-trial*chan*samples/s", "value": b["throughput"],
            "unit": "DM-trial*chan*samples/s", "n_gpus": 1, "steps": b["steps"],
            "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded Gaussian int16 voltages, Poisson chunk arrivals",
            "config": {"workload": workload, "beams": len(streams), "duration_s": args.duration,
                       "ring_storage": args.store, "loop": "pv_serve (C++)",
                       "budget_gb": args.budget_gb,
                       "chunks": b["chunks"], "offered_units": rt_units,
                       "chunk_spectra": "4096-32768 per beam, Poisson, one chunk per chunk duration",
                       "nchan_range": [min(x["nchan"] for x in spec), max(x["nchan"] for x in spec)]},
            "e2e": {"value": b["throughput"], "unit": "DM-trial*chan*samples/s",
                    "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                    "sub_chunk_bytes_mean": float(np.mean(sub_bytes)),
                    "what": "every sub-chunk's voltages copied from its stream's page-locked receive buffer, "
                            "wall time of the whole trace"},
            "serve": b, "plain": p,
            "latency_ms": {"p50": b["latency_p50"] * 1e3, "p99": b["latency_p99"] * 1e3,
                           "p99_after_admission": b["latency_admitted_p99"] * 1e3,
                           "p99_over_chunk_duration": b["latency_over_duration_p99"],
                           "plain_p50": p["latency_p50"] * 1e3,
                           "plain_p99": p["latency_p99"] * 1e3,
                           "plain_p99_over_chunk_duration": p["latency_over_duration_p99"]},
            "batched_over_plain_latency_p99": p["latency_p99"] / max(b["latency_p99"], 1e-9),
            "gpu_launches": b["gpu_launches"], "clocks": clk, "cpu_baseline": None}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# CPU restatement (baseline / reference arm)
# ---------------------------------------------------------------------------

class CpuChain:
    """The oracle's chain on a bounded sample of one chunk: an eighth of the
    subbands through PPF/Stokes/integration (x8), the full-band RFI clipper on
    one chunk of filterbank, and an eighth of the trials dedispersed over every
    channel and the whole chunk (x8)."""

    def __init__(self, cfg, sub_frac=8, trial_frac=8, add_budget=None):
        from oracle import pyoracle as po
        po.build()
        self.po, self.cfg = po, cfg
        nsub, nch, it = cfg["nsub"], cfg["nchan_sub"], cfg["int_time"]
        self.ns = max(1, nsub // sub_frac)
        self.sub_scale = nsub / self.ns
        self.nt = max(1, cfg["tdms"] // trial_frac)
        if add_budget:  # trials so that one sample costs about add_budget adds
            self.nt = int(max(1, min(cfg["tdms"], add_budget // (nsub * nch * cfg["chunk"]))))
        self.trial_scale = cfg["tdms"] / self.nt
        rng = np.random.default_rng(3)
        n = cfg["chunk"] * it * nch
        self.volt = (rng.standard_normal((self.ns, 2, n), dtype=np.float32) * 16 +
                     1j * rng.standard_normal((self.ns, 2, n), dtype=np.float32) * 16).astype(np.complex64)
        coeffs = po.fir_coefficients(8, nch, cfg["window"]).astype(np.float32)
        self.ppf = po.PPF(nch, 8, coeffs)
        self.fb = rng.gamma(8.0, 125.0, size=(cfg["chunk"], nsub, 1, nch)).astype(np.float32)
        nbins = nsub * nch
        self.k, _ = po.dm_shifts(cfg["fch1"], cfg["foff"], nbins)
        self.start = np.float32(cfg["dm_low"]) / np.float32(cfg["tsamp"])
        self.step = np.float32(cfg["dm_step"]) / np.float32(cfg["tsamp"])
        ms = int(po.shift_table(self.k, self.nt, self.start, self.step).max())
        self.buf = rng.standard_normal((nbins, cfg["chunk"] + ms + 1), dtype=np.float32)
        self.rms = float(np.sqrt(np.float32(nch) * np.float32(nsub)))
        self.sample = ("%d of %d subbands through PPF/Stokes/x%d integration (x%.0f), RFI on the "
                       "full %d-channel chunk, %d of %d trials dedispersed and analysed over all "
                       "channels and %d samples (x%.0f)"
                       % (self.ns, nsub, it, self.sub_scale, nbins, self.nt, cfg["tdms"], cfg["chunk"],
                          self.trial_scale))

    def chunk_seconds(self):
        po, cfg = self.po, self.cfg
        t0 = time.perf_counter()
        spec = self.ppf.run(self.volt.reshape(self.ns, 2, -1, cfg["nchan_sub"]))
        st = po.integrate(po.stokes(spec, 1), cfg["int_time"], 1)
        t1 = time.perf_counter()
        r = po.RFI(bp_text(cfg), cr=cfg["cr"], sr=cfg["sr"], history=cfg["history"],
                   zero_dming=cfg.get("zero_dming", 0), mode=0)
        fb = self.fb.copy()
        t2 = time.perf_counter()
        r.run(fb)
        t3 = time.perf_counter()
        out = po.dedisperse(self.buf, cfg["chunk"], self.nt, self.k, self.start, self.step)
        po.analyse(out, cfg["threshold"], self.rms, cfg["bin_pow2"])
        t4 = time.perf_counter()
        del st
        self.last_wall = (t1 - t0) + (t3 - t2) + (t4 - t3)  # what was actually run
        return (t1 - t0) * self.sub_scale + (t3 - t2) + (t4 - t3) * self.trial_scale


def host_cpu():
    """The host's CPU model and logical CPU count, for the CPU baselines."""
    model, impl, part = None, None, None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key, _, val = line.partition(":")
                key, val = key.strip(), val.strip()
                if key == "model name" and model is None:
                    model = val
                elif key == "CPU implementer" and impl is None:
                    impl = val
                elif key == "CPU part" and part is None:
                    part = val
    except OSError:
        pass
    if model is None and part is not None:
        model = {"0xd4f": "Arm Neoverse V2"}.get(part.lower(), "Arm implementer %s part %s" % (impl, part))
    return {"cpu_model": model or "unknown", "nproc": os.cpu_count()}


def cpu_baseline(cfg, args, repeats=1):
    chain = CpuChain(cfg)
    secs = [chain.chunk_seconds() for _ in range(repeats)]
    units = cfg["tdms"] * cfg["nsub"] * cfg["nchan_sub"] * cfg["chunk"]
    return {"value": units / float(np.median(secs)), "unit": "DM-trial*chan*samples/s",
            "cores": chain.po.num_threads(), "kind": "port", **host_cpu(),
            "sample": chain.sample + "; %.1f s per chunk extrapolated" % float(np.median(secs))}


MIX_SAMPLE = 4  # beams of the mix timed on the CPU
MIX_ADDS = 1.2e10  # dedispersion adds per sampled beam


def cpu_mix_sample(cfgs):
    return [CpuChain(c, add_budget=MIX_ADDS) for c in cfgs[:MIX_SAMPLE]]


def cpu_mix_seconds(chains, cfgs):
    """CPU seconds per step of the whole mix: the sampled beams' chain time
    scaled by the mix's work over the sampled beams' work."""
    secs = [ch.chunk_seconds() for ch in chains]
    units = [c["tdms"] * c["nsub"] * c["nchan_sub"] * c["chunk"] for c in cfgs]
    return float(np.sum(secs)) * sum(units) / sum(units[:len(chains)])


def cpu_baseline_mix(cfgs):
    chains = cpu_mix_sample(cfgs)
    secs = cpu_mix_seconds(chains, cfgs)
    units = sum(c["tdms"] * c["nsub"] * c["nchan_sub"] * c["chunk"] for c in cfgs)
    return {"value": units / secs, "unit": "DM-trial*chan*samples/s",
            "cores": chains[0].po.num_threads(), "kind": "port", **host_cpu(),
            "sample": "first %d beams of the mix, each: %s; scaled to the %d-beam step by work "
                      "(%.1f s per step)" % (len(chains), "; ".join(ch.sample for ch in chains),
                                             len(cfgs), secs)}


def run_reference(args, cfgs, workload):
    """The reference arm: the reference algorithm's CPU restatement on the host
    cores, on the same workload (a bounded sample per step, scaled to whole
    steps by work)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    if len(cfgs) == 1:
        chains = [CpuChain(cfgs[0])]
        step_secs = lambda: chains[0].chunk_seconds()  # noqa: E731
        sample = chains[0].sample
    else:
        chains = cpu_mix_sample(cfgs)
        step_secs = lambda: cpu_mix_seconds(chains, cfgs)  # noqa: E731
        sample = ("first %d beams of the %d-beam mix, scaled to the step by work: "
                  % (len(chains), len(cfgs)) + "; ".join(ch.sample for ch in chains))
    for _ in range(args.warmup):
        step_secs()
    secs, walls = [], []
    for _ in range(args.steps):
        secs.append(step_secs())
        walls.append(sum(ch.last_wall for ch in chains))
    units = sum(c["tdms"] * c["nsub"] * c["nchan_sub"] * c["chunk"] for c in cfgs)
    value = units * len(secs) / float(np.sum(secs))
    line = {"impl": "reference", "metric": "DM-trial*chan*samples/s", "value": value,
            "unit": "DM-trial*chan*samples/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(walls)) * 1e3,
            "ms_per_step_what": "host time of the bounded sample each step runs; value is the whole step's "
                                "work over the step's time extrapolated from the sample's stage times",
            "ms_per_step_extrapolated": float(np.mean(secs)) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded Gaussian voltages and filterbank",
            "config": {"workload": workload, "beams": len(cfgs),
                       "nchan_total": sum(c["nsub"] * c["nchan_sub"] for c in cfgs),
                       "tdms_total": sum(c["tdms"] for c in cfgs), "chunk": cfgs[0]["chunk"]},
            "cpu_baseline": {"value": value, "unit": "DM-trial*chan*samples/s",
                             "cores": chains[0].po.num_threads(), "kind": "port", **host_cpu(),
                             "sample": sample + " per step; the reference needs Qt4, Boost, "
                                       "FFTW3 and pelican, so its algorithm's CPU restatement is "
                                       "timed"},
            "e2e": {"value": value, "unit": "DM-trial*chan*samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="pv", choices=["pv", "reference"])
    ap.add_argument("--workload", default="batch64", choices=["batch64", "fullband", "serve128", "io"])
    ap.add_argument("--beams", type=int, default=None, help="number of beams (64 / 128)")
    ap.add_argument("--duration", type=float, default=60.0, help="serve128: seconds of arrivals")
    ap.add_argument("--grace", type=float, default=30.0, help="serve128: seconds to drain")
    ap.add_argument("--budget-gb", type=float, default=160.0, help="serve128: HBM budget")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ingest", default="voltages", choices=["voltages", "udp"],
                    help="batch64: each step's input as int16 voltages or as LOFAR UDP packet streams")
    ap.add_argument("--unpipelined", action="store_true",
                    help="batch64: one dedispersion launch per step after the clippers (the same work)")
    ap.add_argument("--store", default="f32", choices=["f32", "f16", "u8"],
                    help="batch64, serve128: delay-ring storage (FP32, FP16, or uint8 with per-channel scale)")
    ap.add_argument("--rfi-one-cta", action="store_true",
                    help="batch64: every beam's clipper on one CTA (default: beams of more than 1024 "
                         "channels on a cluster of 2 or 4 CTAs)")
    ap.add_argument("--rfi-cluster4", action="store_true",
                    help="batch64: clippers of beams of more than 4096 channels on clusters of 4 CTAs")
    ap.add_argument("--rfi-cluster8", action="store_true",
                    help="batch64: clippers of beams of more than 1024 channels on clusters of 128-thread CTAs")
    ap.add_argument("--tdms", type=int, default=None, help="reduced case for profiling")
    ap.add_argument("--no-serve", dest="serve", action="store_false",
                    help="batch64: skip the short serving run")
    ap.add_argument("--variant", type=int, default=None,
                    help="dedispersion tile variant (0-8) instead of the autotuner's choice (profiling)")
    ap.add_argument("--chunk", type=int, default=None, help="reduced case for profiling")
    ap.add_argument("--nsub", type=int, default=None, help="reduced case for profiling")
    args = ap.parse_args()
    if args.workload == "io":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the io workload times device kernels only; "
                              "its cpu_baseline key holds the CPU restatement's rate"}))
            return
        run_io(args)
        return
    if args.workload == "fullband":
        cfg = fullband_config()
        if args.tdms or args.chunk or args.nsub:
            if args.tdms:
                cfg["tdms"] = args.tdms
                cfg["dm_step"] = cfg["dm_max"] / (cfg["tdms"] - 1)
            cfg["chunk"] = args.chunk or cfg["chunk"]
            cfg["nsub"] = args.nsub or cfg["nsub"]
            cfg["workload"] += "-reduced(tdms=%d,chunk=%d,nsub=%d)" % (cfg["tdms"], cfg["chunk"],
                                                                        cfg["nsub"])
        if args.impl == "reference":
            run_reference(args, [cfg], cfg["workload"])
        else:
            run_pv(args, cfg)
        return
    if args.workload == "serve128":
        args.beams = args.beams or 128
        workload = "serve%d-poisson-%gs-%ggb" % (args.beams, args.duration, args.budget_gb)
        if args.store != "f32":
            workload += "-%s-rings" % args.store
        if args.impl == "reference":
            cfgs = serve_beams(args.beams)
            run_reference(args, cfgs, workload)
        else:
            run_serve(args, workload)
        return
    args.beams = args.beams or 64
    cfgs = batch_configs(args.beams, chunk=args.chunk or 4096)
    workload = "batch%d-mixed-beams-4096samp" % args.beams
    if args.store != "f32":
        workload += "-%s-rings" % args.store
    if args.ingest == "udp":
        workload += "-udp-packets"
    if args.beams != 64 or args.chunk:
        workload += "-reduced(beams=%d,chunk=%d)" % (args.beams, cfgs[0]["chunk"])
    if args.impl == "reference":
        run_reference(args, cfgs, workload)
    else:
        run_batch(args, cfgs, workload)


if __name__ == "__main__":
    main()
