"""Benchmark: TOD samples/s of the polarized-beam convolution on one GB300.

Workload (the production-size plain forward): sky HEALPix nside 1024 float32
I,Q,U (seeded C_ell ~ ell^-2 Gaussian random fields, V = 0); beam nside 2048,
radius 3 deg, elliptical Gaussian FWHM 1.5 deg, ellipticity 0.05, epsilon
0.01; one detector pair; 2,000,000 samples of a constant-elevation sweep
(RA += 360/4096 deg per sample, Dec += 0.05 deg per sweep from -80 deg, psi
uniform); FP64 pointing, FP32 sky and beam.  Synthetic, seeded.

One step = one TUNED forward over all samples with the inputs resident in HBM
(`value`); L2 is flushed (a 256 MiB write) between timed steps.  `e2e` is
the same metric through the C ABI with host buffers: pinned host pointing is
copied in (pisco_set_scan), the forward runs and the TOD comes back
(pisco_forward), every step.  Also reported: the PLAIN form on a bounded
prefix, the rms error of TUNED against the FP64 form, the roofline of the
forward kernel and the CPU baseline (oracle/_ref when it loads on this
host, else the oracle's C restatement) on a bounded prefix.

`--impl reference` times the reference's CPU implementation of the path
(oracle/_ref: the reference Convolver compiled from its own sources, when it
was built for this host; else the oracle port) with all host threads.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "c2_nside1024_beam3deg_2Msamples_sweep"
METRIC = "TOD samples/s (nside 1024 sky, 3 deg beam, tuned FP32/FP64-pointing forward)"
BYTES_PER_PAIR = 48     # sky IQUV f32 + beam a IQUV f32 + beam b IQUV f32
BYTES_PER_SAMPLE = 32   # 3 x 8 B FP64 pointing in + 2 x 4 B FP32 TOD out


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:  # noqa: BLE001
        return os.cpu_count() or 1


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_l2_bytes_per_pair():
    """L2 bytes served per (sample, disc pixel) pair by the tuned forward, from
    the committed ncu summary (line 'l2_bytes_per_pair: <float>')."""
    p = os.path.join(ROOT, "profiles", "tuned_forward_c2_ncu.md")
    if os.path.exists(p):
        with open(p) as f:
            for line in f:
                if line.strip().startswith("l2_bytes_per_pair:"):
                    return float(line.split(":", 1)[1].strip())
    return None


def ncu_traffic_per_launch():
    """DRAM bytes (read + write) per full-size launch of the tuned forward, from
    the committed ncu summary (line 'dram_bytes_per_launch: <int>')."""
    p = os.path.join(ROOT, "profiles", "tuned_forward_c2_dram_traffic.md")
    if os.path.exists(p):
        with open(p) as f:
            for line in f:
                if line.strip().startswith("dram_bytes_per_launch:"):
                    return int(line.split(":", 1)[1].strip())
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:  # noqa: BLE001
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:  # noqa: BLE001
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[2:]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# sample plans the TUNED forward builds per launch of its pair kernel
PLAN_CHUNK = 1 << 22

# ------------------------------------------------------------------ workload
def max_over_ranks(value: float, dist, device) -> float:
    """The largest of every rank's value (the whole job ends with the slowest
    rank); the value itself with one rank."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_workload(device: str, nsamples: int, shard: int = 0, nshards: int = 1):
    from pisco4cmb_gb300 import PolBeam, beam_npix_for_radius, synth

    w = synth.WORKLOADS[2]
    t0 = time.time()
    sky = synth.grf_sky(w["nside_sky"], 2, dtype=np.float32, device=device)
    nsb = w["nside_beam"]
    npb = beam_npix_for_radius(nsb, math.radians(w["radius_deg"]))
    beam = PolBeam(nsb, npb, w["epsilon"], "p")
    fx, fy = synth.elliptical_fwhm(w["fwhm_deg"], w["ellipticity"])
    beam.make_unpol_gaussian_elliptical_beams(fx, fy, 0.0)
    beam.build(w["nside_sky"])
    ra, dec, psi = synth.sweep_scan(nsamples, 2, shard=shard, nshards=nshards)
    return dict(sky=sky, beam=beam, ra=ra, dec=dec, pa=psi, nside_sky=w["nside_sky"],
                gen_s=time.time() - t0)


class _Planes:
    """Beam planes of the reference arm (PolBeam::aBeams / bBeams)."""

    def __init__(self, nside, a, b):
        self.nside, self._a, self._b = nside, a, b

    def planes(self):
        return self._a, self._b


def make_reference_workload(device: str, nsamples: int):
    """The workload of make_workload built without libpisco_gb300: the beam by
    the reference's own PolBeam (oracle/_ref), else by the oracle's
    restatement of it (bit-identical to the reference's, tested)."""
    import oracle
    from pisco4cmb_gb300 import synth

    w = synth.WORKLOADS[2]
    t0 = time.time()
    sky = synth.grf_sky(w["nside_sky"], 2, dtype=np.float32, device=device)
    nsb = w["nside_beam"]
    npb = oracle.beam_npix_for_radius(nsb, math.radians(w["radius_deg"]))
    fx, fy = synth.elliptical_fwhm(w["fwhm_deg"], w["ellipticity"])
    if oracle.ref_available():
        ba, bb, _ = oracle.ref_gaussian_beams(nsb, npb, fx, fy, 0.0, w["epsilon"], w["nside_sky"])
        beam_by = "reference PolBeam (oracle/_ref)"
    else:
        ba, bb = oracle.gaussian_beams(nsb, npb, fx, fy, 0.0, w["epsilon"], w["nside_sky"])
        beam_by = "oracle PolBeam restatement"
    ra, dec, psi = synth.sweep_scan(nsamples, 2)
    return dict(sky=sky, beam=_Planes(nsb, ba, bb), ra=ra, dec=dec, pa=psi,
                nside_sky=w["nside_sky"], gen_s=time.time() - t0, beam_by=beam_by)


# ------------------------------------------------------------------ CPU arm
def cpu_forward(wl, n: int, threads: int, prefer_ref: bool = True):
    """(kind, seconds, tod_a) of the CPU implementation on the first n samples."""
    import oracle

    oracle.build_oracle()
    ba, bb = wl["beam"].planes()
    ra, dec, pa = (wl[k][:n] for k in ("ra", "dec", "pa"))
    use_ref = False
    if prefer_ref and oracle.ref_available():
        try:
            oracle.ref_lib()
            use_ref = True
        except OSError:
            use_ref = False
    t0 = time.perf_counter()
    if use_ref:
        a, _ = oracle.ref_convolve(ra, dec, pa, wl["nside_sky"], wl["sky"], wl["beam"].nside,
                                   ba, bb, nthreads=threads)
    else:
        a, _ = oracle.convolve_f32(ra, dec, pa, wl["nside_sky"], wl["sky"], wl["beam"].nside,
                                   ba, bb, nthreads=threads)
    return ("reference" if use_ref else "port"), time.perf_counter() - t0, a


def cpu_sample_size(wl, threads: int, target_s: float):
    """Samples for about target_s of CPU work: a 256-sample warm-up (thread
    start-up, first touches), then the per-sample cost timed on 4,096 samples
    (about 0.3 s at 16 threads: the ~60 ms fixed cost of a call stays small)."""
    cpu_forward(wl, 256, threads)
    m = max(4096, 64 * threads)
    kind, t, _ = cpu_forward(wl, m, threads)
    per = t / m
    return max(256, min(len(wl["ra"]), int(target_s / max(per, 1e-9)))), kind


def run_reference_arm(args, rank, world):
    if rank != 0:
        return 0
    # input generation is not timed; the sky synthesis uses the GPU when there is one
    try:
        import torch

        gen_dev = "cuda" if torch.cuda.is_available() else "cpu"
    except Exception:  # noqa: BLE001
        gen_dev = "cpu"
    wl = make_reference_workload(gen_dev, 200_000)
    threads = host_cores()
    n, kind = cpu_sample_size(wl, threads, 5.0)
    for _ in range(args.warmup):
        cpu_forward(wl, min(n, 2048), threads)
    times = []
    for _ in range(args.steps):
        _, t, _ = cpu_forward(wl, n, threads)
        times.append(t)
    t_step = sum(times) / len(times)
    v = n / t_step
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "samples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded GRF sky, Gaussian beam, sweep scan)",
            "config": {"workload": WORKLOAD, "sample": "first %d of 2,000,000 sweep samples" % n,
                       "parallelism": "host OpenMP, %d threads" % threads},
            "cpu_baseline": {"value": v, "unit": "samples/s", "cores": threads, "kind": kind,
                             "sample": "first %d samples of the workload" % n},
            "e2e": {"value": v, "unit": "samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm
def run_gpu_arm(args, rank, world, local):
    import torch

    from pisco4cmb_gb300 import GPUConvolver, RunConfig, Scan, Sky

    torch.cuda.set_device(local)
    dev = "cuda:%d" % local
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device(dev))
    # one interleaved shard of the scan per rank: every rank's work equals the
    # one-GPU workload (weak scaling), no collective on the data path
    wl = make_workload(dev, args.samples, shard=rank, nshards=world)
    n = len(wl["ra"])
    sky = wl["sky"]
    conv = GPUConvolver(RunConfig(deviceId=local, ptgPerConv=1 << 22), form="tuned")
    conv.update_sky(Sky(wl["nside_sky"], sky[0], sky[1], sky[2], None))
    conv.update_beam(wl["beam"])
    conv.update_scan(Scan(n, wl["ra"], wl["dec"], wl["pa"]))
    pairs = conv.count_pairs()

    stream = torch.cuda.Stream(device=dev)
    sh = stream.cuda_stream
    out_a = torch.empty(n, dtype=torch.float32, device=dev)
    out_b = torch.empty(n, dtype=torch.float32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def step(form="tuned", m=None):
        conv.forward_device(out_a.data_ptr(), out_b.data_ptr(), n=m or n, stream=sh, form=form)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    conv.sync()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for i in range(args.steps):
                flush.fill_(i & 0xff)
                evs[i][0].record(stream)
                step()
                evs[i][1].record(stream)
        torch.cuda.synchronize()
    conv.sync()
    kernel_ms = [s.elapsed_time(e) for s, e in evs]
    t_total = sum(kernel_ms) / 1e3
    t_total = max_over_ranks(t_total, dist, dev)
    if dist:
        dist.barrier()
    ms_step = t_total / args.steps * 1e3
    value = n * world * args.steps / t_total
    fallbacks = conv.last_fallbacks()

    # plain form on a bounded prefix (it is FP64-per-pair and slow on GB300)
    m_plain = min(n, args.plain_samples)
    with torch.cuda.stream(stream):
        step("plain", m_plain)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step("plain", m_plain)
        e1.record(stream)
    torch.cuda.synchronize()
    plain_sps = m_plain / (e0.elapsed_time(e1) / 1e3)

    # accuracy of TUNED vs FP64 on a bounded prefix (untimed)
    m_acc = min(n, args.accuracy_samples)
    ta = torch.empty(m_acc, dtype=torch.float64, device=dev)
    tb = torch.empty(m_acc, dtype=torch.float64, device=dev)
    fa = torch.empty(m_acc, dtype=torch.float64, device=dev)
    fb = torch.empty(m_acc, dtype=torch.float64, device=dev)
    conv.forward_device(ta.data_ptr(), tb.data_ptr(), out_f64=True, n=m_acc, form="tuned")
    conv.forward_device(fa.data_ptr(), fb.data_ptr(), out_f64=True, n=m_acc, form="fp64")
    conv.sync()
    rms = torch.sqrt(torch.mean(torch.cat([fa, fb]) ** 2)).item()
    err = torch.cat([ta - fa, tb - fb])
    rms_err = torch.sqrt(torch.mean(err ** 2)).item() / rms
    max_err = torch.max(torch.abs(err)).item() / rms
    # worst FP32 decision error (fraction of the FP64 margin) and exactness
    # of the TUNED disc on a bounded prefix
    m_cal = min(n, args.accuracy_samples // 5)
    worst_frac, tuned_pairs = conv.tuned_calibrate(0, m_cal, with_pairs=True)
    conv.update_scan(Scan(m_cal, wl["ra"][:m_cal], wl["dec"][:m_cal], wl["pa"][:m_cal]))
    exact_pairs = conv.count_pairs()
    conv.update_scan(Scan(n, wl["ra"], wl["dec"], wl["pa"]))

    # e2e through the C ABI with pinned host buffers, host<->device copies inside
    ra_h = torch.from_numpy(wl["ra"]).pin_memory()
    dec_h = torch.from_numpy(wl["dec"]).pin_memory()
    pa_h = torch.from_numpy(wl["pa"]).pin_memory()
    a_h = torch.empty(n, dtype=torch.float32).pin_memory()
    b_h = torch.empty(n, dtype=torch.float32).pin_memory()
    import ctypes

    from pisco4cmb_gb300 import _lib

    L = _lib.load()

    def e2e_step():
        _lib.check(L.pisco_set_scan(conv.ctx, n, ctypes.c_void_p(ra_h.data_ptr()),
                                    ctypes.c_void_p(dec_h.data_ptr()),
                                    ctypes.c_void_p(pa_h.data_ptr()), _lib.FLOAT64), conv.ctx, "set_scan")
        _lib.check(L.pisco_forward(conv.ctx, b"p", ctypes.c_void_p(a_h.data_ptr()),
                                   ctypes.c_void_p(b_h.data_ptr()), _lib.FLOAT32, _lib.FORM_TUNED),
                   conv.ctx, "forward")

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    e2e_t = 0.0
    for i in range(args.steps):
        flush.fill_(i & 0xff)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_t += time.perf_counter() - t0
    e2e_t = max_over_ranks(e2e_t, dist, dev)
    e2e_value = n * world * args.steps / e2e_t
    assert np.allclose(a_h.numpy()[:1000], out_a.cpu().numpy()[:1000], rtol=1e-6, atol=1e-4)

    # roofline of the forward kernel (algorithmic bytes per launch / launch time)
    peak, peak_kind = measured_peaks()
    alg_bytes = pairs * BYTES_PER_PAIR + n * BYTES_PER_SAMPLE
    achieved = alg_bytes / (t_total / args.steps) / 1e9
    traffic = ncu_traffic_per_launch()
    # what actually limits the kernel: one dependent L2 gather (the beam) per
    # pair; L2 bytes per pair from ncu, the rate from this run's time
    l2_pp = ncu_l2_bytes_per_pair()
    l2_line = None if l2_pp is None else {
        "bytes_per_pair": l2_pp, "achieved_gbs": pairs * l2_pp / (t_total / args.steps) / 1e9,
        "l1_serves": "the sky reads (all hits)", "l2_serves": "the beam gather (all L1 misses)",
        "source": "profiles/tuned_forward_c2_ncu.md"}

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            threads = host_cores()
            wl_cpu = dict(wl)
            m_cpu, kind = cpu_sample_size(wl_cpu, threads, args.cpu_seconds)
            kind, t_cpu, cpu_a = cpu_forward(wl_cpu, m_cpu, threads)
            cpu = {"value": m_cpu / t_cpu, "unit": "samples/s", "cores": threads, "kind": kind,
                   "sample": "first %d of the %d workload samples, %.1f s" % (m_cpu, n, t_cpu)}
        line = {
            "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded GRF sky C_l~l^-2, elliptical Gaussian PolBeam, sweep scan)",
            "config": {"workload": WORKLOAD, "nsamples": n, "nside_sky": 1024, "nside_beam": 2048,
                       "beam_radius_deg": 3.0, "pairs_per_step": pairs,
                       "pairs_per_sample": pairs / n, "form": "tuned",
                       "l2": "flushed between timed steps (256 MiB write); sky 201 MB > L2",
                       "parallelism": ("one interleaved scan shard per GPU, no collective"
                                       if world > 1 else "single GPU")},
            "e2e": {"value": e2e_value, "unit": "samples/s", "h2d_bytes_per_step": n * 24,
                    "d2h_bytes_per_step": n * 8},
            # per step: the plan kernel and the pair kernel, per 4M-sample chunk
            "gpu_launches": args.steps * 2 * (-(-n // PLAN_CHUNK)),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "kernel": "the forward step: plan_kernel + tuned_kernel",
                         "traffic": traffic,
                         "bytes_model": "48 B/pair x exact disc pairs + 32 B/sample",
                         "note": ("the byte model counts the sky and beam gathers that L1 and L2 "
                                  "serve; DRAM moves `traffic` bytes per pair-kernel launch"),
                         "l2": l2_line},
            "plain": {"value": plain_sps, "unit": "samples/s", "sample": m_plain,
                      "tuned_over_plain": value / world / plain_sps},
            "accuracy": {"rms_err_vs_fp64": rms_err, "max_err_vs_fp64": max_err,
                         "sample": m_acc, "relative_to": "TOD rms",
                         "worst_fp32_decision_error_over_margin": worst_frac,
                         "tuned_disc_pairs_equal_exact": tuned_pairs == exact_pairs,
                         "calibration_sample": m_cal},
            "macs_per_s": pairs * 8 * world * args.steps / t_total,
            "fp64_fallback_pairs_per_step": fallbacks,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "input_gen_s": wl["gen_s"],
        }
        if not args.no_cpu:
            line["reference_gpu"] = reference_gpu_sample(wl, 16384)
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


# ------------------------------------------------------------------ other workloads
def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _study_stream():
    """Makes a fresh (non-default) torch stream current and returns its
    handle: torch events then record on the stream the library launches on.
    (A null handle would select the library context's own stream, which
    torch's default-stream events do not see.)"""
    import torch

    st = torch.cuda.Stream()
    torch.cuda.set_stream(st)
    return st.cuda_stream


def _gaussian_beam(nside_beam, radius_deg, fwhm_deg, ell, nside_sky, epsilon=0.01, phi0=0.0):
    from pisco4cmb_gb300 import PolBeam, beam_npix_for_radius, synth

    npb = beam_npix_for_radius(nside_beam, math.radians(radius_deg))
    beam = PolBeam(nside_beam, npb, epsilon, "p")
    fx, fy = synth.elliptical_fwhm(fwhm_deg, ell)
    beam.make_unpol_gaussian_elliptical_beams(fx, fy, phi0)
    beam.build(nside_sky)
    return beam


def run_c3_precision(args):
    """Precision study: FP32/FP64-pointing TUNED vs all-FP64 on the GPU (and vs
    the CPU FP64 oracle on a small prefix), pole-heavy scan."""
    import torch

    import oracle
    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky, synth

    w = synth.WORKLOADS[3]
    t0 = time.time()
    sky = synth.grf_sky(w["nside_sky"], 3, lmax=w["lmax"], dtype=np.float32, device="cuda")
    beam = _gaussian_beam(w["nside_beam"], w["radius_deg"], w["fwhm_deg"], w["ellipticity"],
                          w["nside_sky"])
    n = args.samples or w["nsamples"]
    ra, dec, pa = synth.pole_heavy_scan(n, 3)
    gen = time.time() - t0
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(w["nside_sky"], sky[0], sky[1], sky[2], None))
    conv.update_beam(beam)
    conv.update_scan(Scan(n, ra, dec, pa))
    pairs = conv.count_pairs()
    out = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(2)]
    cs = _study_stream()
    conv.forward_device(out[0].data_ptr(), out[1].data_ptr(), out_f64=True, form="tuned", stream=cs)
    conv.sync()
    e0, e1 = _events()
    e0.record()
    conv.forward_device(out[0].data_ptr(), out[1].data_ptr(), out_f64=True, form="tuned", stream=cs)
    e1.record()
    torch.cuda.synchronize()
    t_tuned = e0.elapsed_time(e1) / 1e3
    tuned = [x.cpu().numpy() for x in out]
    fb = conv.last_fallbacks()
    # the same forward in sky order (bit-identical TOD); the first launch sorts
    conv.set_sample_order("sky")
    so = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(2)]
    conv.forward_device(so[0].data_ptr(), so[1].data_ptr(), out_f64=True, form="tuned", stream=cs)
    conv.sync()
    e0.record()
    conv.forward_device(so[0].data_ptr(), so[1].data_ptr(), out_f64=True, form="tuned", stream=cs)
    e1.record()
    torch.cuda.synchronize()
    t_sky = e0.elapsed_time(e1) / 1e3
    sky_same = all(np.array_equal(a.cpu().numpy(), b) for a, b in zip(so, tuned))
    conv.set_sample_order("scan")
    m = min(n, args.fp64_samples)
    ref = [torch.empty(m, dtype=torch.float64, device="cuda") for _ in range(2)]
    e0.record()
    conv.forward_device(ref[0].data_ptr(), ref[1].data_ptr(), out_f64=True, n=m, form="fp64",
                        stream=cs)
    e1.record()
    torch.cuda.synchronize()
    t_fp64 = e0.elapsed_time(e1) / 1e3
    ref = [x.cpu().numpy() for x in ref]
    rms = float(np.sqrt(np.mean(np.concatenate(ref) ** 2)))
    err = np.concatenate([tuned[0][:m] - ref[0], tuned[1][:m] - ref[1]])
    pole = np.abs(np.abs(dec[:m]) - np.pi / 2) <= np.radians(1.0)
    errp = np.concatenate([(tuned[0][:m] - ref[0])[pole], (tuned[1][:m] - ref[1])[pole]])
    worst = conv.tuned_calibrate(0, min(n, 20000))
    # CPU FP64 oracle on a small prefix (every 10th sample is a pole pointing)
    mc = min(n, args.cpu_samples)
    ba, bb = beam.planes()
    oa, ob = oracle.convolve_f64(ra[:mc], dec[:mc], pa[:mc], w["nside_sky"],
                                 sky.astype(np.float64), w["nside_beam"], ba.astype(np.float64),
                                 bb.astype(np.float64), nthreads=host_cores())
    errc = np.concatenate([tuned[0][:mc] - oa, tuned[1][:mc] - ob])
    errf = np.concatenate([ref[0][:mc] - oa, ref[1][:mc] - ob])
    line = {"workload": "c3_precision_nside2048_beam1deg", "nsamples": n, "pairs": pairs,
            "tuned_samples_per_s": n / t_tuned, "fp64_gpu_samples_per_s": m / t_fp64,
            "tuned_sky_order": {"samples_per_s": n / t_sky, "over_scan_order": t_tuned / t_sky,
                                "tod_bit_identical": sky_same},
            "fp64_fallback_pairs": fb, "worst_fp32_decision_error_over_margin": worst,
            "tuned_vs_fp64_gpu": {"rms": float(np.sqrt(np.mean(err ** 2)) / rms),
                                  "max": float(np.abs(err).max() / rms), "samples": m,
                                  "pole_samples": int(pole.sum()),
                                  "pole_max": float(np.abs(errp).max() / rms) if errp.size else None},
            "tuned_vs_cpu_fp64_oracle": {"rms": float(np.sqrt(np.mean(errc ** 2)) / rms),
                                         "max": float(np.abs(errc).max() / rms), "samples": mc},
            "fp64_gpu_vs_cpu_fp64_oracle": {"max": float(np.abs(errf).max() / rms),
                                            "samples": mc},
            "relative_to": "TOD rms", "input_gen_s": gen}
    print(json.dumps(line), flush=True)
    return 0


def run_c4_batched(args):
    """48 uneven detector pairs: one autotuned persistent launch vs sequential."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky, synth

    w = synth.WORKLOADS[4]
    nss = w["nside_sky"]
    sky = synth.grf_sky(nss, 4, dtype=np.float32, device="cuda")
    dets = synth.c4_detectors()
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    rows, keep, beams, scans = [], [], [], []
    for d, p in enumerate(dets):
        beam = _gaussian_beam(w["nside_beam"], p["radius_deg"], p["radius_deg"] / 2.5,
                              p["ellipticity"], nss, w["epsilon"])
        conv.set_beam_slot(d, beam)
        ra, dec, pa = synth.sweep_scan(p["nsamples"], 4, stream=100 + d)
        ra, dec = synth.offset_pointing(ra, dec, p["dx_deg"], p["dy_deg"])
        t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
        o = [torch.empty(p["nsamples"], device="cuda") for _ in range(2)]
        keep.append((t, o))
        beams.append(beam)
        scans.append((ra, dec, pa))
        rows.append((d, p["nsamples"], t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(),
                     o[0].data_ptr(), o[1].data_ptr()))
    descs = conv.det_descs(rows)
    total = sum(p["nsamples"] for p in dets)
    cache = os.path.join(os.environ.get("PISCO_TUNE_CACHE", "/tmp"), "pisco_autotune.json")
    chunk, tune_ms = conv.autotune_batched(descs, cache_path=cache)
    _, warps = conv.batched_config()
    cs = _study_stream()
    for _ in range(2):
        conv.forward_batched(descs, stream=cs)
    conv.sync()
    e0, e1 = _events()
    with ClockSampler(0) as clk:
        e0.record()
        for _ in range(args.steps):
            conv.forward_batched(descs, stream=cs)
        e1.record()
        conv.sync()
        torch.cuda.synchronize()
    t_batched = e0.elapsed_time(e1) / 1e3 / args.steps
    batched_out = [[o.cpu().numpy() for o in k[1]] for k in keep]
    # sequential single-detector launches (TUNED and PLAIN), one context each pair
    seq = {}
    for form in ("tuned", "plain"):
        c = GPUConvolver(form=form)
        c.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
        tt = 0.0
        same = True
        frac = 1.0 if form == "tuned" else args.plain_fraction
        nseq = 0
        for d, p in enumerate(dets):
            m = max(1, int(p["nsamples"] * frac))
            c.update_beam(beams[d])
            ra, dec, pa = scans[d]
            c.update_scan(Scan(m, ra[:m], dec[:m], pa[:m]))
            oa = torch.empty(m, device="cuda")
            ob = torch.empty(m, device="cuda")
            e0.record()
            c.forward_device(oa.data_ptr(), ob.data_ptr(), stream=cs)
            e1.record()
            torch.cuda.synchronize()
            tt += e0.elapsed_time(e1) / 1e3
            nseq += m
            if form == "tuned":
                same &= bool(np.array_equal(oa.cpu().numpy(), batched_out[d][0][:m]))
        seq[form] = {"samples_per_s": nseq / tt, "samples": nseq, "bit_identical_to_batched":
                     same if form == "tuned" else None}
        c.close()
    # many short scans: 512 pairs of 2,000 samples (the 48 beams in turn),
    # where one launch per pair leaves most of the GPU idle
    m_small, n_small = 2000, 512
    srows, skeep, sscans = [], [], []
    for k in range(n_small):
        d = k % len(dets)
        ra, dec, pa = scans[d]
        off = (k * 7919) % max(1, dets[d]["nsamples"] - m_small)
        sl = slice(off, off + m_small)
        t = [torch.tensor(np.ascontiguousarray(x[sl]), device="cuda") for x in (ra, dec, pa)]
        o = [torch.empty(m_small, device="cuda") for _ in range(2)]
        skeep.append((t, o))
        sscans.append(d)
        srows.append((d, m_small, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(),
                      o[0].data_ptr(), o[1].data_ptr()))
    sdescs = conv.det_descs(srows)
    s_chunk, _ = conv.autotune_batched(sdescs, cache_path=cache)
    _, s_warps = conv.batched_config()
    conv.forward_batched(sdescs, stream=cs)
    conv.sync()
    e0.record()
    for _ in range(args.steps):
        conv.forward_batched(sdescs, stream=cs)
    e1.record()
    conv.sync()
    torch.cuda.synchronize()
    t_small = e0.elapsed_time(e1) / 1e3 / args.steps
    c = GPUConvolver(form="tuned")
    c.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    tt = 0.0
    same = True
    for k, d in enumerate(sscans):
        c.update_beam(beams[d])
        t, _ = skeep[k]
        c.set_scan_device(m_small, *[x.data_ptr() for x in t])
        oa = torch.empty(m_small, device="cuda")
        ob = torch.empty(m_small, device="cuda")
        e0.record()
        c.forward_device(oa.data_ptr(), ob.data_ptr(), stream=cs)
        e1.record()
        torch.cuda.synchronize()
        tt += e0.elapsed_time(e1) / 1e3
        same &= bool(torch.equal(oa, skeep[k][1][0]))
    c.close()
    small = {"pairs": n_small, "samples_per_pair": m_small, "autotuned_chunk": s_chunk,
             "autotuned_warps_per_block": s_warps,
             "batched_samples_per_s": n_small * m_small / t_small,
             "sequential_tuned_samples_per_s": n_small * m_small / tt,
             "batched_over_sequential_tuned": tt / t_small,
             "bit_identical_to_batched": same}
    line = {"workload": "c4_batched_48pairs_nside512", "ndet": len(dets), "total_samples": total,
            "autotuned_chunk": chunk, "autotuned_warps_per_block": warps,
            "autotune_best_ms": tune_ms,
            "batched_graph_samples_per_s": total / t_batched, "batched_ms": t_batched * 1e3,
            "sequential_tuned": seq["tuned"], "sequential_plain": seq["plain"],
            "batched_over_sequential_tuned": (total / t_batched) / seq["tuned"]["samples_per_s"],
            "batched_over_sequential_plain": (total / t_batched) / seq["plain"]["samples_per_s"],
            "many_short_scans": small, "clocks": clk.summary()}
    print(json.dumps(line), flush=True)
    return 0


def run_c5_adjoint(args):
    """Adjoint (sky and beam gradients) time vs forward time, both variants."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky, synth

    w = synth.WORKLOADS[5]
    nss, nsb = w["nside_sky"], w["nside_beam"]
    sky = synth.grf_sky(nss, 5, dtype=np.float32, device="cuda")
    beam = _gaussian_beam(nsb, w["radius_deg"], w["fwhm_deg"], w["ellipticity"], nss)
    n = w["ndet"] * (args.samples or w["nsamples"])
    ra, dec, pa = synth.sweep_scan(n, 5)
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(nss, sky[0], sky[1], sky[2], None))
    conv.update_beam(beam)
    t = [torch.tensor(x, device="cuda") for x in (ra, dec, pa)]
    conv.set_scan_device(n, *[x.data_ptr() for x in t])
    pairs = conv.count_pairs()
    ta = torch.empty(n, device="cuda")
    tb = torch.empty(n, device="cuda")
    ga = torch.randn(n, device="cuda")
    gb = torch.randn(n, device="cuda")
    gsky = torch.empty((12 * nss * nss, 4), device="cuda")
    gbeam = torch.empty((beam.nPixels, 8), device="cuda")
    e0, e1 = _events()

    def timeit(fn, reps=args.steps):
        fn()
        conv.sync()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        conv.sync()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / reps

    cs = _study_stream()
    t_fwd = timeit(lambda: conv.forward_device(ta.data_ptr(), tb.data_ptr(), form="tuned", stream=cs))
    res = {}
    for det in (True, False):
        for with_beam in (False, True):
            for iqu in (False, True):
                key = (("deterministic" if det else "atomic") +
                       ("_sky_and_beam" if with_beam else "_sky") + ("_iqu" if iqu else "_iquv"))
                res[key] = timeit(lambda: conv.adjoint_device(
                    ga.data_ptr(), gb.data_ptr(), False, gsky.data_ptr(),
                    gbeam.data_ptr() if with_beam else 0, deterministic=det, stream=cs,
                    sky_iqu=iqu))
    # the fused beam-parameter gradient (no beam-map gradient): the model beam
    # on the device, then sky (I, Q, U) + parameter gradients in one adjoint
    params = (w["fwhm_deg"], w["ellipticity"], 0.0, 0.0, 0.0)
    ab = torch.empty((beam.nPixels, 8), device="cuda")
    conv.gaussian_beam_device(nsb, beam.nPixels, w["epsilon"], nss, *params, ab.data_ptr(),
                              set_beam=True)
    grad = torch.empty(5, dtype=torch.float64, device="cuda")
    for det in (True, False):
        for with_sky in (True, False):
            key = (("deterministic" if det else "atomic") +
                   ("_sky_iqu_and_params_fused" if with_sky else "_params_fused"))
            res[key] = timeit(lambda: conv.adjoint_gaussian_device(
                ga.data_ptr(), gb.data_ptr(), False, gsky.data_ptr() if with_sky else 0,
                grad.data_ptr(), params, w["epsilon"], nss, deterministic=det, stream=cs,
                sky_iqu=True))
    line = {"workload": "c5_adjoint_nside256_beam4deg", "nsamples": n, "pairs": pairs,
            "forward_ms": t_fwd * 1e3,
            "adjoint_ms": {k: v * 1e3 for k, v in res.items()},
            "adjoint_over_forward": {k: v / t_fwd for k, v in res.items()}}
    print(json.dumps(line), flush=True)
    return 0


def run_order_study(args):
    """Sky-ordered processing: the c2 TUNED forward on its sweep scan, on the
    same samples shuffled (time order lost, as when many detectors or a
    revisiting scan are concatenated), and on the shuffled samples in sky
    order.  L2 flushed between timed steps."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky

    n = args.samples or 2_000_000
    wl = make_workload("cuda", n)
    sky = wl["sky"]
    perm = np.random.default_rng(20261203).permutation(n)
    cs = _study_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    e0, e1 = _events()
    res = {}
    for name, shuffled, order in (("sweep_scan_order", False, "scan"),
                                  ("sweep_sky_order", False, "sky"),
                                  ("shuffled_scan_order", True, "scan"),
                                  ("shuffled_sky_order", True, "sky")):
        ra, dec, pa = (wl[k][perm] if shuffled else wl[k] for k in ("ra", "dec", "pa"))
        c = GPUConvolver(form="tuned")
        c.update_sky(Sky(1024, sky[0], sky[1], sky[2], None))
        c.update_beam(wl["beam"])
        c.update_scan(Scan(n, ra, dec, pa))
        c.set_sample_order(order)
        a = torch.empty(n, device="cuda")
        b = torch.empty(n, device="cuda")
        for _ in range(2):  # the first call also sorts
            c.forward_device(a.data_ptr(), b.data_ptr(), stream=cs)
        c.sync()
        ts = []
        for i in range(args.steps):
            flush.fill_(i & 0xff)
            e0.record()
            c.forward_device(a.data_ptr(), b.data_ptr(), stream=cs)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        res[name] = {"ms": float(np.median(ts)), "samples_per_s": n / (np.median(ts) / 1e3)}
        c.close()
    line = {"workload": "order_c2_nside1024_beam3deg", "nsamples": n, "timings": res,
            "shuffled_sky_over_scan": res["shuffled_scan_order"]["ms"] / res["shuffled_sky_order"]["ms"]}
    print(json.dumps(line), flush=True)

    # a sky larger than L2 (nside 2048: 805 MB) read by uniformly random pointings
    from pisco4cmb_gb300 import synth

    w = synth.WORKLOADS[3]
    sky3 = synth.grf_sky(w["nside_sky"], 3, lmax=w["lmax"], dtype=np.float32, device="cuda")
    beam3 = _gaussian_beam(w["nside_beam"], w["radius_deg"], w["fwhm_deg"], w["ellipticity"],
                           w["nside_sky"])
    n3 = 1_000_000
    rng = np.random.default_rng(20261204)
    ra3 = rng.uniform(0, 2 * np.pi, n3)
    dec3 = np.arcsin(rng.uniform(-1, 1, n3))
    pa3 = rng.uniform(0, np.pi, n3)
    res3 = {}
    for order in ("scan", "sky"):
        c = GPUConvolver(form="tuned")
        c.update_sky(Sky(w["nside_sky"], sky3[0], sky3[1], sky3[2], None))
        c.update_beam(beam3)
        c.update_scan(Scan(n3, ra3, dec3, pa3))
        c.set_sample_order(order)
        a = torch.empty(n3, device="cuda")
        b = torch.empty(n3, device="cuda")
        for _ in range(2):
            c.forward_device(a.data_ptr(), b.data_ptr(), stream=cs)
        c.sync()
        ts = []
        for i in range(args.steps):
            flush.fill_(i & 0xff)
            e0.record()
            c.forward_device(a.data_ptr(), b.data_ptr(), stream=cs)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        res3[order] = {"ms": float(np.median(ts)), "samples_per_s": n3 / (np.median(ts) / 1e3)}
        c.close()
    line = {"workload": "order_random_fullsky_nside2048_beam1deg", "nsamples": n3, "timings": res3,
            "sky_over_scan": res3["scan"]["ms"] / res3["sky"]["ms"]}
    print(json.dumps(line), flush=True)
    return 0


def run_map_study(args):
    """Binned map-making (SkyMap on the GPU): the c2 scan's two detectors (a at
    0 deg, b at 90 deg; 4,000,000 TOD values) into an nside 1024 map: TOD
    accumulation from device-resident FP64 pointing and TOD, and the solve.
    CPU baseline: the map-making oracle (one thread) on a bounded prefix."""
    import torch

    import oracle
    from pisco4cmb_gb300 import SkyMap

    n = args.samples or 2_000_000
    from pisco4cmb_gb300 import synth

    ra, dec, pa = synth.sweep_scan(n, 2)
    rng = np.random.default_rng(20261203)
    tod = rng.normal(size=(2, n))
    ra2, dec2, pa2 = (np.stack([x, x]) for x in (ra, dec, pa))
    t = [torch.tensor(x.reshape(-1), device="cuda") for x in (ra2, dec2, pa2, tod)]
    pol = np.float32([0.0, np.pi / 2])
    cs = _study_stream()
    m = SkyMap(1024)
    e0, e1 = _events()

    def acc():
        m.accumulate_device(n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), 2, pol,
                            t[3].data_ptr(), f64=True, stream=cs)

    acc()  # warm-up (scratch allocation)
    m.reset()
    ts = []
    for _ in range(args.steps):
        e0.record()
        acc()
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    t_acc = float(np.median(ts)) / 1e3
    e0.record()
    m.solve_map()
    e1.record()
    torch.cuda.synchronize()
    t_solve = e0.elapsed_time(e1) / 1e3
    hits = m.get_hitmap()
    # determinism: a fresh map from the same calls gives the same normal equations
    m2 = SkyMap(1024)
    for _ in range(args.steps):
        m2.accumulate_device(n, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), 2, pol,
                             t[3].data_ptr(), f64=True, stream=cs)
    same = all(np.array_equal(x, y) for x, y in zip(m.get_normal(), m2.get_normal()))
    # CPU: the oracle (single-threaded restatement of skymap.cpp) on a prefix
    k = min(n, 200_000)
    t0 = time.perf_counter()
    oracle.map_accumulate(1024, ra2[:, :k], dec2[:, :k], pa2[:, :k], pol, tod[:, :k])
    t_cpu = time.perf_counter() - t0
    line = {"workload": "map_c2scan_2det_nside1024", "tod_values": 2 * n,
            "accumulate_ms": t_acc * 1e3, "tod_values_per_s": 2 * n / t_acc,
            "solve_ms": t_solve * 1e3, "pixels": 12 * 1024 * 1024,
            "pixels_hit": int((hits > 0).sum()), "pixels_solved": int((hits >= 3).sum()),
            "deterministic": same,
            "cpu_baseline": {"tod_values_per_s": 2 * k / t_cpu, "cores": 1, "kind": "port",
                             "sample": "first %d samples x 2 detectors" % k}}
    print(json.dumps(line), flush=True)
    return 0


def run_beam_study(args):
    """Beam construction on the GPU against the host PolBeam builder, for the
    c2 beam (nside 2048, 3 deg, FWHM 1.5 deg, e 0.05; sky nside 1024), the c3
    beam (nside 4096, 1 deg, FWHM 0.5 deg, e 0.02; sky 2048) and a wide one
    (nside 8192, 5 deg, FWHM 2 deg, e 0.05; sky 2048).  Per case: the host
    builder (make_unpol_gaussian_elliptical_beams + build, one thread), the
    device build from field planes (pisco_beam_build_device; 64 B of fields
    in + 32 B of beam out per pixel), the device Gaussian model and its
    parameter gradient (32 B of gbeam in per pixel), and the largest float ulp
    difference between the device and host builds."""
    import ctypes

    import torch

    from pisco4cmb_gb300 import GPUConvolver, PolBeam, beam_npix_for_radius, synth
    from pisco4cmb_gb300._lib import check, load

    cs = _study_stream()
    conv = GPUConvolver(form="tuned")
    conv.configure_execution()
    e0, e1 = _events()
    hbm_peak, peak_kind = measured_peaks()

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        ts = []
        for _ in range(max(args.steps, 5)):
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.median(ts)) / 1e3

    for name, nsb, rdeg, fwhm, ell, nss in (("c2_beam", 2048, 3.0, 1.5, 0.05, 1024),
                                             ("c3_beam", 4096, 1.0, 0.5, 0.02, 2048),
                                             ("wide_beam", 8192, 5.0, 2.0, 0.05, 2048)):
        npix = beam_npix_for_radius(nsb, math.radians(rdeg))
        fx, fy = synth.elliptical_fwhm(fwhm, ell)
        t0 = time.perf_counter()
        hb = PolBeam(nsb, npix, 0.01, "p")
        hb.make_unpol_gaussian_elliptical_beams(fx, fy, 0.0)
        hb.build(nss)
        t_host = time.perf_counter() - t0
        f = [np.empty(npix, np.float64) for _ in range(4)]
        check(load().pisco_beam_gaussian_fields(nsb, npix, fx, fy, 0.0,
                                                *[x.ctypes.data_as(ctypes.c_void_p) for x in f]))
        fd = torch.tensor(np.stack(f), device="cuda")
        out = torch.empty((npix, 8), dtype=torch.float32, device="cuda")
        gb = torch.randn((npix, 8), dtype=torch.float32, device="cuda")
        grad = torch.empty(5, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        t_build = timed(lambda: conv.build_beam_device(nsb, npix, 0.01, "p", nss, fd.data_ptr(),
                                                       fd.data_ptr(), out.data_ptr(),
                                                       set_beam=False, stream=cs))
        a, b = hb.planes()
        host = np.concatenate([a.T, b.T], axis=1)
        dev = out.cpu().numpy()
        hi = host.view(np.int32).astype(np.int64)
        di = dev.view(np.int32).astype(np.int64)
        ulp = int(np.abs(np.where(hi < 0, -(hi & 0x7FFFFFFF), hi) -
                         np.where(di < 0, -(di & 0x7FFFFFFF), di)).max())
        t_model = timed(lambda: conv.gaussian_beam_device(nsb, npix, 0.01, nss, fwhm, ell, 0.0,
                                                          0.0, 0.0, out.data_ptr(),
                                                          set_beam=False, stream=cs))
        t_grad = timed(lambda: conv.gaussian_beam_param_grad_device(
            nsb, npix, 0.01, nss, fwhm, ell, 0.0, 0.0, 0.0, gb.data_ptr(), False,
            grad.data_ptr(), stream=cs))
        line = {"workload": "beam_" + name, "beam_pixels": npix, "nside_beam": nsb,
                "radius_deg": rdeg, "host_build_ms": t_host * 1e3,
                "device_build_ms": t_build * 1e3,
                "device_build_gbs": 96.0 * npix / t_build / 1e9,
                "device_model_ms": t_model * 1e3, "device_param_grad_ms": t_grad * 1e3,
                "device_param_grad_gbs": 32.0 * npix / t_grad / 1e9,
                "hbm_peak_gbs": hbm_peak, "peak": peak_kind,
                "max_ulp_device_vs_host": ulp,
                "cpu_baseline": {"kind": "port", "cores": 1,
                                 "sample": "whole beam, library host builder "
                                           "(bit-identical to the reference PolBeam)"}}
        print(json.dumps(line), flush=True)
    return 0


def run_bilinear_study(args):
    """Bilinear beam lookup (HEALPix get_interpol, the reference's
    commented-out convolver.cpp:162-185 path) on the c2 workload: TUNED with
    the FP32 stencil over all samples against TUNED nearest, PLAIN bilinear on
    a bounded prefix, and the error against the FP64 form's bilinear lookup on
    that prefix (relative to the TOD rms)."""
    import torch

    from pisco4cmb_gb300 import GPUConvolver, Sky

    n = args.samples or 2_000_000
    wl = make_workload("cuda", n)
    sky = np.asarray(wl["sky"], np.float32)
    cs = _study_stream()
    e0, e1 = _events()
    t = [torch.tensor(np.asarray(wl[k][:n], np.float64), device="cuda") for k in ("ra", "dec", "pa")]
    torch.cuda.synchronize()

    def conv(form, interp, m, f64=False):
        c = GPUConvolver(form=form)
        planes = [sky[k].astype(np.float64) if f64 else sky[k] for k in range(3)]
        c.update_sky(Sky(wl["nside_sky"], planes[0], planes[1], planes[2], None))
        c.update_beam(wl["beam"])
        c.set_interp(interp)
        c.set_scan_device(m, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), stream=cs)
        return c

    def timed(c, m, reps):
        a = torch.empty(m, dtype=torch.float64, device="cuda")
        b = torch.empty(m, dtype=torch.float64, device="cuda")
        c.forward_device(a.data_ptr(), b.data_ptr(), out_f64=True, stream=cs)  # warm-up
        ts = []
        for _ in range(reps):
            e0.record()
            c.forward_device(a.data_ptr(), b.data_ptr(), out_f64=True, stream=cs)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        return float(np.median(ts)), a.cpu().numpy()

    reps = max(3, min(args.steps, 5))
    t_near, _ = timed(conv("tuned", False, n), n, reps)
    cb = conv("tuned", True, n)
    t_bil, a_bil = timed(cb, n, reps)

    # adjoint of the bilinear lookup: deterministic sky (I, Q, U), atomic sky + beam
    rng = np.random.default_rng(20261203)
    g = [torch.tensor(rng.normal(size=n).astype(np.float32), device="cuda") for _ in range(2)]
    gsky = torch.empty((12 * wl["nside_sky"] ** 2, 4), dtype=torch.float32, device="cuda")
    gbeam = torch.empty((wl["beam"].nPixels, 8), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    def adj_time(det, beam):
        cb.adjoint_device(g[0].data_ptr(), g[1].data_ptr(), False, gsky.data_ptr(),
                          gbeam.data_ptr() if beam else 0, deterministic=det, stream=cs,
                          sky_iqu=True)  # warm-up
        e0.record()
        cb.adjoint_device(g[0].data_ptr(), g[1].data_ptr(), False, gsky.data_ptr(),
                          gbeam.data_ptr() if beam else 0, deterministic=det, stream=cs,
                          sky_iqu=True)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    t_adj_det = adj_time(True, False)
    t_adj_atom = adj_time(False, True)
    m = min(n, args.plain_samples)
    t_plain, _ = timed(conv("plain", True, m), m, 1)
    k = min(n, args.fp64_samples)
    _, a64 = timed(conv("fp64", True, k, f64=True), k, 1)
    rms = float(np.sqrt(np.mean(a64 ** 2)))
    d = a_bil[:k] - a64
    line = {"workload": "bilinear_c2_nside1024_beam3deg", "nsamples": n,
            "tuned_nearest": {"ms": t_near * 1e3, "samples_per_s": n / t_near},
            "tuned_bilinear": {"ms": t_bil * 1e3, "samples_per_s": n / t_bil,
                               "over_nearest": t_bil / t_near},
            "adjoint_bilinear": {"deterministic_sky_iqu_ms": t_adj_det * 1e3,
                                 "deterministic_sky_iqu_over_forward": t_adj_det / t_bil,
                                 "atomic_sky_iqu_and_beam_ms": t_adj_atom * 1e3,
                                 "atomic_sky_iqu_and_beam_over_forward": t_adj_atom / t_bil},
            "plain_bilinear": {"samples_per_s": m / t_plain, "sample": m,
                               "tuned_over_plain": (n / t_bil) / (m / t_plain)},
            "tuned_bilinear_vs_fp64_bilinear": {"rms": float(np.sqrt(np.mean(d ** 2))) / rms,
                                                "max": float(np.abs(d).max()) / rms,
                                                "sample": k, "relative_to": "TOD rms"}}
    print(json.dumps(line), flush=True)
    return 0


def reference_gpu_sample(wl, m: int):
    """The reference's own GPU pipeline (K1 + K2 recompiled for sm_103a) on the
    first m samples of the workload, or why it did not run."""
    import oracle

    if not oracle.refgpu_available():
        return {"unavailable": "reference GPU kernels not built (needs the reference tree at "
                               "build time)"}
    try:
        m -= m % 2048
        ba, bb = wl["beam"].planes()
        ra, dec, pa = (np.asarray(wl[k][:m], np.float32) for k in ("ra", "dec", "pa"))
        _, _, t = oracle.refgpu_convolve(ra, dec, pa, wl["nside_sky"],
                                         np.asarray(wl["sky"], np.float32), wl["beam"].nside,
                                         ba, bb, nthreads=host_cores())
    except Exception as e:  # noqa: BLE001  (a baseline must not break the headline line)
        return {"unavailable": str(e)[:200]}
    return {"value": m / t[0], "unit": "samples/s", "kernels_only": m / t[1],
            "sample": "first %d samples" % m,
            "kind": "reference K1+K2 recompiled for sm_103a with GPUConvolver's pipeline"}


def run_refgpu_study(args):
    """The reference's own GPU pipeline on this GB300: its kernels K1 + K2
    (cudaConv2.cu, compiled unmodified for sm_103a) with GPUConvolver's host
    orchestration (query_disc on all host cores, ptgPerConv = 2048 chunks,
    per-chunk copies; oracle/ref_gpu_harness.cpp), on the first
    --samples (default 65,536) samples of the c2 workload, beside this
    library's TUNED forward on the same samples through the same host-array
    call (exec_convolution: host pointing in, host TOD out)."""
    import oracle
    from pisco4cmb_gb300 import GPUConvolver, Scan, Sky

    if not oracle.refgpu_available():
        print(json.dumps({"workload": "refgpu_c2", "unavailable":
                          "reference GPU kernels not built (needs the reference tree at build time)"}))
        return 0
    n = args.samples or 65536
    n -= n % 2048
    wl = make_workload("cuda", n)
    sky = np.asarray(wl["sky"], np.float32)
    ba, bb = wl["beam"].planes()
    ra, dec, pa = (np.asarray(wl[k][:n], np.float32) for k in ("ra", "dec", "pa"))
    cores = host_cores()
    # pixPerDisc as a caller of the reference would set it: the largest disc of the sample
    ra_, rb_, t = oracle.refgpu_convolve(ra, dec, pa, wl["nside_sky"], sky, wl["beam"].nside,
                                         ba, bb, nthreads=cores)
    conv = GPUConvolver(form="tuned")
    conv.update_sky(Sky(wl["nside_sky"], sky[0], sky[1], sky[2], None))
    conv.update_beam(wl["beam"])
    conv.update_scan(Scan(n, ra, dec, pa))
    a = np.zeros(n, np.float32)
    b = np.zeros(n, np.float32)
    conv.exec_convolution(a, b)  # warm-up
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        conv.exec_convolution(a, b)
        ts.append(time.perf_counter() - t0)
    t_ours = float(np.median(ts))
    rms = float(np.sqrt(np.mean(a.astype(np.float64) ** 2)))
    d = np.concatenate([a - ra_, b - rb_]).astype(np.float64)
    line = {"workload": "refgpu_c2", "samples": int(n), "host_cores": cores,
            "reference_gpu": {"samples_per_s": n / t[0], "kernel_samples_per_s": n / t[1],
                              "total_s": t[0], "kernels_s": t[1], "query_disc_s": t[2],
                              "copies_s": t[3],
                              "kind": "reference K1+K2 recompiled for sm_103a, GPUConvolver "
                                      "orchestration, query_disc restated"},
            "tuned_host_api": {"samples_per_s": n / t_ours, "seconds": t_ours},
            "speedup_vs_reference_gpu": t[0] / t_ours,
            "speedup_vs_reference_kernels": t[1] / t_ours,
            "rms_diff_over_tod_rms": float(np.sqrt(np.mean(d ** 2))) / rms,
            "max_diff_over_tod_rms": float(np.abs(d).max()) / rms}
    print(json.dumps(line), flush=True)
    conv.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--samples", type=int, default=2_000_000)
    ap.add_argument("--plain-samples", type=int, default=100_000)
    ap.add_argument("--accuracy-samples", type=int, default=50_000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3", "c4", "c5", "order", "map", "beam",
                             "refgpu", "bilinear"],
                    help="c2 = the headline line; the others print their own study lines")
    ap.add_argument("--fp64-samples", type=int, default=200_000)
    ap.add_argument("--cpu-samples", type=int, default=2_000)
    ap.add_argument("--plain-fraction", type=float, default=0.05)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = env_rank()
    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    if args.workload != "c2":
        import torch

        torch.cuda.set_device(local)
        if args.samples == 2_000_000:
            args.samples = 0  # the workload's own sample count
        return {"c3": run_c3_precision, "c4": run_c4_batched, "c5": run_c5_adjoint,
                "order": run_order_study, "map": run_map_study,
                "beam": run_beam_study, "refgpu": run_refgpu_study,
                "bilinear": run_bilinear_study}[args.workload](args)
    return run_gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
