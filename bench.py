"""Benchmark of the GB300 simus/pfield sweep.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one "step" = one frame): the 128-element scale configuration -- 200,000 scatterers
in x in [-19, 19] mm, z in [5, 50] mm with three anechoic disks, 0.5 dB/cm/MHz, one 0-degree
plane wave -> 128-channel RF (plain fused FP32 simus sweep + this library's irfft + gate), plus the RMS
pressure field on a 256 x 512 grid over the same box.  Inputs are seeded synthetic data.

The JSON line reports RF frames/s (``value``, inputs resident in HBM, L2 flushed before every
step), the same through the public API with host buffers (``e2e``), Green's terms/s, the FP32
roofline of the dominant kernel, the CPU baseline (the oracle: a port of the reference's FP64
NumPy path, timed on this host's cores on a bounded sample and scaled per scatterer/point),
and SM clocks sampled during the timed region.

``--impl reference`` times that CPU path alone, each step a bounded sample, and prints the
same metric with ``"impl": "reference"``.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# The headline metric: frames/s and Green's terms/s of the tensor-core and surrogate paths beside
# the plain FP32 kernel, each at relative L2 <= 1e-3 against FP64.  ``value`` is the plain fused
# FP32 kernel's frame rate on the 200,000-scatterer frame; the tensor-core and surrogate
# figures on their own workloads are in ``vs_plain_fp32`` (and in full under ``paths``).
METRIC = "RF frames/s & Green terms/s: TC/surrogate vs plain FP32 kernel at rel-L2\u22641e-3"
VALUE_IS = "plain fused FP32 kernel: RF frames/s of the 200,000-scatterer frame (simus + 256x512 pfield)"
UNIT = "frames/s"
WORKLOAD = ("cfg2: 128-element linear array (pitch 0.30 mm, width 0.27 mm, fc 5.2 MHz, bw 0.67), "
            "c 1540 m/s, 0.5 dB/cm/MHz, 0-degree plane wave, 200,000 scatterers x in [-19,19] mm, "
            "z in [5,50] mm, rc N(0,1) with three 2 mm anechoic disks; + pfield on 256x512 grid")
L2_FLUSH_BYTES = 512 << 20
# DRAM bytes (read + write) of one simus_ws_kernel launch measured by ncu on an 8,720-scatterer
# chunk, the chunk size of the benchmark frame: the tile geometry blocks read once from HBM
# (then from L2 by the other bands' CTAs) plus the partial spectra.  The bench cannot run ncu;
# the figure is refreshed from a capture whenever the kernel changes.
BAND_KERNEL_DRAM_BYTES = 61_484_032 + 1_643_776


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def _cpu_info():
    model = "unknown"
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                model = line.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    if model == "unknown":
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for line in out.splitlines():
                if "Model name" in line:
                    model = line.split(":", 1)[1].strip()
                    break
        except Exception:
            pass
    return model, len(os.sched_getaffinity(0))


# ------------------------------------------------------------------------------------------
# CPU baseline: the oracle (FP64 NumPy port of the reference's PYTHON strategy)
# ------------------------------------------------------------------------------------------

def _single_thread_blas():
    """Oracle workers run one process per core; each must use one BLAS/OpenMP thread."""
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[v] = "1"


def _oracle_simus_shard(args):
    import oracle.fastsimus_fp64 as O

    scat, rc, delays, plan, params, medium = args
    return O.simus_spectrum_selected(scat, rc, delays, plan, params, medium)


def _oracle_pfield_shard(args):
    import oracle.fastsimus_fp64 as O

    pts, delays, plan, params, medium = args
    return O.pfield_compute(pts, delays, plan, params, medium)


def cpu_frame_time(pool, n_workers, scat, rc, grid_pts, delays, plan, pplan, params, medium, s_sample, g_sample):
    """Seconds per full frame: the simus sweep of s_sample scatterers and the pfield sweep of
    g_sample grid points, each scaled linearly to the full frame (the sweeps are linear in the
    scatterers and in the points), plus the irfft + gate of the frame's spectrum, timed once and
    not scaled (its size does not depend on the scatterer count).  The plans are excluded on
    both arms."""
    import oracle.fastsimus_fp64 as O

    rng = np.random.default_rng(123)
    si = rng.choice(scat.shape[0], s_sample, replace=False)
    gi = rng.choice(grid_pts.shape[0], g_sample, replace=False)
    s_sh = np.array_split(si, n_workers)
    g_sh = np.array_split(gi, n_workers)
    t0 = time.perf_counter()
    parts = pool.map(_oracle_simus_shard, [(scat[i], rc[i], delays, plan, params, medium) for i in s_sh])
    spec = sum(parts) * plan.correction_factor
    t1 = time.perf_counter()
    O.irfft_and_threshold(spec, plan, params.n_elements)
    t2 = time.perf_counter()
    pool.map(_oracle_pfield_shard, [(grid_pts[i], delays, pplan, params, medium) for i in g_sh])
    t3 = time.perf_counter()
    return (t1 - t0) * scat.shape[0] / s_sample + (t2 - t1) + (t3 - t2) * grid_pts.shape[0] / g_sample


def port_calibration():
    """The committed single-core timing of the oracle port against the reference's own FP64
    path on the same inputs (oracle/calibrate_port.py), or None."""
    p = ROOT / "oracle" / "port_calibration.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
    except Exception:
        return None
    return {"simus_port_over_reference": d.get("simus_port_over_reference_mean"),
            "pfield_port_over_reference": d.get("pfield_port_over_reference"), "cpu": d.get("cpu"),
            "source": "oracle/port_calibration.json (oracle/calibrate_port.py: same inputs and plans, one core, "
                      "one BLAS thread)"}


def make_workload(n_scat=200_000, grid_nx=256, grid_nz=512):
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.plan import pfield_precompute, simus_precompute

    params, medium = W.cfg2_probe(), W.cfg2_medium()
    scat, rc = W.cfg2_scatterers(n_scat)
    grid = W.cfg2_grid(grid_nx, grid_nz)
    delays = np.zeros(params.n_elements)
    t0 = time.perf_counter()
    plan = simus_precompute(scat, rc, delays, params, medium)
    pplan = pfield_precompute(grid, delays, params, medium)
    t_plan = time.perf_counter() - t0
    return params, medium, scat, rc, grid, delays, plan, pplan, t_plan


def green_terms(plan, pplan, params, n_scat, n_grid):
    e_u = params.n_elements * plan.n_sub
    return n_scat * e_u * plan.selected_freqs.shape[0] + n_grid * e_u * pplan.selected_freqs.shape[0]


def replica_throughput(local_ms: float, steps: int, dist=None, device="cpu"):
    """Whole-job frames/s of independent replicas, one per rank: every rank ran `steps` frames
    in `local_ms`; the job took as long as its slowest rank.  Returns (frames/s, job ms)."""
    import torch

    world, job_ms = 1, float(local_ms)
    if dist is not None and dist.is_initialized():
        world = dist.get_world_size()
        t = torch.tensor([job_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        job_ms = float(t.item())
    return steps * world / (job_ms * 1e-3), job_ms


def frame_launches(plan, params, n_scat, device) -> int:
    """This library's kernel launches in one timed frame: fsg_simus (set-up, geometry + band
    kernel per scatterer chunk, reduction), the RF epilogue (twiddles, irfft, gate) and
    fsg_pfield (set-up, band kernel, reduction)."""
    from fastsimus_gb300 import _device, _native

    lib = _native.load()
    fplan = _device.plan_tables(plan, device).fsg_plan(plan)
    n = int(lib.fsg_simus_launches(_native.make_probe(params, plan.n_sub), fplan, int(n_scat), 0))
    if n < 0:
        raise RuntimeError("fsg_simus_launches rejected the frame")
    return n + 3 + 3


def algorithmic_flops_simus(plan, params, n_scat, n_tx=1):
    """S * F * (8 E U + 16 E T): recurrence (6) + sub-sum (2) per term, TX and RX complex MAC
    (8 + 8) per (scatterer, element, frequency, transmit)."""
    E, U, F = params.n_elements, plan.n_sub, plan.selected_freqs.shape[0]
    return float(n_scat) * F * (8.0 * E * U + 16.0 * E * n_tx)


def run_reference_arm(args, rank, world):
    if rank != 0:
        print(json.dumps({"impl": "reference", "rank": rank, "skipped": "rank 0 runs the CPU arm"}), file=sys.stderr)
        return
    import multiprocessing as mp

    params, medium, scat, rc, grid, delays, plan, pplan, _ = make_workload(args.scatterers, args.grid_nx, args.grid_nz)
    gpts = grid.reshape(-1, 2)
    model, cores = _cpu_info()
    _single_thread_blas()
    ctx = mp.get_context("spawn")
    s_sample, g_sample = args.cpu_scatterers, args.cpu_points
    with ctx.Pool(cores) as pool:
        for _ in range(max(args.warmup, 0)):
            cpu_frame_time(pool, cores, scat, rc, gpts, delays, plan, pplan, params, medium, max(cores, 64),
                           max(cores, 64))
        times = [cpu_frame_time(pool, cores, scat, rc, gpts, delays, plan, pplan, params, medium, s_sample,
                                g_sample) for _ in range(args.steps)]
    t = float(np.mean(times))
    val = 1.0 / t
    sample = (f"{s_sample} of {scat.shape[0]} scatterers and {g_sample} of {gpts.shape[0]} grid points per step, "
              f"sharded over {cores} processes, sweep times scaled linearly to the full frame; the irfft + gate "
              "of the frame timed once, unscaled")
    line = {
        "metric": METRIC, "value": val, "unit": UNIT, "value_is": VALUE_IS, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "cpu": model, "l2": "n/a (CPU)"},
        "green_terms_per_s": green_terms(plan, pplan, params, scat.shape[0], gpts.shape[0]) * val,
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                         "port_calibration": port_calibration()},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------

class ClockSampler:
    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.gpu)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


def fp32_theoretical_tflops(device, sm_mhz=None):
    """SMs x 128 FP32 lanes x 2 flops x the maximum SM clock (or `sm_mhz`)."""
    import torch

    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = sm_mhz or _peaks().get("sm_max_mhz") or 2070.0
    return sms * 128 * 2 * float(mhz) * 1e6 / 1e12


def fp32_peak_tflops(device):
    """Measured FP32 FMA throughput (TFLOP/s) of this GPU from fsg_fp32_fma_probe."""
    import ctypes

    import torch

    from fastsimus_gb300 import _native

    lib = _native.load()
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    blocks = sms * 8
    out = torch.empty(blocks, dtype=torch.float32, device=device)
    flops = ctypes.c_double()
    stream = torch.cuda.current_stream(device).cuda_stream
    best = 0.0
    for it in range(4):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        _native.check(lib.fsg_fp32_fma_probe(out.data_ptr(), blocks, 1 << 16, ctypes.byref(flops), stream))
        e.record()
        torch.cuda.synchronize()
        if it:
            best = max(best, flops.value / (s.elapsed_time(e) * 1e-3) / 1e12)
    return best


def run_gpu_arm(args, rank, world):
    import torch

    import fastsimus_gb300 as F
    from fastsimus_gb300 import _device, build

    build.build()
    local = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=device)

    params, medium, scat, rc, grid, delays, plan, pplan, t_plan = make_workload(args.scatterers, args.grid_nx,
                                                                                 args.grid_nz)
    n_scat, n_grid = scat.shape[0], grid.shape[0] * grid.shape[1]

    # device-resident inputs
    scat_d = torch.as_tensor(scat, device=device)
    rc_d = torch.as_tensor(rc, device=device)
    grid_d = torch.as_tensor(grid, device=device)
    del_d = torch.as_tensor(delays, device=device)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)

    def step_device():
        res = F.simus_compute(scat_d, rc_d, del_d, plan, params, medium)
        pf = F.pfield_compute(grid_d, del_d, pplan, params, medium)
        return res, pf

    for _ in range(args.warmup):
        step_device()
    torch.cuda.synchronize()

    timer = _device.LaunchTimer()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        _device.set_timer(timer)
        for k in range(args.steps):
            flush.zero_()
            starts[k].record()
            step_device()
            ends[k].record()
        torch.cuda.synchronize()
        _device.set_timer(None)
    dev_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    value, dev_ms = replica_throughput(dev_ms, args.steps, dist, device)
    if dist is not None:
        dist.barrier()
    simus_ms = timer.elapsed_ms("fsg_simus")
    pfield_ms = timer.elapsed_ms("fsg_pfield")

    if args.no_e2e:
        if rank == 0:
            print(json.dumps({"value": value, "simus_ms": float(np.mean(simus_ms)),
                              "pfield_ms": float(np.mean(pfield_ms)), "note": "profiling run (no e2e)"}), flush=True)
        if dist is not None:
            dist.destroy_process_group()
        return

    # end-to-end through the public API with host (pinned) buffers
    scat_h = torch.as_tensor(scat).pin_memory()
    rc_h = torch.as_tensor(rc).pin_memory()
    grid_h = torch.as_tensor(grid).pin_memory()
    del_h = torch.as_tensor(delays).pin_memory()
    res, pf = step_device()
    rf_out = torch.empty(res.rf.shape, dtype=res.rf.dtype).pin_memory()
    pf_out = torch.empty(pf.shape, dtype=pf.dtype).pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in (scat_h, rc_h, grid_h, del_h))
    d2h = rf_out.numel() * rf_out.element_size() + pf_out.numel() * pf_out.element_size()
    e2e_ms = []
    for k in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        r = F.simus_compute(scat_h, rc_h, del_h, plan, params, medium)
        p = F.pfield_compute(grid_h, del_h, pplan, params, medium)
        rf_out.copy_(r.rf, non_blocking=True)
        pf_out.copy_(p, non_blocking=True)
        e.record()
        torch.cuda.synchronize()
        if k >= args.warmup:
            e2e_ms.append(s.elapsed_time(e))
    e2e_value, _ = replica_throughput(sum(e2e_ms), args.steps, dist, device)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    peak = fp32_peak_tflops(device)
    flops = algorithmic_flops_simus(plan, params, n_scat)
    simus_avg = float(np.mean(simus_ms)) if simus_ms else float("nan")
    achieved = flops / (simus_avg * 1e-3) / 1e12
    gt = green_terms(plan, pplan, params, n_scat, n_grid)
    peaks = _peaks()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "value_is": VALUE_IS, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (double-float phase)", "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "parallelism": "replicas" if world > 1 else "1 gpu",
                   "l2": f"flushed before every timed step ({L2_FLUSH_BYTES >> 20} MiB write)",
                   "n_freq_simus": int(plan.selected_freqs.shape[0]), "n_freq_pfield": int(pplan.selected_freqs.shape[0]),
                   "n_sub": int(plan.n_sub), "plan_host_s": t_plan},
        "green_terms_per_s": gt * value,
        "simus_ms": simus_avg, "pfield_ms": float(np.mean(pfield_ms)) if pfield_ms else None,
        "gpu_launches": args.steps * frame_launches(plan, params, n_scat, device),
        "roofline": {"kernel": "simus_ws_kernel", "bound": "fp32", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                     "traffic": BAND_KERNEL_DRAM_BYTES, "traffic_unit": "bytes per sweep-kernel launch",
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one simus_ws_kernel "
                                       "launch on an 8,720-scatterer chunk (the chunk size of this frame), "
                                       "python bench.py --steps 1 --warmup 1 --no-e2e --scatterers 20000",
                     "peak_source": "measured in-run by fsg_fp32_fma_probe (FP32 FMA chains); MEASURED_PEAKS.json "
                                    "holds only HBM and bf16 tensor peaks",
                     "peak_theoretical": fp32_theoretical_tflops(device),
                     "frac_vs_theoretical": achieved / fp32_theoretical_tflops(device),
                     "theoretical_source": "SMs x 128 FP32 lanes x 2 x max SM clock",
                     "algorithmic_flops_per_launch": flops,
                     "hbm_peak_gbs": peaks.get("hbm_gbs")},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline:
        import multiprocessing as mp

        model, cores = _cpu_info()
        _single_thread_blas()
        ctx = mp.get_context("spawn")
        with ctx.Pool(cores) as pool:
            cpu_frame_time(pool, cores, scat, rc, grid.reshape(-1, 2), delays, plan, pplan, params, medium,
                           cores, cores)
            t = cpu_frame_time(pool, cores, scat, rc, grid.reshape(-1, 2), delays, plan, pplan, params, medium,
                               args.cpu_scatterers, args.cpu_points)
        line["cpu_baseline"] = {
            "value": 1.0 / t, "unit": UNIT, "cores": cores, "kind": "port", "cpu": model,
            "sample": f"{args.cpu_scatterers} scatterers + {args.cpu_points} grid points of the frame, sharded over "
                      f"{cores} processes, sweeps scaled linearly to {n_scat} scatterers + {n_grid} points; "
                      "the irfft + gate of the frame timed once, unscaled",
            "port_calibration": port_calibration()}
    if not args.no_ref_gpu and world == 1:
        line["reference_gpu_kernel"] = reference_gpu_leg(args, device, scat, rc, delays, plan, params, medium,
                                                         flush, simus_avg)
    if not args.no_paths and world == 1:
        line["paths"] = other_paths(args)
        line["vs_plain_fp32"] = vs_plain_summary(line["paths"])
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def reference_gpu_leg(args, device, scat, rc, delays, plan, params, medium, flush, our_simus_ms) -> dict:
    """The reference's own CUDA kernel (simus_fused.cu, compiled from its source for sm_103a, stock
    launch shape) on the same frame and GPU: time per sweep (zeroed outputs + kernel, CUDA
    events, L2 flushed), and its accuracy against this package's sweep on the full frame and
    against the FP64 oracle on a 512-scatterer sample.  Failure is recorded, not raised."""
    import torch

    from tests._golden import max_phase_err, rel_l2

    try:
        from oracle import ref_gpu
        import oracle.fastsimus_fp64 as O
        from fastsimus_gb300.simus import simus_gb300

        E, U, nf = params.n_elements, int(plan.n_sub), int(plan.selected_freqs.shape[0])
        ok, why = ref_gpu.available(E, U, nf)
        if not ok:
            return {"unavailable": why}
        k = ref_gpu.RefSimusKernel(E, U, nf, device)
        d = k.prepare(scat, rc, delays, plan, params, medium)
        re, im = k.outputs()
        for _ in range(max(args.warmup, 2)):
            k.launch(d, re, im)
        torch.cuda.synchronize()
        ms = []
        for _ in range(max(args.steps, 3)):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            k.launch(d, re, im)
            e.record()
            torch.cuda.synchronize()
            ms.append(s.elapsed_time(e))
        t = float(np.mean(ms))
        c128 = lambda t: t.cpu().numpy().astype(np.complex128)  # noqa: E731
        ref_full = c128(torch.complex(re, im).reshape(E, nf).T)
        ones = np.ones(E)
        ours_full = c128(simus_gb300(scat, rc, params, plan, medium, delays, ones))
        idx = np.random.default_rng(7).choice(scat.shape[0], 512, replace=False)
        ref_s = c128(k.spectrum(scat[idx], rc[idx], delays, plan, params, medium))
        ours_s = c128(simus_gb300(scat[idx], rc[idx], params, plan, medium, delays, ones))
        gold = O.simus_spectrum_selected(scat[idx], rc[idx], delays, plan, params, medium)
        k.close()
        terms = scat.shape[0] * E * U * nf
        return {
            "source": "src/fast_simus/kernels/simus_fused.cu compiled by oracle/ref_gpu_build.py (nvcc sm_103a, "
                      "--use_fast_math, the -D set and 256x128 launch of kernels/cuda_simus.py)",
            "sweep_ms": t, "gb300_sweep_ms": our_simus_ms, "speedup_gb300_vs_reference_kernel": t / our_simus_ms,
            "green_terms_per_s": terms / (t * 1e-3),
            "relL2_vs_gb300_full_frame": rel_l2(ref_full, ours_full),
            "max_phase_err_rad_vs_gb300_full_frame": max_phase_err(ref_full, ours_full),
            "relL2_vs_fp64_oracle_512": rel_l2(ref_s, gold),
            "max_phase_err_rad_vs_fp64_oracle_512": max_phase_err(ref_s, gold),
            "gb300_relL2_vs_fp64_oracle_512": rel_l2(ours_s, gold),
            "gb300_max_phase_err_rad_vs_fp64_oracle_512": max_phase_err(ours_s, gold),
        }
    except Exception as exc:  # recorded in the JSON line
        return {"error": f"{type(exc).__name__}: {exc}"}


def vs_plain_summary(paths: dict) -> dict:
    """The comparison the headline metric names, read from the path measurements: each path's
    RF frames/s and Green's terms/s beside the plain FP32 kernel on the same workload and GPU,
    with its error against the FP32 / FP64 results."""
    out = {}
    tc = paths.get("tensor_core_cfg4", {})
    if "paths" in tc:
        t, pl = tc["paths"].get("tc", {}), tc["paths"].get("plain_fp32_single_transmit", {})
        out["tensor_core"] = {
            "workload": "31 plane waves x 262,144 scatterers, 64 elements",
            "frames_per_s": t.get("frames_per_s"), "green_terms_per_s": t.get("green_terms_per_s"),
            "plain_fp32_frames_per_s": pl.get("frames_per_s"), "plain_fp32_green_terms_per_s": pl.get("green_terms_per_s"),
            "speedup_vs_plain": tc.get("speedup_tc_vs_plain"),
            "relL2_vs_fp64_oracle": t.get("relL2_vs_fp64_oracle"), "relL2_vs_plain_fp32": t.get("relL2_vs_plain_fp32")}
    elif tc:
        out["tensor_core"] = tc
    su = paths.get("surrogate_cfg5", {})
    if "simus_1M_x75" in su:
        q = su["simus_1M_x75"]
        out["surrogate"] = {k: q.get(k) for k in q if k != "breakdown_sample_s"}
        out["surrogate"]["workload"] = "1,000,000 scatterers x 75 plane waves over the cfg1 box"
        out["surrogate"]["val_rel_l2"] = su.get("training", {}).get("val_rel_l2")
        out["surrogate"]["training_frac_of_bf16_peak"] = su.get("roofline", {}).get("frac")
    elif su:
        out["surrogate"] = su
    return out


def other_paths(args) -> dict:
    """Summaries of the batched (cfg3), tensor-core (cfg4) and surrogate (cfg5) paths, measured
    in the same run; a failure in one is recorded in the line, not raised."""
    import copy

    out = {}
    for name, fn, kw in (("batched_fp32_cfg3", run_batched_workload, {"autotune_quick": True}),
                         ("tensor_core_cfg4", run_tc_workload, {}),
                         ("surrogate_cfg5", run_surrogate_workload, {}),
                         ("beamform_das_cfg3", run_beamform_workload, {})):
        a = copy.copy(args)
        a.scatterers = 200_000  # each workload uses its own size
        a.steps, a.warmup = 3, 2
        for k, v in kw.items():
            setattr(a, k, v)
        try:
            r = fn(a)
            keep = ("metric", "value", "unit", "ms_per_step", "green_terms_per_s", "sweep_ms", "roofline", "paths",
                    "speedup_tc_vs_plain", "speedup_tc_vs_fp32_batched", "config", "training",
                    "field_rel_l2_1M_queries", "per_query_s", "simus_1M_x75", "clocks",
                    "rf2iq_ms", "das_ms",
                    "das_terms_per_s", "cpu_baseline", "parity_rel_l2_sample")
            out[name] = {k: r[k] for k in keep if k in r}
            if "training" in out[name]:
                out[name]["training"] = {k: v for k, v in out[name]["training"].items() if k != "history"}
        except Exception as exc:  # recorded in the JSON line
            out[name] = {"error": f"{type(exc).__name__}: {exc}"}
    return out


def run_beamform_workload(args):
    """Imaging of the cfg3 firings downstream of simus: one seeded phantom of the cfg3 set
    simulated for 75 plane waves at +-16 deg by the batched sweep, then rf2iq of the 75 RF
    frames and the compounded delay-and-sum of all firings on a 256 x 512 grid of the cfg3 box
    (x in [-10, 10] mm, z in [5, 30] mm), linear interpolation, default f-number.  A step is
    rf2iq + das on HBM-resident RF (kernels timed with CUDA events on the launching stream).
    The CPU baseline runs the FP64 oracle on a bounded sample (2 firings x 4,096 pixels),
    scaled to the full image; the same sample gives the parity figure."""
    import ctypes

    import torch

    from fastsimus_gb300 import _device, _native, build
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus
    from fastsimus_gb300.beamform import RF2IQ_ORDER, DasParam, _das_call, _lowpass, _pixels, das, rf2iq

    build.build()
    device = torch.device("cuda", _env_int("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    p, m = W.cfg1_probe(), W.cfg1_medium()
    angles = np.linspace(-16.0, 16.0, getattr(args, "transmits", 75))
    delays = np.asarray(W.plane_wave_delays(p, m, angles), dtype=np.float64)
    b = BatchedSimus(W.cfg3_phantoms(1), delays, p, m)
    b.run()
    rf = b.rfs[0]  # (n_tx, n_samples, E) float32, HBM-resident
    plan = b.plans[0]
    fs = plan.n_fft * float(plan.selected_freqs[1] - plan.selected_freqs[0])  # exact RF sample rate
    nt, ns, ne = rf.shape
    xs, zs = np.linspace(-10e-3, 10e-3, 256), np.linspace(5e-3, 30e-3, 512)
    x, z = np.meshgrid(xs, zs)
    param = DasParam.from_params(p, m, fs=fs)
    lib = _native.load()
    stream = _device.stream_handle(device)
    sos, zq = _lowpass(fs, p.freq_center, None)
    dp = ctypes.POINTER(ctypes.c_double)
    iq = torch.empty((nt, ne, ns), dtype=torch.complex64, device=device)
    img = torch.empty(x.size, dtype=torch.complex64, device=device)
    pix, _ = _pixels(x, z, device)
    txd = torch.as_tensor(delays, device=device)
    probe, dpar = _das_call(param, "linear", True)

    def step(ev=None):
        if ev:
            ev[0].record()
        _native.check(lib.fsg_rf2iq(rf.data_ptr(), nt, ns, ne, fs, p.freq_center, 0.0, sos.shape[0],
                                    sos.ctypes.data_as(dp), zq.ctypes.data_as(dp), 3 * (RF2IQ_ORDER + 1),
                                    iq.data_ptr(), stream))
        if ev:
            ev[1].record()
        _native.check(lib.fsg_das(ctypes.byref(probe), ctypes.byref(dpar), iq.data_ptr(), nt, ns, txd.data_ptr(),
                                  pix.data_ptr(), pix.shape[0], img.data_ptr(), stream))
        if ev:
            ev[2].record()

    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    t_iq, t_das = [], []
    with ClockSampler(device.index or 0) as clocks:
        # ~0.5 s of steps, so the clock sampler (every 200 ms) sees the timed region
        for _ in range(max(args.steps, 300)):
            flush.zero_()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            step(ev)
            torch.cuda.synchronize()
            t_iq.append(ev[0].elapsed_time(ev[1]))
            t_das.append(ev[1].elapsed_time(ev[2]))
    iq_ms, das_ms = float(np.median(t_iq)), float(np.median(t_das))
    terms = x.size * nt * ne
    # CPU oracle on a bounded sample, and the GPU image of the same sample for parity
    from oracle import das_fp64 as D

    rng = np.random.default_rng(0)
    sel = rng.choice(x.size, 4096, replace=False)
    fr = [0, nt - 1]
    px, pz = x.reshape(-1)[sel], z.reshape(-1)[sel]
    rf_h = rf[fr].cpu().numpy().astype(np.float64)
    t0 = time.perf_counter()
    iq_h = np.stack([D.rf2iq(rf_h[k], fs, p.freq_center) for k in range(len(fr))])
    ref = D.das(iq_h, px, pz, delays[fr], n_elements=ne, pitch=p.pitch, radius=p.radius, c=m.speed_of_sound, fs=fs,
                fc=p.freq_center, fnumber=D.default_fnumber(p.element_width, p.freq_center, m.speed_of_sound))
    t_cpu = time.perf_counter() - t0
    got = das(rf2iq(rf[fr], fs, p.freq_center), px, pz, delays[fr], param).cpu().numpy()
    parity = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    cpu_image_s = t_cpu * (x.size / sel.size) * (nt / len(fr))
    return {
        "metric": "compounded images/s (rf2iq + delay-and-sum of 75 plane-wave firings, 256 x 512 pixels)",
        "value": 1e3 / (iq_ms + das_ms), "unit": "images/s", "ms_per_step": iq_ms + das_ms,
        "rf2iq_ms": iq_ms, "das_ms": das_ms, "das_terms_per_s": terms / (das_ms * 1e-3),
        "config": {"workload": "cfg3 probe (64 elements), one cfg3 phantom, 75 plane waves +-16 deg, "
                               "256 x 512 grid over x [-10, 10] mm, z [5, 30] mm",
                   "n_samples": ns, "fs_hz": fs, "fnumber": D.default_fnumber(p.element_width, p.freq_center,
                                                                               m.speed_of_sound),
                   "l2": "flushed (512 MiB write) before every step"},
        "cpu_baseline": {"value": 1.0 / cpu_image_s, "unit": "images/s", "cores": 1, "kind": "port",
                         "sample": f"2 firings x {sel.size} pixels, scaled x{x.size * nt / (sel.size * len(fr)):.0f}"},
        "parity_rel_l2_sample": parity,
        "clocks": clocks.summary(),
    }


def run_batched_workload(args):
    """cfg3: 75 plane waves x 16 phantoms (log-uniform 10k-200k scatterers) in one persistent
    launch, tile shapes from the autotuner, the whole batch replayed from a CUDA graph."""
    import torch

    from fastsimus_gb300 import _device, build
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    build.build()
    device = torch.device("cuda", _env_int("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    p, m = W.cfg1_probe(), W.cfg1_medium()
    phantoms = W.cfg3_phantoms(getattr(args, "phantoms", 16))
    delays = W.plane_wave_delays(p, m, np.linspace(-16.0, 16.0, getattr(args, "transmits", 75)))
    t0 = time.perf_counter()
    b = BatchedSimus(phantoms, delays, p, m)
    t_plan = time.perf_counter() - t0
    t0 = time.perf_counter()
    from fastsimus_gb300.batched import BatchTuning, fp32_search_space

    # tile-shape search: every compiled FP32 shape x two chunk sizes for this batch, timed on a
    # slice of the batch (its first phantoms: same probe, firings and per-item shapes); the
    # winner runs the full batch
    space = fp32_search_space(p.n_elements, sum(int(s.shape[0]) for s, _ in b.phantoms))
    n_slice = min(len(phantoms), 3)
    tuner = BatchedSimus(phantoms[:n_slice], delays, p, m, plans=b.plans[:n_slice])
    best = tuner.autotune(candidates=space, cache=False)
    tune_log = sorted(({"ms": round(t, 3), **c} for t, c in tuner.tune_log), key=lambda r: r["ms"])
    del tuner
    b.set_tuning(best)
    t_tune = time.perf_counter() - t0
    b.capture()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)
    for _ in range(args.warmup):
        b.replay()
    torch.cuda.synchronize()
    timer = _device.LaunchTimer()
    ms = []
    with ClockSampler(device.index or 0) as clocks:
        for _ in range(args.steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            b.replay()
            e.record()
            torch.cuda.synchronize()
            ms.append(s.elapsed_time(e))
    # kernel-only time of the sweep (eager launch with events on the launching stream)
    _device.set_timer(timer)
    for _ in range(2):
        b.launch_sweep()
    torch.cuda.synchronize()
    _device.set_timer(None)
    sweep_ms = float(np.mean(timer.elapsed_ms("fsg_simus_batched")))
    frames = len(phantoms) * delays.shape[0]
    n_scat = [int(s.shape[0]) for s, _ in b.phantoms]
    flops = sum(algorithmic_flops_simus(pl, p, n, n_tx=delays.shape[0]) for pl, n in zip(b.plans, n_scat))
    terms = sum(n * p.n_elements * pl.n_sub * pl.selected_freqs.shape[0] * delays.shape[0]
                for pl, n in zip(b.plans, n_scat))
    step_ms = float(np.mean(ms))
    peak = fp32_peak_tflops(device)
    line = {"metric": "RF frames/s (batched FP32: 75 plane waves x 16 phantoms, one persistent launch, CUDA graph)",
            "value": frames / (step_ms * 1e-3), "unit": "frames/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": f"cfg3: cfg1 probe, {delays.shape[0]} plane waves in [-16,16] deg, "
                                   f"{len(phantoms)} phantoms, scatterers {min(n_scat)}..{max(n_scat)} "
                                   f"(total {sum(n_scat)})", "tuning": best.__dict__,
                       "l2": "flushed before every replay", "plan_host_s": t_plan, "autotune_s": t_tune},
            "green_terms_per_s": terms / (step_ms * 1e-3),
            "sweep_ms": sweep_ms,
            "roofline": {"kernel": "batched_kernel", "bound": "fp32", "achieved": flops / (sweep_ms * 1e-3) / 1e12,
                         "peak": peak, "unit": "TFLOP/s", "frac": flops / (sweep_ms * 1e-3) / 1e12 / peak,
                         "algorithmic_flops_per_launch": flops},
            "autotune": {"searched_on": f"the first {n_slice} phantoms of the batch, one sweep per candidate",
                         "space": [c.__dict__ for c in space], "log_ms": tune_log, "winner": best.__dict__},
            "clocks": clocks.summary()}
    # the same batch on the tensor cores (BF16 hi/lo, 1e-3 accuracy class), checked against the
    # FP32 spectra above
    try:
        ref = [o.clone() for o in b.outs]
        tcb = BatchedSimus(phantoms, delays, p, m, backend="tc", plans=b.plans)
        tc_best = tcb.autotune(candidates=[BatchTuning(fb, c, 1) for fb in (1, 2) for c in (8192, 16384)], cache=False)
        tcb.capture()
        for _ in range(args.warmup):
            tcb.replay()
        torch.cuda.synchronize()
        tms = []
        for _ in range(args.steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            tcb.replay()
            e.record()
            torch.cuda.synchronize()
            tms.append(s.elapsed_time(e))
        rel = [float(torch.linalg.vector_norm(a - r) / torch.linalg.vector_norm(r)) for a, r in zip(tcb.outs, ref)]
        tc_ms = float(np.mean(tms))
        line["paths"] = {"tc": {"frames_per_s": frames / (tc_ms * 1e-3), "ms_per_batch": tc_ms,
                                "speedup_vs_fp32_batched": step_ms / tc_ms, "tuning": tc_best.__dict__,
                                "status": tcb.device_status(), "relL2_vs_fp32_max": max(rel),
                                "relL2_vs_fp32_median": float(np.median(rel))}}
    except Exception as exc:  # recorded in the line
        line["paths"] = {"tc": {"error": f"{type(exc).__name__}: {exc}"}}
    return line


def _oracle_rf_shard(args):
    import oracle.fastsimus_fp64 as O

    scat, rc, delays, plan, params, medium = args
    return O.simus_spectrum_selected(scat, rc, delays, plan, params, medium)


def run_tc_workload(args):
    """cfg4: 31 plane waves in [-12, 12] deg, 262,144 scatterers (5 % bright x10), cfg1 probe.
    Times the tcgen05 BF16 hi/lo path, the FP32 batched path and the plain single-transmit
    kernel looped over firings, and measures the tensor-core path's RF error against the FP64
    oracle on 3 firings x a 16,384-scatterer subsample (linearity makes the subsample a valid
    check of the same arithmetic)."""
    import multiprocessing as mp

    import torch

    import fastsimus_gb300 as F
    from fastsimus_gb300 import _device, build
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus

    _single_thread_blas()
    build.build()
    device = torch.device("cuda", _env_int("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    p, m = W.cfg1_probe(), W.cfg1_medium()
    scat, rc = W.cfg4_scatterers(args.scatterers if args.scatterers != 200_000 else 262_144)  # 262,144 by default
    angles = np.linspace(-12.0, 12.0, 31)
    delays = W.plane_wave_delays(p, m, angles)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=device)

    def time_graph(b, steps):
        b.capture()
        for _ in range(args.warmup):
            b.replay()
        torch.cuda.synchronize()
        ms = []
        for _ in range(steps):
            flush.zero_()
            st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            st.record()
            b.replay()
            en.record()
            torch.cuda.synchronize()
            ms.append(st.elapsed_time(en))
        return float(np.mean(ms))

    if args.tc_only:  # profiling case: the tensor-core sweep alone
        tc = BatchedSimus([(scat, rc)], delays, p, m, backend="tc")
        for _ in range(max(1, args.steps)):
            tc.launch_sweep()
        torch.cuda.synchronize()
        return {"tc_only": True, "status": tc.device_status()}
    out = {}
    with ClockSampler(device.index or 0) as clocks:
        tc = BatchedSimus([(scat, rc)], delays, p, m, backend="tc")
        plan = tc.plans[0]
        best_tc = tc.autotune(cache=False)
        tc_ms = time_graph(tc, args.steps)
        assert tc.device_status() == 0
        tc_spec = tc.outs[0].clone()
        fp = BatchedSimus([(scat, rc)], delays, p, m, plans=[plan], backend="fp32")
        fp_ms = time_graph(fp, max(1, args.steps // 2))
        fp_spec = fp.outs[0].clone()
        # plain single-transmit kernel, one call per firing (the reference's usage)
        scat_d, rc_d = torch.as_tensor(scat, device=device), torch.as_tensor(rc, device=device)
        del_d = torch.as_tensor(delays, device=device)
        for t in range(2):
            F.simus_compute(scat_d, rc_d, del_d[t], plan, p, m)
        torch.cuda.synchronize()
        flush.zero_()
        st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        st.record()
        plain_spec = [F.simus_compute(scat_d, rc_d, del_d[t], plan, p, m).spectrum for t in range(len(angles))]
        en.record()
        torch.cuda.synchronize()
        plain_ms = st.elapsed_time(en)
    plain = torch.stack(plain_spec, 0)

    def rel(a, b):
        a, b = a.to(torch.complex128), b.to(torch.complex128)
        return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))

    # accuracy of the tensor-core path against the FP64 oracle on a subsample
    n_sub_s = args.tc_oracle_scatterers
    sub = np.random.default_rng(5).choice(scat.shape[0], n_sub_s, replace=False)
    firings = [0, len(angles) // 2, len(angles) - 1]
    tc_sub = BatchedSimus([(scat[sub], rc[sub])], delays, p, m, plans=[plan], backend="tc")
    tc_sub.run()
    sub_spec = tc_sub.outs[0].cpu().numpy()
    model, cores = _cpu_info()
    errs, phases = [], []
    i0, nf = plan.freq_idx_start, plan.selected_freqs.shape[0]
    with mp.get_context("spawn").Pool(cores) as pool:
        for t in firings:
            shards = np.array_split(sub, cores)
            parts = pool.map(_oracle_rf_shard, [(scat[i], rc[i], delays[t], plan, p, m) for i in shards])
            ref_sel = sum(parts) * plan.correction_factor
            got = sub_spec[t, i0:i0 + nf].astype(np.complex128)
            errs.append(float(np.linalg.norm(got - ref_sel) / np.linalg.norm(ref_sel)))
            mask = np.abs(ref_sel) > 1e-3 * np.abs(ref_sel).max()
            phases.append(float(np.max(np.abs(np.angle(got[mask] / ref_sel[mask])))))
    frames = len(angles)
    E, U, Fq = p.n_elements, plan.n_sub, plan.selected_freqs.shape[0]
    terms = scat.shape[0] * E * U * Fq * frames
    alg = algorithmic_flops_simus(plan, p, scat.shape[0], n_tx=frames)
    tensor_flops = 3 * 2 * (2 * 128 * 64 * 64) * (scat.shape[0] / 64) * Fq  # executed: TX + RX real GEMMs x 3 products
    peaks = _peaks()
    bf16_peak = peaks.get("bf16_tflops", 1890.4)
    line = {
        "metric": "RF frames/s & Green terms/s: tcgen05 BF16 hi/lo path vs plain FP32 kernel at relL2<=1e-3",
        "value": frames / (tc_ms * 1e-3), "unit": "frames/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": tc_ms, "higher_is_better": True, "dtype": "bf16x3 (hi/lo) tensor, f32 accumulate",
        "data": "synthetic (seeded)",
        "config": {"workload": f"cfg4: cfg1 probe, 31 plane waves in [-12,12] deg, {scat.shape[0]} scatterers, "
                               "5% x10 bright", "n_freq": int(Fq), "tuning_tc": best_tc.__dict__,
                   "l2": "flushed before every timed step"},
        "green_terms_per_s": terms / (tc_ms * 1e-3),
        "paths": {
            "tc": {"frames_per_s": frames / (tc_ms * 1e-3), "green_terms_per_s": terms / (tc_ms * 1e-3),
                   "ms_per_batch": tc_ms, "relL2_vs_plain_fp32": rel(tc_spec, plain),
                   "relL2_vs_fp64_oracle": errs, "max_phase_err_rad_vs_fp64": phases,
                   "oracle_subset": f"firings {firings} (angles {[float(angles[i]) for i in firings]}) on "
                                    f"{n_sub_s} random scatterers, oracle on {cores} cores"},
            "fp32_batched": {"frames_per_s": frames / (fp_ms * 1e-3), "green_terms_per_s": terms / (fp_ms * 1e-3),
                             "ms_per_batch": fp_ms, "relL2_vs_plain_fp32": rel(fp_spec, plain)},
            "plain_fp32_single_transmit": {"frames_per_s": frames / (plain_ms * 1e-3),
                                           "green_terms_per_s": terms / (plain_ms * 1e-3),
                                           "ms_per_batch": plain_ms},
        },
        "speedup_tc_vs_plain": plain_ms / tc_ms, "speedup_tc_vs_fp32_batched": fp_ms / tc_ms,
        "roofline": {"kernel": "tc_kernel", "bound": "tensor", "achieved": alg / (tc_ms * 1e-3) / 1e12,
                     "peak": bf16_peak, "unit": "TFLOP/s", "frac": alg / (tc_ms * 1e-3) / 1e12 / bf16_peak,
                     "algorithmic_flops_per_launch": alg,
                     "count": "algorithmic S F (8 E U + 16 E T): the hi/lo split counted once",
                     "executed_tensor_tflops": tensor_flops / (tc_ms * 1e-3) / 1e12,
                     "executed_frac": tensor_flops / (tc_ms * 1e-3) / 1e12 / bf16_peak,
                     "executed_note": "bf16 tensor flops as issued: TX + RX real GEMMs x 3 hi/lo products",
                     "peak_source": "MEASURED_PEAKS.json bf16_tflops (measured)" if "bf16_tflops" in peaks
                     else "fallback 1890.4"},
        "clocks": clocks.summary(),
    }
    return line


def run_surrogate_workload(args):
    """cfg5: Fourier-feature MLP (64 features, 4 x 256 SiLU, BF16 weights; a head of five
    carrier amplitudes) trained by the library's tcgen05 kernels on 2M exact transmit-field
    samples over the cfg1 box, the band fc (1 +- B/2) and +-16 degrees; then used in simus for
    1,000,000 scatterers x 75 plane waves with the exact kernel judging every (64-scatterer
    tile, firing) unit and recomputing units above 1e-3, and answering every query outside the
    network's domain (frequencies outside its band).  The simus part runs on a bounded sample
    of the phantom and is scaled by scatterer count; the exact FP32 batched sweep is timed on
    the full phantom."""
    import torch

    from fastsimus_gb300 import build
    from fastsimus_gb300 import workloads as W
    from fastsimus_gb300.batched import BatchedSimus, shared_plan
    from fastsimus_gb300.surrogate import TxFieldSurrogate, cfg5_box, mlp_flops_per_sample, simus_with_surrogate

    build.build()
    device = torch.device("cuda", _env_int("LOCAL_RANK", 0))
    torch.cuda.set_device(device)
    p, m = W.cfg1_probe(), W.cfg1_medium()
    box = cfg5_box(p)
    sur = TxFieldSurrogate(p, m, box, seed=0)
    with ClockSampler(device.index or 0) as clocks:
        rep = sur.train(n_train=args.sur_train, steps=args.sur_steps, evals=3)
    peaks = _peaks()
    bf16_peak = peaks.get("bf16_tflops_sustained", peaks.get("bf16_tflops", 1890.4))
    # per-query costs: network inference (tcgen05 forward + carriers) vs the exact field kernel
    q = sur.sample_domain(1 << 20, seed=9)
    for _ in range(2):
        sur.predict(q)
        sur.exact(q)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    pred = sur.predict(q)
    ev[1].record()
    ex = sur.exact(q)
    ev[2].record()
    torch.cuda.synchronize()
    t_net_q = ev[0].elapsed_time(ev[1]) * 1e-3 / q.shape[0]
    t_exact_q = ev[1].elapsed_time(ev[2]) * 1e-3 / q.shape[0]
    val_rel = float(torch.linalg.vector_norm(pred - ex) / torch.linalg.vector_norm(ex))

    def simus_case(scat, rc, angles_deg):
        angles = np.deg2rad(angles_deg)
        delays = W.plane_wave_delays(p, m, angles_deg)
        plan = shared_plan(scat, rc, list(delays), p, m)
        sub = np.random.default_rng(2).choice(scat.shape[0], args.sur_sample, replace=False)
        simus_with_surrogate(sur, scat[sub[:128]], rc[sub[:128]], angles, plan, tol=1e-3, exact_reference=False)
        res = simus_with_surrogate(sur, scat[sub], rc[sub], angles, plan, tol=1e-3)
        ex_full = BatchedSimus([(scat, rc)], delays, p, m, plans=[plan], backend="fp32")
        ex_full.run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ex_full.run()
        torch.cuda.synchronize()
        t_exact_full = time.perf_counter() - t0
        scale = scat.shape[0] / args.sur_sample
        t_sur_full = res["t_surrogate_total_s"] * scale
        frames = len(angles)
        terms = scat.shape[0] * p.n_elements * plan.n_sub * plan.selected_freqs.shape[0] * frames
        return {"surrogate_s_scaled": t_sur_full, "exact_fp32_batched_s": t_exact_full,
                "gain_vs_exact": t_exact_full / t_sur_full, "frames_per_s_surrogate": frames / t_sur_full,
                "frames_per_s_exact": frames / t_exact_full,
                "green_terms_per_s_surrogate": terms / t_sur_full, "green_terms_per_s_exact": terms / t_exact_full,
                "fallback_fraction": res["fallback_fraction"], "network_query_share": res["network_query_share"],
                "units_in_domain": res["units_in_domain"], "units_failed_check": res["units_failed_check"],
                "unit_rel_err_median": res["unit_rel_err_median"], "unit_rel_err_max": res["unit_rel_err_max"],
                "rf_rel_l2_vs_exact": res["rf_rel_l2_vs_exact"],
                "sample_scatterers": args.sur_sample,
                "breakdown_sample_s": {k: res[k] for k in ("t_network_s", "t_exact_outside_domain_s",
                                                           "t_check_fallback_s", "t_rx_s")}}

    full_s, full_rc = W.cfg4_scatterers(1_000_000, seed=1)
    cfg5 = simus_case(full_s, full_rc, np.linspace(-16.0, 16.0, 75))
    line = {
        "metric": "RF frames/s & Green terms/s: surrogate (exact fallback at 1e-3) vs exact FP32 path",
        "value": cfg5["frames_per_s_surrogate"], "unit": "frames/s", "n_gpus": 1, "higher_is_better": True,
        "dtype": "bf16 weights, bf16 hi/lo activations, f32 accumulate (tcgen05 training and inference); "
                 "f32 exact fallback",
        "data": "synthetic (seeded)",
        "config": {"workload": "cfg5: cfg1 probe; train on 2M samples (x, z, f, theta) over the cfg1 box "
                               "x [-10, 10] mm, z [5, 30] mm, |theta| <= 16 deg, f in fc(1 +- B/2); use 1,000,000 "
                               "scatterers x 75 plane waves at [-16, 16] deg",
                   "train_samples": args.sur_train, "steps": rep["steps"], "batch": rep["batch"],
                   "carriers": "plane wave, 2 aperture-edge waves, 2 grating lobes"},
        "training": {k: rep[k] for k in ("train_s", "data_s", "steps", "batch", "ms_per_step", "samples_per_s",
                                         "algorithmic_tflops", "val_rel_l2")},
        "field_rel_l2_1M_queries": val_rel,
        "per_query_s": {"network": t_net_q, "exact_kernel": t_exact_q, "ratio_network_over_exact": t_net_q / t_exact_q,
                        "network_tc_status": sur.tc_status()},
        "simus_1M_x75": cfg5,
        "clocks": clocks.summary(),
    }
    line["training"]["history"] = rep["history"]
    line["roofline"] = {"kernel": "mlp_train (fb + dw + adam per step)", "bound": "tensor",
                        "achieved": rep["algorithmic_tflops"], "peak": bf16_peak, "unit": "TFLOP/s",
                        "frac": rep["algorithmic_tflops"] / bf16_peak,
                        "count": f"3 x {mlp_flops_per_sample(sur.n_out):.0f} flops per training sample (forward, "
                                 "input and weight gradients; the hi/lo split of the forward activations counted once)",
                        "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (training is a long loop)"
                        if "bf16_tflops_sustained" in peaks else "fallback"}
    return line


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-scatterers", type=int, default=50_000, help="CPU baseline sample (25%% of the frame)")
    ap.add_argument("--cpu-points", type=int, default=32_768, help="CPU baseline grid sample (25%% of the grid)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="device timing only (profiling runs)")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip the reference CUDA kernel leg of the default line")
    ap.add_argument("--no-paths", action="store_true", help="skip the batched / tensor-core / surrogate summaries")
    ap.add_argument("--scatterers", type=int, default=200_000, help="smaller values make profiling cases")
    ap.add_argument("--grid-nx", type=int, default=256)
    ap.add_argument("--grid-nz", type=int, default=512)
    ap.add_argument("--workload", choices=["cfg2", "cfg3", "cfg4", "cfg5", "das"], default="cfg2",
                    help="cfg2: plain simus + pfield frame (default); cfg3: batched 75 waves x 16 phantoms; "
                         "cfg4: tensor-core path vs FP32 paths, 31 waves x 262,144 scatterers; cfg5: surrogate; "
                         "das: rf2iq + delay-and-sum of 75 cfg3 firings")
    ap.add_argument("--tc-oracle-scatterers", type=int, default=16384)
    ap.add_argument("--tc-only", action="store_true", help="cfg4 profiling case: only the tensor-core sweep")
    ap.add_argument("--sur-train", type=int, default=2_000_000)
    ap.add_argument("--sur-steps", type=int, default=60_000)
    ap.add_argument("--sur-sample", type=int, default=1024)
    ap.add_argument("--phantoms", type=int, default=16)
    ap.add_argument("--transmits", type=int, default=75)
    args = ap.parse_args()
    rank, world = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1)
    if args.impl == "reference":
        run_reference_arm(args, rank, world)
    elif args.workload == "cfg3":
        print(json.dumps(run_batched_workload(args)), flush=True)
    elif args.workload == "cfg4":
        print(json.dumps(run_tc_workload(args)), flush=True)
    elif args.workload == "cfg5":
        print(json.dumps(run_surrogate_workload(args)), flush=True)
    elif args.workload == "das":
        print(json.dumps(run_beamform_workload(args)), flush=True)
    else:
        run_gpu_arm(args, rank, world)


if __name__ == "__main__":
    main()
