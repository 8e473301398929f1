#!/usr/bin/env python
"""Benchmark: fused FP64 sequential trace of the 12-surface TMA + corrector
system (16M rays, 6 wavelengths) on one GB300, in ray-surface ops/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

One step = one out-of-place trace of the whole ray batch (inputs resident in
HBM, 1.2 GB > L2, so no L2 flush is needed).  Prints one JSON line (rank 0).
Under torchrun each rank traces its own batch (weak scaling, no collective
on the data path); the reported time is the max over ranks.

``--impl reference`` times the reference algorithm on the host cores instead:
the oracle's C restatement of the reference trace (oracle/), all threads, on a
bounded sample of the same workload.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ray-surface ops/s (FP64 trace)"
UNIT = "ray-surface/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="tma_corrector")
    p.add_argument("--nrays", type=int, default=16 * 1024 * 1024)
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-huygens", action="store_true")
    p.add_argument("--no-paraboloid", action="store_true")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--batch-states", type=int, default=4096)
    p.add_argument("--no-surrogate", action="store_true")
    p.add_argument("--no-guard", action="store_true", help="surrogate without the vignetting guard")
    p.add_argument("--surrogate-samples", type=int, default=2_000_000)
    p.add_argument("--surrogate-epochs", type=int, default=24)
    p.add_argument("--per-stage", type=int, default=None, metavar="REPS",
                   help="instead of the bench line: the workload's optic truncated after each interface, one "
                        "untimed launch each, then REPS timed ones (0: the single launch only, for an ncu census "
                        "of one launch per truncation); prints one JSON line of per-interface times")
    return p.parse_args()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def reduce_step_time(ms, world, device):
    """Timed region of the whole job: the max over ranks (every rank must
    call it; identity for one rank)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world, per_unit, steps, ms):
    """Whole-job rate: the units all ranks processed over the job's time
    (weak scaling: every rank traces its own batch)."""
    return units_per_rank * world * per_unit * steps / (ms * 1e-3)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 9]
        sm = [float(r[1]) for r in rows if r[1].replace('.', '', 1).isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace('.', '', 1).isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def _oracle():
    """The oracle (C restatement of the reference trace) and its own optic
    builder: the CPU legs never load the product package or its library."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as ora
    import optics as OO
    return ora, OO


def cpu_workload(workload):
    ora, OO = _oracle()
    build_optic, make_rays, nsurf = OO.workloads().WORKLOADS[workload]
    return ora, build_optic(OO), make_rays, nsurf


def time_cpu(workload, nrays, threads=None):
    ora, opt, make_rays, nsurf = cpu_workload(workload)
    threads = threads or ora.threads()
    rays = ora.Rays(*make_rays(nrays, seed=1000))
    t1 = time.perf_counter()
    ora.trace(opt, rays, nthreads=threads)
    dt = time.perf_counter() - t1
    return nrays * nsurf / dt, dt, threads


def cpu_baseline(workload, target_s=12.0):
    """Bounded CPU sample: grow the ray count until one trace takes ~1 s,
    then repeat to ~target_s of CPU work; report the median throughput."""
    n = 1 << 16
    rate, dt, threads = time_cpu(workload, n)
    while dt < 1.0 and n < (1 << 23):
        n *= 2
        rate, dt, threads = time_cpu(workload, n)
    rates = [rate]
    spent = dt
    while spent < target_s:
        r, d, _ = time_cpu(workload, n, threads)
        rates.append(r)
        spent += d
    # one thread, on a sample of about 2 s
    n1 = max(1 << 12, int(n * 2.0 / (dt * threads)))
    r1, d1, _ = time_cpu(workload, n1, 1)
    return {"value": statistics.median(rates), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{workload}: {n} rays x {len(rates)} repeats ({spent:.1f} s of CPU trace), "
                      f"oracle C restatement of the reference trace, OpenMP {threads} threads",
            "one_thread": {"value": r1, "unit": UNIT, "cores": 1, "sample": f"{n1} rays, {d1:.1f} s"}}


def run_reference(args):
    """The reference's trace algorithm on the host cores (the oracle's C
    restatement, OpenMP over all threads) on the same configuration as the
    GPU arm: the full ray batch of each rank-0 step, same seeds, traced in
    place from a fresh copy of the inputs (copy outside the timed region)."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    ora, opt, make_rays, nsurf = cpu_workload(args.workload)
    threads = ora.threads()
    n = args.nrays
    pristine = ora.Rays(*make_rays(n, seed=4242))
    rays = pristine.copy()
    total = 0.0
    for it in range(args.warmup + args.steps):
        np.copyto(rays.d, pristine.d)
        np.copyto(rays.b, pristine.b)
        rays.origin, rays.rot = pristine.origin.copy(), pristine.rot.copy()
        t1 = time.perf_counter()
        ora.trace(opt, rays, nthreads=threads)
        dt = time.perf_counter() - t1
        if it >= args.warmup:
            total += dt
    value = n * nsurf * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.workload}: {nsurf}-surface trace of {n} rays per step (seed 4242, as "
                               "the GPU arm's rank 0), 6 wavelengths 350-1000 nm, Sellmeier silica",
                   "rays_per_step": n, "surfaces": nsurf, "l2": "host arrays, 1.2 GB per step"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"the full {n}-ray batch per step, oracle C restatement of the reference "
                                   f"trace, OpenMP {threads} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def load_counters(key):
    """Per-unit counters of one kernel on one workload from the committed ncu
    summaries (profiles/kernel_counters.json): DRAM bytes and executed FP64
    instructions per ray, measured on a case larger than L2."""
    path = os.path.join(ROOT, "profiles", "kernel_counters.json")
    try:
        with open(path) as f:
            return json.load(f).get(key)
    except (OSError, ValueError):
        return None


def executed_fp64_flops(c):
    """Executed FP64 flops per unit from an ncu census: DADD + DMUL + 2 DFMA."""
    if not c or "fp64_dfma_per_ray" not in c:
        return None
    return c["fp64_dadd_per_ray"] + c["fp64_dmul_per_ray"] + 2 * c["fp64_dfma_per_ray"]


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def host_trace_e2e(L, _lib, prog, arrs, n, niter, steps, sp, chunk=1 << 19):
    """The trace through the C-ABI host-buffer entry point (bt_optic_trace_host):
    pinned host arrays in, results back in them; host clock around each call
    (inputs restored between calls, outside the clock).  Returns (median ms
    per call, h2d bytes, d2h bytes)."""
    import torch
    host = [torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).pin_memory() for x in arrs[:9]]
    hflags = [torch.from_numpy(np.ascontiguousarray(x, dtype=np.uint8)).pin_memory() for x in arrs[9:]]
    pristine = [h.clone() for h in host] + [f.clone() for f in hflags]
    hrv = _lib.BtRayVector(*[h.data_ptr() for h in host], *[f.data_ptr() for f in hflags], n)
    times = []
    for it in range(1 + steps):
        for dst, src in zip(host + hflags, pristine):
            dst.copy_(src)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        _lib.check(L.bt_optic_trace_host(prog._optic.ptr, ctypes.byref(hrv), niter, chunk, sp))
        dt = (time.perf_counter() - t1) * 1e3
        if it > 0:
            times.append(dt)
    return (statistics.median(times) if times else 0.0), n * (9 * 8 + 2), n * (8 * 8 + 2)


def bench_paraboloid(bt, fp64_peak, n=1_000_000, reps=20, cpu=True):
    """The f/4 paraboloid mirror onto a flat detector, 1e6 rays (2 surfaces):
    device-timed out-of-place trace with L2 flushed between steps (the
    148 MB of rays are about L2's size), e2e through the host-buffer entry
    point, and the oracle on the host cores on the same 1e6 rays."""
    import torch
    from batoid_gb300 import _lib, _device as D, workloads as W, workcount as WC
    opt = W.paraboloid_optic(bt)
    arrs = W.paraboloid_rays(n, seed=57721)
    rv_in = bt.RayVector(*arrs)
    rv_out = bt.RayVector._empty(n)
    prog = opt._program(rv_in.coordSys)
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    niter = bt.global_vars._batoid_niter
    a, b = rv_in._rv, rv_out._rv
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=D.device())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    times = []
    for it in range(3 + reps):
        flush.fill_(it & 0xff)
        e0.record(stream)
        _lib.check(L.bt_optic_trace_into(prog._optic.ptr, a, b, niter, sp))
        e1.record(stream)
        torch.cuda.synchronize()
        if it >= 3:
            times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    nsurf = 2
    bpr = WC.READ_BYTES_PER_RAY + WC.WRITE_BYTES_PER_RAY
    gbs = bpr * n / (ms * 1e-3) / 1e9
    hbm_peak = measured_peaks().get("hbm_gbs", 6800.0)
    c = load_counters("k_trace_ff/paraboloid")
    out = {"workload": f"paraboloid: f/4 mirror (R 8 m, annulus 0.2-0.5 m) + flat detector, {n} rays, "
                       "field +-0.5 deg, 500 nm, vacuum",
           "value": n * nsurf / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms, "steps": reps,
           "l2": "flushed between steps (256 MB write)",
           "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                        "bytes_per_ray": bpr, "peak_source": "MEASURED_PEAKS.json hbm_gbs",
                        "traffic": (c["dram_bytes_per_ray"] * n if c else None)}}
    if c and "warp_inst_per_ray" in c:
        sms = ctypes.c_int(0)
        _lib.check(L.bt_device_sm_count(ctypes.byref(sms)))
        peak = 4 * sms.value * 2.07
        ach = c["warp_inst_per_ray"] * n / (ms * 1e-3) / 1e9
        out["issue"] = {"achieved": ach, "peak": peak, "unit": "G warp-instructions/s", "frac": ach / peak,
                        "peak_source": f"4 schedulers x {sms.value} SMs x 2.07 GHz"}
    fpr = executed_fp64_flops(c)
    if fpr and fp64_peak:
        ach = fpr * n / (ms * 1e-3) / 1e12
        out["fp64"] = {"executed_flops_per_ray": fpr, "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                       "frac": ach / fp64_peak}
    e2e_ms, h2d, d2h = host_trace_e2e(L, _lib, prog, arrs, n, niter, 5, sp, chunk=1 << 18)
    out["e2e"] = {"value": n * nsurf / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                  "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                  "path": "bt_optic_trace_host, pinned host arrays, 256k-ray chunks on 3 streams"}
    if cpu:
        ora, copt, make_rays, _ = cpu_workload("paraboloid")
        pristine = ora.Rays(*make_rays(n, seed=57721))
        rates = []
        spent = 0.0
        while spent < 5.0 or len(rates) < 3:
            rays = pristine.copy()
            t1 = time.perf_counter()
            ora.trace(copt, rays)
            d = time.perf_counter() - t1
            spent += d
            rates.append(n * nsurf / d)
        out["cpu_baseline"] = {"value": statistics.median(rates), "unit": UNIT, "cores": ora.threads(),
                               "kind": "port", "sample": f"the full {n}-ray batch x {len(rates)} repeats, "
                                                          "oracle C restatement of the reference trace"}
        out["speedup_vs_cpu"] = out["value"] / out["cpu_baseline"]["value"]
        out["e2e_speedup_vs_cpu"] = out["e2e"]["value"] / out["cpu_baseline"]["value"]
    return out


HUYGENS_FIELDS = [(fx, fy) for fy in (-1.2, 0.0, 1.2) for fx in (-1.2, 0.0, 1.2)]  # degrees


def bench_huygens(bt, opt, nx=256, npix=128, pitch=2e-6, wavelength=620e-9, check_pixels=48, cpu=True,
                  fp32_peak=None, reps=5):
    """Huygens PSF of the 12-surface system: 9 field points (3x3 grid over
    +-1.2 deg), 256x256 pupil grid each, 128x128 pixels at 2 um around each
    field's chief ray.  Device-timed: one trace launch for all fields, and
    one launch set of the phasor sums for all fields
    (bt_huygens_amplitudes_fields).  Error: PSF on sampled pixels vs the
    FP64 per-pixel sum (device sumAmplitude kernel, the reference's
    algorithm), relative to each field's PSF peak."""
    import torch
    from batoid_gb300 import _lib, _device as D, analysis as A
    from batoid_gb300.rayVector import concatenateRayVectors
    L = _lib.lib()
    F = len(HUYGENS_FIELDS)
    thx = np.deg2rad([f[0] for f in HUYGENS_FIELDS])
    thy = np.deg2rad([f[1] for f in HUYGENS_FIELDS])
    n = nx * nx
    rays = concatenateRayVectors([bt.RayVector.asGrid(optic=opt, wavelength=wavelength, theta_x=thx[f],
                                                      theta_y=thy[f], nx=nx) for f in range(F)])
    stream = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    opt.trace(rays)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_trace = e0.elapsed_time(e1)
    cidx = (nx // 2) * nx + nx // 2
    pts = np.ascontiguousarray([[rays.x[f * n + cidx], rays.y[f * n + cidx], 0.0] for f in range(F)])
    t0 = np.ascontiguousarray([float(rays.t[f * n]) for f in range(F)])
    lat = np.ascontiguousarray(np.tile([pitch, 0.0, 0.0, pitch], (F, 1)))
    re = D.empty(F * npix * npix)
    im = D.empty(F * npix * npix)
    dp = _lib.c_double_p

    def sums():
        _lib.check(L.bt_huygens_amplitudes_fields(rays._rv, F, pts.ctypes.data_as(dp), lat.ctypes.data_as(dp),
                                                  t0.ctypes.data_as(dp), npix, npix, 1, D.ptr(re), D.ptr(im),
                                                  D.stream_ptr()))

    sums()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        sums()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_psf = e0.elapsed_time(e1) / reps
    psf = (D.to_host(re) ** 2 + D.to_host(im) ** 2).reshape(F, npix, npix)
    valid = (~rays.failed & ~rays.vignetted)
    pairs_valid = int(valid.sum()) * npix * npix
    pairs = F * n * npix * npix  # the kernel sums every grid ray (excluded ones with zero weight)
    rng = np.random.default_rng(5)
    max_err = 0.0
    for f in range(F):
        view = bt.RayVector._fromBuffers(rays._d[:, f * n:(f + 1) * n], rays._b[:, f * n:(f + 1) * n],
                                         rays.coordSys)
        peak = psf[f].max()
        for a, b in rng.integers(0, npix, (check_pixels // 4, 2)):
            P = (pts[f][0] + (b - npix // 2) * pitch, pts[f][1] + (a - npix // 2) * pitch, 0.0)
            ref = view.sumAmplitude(P, t0[f])
            max_err = max(max_err, abs(abs(ref) ** 2 - psf[f, a, b]) / peak)
    # through the public API: one huygensPSFs call vs nine huygensPSF calls
    # (host clock around ray generation, trace, sums and the copy back)
    A.huygensPSFs(opt, thx, thy, wavelength, nx=nx, dx=pitch, nxOut=npix)  # warm-up
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    multi = A.huygensPSFs(opt, thx, thy, wavelength, nx=nx, dx=pitch, nxOut=npix)
    ms_multi = (time.perf_counter() - t1) * 1e3
    A.huygensPSF(opt, thx[0], thy[0], wavelength, nx=nx, dx=pitch, nxOut=npix)  # warm-up
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    single = [A.huygensPSF(opt, thx[f], thy[f], wavelength, nx=nx, dx=pitch, nxOut=npix) for f in range(F)]
    ms_per_field_api = (time.perf_counter() - t1) * 1e3
    out = {
        "workload": f"{F} fields x {nx}x{nx} pupil rays x {npix}x{npix} px at {pitch*1e6:.0f} um, "
                    f"{wavelength*1e9:.0f} nm, tma_corrector",
        "fields_per_s": F / ((ms_trace + ms_psf) * 1e-3),
        "ray_pixel_pairs_per_s": pairs / (ms_psf * 1e-3),
        "valid_ray_pixel_pairs_per_s": pairs_valid / (ms_psf * 1e-3),
        "ms_trace": ms_trace, "ms_psf": ms_psf, "ms_total": ms_trace + ms_psf,
        "gpu_launches": {"trace": 1, "psf": 3},
        "psf_max_err_rel_peak": max_err,
        "err_reference": "FP64 per-pixel phasor sum (bt_rv_sum_amplitude) on sampled pixels of every field",
        "api_wall_ms": {"huygensPSF_per_field": ms_per_field_api, "huygensPSFs_one_call": ms_multi},
        "fields_per_s_one_call": F / (ms_multi * 1e-3),
        "one_call_vs_per_field_max_abs_diff": max(float(np.abs(m.array - o.array).max()) for m, o in zip(multi, single)),
    }
    if fp32_peak:
        ach = 10.0 * pairs / (ms_psf * 1e-3) / 1e12
        out["roofline"] = {"bound": "fp32", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s",
                           "frac": ach / fp32_peak, "flops_per_pair": 10,
                           "peak_source": "FFMA loop measured in this run (bt_measure_fp32_peak)",
                           "note": "prep + phasor sums + reduce of all fields over their event time"}
    if cpu:
        # oracle (C, all threads): per-pixel sumAmplitude on a pixel sample, extrapolated
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as ora
        f = 4
        sl = slice(f * n, (f + 1) * n)
        host = ora.Rays(*[getattr(rays, k)[sl] for k in ora.Rays.FIELDS], rays.vignetted[sl], rays.failed[sl])
        npx = 64
        t1 = time.perf_counter()
        for k in range(npx):
            ora.sum_amplitude(host, (pts[f][0] + k * pitch, pts[f][1], 0.0), t0[f])
        per_px = (time.perf_counter() - t1) / npx
        out["cpu_baseline"] = {"s_per_pixel": per_px, "cores": ora.threads(), "kind": "port",
                               "extrapolated_s_total": per_px * npix * npix * F,
                               "sample": f"{npx} pixels of one field, oracle sumAmplitude (reference algorithm)"}
        out["speedup_vs_cpu"] = out["cpu_baseline"]["extrapolated_s_total"] / (ms_psf * 1e-3)
    return out


BATCH_FIELDS = [(fx, fy) for fy in (-1.2, 0.0, 1.2) for fx in (-1.2, 0.0, 1.2)]


def batch_states(pt, nstates, seed=31337):
    """Seeded perturbed states: M2 and camera shifts U(+-1 mm) and tilts
    U(+-10 arcsec), 20 bending amplitudes N(0, 100 nm); pupil grids
    U{32..128}; wavelengths from the six 350-1000 nm values."""
    rng = np.random.default_rng(seed)
    tilt = np.deg2rad(10.0 / 3600.0)
    rigid = rng.uniform(-1.0, 1.0, (nstates, 10)) * np.tile([1e-3, 1e-3, 1e-3, tilt, tilt], 2)
    bend = rng.normal(0.0, 100e-9, (nstates, pt.nmodes))
    nx = rng.integers(32, 129, nstates)
    wl = np.linspace(350e-9, 1000e-9, 6)[rng.integers(0, 6, nstates)]
    return np.concatenate([rigid, bend], axis=1), nx, wl


def bench_batched(bt, nstates=4096, reps=3, cpu=True, fp64_peak_tflops=None):
    """Batched wavefronts: 4096 perturbed states x 9 fields, Zernike fit
    (jmax 28, annular) per (state, field), one persistent graph-captured
    launch per batch.  Device-timed with the states' tables resident; e2e
    from host dofs through PerturbedTelescope.zernike."""
    import torch
    from batoid_gb300 import _device as D, workloads as W
    from batoid_gb300.autotune import batch_config
    from batoid_gb300.batch import PerturbedTelescope
    from batoid_gb300.modes import ModeSet
    optic = W.tma_optic(bt)
    modes = ModeSet(nmodes=20, n=512)
    pt = PerturbedTelescope(optic, modes=modes, fields=np.deg2rad(BATCH_FIELDS), jmax=28)
    dofs, nx, wl = batch_states(pt, nstates)
    pt.prepare(np.arange(32, 129))
    threads, ctas = batch_config(pt)
    inp = pt.device_inputs(dofs, nx, wl)
    F, J = len(BATCH_FIELDS), pt.jmax
    coefs = torch.empty(nstates * F * (J + 1), dtype=torch.float64, device=D.device())
    status = torch.empty(nstates * F, dtype=torch.int32, device=D.device())
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        # capture + first replay, marked for profilers (ncu --nvtx-include "batched_wavefronts/")
        torch.cuda.nvtx.range_push("batched_wavefronts")
        pt.launch(inp, coefs, status, threads, ctas, graph=True)
        torch.cuda.nvtx.range_pop()
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            pt.launch(inp, coefs, status, threads, ctas, graph=True)
        e1.record(stream)
        stream.synchronize()
    ms = e0.elapsed_time(e1) / reps
    st = D.to_host(status)
    rays = int(np.sum(nx.astype(np.int64) ** 2)) * F
    stages = pt.prog.nstages + 1
    jobs = nstates * F
    # end to end: host dofs -> tables -> device -> kernel -> coefficients on the host
    t1 = time.perf_counter()
    host = pt.zernike(dofs, nx, wl, threads=threads, ctas_per_sm=ctas)
    e2e_s = time.perf_counter() - t1
    out = {
        "workload": f"{nstates} states x {F} fields, pupil grids 32-128 (seeded), jmax 28 annular fit, "
                    "M2/camera rigid dofs + 20 bending modes (512x512 bicubic), tma_corrector",
        "wavefronts_per_s": jobs / (ms * 1e-3),
        "ray_surface_per_s": rays * stages / (ms * 1e-3),
        "ms_per_batch": ms, "rays_per_batch": rays, "jobs": jobs,
        "launch": {"threads": threads, "ctas_per_sm": ctas, "graph": True, "kernels_per_batch": 1},
        "failed_fits": int(np.sum(st != 0)),
        "e2e": {"wavefronts_per_s": jobs / e2e_s, "s_per_batch": e2e_s,
                "h2d_bytes": int(sum(t.numel() * t.element_size() for k, t in inp.items() if k != "nstates")),
                "d2h_bytes": int(coefs.numel() * 8 + status.numel() * 4),
                "path": "PerturbedTelescope.zernike (host tables, copies, launch, copies back)"},
    }
    # issue roofline of the batched kernel from its ncu census (warp
    # instructions per pupil ray, fit included); executed FP64 flops and the
    # reference-flop count beside it
    c = load_counters("k_batch_zernike/tma_bending")
    roof = {"bound": "issue", "achieved": None, "peak": None, "unit": "G warp-instructions/s", "frac": None,
            "kernel": "k_batch_zernike"}
    if c and "warp_inst_per_ray" in c:
        from batoid_gb300 import _lib
        sms = ctypes.c_int(0)
        _lib.check(_lib.lib().bt_device_sm_count(ctypes.byref(sms)))
        peak = 4 * sms.value * 2.07
        ach = c["warp_inst_per_ray"] * rays / (ms * 1e-3) / 1e9
        roof.update({"achieved": ach, "peak": peak, "frac": ach / peak, "warp_inst_per_ray": c["warp_inst_per_ray"],
                     "peak_source": f"4 schedulers x {sms.value} SMs x 2.07 GHz",
                     "traffic": c.get("dram_bytes_per_ray", 0.0) * rays})
    if fp64_peak_tflops:
        from batoid_gb300 import workcount as WC
        fpr = WC.wavefront_flops_per_ray(pt.perturbed(dofs[0]), J)
        ach = fpr * rays / (ms * 1e-3) / 1e12
        efpr = executed_fp64_flops(c)
        if efpr:
            each = efpr * rays / (ms * 1e-3) / 1e12
            roof["fp64"] = {"executed_flops_per_ray": efpr, "achieved": each, "peak": fp64_peak_tflops,
                            "unit": "TFLOP/s", "frac": each / fp64_peak_tflops,
                            "peak_source": "DFMA loop measured in this run (bt_measure_fp64_peak)"}
        roof["reference_flops"] = {"flops_per_ray": fpr, "tflops": ach, "ratio_to_peak": ach / fp64_peak_tflops,
                                   "convention": "FP64 operations of the reference's own expressions "
                                                 "(workcount.wavefront_flops_per_ray); not executed as such"}
    out["roofline"] = roof
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import wavefront as owf
        from batoid_gb300.utils import fieldToDirCos
        sample = [(s, s % F) for s in range(0, nstates, max(1, nstates // 6))][:6]
        srays = 0
        maxdiff = 0.0
        t1 = time.perf_counter()
        for s, f in sample:
            c = owf.zernike(pt.perturbed(dofs[s]), fieldToDirCos(*np.deg2rad(BATCH_FIELDS[f])), wl[s], int(nx[s]),
                            J, pt.eps)
            srays += int(nx[s]) ** 2
            maxdiff = max(maxdiff, float(np.max(np.abs(c - host[s, f])) * wl[s]))
        dt = time.perf_counter() - t1
        import oracle as ora
        out["cpu_baseline"] = {"s_per_ray": dt / srays, "cores": ora.threads(), "kind": "port",
                               "extrapolated_s_per_batch": dt / srays * rays,
                               "sample": f"{len(sample)} (state, field) jobs, oracle trace + numpy lstsq "
                                         "(reference wavefront/zernike algorithm)"}
        out["speedup_vs_cpu"] = out["cpu_baseline"]["extrapolated_s_per_batch"] / (ms * 1e-3)
        out["max_coef_diff_m_vs_oracle"] = maxdiff
    return out


def bench_surrogate(bt, train_samples=2_000_000, heldout_states=7282, epochs=24, threshold_nm=2.0, cpu=True,
                    guard_on=True):
    """Learned surrogate: MLP 33 -> 4 x 512 GELU -> 28 (+ error head), BF16
    tensor-core kernels with FP32 accumulation, trained on batched-trace
    data (nx 32 pupil grids, 9 fields, 6 wavelengths); evaluated on held-out
    states against the batched trace, with fallback to the trace above
    threshold_nm of calibrated predicted RMS wavefront error."""
    import torch
    from batoid_gb300 import _device as D, workloads as W
    from batoid_gb300.autotune import batch_config
    from batoid_gb300.batch import PerturbedTelescope
    from batoid_gb300.modes import ModeSet
    from batoid_gb300.surrogate import WavefrontSurrogate, rms_nm
    optic = W.tma_optic(bt)
    pt = PerturbedTelescope(optic, modes=ModeSet(nmodes=20, n=512), fields=np.deg2rad(BATCH_FIELDS), jmax=28)
    sur = WavefrontSurrogate(pt, W.WAVELENGTHS, nx=32)
    pt.prepare([32])
    threads, ctas = batch_config(pt)
    F = len(BATCH_FIELDS)
    t1 = time.perf_counter()
    dofs, widx = sur.sample_states((train_samples + F - 1) // F, seed=101)
    coefs = sur.trace(dofs, widx, threads=threads, ctas_per_sm=ctas)
    datagen_s = time.perf_counter() - t1
    feat, grp, w = sur.features(dofs, widx)
    t1 = time.perf_counter()
    sur.train(feat, grp, w, coefs, epochs=epochs, batch=8192, lr=1e-3)
    train_s = time.perf_counter() - t1
    steps = epochs * (len(feat) // 8192)
    t1 = time.perf_counter()
    guard = sur.build_guard() if guard_on else None
    guard_s = time.perf_counter() - t1
    vd, vw = sur.sample_states(4096, seed=202)
    vc = sur.trace(vd, vw, threads=threads, ctas_per_sm=ctas)
    vf, vg, vwl = sur.features(vd, vw)
    kappa = sur.calibrate(vf, vg, vwl, vc)
    # held-out: the batched trace (device-resident inputs, graph replay) is the ground truth and the baseline
    hd, hw = sur.sample_states(heldout_states, seed=303)
    inp = pt.device_inputs(hd, 32, W.WAVELENGTHS[hw])
    N = heldout_states * F
    tc = torch.empty(N * 29, dtype=torch.float64, device=D.device())
    ts = torch.empty(N, dtype=torch.int32, device=D.device())
    stream = torch.cuda.Stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        pt.launch(inp, tc, ts, threads, ctas, graph=True)
        stream.synchronize()
        e0.record(stream)
        for _ in range(3):
            pt.launch(inp, tc, ts, threads, ctas, graph=True)
        e1.record(stream)
        stream.synchronize()
    trace_ms = e0.elapsed_time(e1) / 3
    truth = D.to_host(tc).reshape(N, 29)
    hf, hg, hwl = sur.features(hd, hw)
    feat_d = torch.from_numpy(hf).to(D.device())
    grp_d = torch.from_numpy(hg).to(D.device())
    w_d = D.to_device(hwl)
    out = torch.empty((N, 29), dtype=torch.float64, device=D.device())
    err = torch.empty(N, dtype=torch.float32, device=D.device())
    gflag = torch.zeros(N, dtype=torch.int32, device=D.device())

    def infer():
        sur.predict_device(feat_d, grp_d, w_d, out, err)
        if guard is not None:
            guard.flags_device(feat_d, grp_d, gflag)

    with torch.cuda.stream(stream):
        # untimed first pass, marked for profilers (ncu --nvtx-include "surrogate_inference/")
        torch.cuda.nvtx.range_push("surrogate_inference")
        infer()
        torch.cuda.nvtx.range_pop()
        stream.synchronize()
        e0.record(stream)
        for _ in range(10):
            infer()
        e1.record(stream)
        stream.synchronize()
    infer_ms = e0.elapsed_time(e1) / 10
    pred = D.to_host(out)
    perr = D.to_host(err) * kappa
    gfl = D.to_host(gflag).astype(bool)
    fb = (perr > threshold_nm) | gfl
    jobs = np.flatnonzero(fb)
    fb_ms = 0.0
    if len(jobs):
        order = torch.from_numpy(jobs.astype(np.int32)).to(D.device())
        fc = torch.empty(N * 29, dtype=torch.float64, device=D.device())
        with torch.cuda.stream(stream):
            e0.record(stream)
            pt.launch(inp, fc, ts, threads, ctas, order=order)
            e1.record(stream)
            stream.synchronize()
        fb_ms = e0.elapsed_time(e1)
        pred[fb] = D.to_host(fc).reshape(N, 29)[fb]
    lin = np.concatenate([np.zeros((N, 1)), sur.linear(hf, hg)], axis=1)
    e_lin = rms_nm(lin, truth, hwl)
    raw, _ = sur.predict(hf, hg, hwl)
    e_raw = rms_nm(raw, truth, hwl)
    e_fin = rms_nm(pred, truth, hwl)

    def stats(e):
        return {"mean_nm": float(np.mean(e)), "p50_nm": float(np.median(e)), "p99_nm": float(np.quantile(e, 0.99)),
                "max_nm": float(np.max(e)), "frac_above_threshold": float(np.mean(e > threshold_nm))}

    # the largest surrogate errors: is the batched truth right there?  Recompute
    # those samples with the CPU oracle of batoid.zernike
    worst = np.argsort(-e_raw)[:4]
    above = np.flatnonzero(e_fin > threshold_nm)
    zmax = np.max(np.abs(hd / sur.dof_scale), axis=1)
    tail_profile = {"count": int(len(above)),
                    "fields": np.bincount(above % F, minlength=F).tolist(),
                    "wavelength_nm": np.bincount(hw[above // F], minlength=len(W.WAVELENGTHS)).tolist(),
                    "median_max_abs_dof_z": float(np.median(zmax[above // F])) if len(above) else None,
                    "median_max_abs_dof_z_all": float(np.median(zmax)),
                    "distinct_states": int(len(np.unique(above // F)))}
    outliers = []
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import wavefront as owf
        from batoid_gb300.utils import fieldToDirCos
        for n in worst:
            s_, f_ = divmod(int(n), F)
            c = owf.zernike(pt.perturbed(hd[s_]), fieldToDirCos(*np.deg2rad(BATCH_FIELDS[f_])), hwl[n], 32, 28, pt.eps)
            outliers.append({"sample": int(n), "surrogate_err_nm": float(e_raw[n]), "linear_err_nm": float(e_lin[n]),
                             "batched_vs_oracle_m": float(np.max(np.abs(c - truth[n])) * hwl[n]),
                             "dofs_max_abs_normalised": float(np.max(np.abs(hd[s_] / sur.dof_scale)))})
    except Exception as exc:  # diagnostic only
        outliers.append({"error": repr(exc)})
    flops_fwd = 2.0 * (33 * 512 + 3 * 512 * 512 + 512 * 28)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    bf16_sus = peaks.get("bf16_tflops_sustained", 1700.0)
    train_tflops = 3 * flops_fwd * sur.timing["samples"] / sur.timing["network_s"] / 1e12
    infer_tflops = flops_fwd * N / (infer_ms * 1e-3) / 1e12
    out_d = {
        "workload": f"MLP 33 -> 4x512 GELU -> 28 + error head, bf16/fp32-accumulate tcgen05 kernels; trained on "
                    f"{len(feat)} (state, field) samples of the 4096-state generator (nx 32), evaluated on "
                    f"{N} held-out samples vs the batched trace",
        "wavefronts_per_s_with_fallback": N / ((infer_ms + fb_ms) * 1e-3),
        "wavefronts_per_s_surrogate_only": N / (infer_ms * 1e-3),
        "wavefronts_per_s_batched_trace": N / (trace_ms * 1e-3),
        "speedup_vs_batched_trace": trace_ms / (infer_ms + fb_ms),
        "fallback_fraction": float(np.mean(fb)), "threshold_nm": threshold_nm, "error_calibration_kappa": kappa,
        "rms_error_with_fallback": stats(e_fin), "rms_error_surrogate_only": stats(e_raw),
        "rms_error_linear_model_only": stats(e_lin),
        "ms": {"inference": infer_ms, "fallback_trace": fb_ms, "batched_trace": trace_ms, "datagen_s": datagen_s,
               "train_s": train_s},
        "training": {"steps": steps, "batch": 8192, "epochs": epochs,
                     "samples_per_s": sur.timing["samples"] / sur.timing["network_s"],
                     "network_s": sur.timing["network_s"], "linear_fit_s": sur.timing["linear_fit_s"],
                     "graph": True,
                     "note": "samples_per_s: network training steps (CUDA-graph replay of gather, forward, loss, "
                             "backward, Adam) over their synchronized wall time; the host least-squares fit of the "
                             "linear model is linear_fit_s"},
        "roofline_training": {"bound": "tensor", "achieved": train_tflops, "peak": bf16_sus, "unit": "TFLOP/s",
                              "frac": train_tflops / bf16_sus, "flops_per_sample": 3 * flops_fwd,
                              "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (seconds-long loop)",
                              "note": "3 x forward flops per sample (forward, data gradient, weight gradient)"},
        "roofline_inference": {"bound": "tensor", "achieved": infer_tflops, "peak": bf16_peak, "unit": "TFLOP/s",
                               "frac": infer_tflops / bf16_peak, "flops_per_sample": flops_fwd,
                               "note": "whole inference pipeline (pack, 5 GEMMs, combine) over its event time"},
        "gpu_launches_per_inference": 8 if guard is not None else 7,
        "vignetting_guard": None if guard is None else {
            "flagged_fraction": float(np.mean(gfl)), "fallback_by_error_head_only": float(np.mean(perr > threshold_nm)),
            "kept_margins_per_group_max": int(guard.nkept.max()),
            "pruned_margins": int(getattr(guard, "dropped", 0)),
            "kept_margins_per_group_mean": float(guard.nkept.mean()), "groups": int(guard.G), "build_s": guard_s,
            "flagged_and_above_threshold_raw": int(np.sum(gfl & (e_raw > threshold_nm))),
            "above_threshold_raw": int(np.sum(e_raw > threshold_nm)),
            "note": "first-order model of the aperture margins of the nx 32 grid rays (central differences of "
                    "traceFull on the nominal optic); a sample whose predicted margins may cross an aperture "
                    "edge falls back to the batched trace"},
        "largest_errors": outliers,
        "above_threshold_profile": tail_profile,
    }
    return out_d


def run_gpu(args):
    import torch
    import torch.distributed as dist
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import batoid_gb300 as bt
    from batoid_gb300 import _lib, _device as D, workloads as W, workcount as WC
    build_optic, make_rays, nsurf = W.WORKLOADS[args.workload]
    opt = build_optic(bt)
    n = args.nrays
    arrs = make_rays(n, seed=4242 + rank)
    rv_in = bt.RayVector(*arrs)
    rv_out = bt.RayVector._empty(n)
    prog = opt._program(rv_in.coordSys)
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    niter = bt.global_vars._batoid_niter
    a, b = rv_in._rv, rv_out._rv

    def step():
        _lib.check(L.bt_optic_trace_into(prog._optic.ptr, a, b, niter, sp))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    ms = reduce_step_time(ms, world, "cuda")
    ms_per_step = ms / args.steps
    total_rays = n * world
    value = job_throughput(n, world, nsurf, args.steps, ms)

    # sanity: the benchmark traced real rays
    vig = float(rv_out.field("vignetted").float().mean().item())

    # Roofline of the fused trace kernel (k_trace_ff, one launch per step).
    # It is bound by instruction issue (float-float arithmetic on the FP32 and
    # integer pipes; the FP64 pipe ~20 % busy): achieved = the warp
    # instructions it executes per ray (committed ncu census of the same
    # kernel and workload) x rays / step time, peak = 4 schedulers x SMs x
    # the SM clock sampled during the timed region.  The FP64 view (executed
    # DADD + DMUL + 2 DFMA vs the in-run DFMA probe) and the reference-flop
    # count are reported beside it.
    fpeak = ctypes.c_double(0.0)
    _lib.check(L.bt_measure_fp64_peak(1 << 14, ctypes.byref(fpeak), sp))
    ref_flops_per_ray = WC.optic_flops_per_ray(opt, niter)
    ref_tflops = ref_flops_per_ray * n / (ms_per_step * 1e-3) / 1e12
    counters = load_counters(f"k_trace_ff/{args.workload}")
    exec_fpr = executed_fp64_flops(counters)
    exec_tflops = exec_fpr * n / (ms_per_step * 1e-3) / 1e12 if exec_fpr else None
    sms = ctypes.c_int(0)
    _lib.check(L.bt_device_sm_count(ctypes.byref(sms)))
    sm_ghz = (clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0) / 1e3
    issue_peak = 4 * sms.value * sm_ghz  # G warp instructions / s
    issue_ach = (counters["warp_inst_per_ray"] * n / (ms_per_step * 1e-3) / 1e9
                 if counters and "warp_inst_per_ray" in counters else None)
    bytes_per_ray = WC.READ_BYTES_PER_RAY + WC.WRITE_BYTES_PER_RAY
    hbm_gbs = bytes_per_ray * n / (ms_per_step * 1e-3) / 1e9
    hbm_peak = measured_peaks().get("hbm_gbs", 6800.0)

    # end to end through the C-ABI with pinned host buffers
    e2e_ms, h2d, d2h = host_trace_e2e(L, _lib, prog, arrs, n, niter, args.e2e_steps, sp)
    e2e_value = total_rays * nsurf / (e2e_ms * 1e-3) if e2e_ms > 0 else None

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.workload)
    paraboloid = None
    if rank == 0 and not args.no_paraboloid:
        paraboloid = bench_paraboloid(bt, fpeak.value, cpu=not args.no_cpu_baseline)
    huygens = None
    if rank == 0 and not args.no_huygens:
        del rv_in, rv_out
        fp32 = ctypes.c_double(0.0)
        _lib.check(L.bt_measure_fp32_peak(1 << 14, ctypes.byref(fp32), sp))
        huygens = bench_huygens(bt, opt, cpu=not args.no_cpu_baseline, fp32_peak=fp32.value)
    batched = None
    if rank == 0 and not args.no_batch:
        batched = bench_batched(bt, nstates=args.batch_states, cpu=not args.no_cpu_baseline,
                                fp64_peak_tflops=fpeak.value)
    surrogate = None
    if rank == 0 and not args.no_surrogate:
        surrogate = bench_surrogate(bt, train_samples=args.surrogate_samples, epochs=args.surrogate_epochs,
                                    guard_on=not args.no_guard)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded rays and optic)",
            "config": {"workload": f"{args.workload}: {nsurf}-surface trace of {n} rays per GPU, "
                                   "6 wavelengths 350-1000 nm, Sellmeier silica",
                       "rays_per_gpu": n, "surfaces": nsurf, "niter": niter,
                       "l2": "inputs larger than L2 (1.2 GB per step), no flush",
                       "vignetted_fraction": vig},
            "roofline": {"bound": "issue", "achieved": issue_ach, "peak": issue_peak,
                         "unit": "G warp-instructions/s",
                         "frac": issue_ach / issue_peak if issue_ach else None,
                         "traffic": (counters["dram_bytes_per_ray"] * n if counters else None),
                         "peak_source": f"4 schedulers x {sms.value} SMs x {sm_ghz:.3f} GHz (clock sampled in "
                                        "the timed region)",
                         "kernel": "k_trace_ff",
                         "counters": counters,
                         "fp64": {"achieved": exec_tflops, "peak": fpeak.value, "unit": "TFLOP/s",
                                  "frac": exec_tflops / fpeak.value if (exec_tflops and fpeak.value) else None,
                                  "executed_flops_per_ray": exec_fpr,
                                  "peak_source": "DFMA loop measured in this run (bt_measure_fp64_peak)"},
                         "reference_flops": {"flops_per_ray": ref_flops_per_ray, "tflops": ref_tflops,
                                             "ratio_to_peak": ref_tflops / fpeak.value if fpeak.value else None,
                                             "convention": "FP64 operations of the reference's own expressions "
                                                           "(batoid_gb300/workcount.py); the kernel executes "
                                                           "fewer (FP32 derivatives, float-float polynomials)"},
                         "hbm": {"achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s",
                                 "frac": hbm_gbs / hbm_peak, "bytes_per_ray": bytes_per_ray,
                                 "peak_source": "MEASURED_PEAKS.json hbm_gbs"}},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": e2e_ms, "path": "bt_optic_trace_host, pinned host arrays, 512k-ray chunks on 3 streams"},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": args.steps,
            "paraboloid": paraboloid,
            "huygens_psf": huygens,
            "batched_wavefronts": batched,
            "surrogate": surrogate,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_per_stage(args):
    """Cost of each interface of the workload's optic: the optic truncated
    after interface k (k = 1..N), traced out of place on the workload's
    rays; the difference of consecutive truncations is interface k's time
    (the first also carries the kernel's ray loads and stores)."""
    import torch
    import batoid_gb300 as bt
    from batoid_gb300 import _lib, workloads as W
    build_optic, make_rays, _ = W.WORKLOADS[args.workload]
    opt = build_optic(bt)

    def leaves(o):
        return [x for it in o.items for x in leaves(it)] if hasattr(o, "items") else [o]

    ifs = leaves(opt)
    n = args.nrays
    rv_in = bt.RayVector(*make_rays(n, seed=4242))
    rv_out = bt.RayVector._empty(n)
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    niter = bt.global_vars._batoid_niter
    rows, prev = [], 0.0
    for k in range(1, len(ifs) + 1):
        sub = bt.CompoundOptic(ifs[:k], name=f"first_{k}", inMedium=opt.inMedium, outMedium=opt.outMedium)
        prog = sub._program(rv_in.coordSys)

        def step():
            _lib.check(L.bt_optic_trace_into(prog._optic.ptr, rv_in._rv, rv_out._rv, niter, stream.cuda_stream))

        step()
        torch.cuda.synchronize()
        ms = None
        if args.per_stage > 0:
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.per_stage):
                step()
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.per_stage
        rows.append({"interface": ifs[k - 1].name, "surface": type(ifs[k - 1].surface).__name__,
                     "ms_through": ms, "ms_interface": None if ms is None else ms - prev})
        prev = ms or 0.0
    print(json.dumps({"per_stage": rows, "workload": args.workload, "rays": n, "reps": args.per_stage}))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.per_stage is not None:
        run_per_stage(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
