"""Throughput benchmark of the per-ray imaging path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision fp64|mixed|mixed_strict|mixed_df|all]
                    [--workload render256|stress1024]

One "step" is one full render of the workload's image through the fused
persistent kernels: every ray of the image traced, sampled and solved.
Default workload (``render256``): render of the seeded 256^3-cell synthetic
snapshot at 256x256 pixels (a=0.94, 17 deg, 230 GHz, <= 8192 steps), timed
in every form -- plain FP64 and the mixed FP32/FP64 forms (mixed,
mixed_strict, mixed_df) -- with each mixed form's flux and per-pixel error
against the FP64 image of the same run.  The headline value is the mixed
form's rays/s.  The default run also prints: the FP64 image checked
against the oracle's render of the same rays (``fp64_vs_oracle``) and each
mixed form's error against it (``mixed_vs_oracle``), the FP64 form end to
end (``e2e_fp64``, ``fp64_vs_reference``), the standalone sampling stage
(``sampling_stage``), the served Poisson stream (``serving``), the
1024x1024 stress render in both forms (``stress1024``) and the 27-image
512x512 mixed-precision sweep (``sweep512``).  ``--workload stress1024``:
the 512^3-cell snapshot at 1024x1024, three frequencies in one pass,
<= 16384 steps, as the headline.  Printed on rank 0 as one JSON line.

``--impl reference`` times the reference algorithm on the host cores
instead: the C restatement of Mahakala's make_image (oracle/, FP64, all
host threads) on a bounded, strided subset of the same image's rays.
The reference itself (Python + JAX) cannot run on the GPU machine.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# algorithmic FLOPs (add/sub/mul/div/sqrt = 1, FMA = 2, transcendental = 1),
# counted from the FP64 device code: one accepted RK4 step (4 closed-form
# accelerations of 184 + RK4 combine 136 + radius_cal 18 + step rule 3) and
# one in-snapshot sample at one frequency (lookup 34, trilinear 168, metric
# 20, fluid frame 92, electrons/units 24, synchrotron 36, transfer 5)
FLOP_PER_STEP = 4 * 184 + 136 + 18 + 3
FLOP_PER_SAMPLE = 34 + 168 + 20 + 92 + 24 + 36 + 5
FLOP_PER_EXTRA_NU = 41

L2_FLUSH_BYTES = 256 << 20

# cycles per RK4 step of one warp alone running the near-hole phase's
# integration step (four float accelerations, the stage combinations and the
# float-pair state update; GB300, clock64 over 400 steps of 32 rays from the
# near-hole queue of the 256x256 render): the latency floor of phase B's
# serial chain
CHAIN_FLOOR_CYCLES = 1270

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# each mixed-form kernel (phases A, B, C) on the 256x256 workload: A and C
# from one capture of `ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,
# gpu__time_duration.sum -k regex:render_ -s 9 -c 3`, B (the four-warp
# near-hole pipeline) from `ncu --set full -k regex:render_zone_kernel -s 3
# -c 1`, both over
# `python bench.py --precision mixed --steps 2 --warmup 3 --quick --serving 0 --sampling-rays 0`
NCU_TRAFFIC_RENDER256 = {"A": 106.92e6 + 3.01e6, "B": 76.74e6 + 1.58e6, "C": 113.40e6 + 0.16e6}

# FP64 FLOP (DFMA = 2) per point of the standalone sampling stage, from ncu's
# DADD/DMUL/DFMA thread-instruction counters on fluid_scalars_kernel (64x64
# camera over the 256^3-cell snapshot, 19 % of points inside it)
SAMPLING_FP64_FLOP_PER_POINT = 399


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="all", choices=["fp64", "mixed", "mixed_strict", "mixed_df", "all"],
                   help="all: time every form, headline the mixed form and report each mixed "
                        "form's error vs FP64")
    p.add_argument("--workload", default="render256", choices=["render256", "stress1024", "vacuum128"])
    p.add_argument("--cpu-sample-rays", type=int, default=0, help="rays per CPU baseline sample (0 = auto)")
    p.add_argument("--resolution", type=int, default=0, help="override the image size (profiling small cases)")
    p.add_argument("--serving", type=int, default=60,
                   help="requests in the served Poisson stream (0 = skip the serving measurement)")
    p.add_argument("--sampling-rays", type=int, default=-1,
                   help="rays per side of the standalone sampling-stage measurement (0 = skip; default 128)")
    p.add_argument("--stress", type=int, default=1,
                   help="1: the default run also times the 1024x1024 three-frequency stress render in the mixed "
                        "form and in FP64 (the 'stress1024' key); 0: skip it")
    p.add_argument("--sweep", type=int, default=1,
                   help="1: the default run also renders the 27-image 512x512 mixed-precision sweep (spin x "
                        "inclination x R_high, each image in FP64 and mixed; the 'sweep512' key); 0: skip it")
    p.add_argument("--quick", action="store_true",
                   help="device timing only: skip the FMA probes, the end-to-end pass and the CPU baseline")
    return p.parse_args()


def workload(name, resolution=0, precision="fp64"):
    import dataclasses
    from mahakala_gb300 import configs
    spec = configs.RENDER_256 if name == "render256" else configs.STRESS_1024
    if resolution:
        spec = dataclasses.replace(spec, resolution=int(resolution))
    desc = (f"{precision} render {spec.resolution}x{spec.resolution} of a "
            f"{spec.snapshot.nblocks * spec.snapshot.cells_per_block}^3-cell synthetic snapshot "
            f"({spec.snapshot.nblocks}^3 meshblocks of {spec.snapshot.cells_per_block}^3), a={spec.bhspin}, "
            f"i={spec.inclination} deg, fov +-{spec.half_fov} M, "
            f"{'/'.join(f'{f / 1e9:g}' for f in spec.freqs)} GHz, <= {spec.max_nsteps} steps")
    return spec, desc


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def clocks_sampler():
    path = tempfile.mktemp(prefix="mk_clocks_", suffix=".csv")
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                                stdout=f, stderr=subprocess.DEVNULL)
        return proc, f, path
    except (OSError, FileNotFoundError):
        return None, None, path


def clocks_summary(proc, f, path, gpu_index):
    if proc is None:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    proc.terminate()
    try:
        proc.wait(timeout=5)
    except subprocess.TimeoutExpired:
        proc.kill()
    f.close()
    sm, smax, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9 or parts[0] != str(gpu_index):
            continue
        try:
            sm.append(float(parts[1]))
            smax = float(parts[2])
        except ValueError:
            continue
        for name, v in zip(names, parts[5:9]):
            if v.lower() == "active":
                reasons.add(name)
    os.unlink(path)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
            "samples": len(sm)}


def measure_fma_peak(torch, kind):
    """FMA probe: achieved FLOP/s of 8 independent FMA chains per thread
    (kind MK_FP64 or MK_MIXED = FP32), or 8 chains of paired FP32 FMAs
    (MK_PROBE_FFMA2, 16 FMAs per iteration)."""
    from mahakala_gb300 import _lib
    lib = _lib.load()
    sms = lib.mk_device_sm_count()
    blocks, threads = sms * 8, 256
    iters = 4096 if kind == _lib.MK_FP64 else 65536
    fma_per_iter = 16 if kind == _lib.MK_PROBE_FFMA2 else 8
    out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        _lib.call("mk_probe_fma", kind, blocks, threads, iters, out.data_ptr(), s.cuda_stream)
        e1.record(s)
        e1.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        best = max(best, 2.0 * fma_per_iter * iters * blocks * threads / t)
    return best


def sm_max_mhz(gpu_index):
    """The GPU's maximum SM clock (MHz) from nvidia-smi, else the measured-peak
    file's figure, else None."""
    try:
        out = subprocess.run(["nvidia-smi", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits",
                              "-i", str(gpu_index)], capture_output=True, text=True, timeout=20).stdout
        return float(out.strip().splitlines()[0])
    except (OSError, ValueError, IndexError, subprocess.SubprocessError):
        pass
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["sm_max_mhz"])
    except (OSError, KeyError, ValueError):
        return None


def probe_peaks(torch, gpu_index):
    """ALU peaks of this GPU: the FP64 FMA probe, the FP32 FMA probe, the
    paired-FP32 FMA probe and the FP32 issue limit SMs x 128 lanes x 2 FLOP
    x the maximum SM clock.  The FP32 roofline peak is the largest of the
    last three (a kernel cannot beat any of them)."""
    from mahakala_gb300 import _lib
    sms = _lib.load().mk_device_sm_count()
    mhz = sm_max_mhz(gpu_index)
    p64 = measure_fma_peak(torch, _lib.MK_FP64)
    p32 = measure_fma_peak(torch, _lib.MK_MIXED)
    p2 = measure_fma_peak(torch, _lib.MK_PROBE_FFMA2)
    theo = sms * 128 * 2 * mhz * 1e6 if mhz else 0.0
    return {"fp64": p64, "fp32": max(p32, p2, theo), "fp32_probe": p32, "ffma2_probe": p2,
            "fp32_theoretical": theo, "sms": sms, "sm_max_mhz": mhz}


def cpu_sample_pixels(res, want):
    stride = max(1, int(round((res * res / max(want, 1)) ** 0.5)))
    ix, iy = np.meshgrid(np.arange(0, res, stride), np.arange(0, res, stride), indexing="ij")
    return (ix * res + iy).reshape(-1), stride


def cpu_baseline(spec, arrays, rays_wanted, threads):
    """The oracle (C restatement of the reference, FP64) on a strided pixel
    subset of the same image; returns (rays/s, sample description, oracle
    run).  The oracle run -- its image, steps and pixel indices, plus an
    untimed second run with each initial wavevector perturbed by 1e-12 that
    tells well-conditioned rays from grazing ones -- is the checker the
    FP64 GPU image is compared against."""
    import oracle
    os.environ["OMP_NUM_THREADS"] = str(threads)
    snap = oracle.OracleSnapshot(arrays)
    pix, stride = cpu_sample_pixels(spec.resolution, rays_wanted)
    s0 = oracle.initialize_geodesics_at_camera(spec.bhspin, spec.inclination, spec.camera_distance,
                                               -spec.half_fov, spec.half_fov, spec.resolution)[pix]
    args = (spec.mass_scale, spec.M_bh, spec.r_high, list(spec.freqs), spec.max_nsteps, spec.r_low)
    t0 = time.perf_counter()
    img, steps = oracle.render_rays(snap, s0, *args)
    dt = time.perf_counter() - t0
    pimg, psteps = oracle.render_rays(snap, oracle.perturbed(s0), *args)
    what = "the whole image" if stride == 1 else f"every {stride}th pixel in x and y of the same image"
    run = dict(pix=pix, img=img, steps=steps, pert_img=pimg, pert_steps=psteps)
    return len(pix) / dt, (f"{len(pix)} rays ({what}), full FP64 physics, {threads} OpenMP threads; "
                           f"{dt:.1f} s"), run


def oracle_checks(res, run, nnu):
    """fp64_vs_oracle: the FP64 GPU image at the oracle's pixels against the
    oracle's image (oracle.image_parity: equal steps, pixels and flux within
    1e-8 on the well-conditioned rays); mixed_vs_oracle: each mixed form's
    flux and max pixel error against the oracle's image directly (floor
    1e-4 of the maximum), beside its bars (1e-3, 1e-2)."""
    import oracle
    from mahakala_gb300 import metrics
    pix = run["pix"]
    out = {}
    if "fp64" in res:
        r = res["fp64"]
        img = r["image"].reshape(nnu, -1)[:, pix].cpu().numpy()
        steps = r["req"].out["nsteps"].reshape(-1)[pix].cpu().numpy()
        out["fp64_vs_oracle"] = oracle.image_parity(img, steps, run["img"], run["steps"], run["pert_img"],
                                                    run["pert_steps"])
    for form in ("mixed", "mixed_strict", "mixed_df"):
        if form in res:
            img = res[form]["image"].reshape(nnu, -1)[:, pix].cpu().numpy()
            out[form + "_vs_oracle"] = {
                "flux_rel_err": max(metrics.flux_rel_err(img[c], run["img"][c]) for c in range(nnu)),
                "max_pixel_rel_err": max(metrics.max_pixel_rel_err(img[c], run["img"][c]) for c in range(nnu)),
                "rays": int(len(pix)), "bars": {"flux": 1e-3, "pixel": 1e-2},
                "pixel_floor": "max(|I_oracle|, 1e-4 max I_oracle)"}
    return out


def run_reference(args):
    """Reference arm: the reference algorithm (C restatement) on host cores."""
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    if args.workload == "vacuum128":
        run_reference_vacuum(args)
        return
    spec, desc = workload(args.workload, args.resolution, "fp64")
    arrays = spec.snapshot.build()
    threads = os.cpu_count() or 1
    # a quarter of the image per step (about 1 s of all-core CPU work for the
    # 256x256 workload), shifted each step
    want = args.cpu_sample_rays or (spec.resolution ** 2) // 4
    import oracle
    os.environ["OMP_NUM_THREADS"] = str(threads)
    snap = oracle.OracleSnapshot(arrays)
    pix, stride = cpu_sample_pixels(spec.resolution, want)
    s0_all = oracle.initialize_geodesics_at_camera(spec.bhspin, spec.inclination, spec.camera_distance,
                                                   -spec.half_fov, spec.half_fov, spec.resolution)
    times = []
    for k in range(args.warmup + args.steps):
        # each step a different strided subset (offset by k), so no ray repeats
        sub = (pix + k) % (spec.resolution * spec.resolution)
        t0 = time.perf_counter()
        oracle.render_rays(snap, s0_all[sub], spec.mass_scale, spec.M_bh, spec.r_high, list(spec.freqs),
                           spec.max_nsteps, spec.r_low)
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    rays = len(pix)
    value = rays * len(times) / sum(times)
    sample = (f"{rays} rays per step (every {stride}th pixel, shifted each step) of the same image, "
              f"full FP64 physics, {threads} OpenMP threads")
    line = {"metric": "rays/s", "value": value, "unit": "rays/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded snapshot)",
            "config": {"workload": desc, "precision": "fp64"}, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "rays/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "images_per_s": value / (spec.resolution ** 2) * len(spec.freqs),
            "note": "the reference is Python+JAX; jax is not installable offline, so its algorithm runs as the "
                    "C restatement in oracle/ (pinned to the reference's own outputs)"}
    print(json.dumps(line), flush=True)


def run_reference_vacuum(args):
    """Reference arm of the vacuum workload: the C restatement's integrator
    (reference rule) on all host threads, half of the rays per step."""
    import oracle
    from mahakala_gb300 import configs
    c = configs.VACUUM_SHADOW
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    s0 = oracle.initialize_geodesics_at_camera(c["bhspin"], c["inclination"], c["distance"], -c["half_fov"],
                                               c["half_fov"], c["resolution"])
    n = s0.shape[0]
    times = []
    for k in range(args.warmup + args.steps):
        sub = s0[(k % 2)::2]
        t0 = time.perf_counter()
        oracle.integrate(sub, c["max_nsteps"], 40.0, 1e-4, c["bhspin"])
        if k >= args.warmup:
            times.append(time.perf_counter() - t0)
    rays = (n + 1) // 2
    value = rays * len(times) / sum(times)
    line = {"metric": "rays/s", "value": value, "unit": "rays/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (camera grid; vacuum)",
            "config": {"workload": f"vacuum trace {c['resolution']}x{c['resolution']}, reference rule"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "rays/s", "cores": threads, "kind": "port",
                             "sample": f"{rays} rays per step (alternate halves of the camera grid), "
                                       f"{threads} OpenMP threads"},
            "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_render(torch, prep, stream, steps, warmup, flush, barrier, min_warmup=3):
    """W warm-up launches, then K launches each timed by CUDA events on the
    launching stream with an L2 flush (untimed) before each.  The library
    also records events on that stream around each of the render's kernels
    (one for FP64, phases A/B/C for the mixed forms); returns the step times
    (s) and the per-kernel times (s) of every timed step."""
    import ctypes
    from mahakala_gb300 import _lib
    for _ in range(max(warmup, min_warmup)):
        prep.launch(stream)
    torch.cuda.synchronize()
    barrier()
    ev, phases = [], []
    _lib.call("mk_set_tuning", b"phase_events", 1)
    try:
        for _ in range(steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            prep.launch(stream)
            e1.record(stream)
            ev.append((e0, e1))
            ms, n = (ctypes.c_float * 3)(), ctypes.c_int32()
            _lib.call("mk_render_phase_ms", ms, ctypes.byref(n))   # waits for this step
            phases.append([ms[i] * 1e-3 for i in range(n.value)])
    finally:
        _lib.call("mk_set_tuning", b"phase_events", 0)
    barrier()
    return [a.elapsed_time(b) * 1e-3 for a, b in ev], phases


def run_serving(torch, model0, n, precisions, latency_bound=2.0):
    """Config-4 stream: Poisson arrivals at 20/s over two resident snapshots
    (seeds 0 and 1), mixed resolutions/spins/inclinations/frequencies/R_high,
    continuous batching over four CUDA-graph slots.  Per form: p50/p99
    latency, served rays/s, the p99 of each request's latency divided by
    its isolated single-image render time, and the offered load (the
    requests' isolated render time summed over the arrival span: above 1
    the GPU cannot keep up at that rate).  The same stream is served a
    second time with latency-bound admission (requests that cannot finish
    within latency_bound x their predicted isolated latency are shed; the
    predictor is each resolution's latency served alone, calibrated on
    separate requests before the stream: the fastest and slowest of each
    resolution)."""
    from mahakala_gb300 import configs
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.serving import (DeviceExecutor, Scheduler, isolated_latencies, isolated_times,
                                        latency_report, poisson_stream, serve_stream)
    c = configs.SERVING
    model1 = AthenakFluidModel(c["snapshots"][1].build(), 0.94, fluid_gamma=13. / 9)
    models = [model0, model1]
    out = {"requests": n, "rate_hz": c["rate_hz"], "snapshots": "256^3-cell synthetic, seeds 0 and 1",
           "slots": 4, "buckets": None}
    for form in precisions:
        arrivals, reqs = poisson_stream(models, n, rate_hz=c["rate_hz"], seed=c["seed"])
        ex = DeviceExecutor(models, precision=form, nslots=4)
        out["buckets"] = list(ex.buckets)

        def factory(**kw):
            return Scheduler(ex, hbm_budget=ex.resident_bytes + (8 << 30), **kw)
        sched = factory()
        torch.cuda.synchronize()
        tickets, wall = serve_stream(sched, arrivals, reqs)
        # isolated reference 1: each request served alone through the same
        # server path (graph replay, copies, polling)
        iso_e2e = isolated_latencies(factory, reqs)
        rep = latency_report(tickets, wall, isolated={t.id: iso_e2e[i] for i, t in enumerate(tickets)})
        rep["isolated_ms_p50"] = 1e3 * float(np.percentile(iso_e2e, 50))
        rep["isolated_ms_p99"] = 1e3 * float(np.percentile(iso_e2e, 99))
        rep["p99_over_isolated_p99"] = rep["p99_ms"] / rep["isolated_ms_p99"]
        # isolated reference 2: the render kernels alone (CUDA events)
        iso, _ = isolated_times(reqs, form)
        dev = latency_report(tickets, wall, isolated={t.id: iso[i] for i, t in enumerate(tickets)})
        rep["device_only"] = {"slowdown_p50": dev["slowdown_p50"], "slowdown_p99": dev["slowdown_p99"],
                              "isolated_ms_p50": 1e3 * float(np.percentile(iso, 50)),
                              "isolated_ms_p99": 1e3 * float(np.percentile(iso, 99))}
        span = float(arrivals[-1])
        rep["offered_load"] = sum(iso) / span
        rep["offered_load_e2e"] = sum(iso_e2e) / span
        rep["offered_load_note"] = ("sum of the requests' isolated render times (device; e2e: through the "
                                    "server alone) over the arrival span: above 1 the GPU cannot keep up")
        rep["isolated_note"] = ("slowdown = stream latency / the same request's latency served alone through the "
                                "same scheduler; device_only divides by its render kernels' time alone")
        rep["nonfinite_images"] = int(sum(not np.all(np.isfinite(t.image)) for t in tickets if t.image is not None))
        rep["batches"] = len(sched.batches)
        rep["mean_requests_per_batch"] = float(np.mean([b["requests"] for b in sched.batches]))
        # latency-bound admission: calibrate a per-resolution predictor on
        # requests that are not in the stream, then serve the stream again
        _, cal = poisson_stream(models, 16, rate_hz=c["rate_hz"], seed=c["seed"] + 1)
        by_res = {}
        for r in cal:
            by_res.setdefault(int(r.resolution), []).append(r)
        # per resolution, the fastest and the slowest calibration request: a
        # request's isolated time varies with spin and view (several-fold
        # for FP64 64^2 renders, whose time is their longest ray's chain), so
        # its own bound takes the low figure and the work it puts ahead of
        # later requests the high one
        cal_t = {res: isolated_latencies(factory, rs) for res, rs in by_res.items()}
        table = {res: (float(np.min(v)), float(np.max(v))) for res, v in cal_t.items()}
        known = sorted(table)

        def predict(r):
            res = int(r.resolution)
            if res in table:
                return table[res]
            near = min(known, key=lambda k: abs(k - res))
            return tuple(x * (res / near) ** 2 for x in table[near])
        bsched = factory(latency_bound=latency_bound, predict=predict)
        torch.cuda.synchronize()
        btickets, bwall = serve_stream(bsched, arrivals, reqs)
        brep = latency_report(btickets, bwall, isolated={t.id: iso_e2e[i] for i, t in enumerate(btickets)})
        served_iso = [iso_e2e[i] for i, t in enumerate(btickets) if t.status == "done"]
        if served_iso:
            brep["isolated_ms_p99"] = 1e3 * float(np.percentile(served_iso, 99))
            brep["p99_over_isolated_p99"] = brep["p99_ms"] / brep["isolated_ms_p99"]
        brep["latency_bound"] = latency_bound
        brep["predictor_ms"] = {str(k): [1e3 * v[0], 1e3 * v[1]] for k, v in sorted(table.items())}
        brep["predictor"] = ("per resolution, the fastest (own bound) and slowest (work ahead of others) isolated "
                             "latency of 16 calibration requests not in the stream")
        pred = [predict(r)[0] for r in reqs]
        over = [t.latency / pred[i] for i, t in enumerate(btickets) if t.status == "done"]
        if over:
            brep["latency_over_predicted_p99"] = float(np.percentile(over, 99))
        brep["note"] = ("requests predicted to miss latency_bound x their isolated latency are shed (status "
                        "'shed', counted apart from served); p99 over the served requests")
        rep["bounded"] = brep
        out[form] = rep
        del ex, sched, bsched
        torch.cuda.empty_cache()
    return out


def hbm_peak():
    """Measured copy bandwidth of this GPU model (GB/s) and its source."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs, STREAM-style copy)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback (6.8 TB/s, one earlier GB300 copy measurement)"


def sampling_stage(torch, model, spec, flush, stream, fp64_peak, rays_per_side=128, reps=3):
    """The sampling stage alone (get_fluid_scalars_from_geodesics as the
    standalone mk_fluid_scalars kernel) over the reference's trajectory rows
    of a rays_per_side^2 camera with the workload's view: every row of every
    ray, as the reference samples them.  Algorithmic bytes per point: 64 B
    state read + 40 B written, plus the 8-corner x 8-primitive float32
    gather (256 B) for points inside the snapshot."""
    import ctypes
    from mahakala_gb300 import _lib
    from mahakala_gb300.geodesics import geodesic_integrator, initialize_geodesics_at_camera
    s0 = initialize_geodesics_at_camera(spec.bhspin, spec.inclination, spec.camera_distance, -spec.half_fov,
                                        spec.half_fov, rays_per_side)
    S, _ = geodesic_integrator(spec.max_nsteps, s0, 40.0, 1e-4, spec.bhspin)
    nt = S.shape[0]
    pts = S.reshape(-1, 8)
    n = pts.shape[0]
    view = ctypes.byref(model.snapshot.view)
    blk = torch.empty(n, dtype=torch.int32, device="cuda")
    prims = torch.empty((n, 8), dtype=torch.float64, device="cuda")
    _lib.call("mk_fluid_prims", view, pts.data_ptr(), n, prims.data_ptr(), blk.data_ptr(), stream.cuda_stream)
    inside = int((blk >= 0).sum().item())
    del prims, blk
    out = torch.empty((n, 5), dtype=torch.float64, device="cuda")
    cosf = float(np.cos(np.pi / 3))

    def call():
        _lib.call("mk_fluid_scalars", view, float(spec.bhspin), pts.data_ptr(), n, cosf, out.data_ptr(),
                  stream.cuda_stream)
    for _ in range(3):
        call()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call()
        e1.record(stream)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t = statistics.mean(ts)
    nbytes = n * (64 + 40) + inside * 256
    flops = SAMPLING_FP64_FLOP_PER_POINT * n
    peak, src = hbm_peak()
    del S, pts, out
    torch.cuda.empty_cache()
    return {"kernel": "fluid_scalars_kernel", "bound": "fp64", "rays": rays_per_side ** 2, "rows": nt,
            "points": n, "in_snapshot": inside, "ms": 1e3 * t, "algorithmic_bytes": nbytes,
            "hbm": {"achieved": nbytes / t / 1e9, "peak": peak, "unit": "GB/s", "frac": nbytes / t / 1e9 / peak,
                    "peak_source": src},
            "fp64": {"achieved": flops / t / 1e12, "peak": fp64_peak / 1e12, "unit": "TFLOP/s",
                     "frac": flops / t / fp64_peak, "flop_per_point": SAMPLING_FP64_FLOP_PER_POINT},
            "traffic": None,
            "note": "every point needs the metric, fluid frame and arccos in binary64 to return the reference's "
                    "values, so the stage is FP64-pipe bound (ncu on the 64x64 case: 87.5 % FP64 pipe, 2.6 % DRAM); "
                    "FLOP per point from ncu's FP64 instruction counters on the same case"}


def stress_record(torch, stream, flush, peaks):
    """The 1024x1024 stress render (512^3-cell snapshot, a=0.94, 60 deg,
    86/230/345 GHz in one ray pass, <= 16384 steps) in the mixed form and in
    FP64, each CUDA-event timed with per-kernel times, with each mixed
    channel's flux and pixel error against the FP64 image.  Mixed: 3
    warm-up and 3 timed renders; FP64 (1.3 s a render): 1 and 1."""
    from mahakala_gb300 import configs, metrics
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.images import PreparedRender
    spec, desc = workload("stress1024", 0, "mixed and fp64")
    t0 = time.perf_counter()
    model = AthenakFluidModel(spec.snapshot.build(), spec.snapshot.bhspin, fluid_gamma=spec.snapshot.fluid_gamma)
    t_build = time.perf_counter() - t0
    rays, nnu = spec.resolution ** 2, len(spec.freqs)
    per_sample = FLOP_PER_SAMPLE + FLOP_PER_EXTRA_NU * (nnu - 1)
    out = {"workload": desc, "snapshot_build_s": t_build, "mass_scale": spec.mass_scale}
    imgs = {}
    for form, reps, warm in (("mixed", 3, 3), ("fp64", 1, 1)):
        prep = PreparedRender([spec.request(model)], precision=form, with_steps=True)
        times, phases = time_render(torch, prep, stream, reps, warm, flush, torch.cuda.synchronize,
                                    min_warmup=warm)
        t = statistics.mean(times)
        steps, samples = prep.work_totals()
        flops = steps * FLOP_PER_STEP + samples * per_sample
        pk = peaks["fp64"] if form == "fp64" else peaks["fp32"]
        out[form] = {"rays_per_s": rays / t, "ms": 1e3 * t, "images_per_s": nnu / t,
                     "phase_ms": [1e3 * statistics.mean(p[i] for p in phases) for i in range(len(phases[0]))],
                     "accepted_steps": steps, "samples": samples, "ray_steps_per_s": steps / t,
                     "achieved_tflops": flops / t / 1e12, "peak_tflops": pk / 1e12, "frac": flops / t / pk,
                     "max_step_optical_depth": prep.max_step_optical_depth(), "timed_renders": reps}
        imgs[form] = (prep.images[0].clone(), prep.requests[0].out["status"].clone())
        del prep
    errs = [metrics.compare(imgs["mixed"][0][c], imgs["fp64"][0][c], imgs["mixed"][1], imgs["fp64"][1], spec.fov)
            for c in range(nnu)]
    out["mixed_vs_fp64"] = {"speedup": out["fp64"]["ms"] / out["mixed"]["ms"],
                            "channels_ghz": [f / 1e9 for f in spec.freqs],
                            "flux_rel_err": [e["flux_rel_err"] for e in errs],
                            "max_pixel_rel_err": [e["max_pixel_rel_err"] for e in errs],
                            "shadow_diameter": errs[0]["shadow_diameter"],
                            "shadow_diameter_fp64": errs[0]["shadow_diameter_fp64"],
                            "pixel_floor": "max(|I_fp64|, 1e-4 max I_fp64)"}
    del imgs, model
    torch.cuda.empty_cache()
    return out


def run_vacuum(args):
    """Config-1 vacuum trace: 128x128 rays, a=0.94, 60 deg, +-10 M, <= 4096
    steps, end states only (no trajectory rows), under the reference step
    rule (div 40, tol 1e-4) and the fixed-fraction rule."""
    import torch
    from mahakala_gb300 import _lib, build
    from mahakala_gb300 import configs
    from mahakala_gb300.geodesics import initialize_geodesics_at_camera, step_policy, trace
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    build.build()
    _lib.load()
    c = configs.VACUUM_SHADOW
    n = c["resolution"] ** 2
    s0 = initialize_geodesics_at_camera(c["bhspin"], c["inclination"], c["distance"], -c["half_fov"],
                                        c["half_fov"], c["resolution"])
    pols = {"reference": step_policy(c["max_nsteps"]),
            "fixed": step_policy(c["max_nsteps"], kind="fixed", hfrac=c["hfrac"], hmin=c["hmin"], hmax=c["hmax"],
                                 capture=c["capture"], r_escape=c["r_escape"])}
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    peak64 = measure_fma_peak(torch, _lib.MK_FP64)
    proc, fh, cpath = clocks_sampler() if rank == 0 else (None, None, None)
    lines = {}
    for name, pol in pols.items():
        for _ in range(max(args.warmup, 3)):
            r = trace(s0, c["bhspin"], pol)
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = trace(s0, c["bhspin"], pol)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        t = statistics.mean(ts)
        K = r["K"].cpu().numpy().astype(np.int64)
        steps = int(K.sum())
        flops = steps * FLOP_PER_STEP
        # end to end: host initial states in, host end states and step counts out
        s0_host = s0.cpu().pin_memory()
        e2e = []
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rr = trace(s0_host.to("cuda", non_blocking=True), c["bhspin"], pol)
            _ = rr["state"].cpu(), rr["K"].cpu(), rr["why"].cpu()
            e2e.append(time.perf_counter() - t0)
        lines[name] = {"rays_per_s": n / t, "ms_per_step": 1e3 * t, "ray_steps": steps,
                       "ray_steps_per_s": steps / t, "e2e_rays_per_s": n / statistics.mean(e2e),
                       "roofline": {"bound": "fp64", "achieved": flops / t / 1e12, "peak": peak64 / 1e12,
                                    "unit": "TFLOP/s", "frac": flops / t / peak64, "traffic": None,
                                    "kernel": "integrate_%s_kernel" % ("reference" if name == "reference"
                                                                        else "fixed")}}
    clocks = clocks_summary(proc, fh, cpath, local) if rank == 0 else None
    if rank != 0:
        return
    import oracle
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    s0h = s0.cpu().numpy()
    t0 = time.perf_counter()
    oracle.integrate(s0h, c["max_nsteps"], 40.0, 1e-4, c["bhspin"])
    cpu_t = time.perf_counter() - t0
    head = lines["reference"]
    line = {"metric": "rays/s", "value": world * head["rays_per_s"], "unit": "rays/s", "n_gpus": world,
            "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": head["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (camera grid; vacuum, no snapshot)",
            "config": {"workload": f"vacuum trace {c['resolution']}x{c['resolution']}, a={c['bhspin']}, "
                                   f"i={c['inclination']} deg, +-{c['half_fov']} M, <= {c['max_nsteps']} steps, "
                                   "end states only (reference rule div 40, tol 1e-4; fixed-fraction rule beside)",
                       "l2": f"flushed between steps ({L2_FLUSH_BYTES >> 20} MB write, untimed)",
                       "parallelism": f"replicas x{world}"},
            "reference_rule": head, "fixed_rule": lines["fixed"], "roofline": head["roofline"],
            "cpu_baseline": {"value": n / cpu_t, "unit": "rays/s", "cores": threads, "kind": "port",
                             "sample": f"all {n} rays, reference rule, oracle C restatement ({cpu_t:.1f} s)"},
            "e2e": {"value": head["e2e_rays_per_s"], "unit": "rays/s", "h2d_bytes_per_step": n * 64,
                    "d2h_bytes_per_step": n * (64 + 8),
                    "api": "mahakala_gb300.geodesics.trace (host initial states -> host end states)"},
            "gpu_launches": args.steps, "clocks": clocks}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.workload == "vacuum128" and args.impl == "ours":
        run_vacuum(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from mahakala_gb300 import _lib, build, metrics
    build.build()
    _lib.load()
    from mahakala_gb300.grmhd.athenak import AthenakFluidModel
    from mahakala_gb300.images import PreparedRender, image_flux_jy, make_image

    forms = ["fp64", "mixed", "mixed_strict", "mixed_df"] if args.precision == "all" else [args.precision]
    head = "mixed" if "mixed" in forms else forms[0]
    spec, desc = workload(args.workload, args.resolution, head)
    t_gen = time.perf_counter()
    arrays = spec.snapshot.build()
    t_gen = time.perf_counter() - t_gen
    model = AthenakFluidModel(arrays, spec.snapshot.bhspin, fluid_gamma=spec.snapshot.fluid_gamma)
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    peaks = probe_peaks(torch, local) if not args.quick else None
    peak64 = peaks["fp64"] if peaks else float("nan")
    peak32 = peaks["fp32"] if peaks else float("nan")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    rays = spec.resolution ** 2
    nnu = len(spec.freqs)
    res = {}
    proc, fh, cpath = clocks_sampler() if rank == 0 else (None, None, None)
    for form in forms:
        req = spec.request(model)
        prep = PreparedRender([req], precision=form, with_steps=True)
        times, phases = time_render(torch, prep, stream, args.steps, args.warmup, flush, barrier)
        t_step = statistics.mean(times)
        t_phase = [statistics.mean(p[i] for p in phases) for i in range(len(phases[0]))]
        if world > 1:
            t = torch.tensor([t_step], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            t_step = float(t.item())
        steps_total, samples_total = prep.work_totals()
        split = prep.precision_split() if form.startswith("mixed") else (0, 0, steps_total)
        samples64 = prep.samples_fp64() if form.startswith("mixed") else samples_total
        work_b = prep.phase_b_work() if form == "mixed" else None
        work_c = prep.phase_c_work() if form.startswith("mixed") else None
        res[form] = dict(prep=prep, req=req, t_step=t_step, t_phase=t_phase, steps=steps_total,
                         zone_run_max=prep.zone_run_max() if form == "mixed" else None, work_b=work_b, work_c=work_c,
                         samples=samples_total, samples64=samples64,
                         split=split, image=prep.images[0].clone(), status=req.out["status"].clone(),
                         max_tau=prep.max_step_optical_depth())
    clocks = clocks_summary(proc, fh, cpath, local) if rank == 0 else None

    sampling = None
    srays = args.sampling_rays if args.sampling_rays >= 0 else 128
    if srays:
        sampling = sampling_stage(torch, model, spec, flush, stream, peak64 if not args.quick else float("nan"),
                                  rays_per_side=srays)

    serving = None
    if args.serving and not args.quick and args.workload == "render256" and rank == 0:
        # one GPU's serving stream (the other replicas would repeat it)
        serving = run_serving(torch, model, args.serving, [f for f in ("mixed", "fp64") if f in forms])

    sweep = None
    if args.sweep and not args.quick and args.workload == "render256" and not args.resolution and rank == 0:
        from mahakala_gb300 import sweep as sweepmod
        t0 = time.perf_counter()
        rep = sweepmod.run(512, "mixed", model=model)
        keep = ("spin", "inclination", "r_high", "fp64_ms", "mixed_ms", "speedup", "max_pixel_rel_err",
                "flux_rel_err", "shadow_diameter_rel_err", "max_step_optical_depth")
        sweep = dict(rep, rows=[{k: r[k] for k in keep} for r in rep["rows"]], wall_s=time.perf_counter() - t0,
                     timing="one warm launch per form and image, CUDA events")

    stress = None
    if args.stress and not args.quick and args.workload == "render256" and not args.resolution and rank == 0:
        stress = stress_record(torch, stream, flush, peaks)

    # end to end through the public API: host request in, NumPy image out
    # (W untimed calls first, like the device timing).  Each timed call is
    # preceded, outside the timed region, by the same L2 flush as the
    # device-timed steps, so both measure from the same GPU state; the same
    # calls back to back with no flush are reported beside it
    # (e2e_back_to_back)
    def e2e_series(precision, flushed):
        out = []
        for k in range(0 if args.quick else max(args.warmup, 3) + args.steps):
            if flushed:
                flush.fill_(1.0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            make_image(model, camera_inclination=spec.inclination, camera_distance=spec.camera_distance,
                       mass_scale=spec.mass_scale, M_bh=spec.M_bh, r_high=spec.r_high,
                       observing_frequency=list(spec.freqs) if nnu > 1 else spec.freqs[0], fov=spec.fov,
                       resolution=spec.resolution, max_nsteps=spec.max_nsteps, precision=precision)
            if k >= max(args.warmup, 3):
                out.append(time.perf_counter() - t0)
        return out

    e2e_times = e2e_series(head, True)
    e2e_t = statistics.mean(e2e_times) if e2e_times else float("nan")
    e2e_b2b = e2e_series(head, False)
    e2e_b2b_t = statistics.mean(e2e_b2b) if e2e_b2b else float("nan")
    # the FP64 form end to end too (like for like against the FP64 CPU path)
    e2e64_times = e2e_series("fp64", True) if head != "fp64" and "fp64" in forms else []
    e2e64_t = statistics.mean(e2e64_times) if e2e64_times else float("nan")
    if world > 1 and e2e_times:  # the slowest replica sets the job's rate
        t = torch.tensor([e2e_t, e2e64_t, e2e_b2b_t], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_t, e2e64_t, e2e_b2b_t = float(t[0].item()), float(t[1].item()), float(t[2].item())
    L_unit = model.get_units(spec.M_bh, spec.mass_scale)["L_unit"]

    def roofline(form):
        """Roofline of the form's dominant kernel, timed by the CUDA events
        the library records around each kernel of every timed step."""
        r = res[form]
        per_sample = FLOP_PER_SAMPLE + FLOP_PER_EXTRA_NU * (nnu - 1)
        src = ("FP64: the FMA probe measured in this run (mk_probe_fma); FP32: the largest of the FP32 FMA "
               "probe, the paired-FP32 FMA probe and the issue limit SMs x 128 x 2 FLOP x the maximum SM clock; "
               "the measured-peak file holds no FP64/FP32 ALU figure")
        if form == "fp64":
            kernels = [("render_fp64_kernel", "fp64", r["steps"] * FLOP_PER_STEP + r["samples"] * per_sample,
                        r["t_phase"][0], peak64, None)]
        else:
            to64, back32, steps64 = r["split"]
            stb, smb = r["work_b"] if r["work_b"] else (steps64, r["samples64"])
            stc, smc = r["work_c"]
            tA, tB, tC = r["t_phase"][:3]
            fa = (r["steps"] - stb - stc) * FLOP_PER_STEP + (r["samples"] - smb - smc) * per_sample
            zone = stb * FLOP_PER_STEP + smb * per_sample
            fc = stc * FLOP_PER_STEP + smc * per_sample
            if form == "mixed":  # float accelerations and emission, float-pair state, compensated sums
                kb = ("render_zone_kernel (phase B: near the hole and after; beside C)", "fp32", zone, tB, peak32, "B")
                kc = ("render_f32_kernel (phase C: parked outbound rays; beside B)", "fp32", fc, tC, peak32, "C")
            else:
                kb = ("render_fp64_kernel (phase B, near the hole)", "fp64", zone, tB, peak64, None)
                kc = ("render_f32_kernel (phase C)", "fp32", fc, tC, peak32, None)
            kernels = [("render_f32_kernel (phase A)", "fp32", fa, tA, peak32, "A"), kb, kc]
        measured = (NCU_TRAFFIC_RENDER256 if form == "mixed" and args.workload == "render256" and not args.resolution
                    else {})
        table = [{"kernel": k, "bound": b, "flop": fl, "ms": 1e3 * t, "achieved": fl / t / 1e12 if t else None,
                  "peak": pk / 1e12, "frac": fl / t / pk if t else None,
                  "traffic": measured.get(tag) if tag else None}
                 for k, b, fl, t, pk, *rest in kernels for tag in [rest[0] if rest else None]]
        top = max(table, key=lambda e: e["ms"])
        out = {"bound": top["bound"], "achieved": top["achieved"], "peak": top["peak"], "unit": "TFLOP/s",
               "frac": top["frac"], "traffic": top["traffic"], "kernel": top["kernel"], "flop_per_launch": top["flop"],
               "kernel_ms": top["ms"], "peak_source": src, "kernels": table,
               "peak_fp32_tflops": peak32 / 1e12, "peak_fp64_tflops": peak64 / 1e12,
               "peaks_tflops": {k: (v / 1e12 if k.startswith(("fp", "ffma")) else v)
                                for k, v in (peaks or {}).items()}}
        if top["traffic"] is not None:
            out["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch of this "
                                     "kernel on this workload (bytes per launch); the kernels are ALU- and "
                                     "latency-bound, the gathers hit L1/L2")
        if form == "fp64":
            out["traffic_note"] = ("ncu on the 192x192 case: 242 MB DRAM read per launch; the kernel is "
                                   "FP64-pipe bound (71 % FP64 pipe, 0.04 % DRAM)")
        else:
            out["note"] = ("phase B runs the serial chain of its longest ray (zone_run_max steps): one integrating "
                           "warp per block, three sampling warps beside it on the other sub-partitions; "
                           "latency-bound, not throughput-bound")
            if form == "mixed" and r["zone_run_max"]:
                # the bound that applies to a serial chain: cycles per step of
                # its integrating warp against that warp's RK4 step alone
                mhz = (clocks or {}).get("sm_mhz") or sm_max_mhz(local) or float("nan")
                cps = tB * mhz * 1e6 / r["zone_run_max"]
                out["chain"] = {"steps": r["zone_run_max"], "cycles_per_step": cps,
                                "floor_cycles_per_step": CHAIN_FLOOR_CYCLES, "frac": CHAIN_FLOOR_CYCLES / cps,
                                "sm_mhz": mhz,
                                "floor_source": ("one warp alone running the integrating warp's RK4 step (four float "
                                                 "accelerations, stage combinations, float-pair state update) on "
                                                 "GB300, clock64 over 400 steps; the phase's time over zone_run_max "
                                                 "steps at the sampled SM clock gives cycles_per_step")}
        return out

    def form_line(form):
        r = res[form]
        to64, back32, steps64 = r["split"]
        return {"rays_per_s": world * rays / r["t_step"], "ms_per_step": 1e3 * r["t_step"],
                "images_per_s": world * nnu / r["t_step"], "ray_steps_per_s": world * r["steps"] / r["t_step"],
                "accepted_steps": r["steps"], "samples": r["samples"], "steps_per_ray": r["steps"] / rays,
                "rays_to_fp64": to64, "rays_back_to_fp32": back32, "steps_in_fp64": steps64,
                "zone_run_max": r["zone_run_max"],
                "phase_b_steps_samples": list(r["work_b"]) if r["work_b"] else None,
                "phase_c_steps_samples": list(r["work_c"]) if r["work_c"] else None,
                "max_step_optical_depth": r["max_tau"],
                "flux_jy": [float(x) for x in np.atleast_1d(image_flux_jy(r["image"], spec.fov, spec.distance_cm,
                                                                         L_unit))],
                "roofline": roofline(form)}

    t_head = res[head]["t_step"]
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    threads = os.cpu_count() or 1
    if args.quick:
        cpu_val, cpu_sample, cpu_run = None, "skipped (--quick)", None
    else:
        # the whole image up to 262,144 rays (a strided quarter of the 1024x1024
        # workload): ~3 s on 16 cores at 256x256, ~16 s at 1024x1024
        cpu_val, cpu_sample, cpu_run = cpu_baseline(spec, arrays,
                                                    args.cpu_sample_rays or min(spec.resolution ** 2, 1 << 18),
                                                    threads)
    line = {
        "metric": "rays/s", "value": world * rays / t_head, "unit": "rays/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * t_head, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"fp64": "f64", "mixed": "f32+f64", "mixed_strict": "f32+f64",
                                           "mixed_df": "f32+f32x2"}[head],
        "data": "synthetic (seeded snapshot, no external data)",
        "config": {"workload": desc, "precision": head,
                   "l2": f"flushed between steps ({L2_FLUSH_BYTES >> 20} MB write, untimed)",
                   "parallelism": f"replicas x{world} (rays independent; no collective)",
                   "mass_scale": spec.mass_scale},
        "images_per_s": world * nnu / t_head,
    }
    for form in forms:
        line[form] = form_line(form)
    for form in ("mixed", "mixed_strict", "mixed_df"):
        if "fp64" not in res or form not in res:
            continue
        a, b = res[form], res["fp64"]
        errs = [metrics.compare(a["image"][c], b["image"][c], a["status"], b["status"], spec.fov)
                for c in range(nnu)]
        line[form + "_vs_fp64"] = {"speedup": b["t_step"] / a["t_step"],
                                   "flux_rel_err": max(e["flux_rel_err"] for e in errs),
                                   "max_pixel_rel_err": max(e["max_pixel_rel_err"] for e in errs),
                                   "shadow_diameter": errs[0]["shadow_diameter"],
                                   "shadow_diameter_fp64": errs[0]["shadow_diameter_fp64"],
                                   "pixel_floor": "max(|I_fp64|, 1e-4 max I_fp64)"}
    if cpu_run is not None:
        line.update(oracle_checks(res, cpu_run, nnu))
    line.update({
        "roofline": roofline(head),
        "cpu_baseline": {"value": cpu_val, "unit": "rays/s", "cores": threads, "kind": "port",
                         "sample": cpu_sample},
        "e2e": {"value": world * rays / e2e_t, "unit": "rays/s", "h2d_bytes_per_step": len(res[head]["prep"].table_bytes),
                "d2h_bytes_per_step": int(rays * nnu * 8) + 8,  # the image and the launch's wait-error word
                "api": f"mahakala_gb300.images.make_image(precision='{head}') (host request -> NumPy image)",
                "l2": "flushed before each call (256 MB write, untimed), as the device-timed steps"},
        "e2e_back_to_back": {"value": world * rays / e2e_b2b_t, "unit": "rays/s",
                             "note": "the same make_image calls back to back, no flush between them"},
        "e2e_fp64": ({"value": world * rays / e2e64_t, "unit": "rays/s",
                      "h2d_bytes_per_step": len(res["fp64"]["prep"].table_bytes),
                      "d2h_bytes_per_step": int(rays * nnu * 8) + 8,
                      "api": "mahakala_gb300.images.make_image(precision='fp64') (host request -> NumPy image)",
                      "l2": "flushed before each call (256 MB write, untimed)"}
                     if e2e64_times else None),
        "fp64_vs_reference": ({"e2e_ratio": (world * rays / e2e64_t) / cpu_val,
                               "device_ratio": (world * rays / res["fp64"]["t_step"]) / cpu_val,
                               "note": "FP64 GPU form over the FP64 CPU path (cpu_baseline), like for like"}
                              if e2e64_times and cpu_val else None),
        "serving": serving,
        "sampling_stage": sampling,
        "stress1024": stress,
        "sweep512": sweep,
        # per render: FP64 one kernel; mixed forms A, B, C, plus the camera-state
        # kernel when the launch exceeds one wave of phase A at 4 blocks per SM
        "gpu_launches": args.steps * (1 if head == "fp64" else
                                      3 + int(rays > _lib.load().mk_device_sm_count() * 4 * 128)),
        "phase_ms": {f: [1e3 * t for t in res[f]["t_phase"]] for f in forms},
        "clocks": clocks,
        "snapshot_build_s": t_gen,
    })
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
