"""Mixed-precision error sweep: the 256^3-cell snapshot rendered at
512x512 for spins {0, 0.5, 0.94} x inclinations {17, 60, 85} deg x R_high
{1, 10, 40}, each image in FP64 and in the mixed form, reporting per image
the max per-pixel relative error (floor 1e-4 of the image maximum), the
total-flux error and the shadow diameter of each form, plus the times.

    python -m mahakala_gb300.sweep [--resolution 512] [--precision mixed] [--out report.json]
"""

import argparse
import itertools
import json
import sys
import time


def run(resolution=512, precision="mixed", spins=None, inclinations=None, r_highs=None, model=None, log=None):
    import torch

    from . import configs, metrics
    from .grmhd.athenak import AthenakFluidModel
    from .images import PreparedRender
    c = configs.MIXED_SWEEP
    spins = spins or c["spins"]
    inclinations = inclinations or c["inclinations"]
    r_highs = r_highs or c["r_highs"]
    spec = configs.RENDER_256
    if model is None:
        model = AthenakFluidModel(spec.snapshot.build(), spec.snapshot.bhspin, fluid_gamma=spec.snapshot.fluid_gamma)
    rows = []
    for a, inc, rh in itertools.product(spins, inclinations, r_highs):
        ms = configs.stable_mass_scale(rh, inc, spec.freqs[0])
        out = {}
        for form in ("fp64", precision):
            req = spec.request(model, bhspin=a, camera_inclination=inc, r_high=rh, mass_scale=ms,
                               resolution=resolution)
            prep = PreparedRender([req], precision=form, with_steps=True)
            prep.launch()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            prep.launch()
            e1.record()
            e1.synchronize()
            out[form] = dict(ms=e0.elapsed_time(e1), image=prep.images[0][0].cpu().numpy(),
                             status=req.out["status"].cpu().numpy(), tau=prep.max_step_optical_depth())
        m = metrics.compare(out[precision]["image"], out["fp64"]["image"], out[precision]["status"],
                            out["fp64"]["status"], spec.fov)
        row = dict(spin=a, inclination=inc, r_high=rh, mass_scale=ms, fp64_ms=out["fp64"]["ms"],
                   mixed_ms=out[precision]["ms"], speedup=out["fp64"]["ms"] / out[precision]["ms"],
                   max_step_optical_depth=out["fp64"]["tau"], **m)
        rows.append(row)
        if log:
            print(json.dumps(row), file=log, flush=True)
    worst = dict(max_pixel_rel_err=max(r["max_pixel_rel_err"] for r in rows),
                 flux_rel_err=max(r["flux_rel_err"] for r in rows),
                 shadow_diameter_rel_err=max(r["shadow_diameter_rel_err"] for r in rows),
                 min_speedup=min(r["speedup"] for r in rows),
                 total_speedup=sum(r["fp64_ms"] for r in rows) / sum(r["mixed_ms"] for r in rows))
    return dict(resolution=resolution, precision=precision, images=len(rows), worst=worst, rows=rows)


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--resolution", type=int, default=512)
    p.add_argument("--precision", default="mixed", choices=["mixed", "mixed_strict", "mixed_df"])
    p.add_argument("--out", default=None)
    args = p.parse_args(argv)
    t0 = time.time()
    rep = run(args.resolution, args.precision, log=sys.stderr)
    rep["wall_s"] = time.time() - t0
    text = json.dumps(rep)
    if args.out:
        with open(args.out, "w") as f:
            f.write(text)
    print(json.dumps(dict(rep, rows=None)))


if __name__ == "__main__":
    main()
