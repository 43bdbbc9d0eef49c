"""Errors of the mixed-precision method (FP32 stencils and V-cycles inside the
FP64 defect-correction loop, optionally with the learned guess) against the
plain FP64 method on the same run, field by field.

  python -m osinco3d_gb300.accuracy --case mixing --steps 20
  python -m osinco3d_gb300.accuracy --case tgv --n 256 --steps 20
  python -m osinco3d_gb300.accuracy --case jet --nx 385 --ny 193 --nz 193 --steps 20

Both runs start from the same host fields and solve every Poisson problem to
the same eps with the multigrid solver; one JSON line reports, per field,
max|mixed - fp64| / max|fp64| and the rms ratio, with each run's ms per step
and V-cycles per step.  For the pressure (mean removed) it also reports the
absolute error, the largest pressure fluctuation and the error relative to
the dynamic pressure max |u|^2.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import o3d


def _run(params, fields, steps: int, names) -> tuple[dict, float, float]:
    with o3d.Context(params) as ctx:
        for nm, f in zip(names, fields):
            ctx.upload(nm, f)
        ms, cyc = [], []
        for it in range(1, steps + 1):
            info = ctx.step(it)
            if info.poisson_status != 0:
                raise RuntimeError(f"Poisson solve status {info.poisson_status} at step {it}")
            ms.append(info.step_ms)
            cyc.append(info.poisson_cycles)
        out = {nm: ctx.download(nm) for nm in names}
    return out, float(np.mean(ms[2:] if len(ms) > 2 else ms)), float(np.mean(cyc))


def compare(params64, params_mixed, fields, names, steps: int) -> dict:
    ref, ms64, c64 = _run(params64, fields, steps, names)
    mix, msm, cm = _run(params_mixed, fields, steps, names)
    errs = {}
    for nm in names:
        a, b = mix[nm], ref[nm]
        if nm == "pp":  # the pressure is defined up to a constant
            a = a - a.mean()
            b = b - b.mean()
        d = a - b
        errs[nm] = {"max_rel": float(np.abs(d).max() / max(np.abs(b).max(), 1e-300)),
                    "rms_rel": float(np.sqrt((d * d).mean()) / max(np.sqrt((b * b).mean()), 1e-300))}
        if nm == "pp":
            # the pressure's scales: its own fluctuation, and the dynamic
            # pressure max |u|^2 of the run
            u2 = max(float(np.abs(ref[c]).max()) for c in ("ux", "uy", "uz")) ** 2
            errs[nm]["max_abs"] = float(np.abs(d).max())
            errs[nm]["p_fluct_max"] = float(np.abs(b).max())
            errs[nm]["max_rel_u2"] = float(np.abs(d).max() / u2)
    return {"steps": steps, "errors": errs, "fp64": {"ms_per_step": ms64, "vcycles_per_step": c64},
            "mixed": {"ms_per_step": msm, "vcycles_per_step": cm}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", choices=["mixing", "tgv", "jet"], default="mixing")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--nx", type=int, default=512)
    ap.add_argument("--ny", type=int, default=256)
    ap.add_argument("--nz", type=int, default=256)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--eps", type=float, default=1e-8)
    ap.add_argument("--guess", choices=["previous", "extrapolated", "extrapolated2"], default="previous",
                    help="initial guess of every pressure solve (both runs)")
    ap.add_argument("--pre", type=int, default=0, help="multigrid pre-smoothing sweeps (0: the default)")
    ap.add_argument("--post", type=int, default=0, help="multigrid post-smoothing sweeps (0: the default)")
    ap.add_argument("--mg-omega", type=float, default=0.0, help="smoother relaxation (0: the default)")
    ap.add_argument("--mixed-only", action="store_true",
                    help="run the mixed method alone (for a launch list of its step) and print its timing")
    args = ap.parse_args()
    guess = {"previous": o3d.GUESS_PREVIOUS, "extrapolated": o3d.GUESS_EXTRAPOLATED,
             "extrapolated2": o3d.GUESS_EXTRAPOLATED2}[args.guess]
    mg = dict(solver=o3d.SOLVER_MG, eps=args.eps, kmax=200, guess=guess, mg_pre=args.pre, mg_post=args.post,
              mg_omega=args.mg_omega)
    if args.case == "mixing":
        p64 = o3d.mixing_layer_params(args.nx, args.ny, args.nz, precision=o3d.PREC_FP64, **mg)
        pmx = o3d.mixing_layer_params(args.nx, args.ny, args.nz, precision=o3d.PREC_MIXED, **mg)
        fields = o3d.mixing_layer_fields(p64)
        names = ("ux", "uy", "uz", "pp", "phi")
        workload = (f"temporal mixing layer {args.nx}x{args.ny}x{args.nz}, 60x30x30, Re 3000, LES c_s 0.17, "
                    f"scalar Sc 1, AB3, CFL 0.2, seeded noise 0.05")
    elif args.case == "jet":
        p64 = o3d.coplanar_jet_params(args.nx, args.ny, args.nz, precision=o3d.PREC_FP64, **mg)
        pmx = o3d.coplanar_jet_params(args.nx, args.ny, args.nz, precision=o3d.PREC_MIXED, **mg)
        fields = o3d.coplanar_jet_fields(p64)
        names = ("ux", "uy", "uz", "pp", "phi")
        workload = (f"co-planar jet {args.nx}x{args.ny}x{args.nz}, 20x10x10, x open, y/z free-slip, Re 2200, "
                    f"LES c_s 0.17, scalar Sc 0.7, AB3, CFL 0.25, seeded noise 0.05")
    else:
        p64 = o3d.tgv_params(args.n, precision=o3d.PREC_FP64, **mg)
        pmx = o3d.tgv_params(args.n, precision=o3d.PREC_MIXED, **mg)
        fields = o3d.tgv_fields(p64)
        names = ("ux", "uy", "uz", "pp")
        workload = f"Taylor-Green vortex {args.n}^3, Re 1600, AB3, CFL 0.2"
    if args.mixed_only:
        _, ms, cyc = _run(pmx, fields, args.steps, names)
        print(json.dumps({"workload": workload, "mixed": {"ms_per_step": ms, "vcycles_per_step": cyc}}))
        return
    res = compare(p64, pmx, fields, names, args.steps)
    res["workload"] = workload
    res["poisson_eps"] = args.eps
    print(json.dumps(res))


if __name__ == "__main__":
    main()
