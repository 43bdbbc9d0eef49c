"""Taylor-Green statistics series computed on the GPU, row for row as the
reference's time loop writes them: statistics_calc (src/utils.f90:243-375)
at t = 0 and after every 25th step (src/osinco3d_main.f90:167-181), 17
columns per row (t, E_k, eps, eps2, dzeta, 3 mean squares of u, 9 of its
gradient).

  python -m osinco3d_gb300.series re1600_dns --tmax 10.5 --out tgv1600.dat
  python -m osinco3d_gb300.series re2500_les --precision fp64 --tmax 5 --out tgv2500.dat

The cases are the reference's two shipped examples:

- re1600_dns: examples/tgv_re1600_dns, free-slip [0, pi]^3 on 185^3 nodes,
  Re 1600, AB3, dt = 0.05 pi / 184 (the time step its statistics file was
  written with: 25 steps per 0.02134).
- re2500_les: examples/tgv_re2500_les, free-slip [0, pi]^3 on 129^3 nodes,
  Re 2500, AB3, dt = 5e-4, Smagorinsky LES with c_s = 0.17.

The reference solved the pressure by lexicographic SOR to eps = 1e-4 (DNS)
and 1e-6 (LES); here any of the library's solvers can be chosen, by default
the multigrid to eps = 1e-8.  The passive scalar of the DNS example does not
feed back on the velocity and is left out.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import o3d

CASES = {
    "re1600_dns": dict(n=185, re=1600.0, dt=0.05 * math.pi / 184.0, iles=0),
    "re2500_les": dict(n=129, re=2500.0, dt=5e-4, iles=1, cs=0.17),
}
EVERY = 25  # statistics cadence of the reference's loop


def tgv_free_slip_params(n: int, re: float, dt: float, iles: int = 0, cs: float = 0.17, **kw) -> o3d.Params:
    """Free-slip Taylor-Green box [0, pi]^3 on n^3 nodes (dx = pi / (n - 1)),
    AB3, as the reference's example parameter files set it up."""
    base = dict(nx=n, ny=n, nz=n, xlx=math.pi, yly=math.pi, zlz=math.pi,
                nbcx1=1, nbcxn=1, nbcy1=1, nbcyn=1, nbcz1=1, nbczn=1,
                itscheme=3, re=re, dt=dt, iles=iles, cs=cs, nscr=0)
    base.update(kw)
    return o3d.default_params(**base)


def run(params: o3d.Params, nsteps: int, every: int = EVERY, fields=None, progress=None) -> dict:
    """Runs nsteps steps from the Taylor-Green initial state (or `fields` =
    ux, uy, uz, pp); returns the statistics rows (t = 0 and every `every`
    steps), the Poisson work per step and the device time."""
    ux, uy, uz, pp = fields if fields is not None else o3d.tgv_fields(params)
    rows, cycles, iters, step_ms, warnings = [], [], [], [], 0
    with o3d.Context(params) as ctx:
        for nm, f in zip(("ux", "uy", "uz", "pp"), (ux, uy, uz, pp)):
            ctx.upload(nm, f)
        rows.append(ctx.statistics_calc(0.0))
        t0 = time.perf_counter()
        for it in range(1, nsteps + 1):
            info = ctx.step(it)
            if info.diverged:
                raise RuntimeError(f"velocity diverged at step {it}")
            # the reference goes on after a capped or stagnated SOR solve
            warnings += info.poisson_status != o3d.OK
            cycles.append(info.poisson_cycles)
            iters.append(info.poisson_iters)
            step_ms.append(info.step_ms)
            if it % every == 0:
                rows.append(ctx.statistics_calc(it * params.dt))
                if progress and (it // every) % progress == 0:
                    print(f"step {it}: t = {it * params.dt:.4f}, E_k = {rows[-1][1]:.10e}", flush=True)
        wall = time.perf_counter() - t0
    return {"rows": np.array(rows), "poisson_iters": np.array(iters), "vcycles": np.array(cycles),
            "step_ms": np.array(step_ms), "wall_s": wall, "poisson_warnings": warnings}


def compare_with(rows: np.ndarray, ref: np.ndarray, cols=(1, 2, 3, 4)) -> dict:
    """Relative differences of the columns `cols` between computed rows and
    reference rows at the same times (matched to 1e-6 of the row spacing),
    and the time and value of each series' peak dissipation."""
    t = rows[:, 0]
    spacing = ref[1, 0] - ref[0, 0]
    idx = [int(np.argmin(np.abs(t - tr))) for tr in ref[:, 0]]
    keep = [q for q, i in enumerate(idx) if abs(t[i] - ref[q, 0]) < 1e-6 * spacing + 1e-12]
    a = rows[[idx[q] for q in keep]]
    b = ref[keep]
    out = {"rows_compared": len(keep), "t_last": float(b[-1, 0])}
    for c in cols:
        rel = np.abs(a[:, c] - b[:, c]) / np.abs(b[:, c])
        out[f"col{c + 1}_max_rel"] = float(rel.max())
        out[f"col{c + 1}_rms_rel"] = float(np.sqrt((rel * rel).mean()))
    for c in (2, 3):
        ia, ib = int(np.argmax(a[:, c])), int(np.argmax(b[:, c]))
        out[f"col{c + 1}_peak"] = {"t": float(a[ia, 0]), "value": float(a[ia, c]),
                                   "ref_t": float(b[ib, 0]), "ref_value": float(b[ib, c])}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--solver", choices=["mg", "sor"], default="mg")
    ap.add_argument("--eps", type=float, default=1e-8)
    ap.add_argument("--omega", type=float, default=1.887, help="SOR relaxation (the DNS example's)")
    ap.add_argument("--idyn", type=int, default=0)
    ap.add_argument("--tmax", type=float, default=10.5)
    ap.add_argument("--guess", choices=["previous", "extrapolated"], default="extrapolated")
    ap.add_argument("--reference", help="the reference's statistics file to compare with")
    ap.add_argument("--out", help="write the rows here, in the reference's 17-column format")
    args = ap.parse_args()
    cs = CASES[args.case]
    prm = tgv_free_slip_params(
        cs["n"], cs["re"], cs["dt"], cs["iles"], cs.get("cs", 0.17),
        precision=o3d.PREC_MIXED if args.precision == "mixed" else o3d.PREC_FP64,
        solver=o3d.SOLVER_MG if args.solver == "mg" else o3d.SOLVER_SOR, eps=args.eps, kmax=100000,
        omega=args.omega, idyn=args.idyn,
        guess=o3d.GUESS_EXTRAPOLATED if args.guess == "extrapolated" else o3d.GUESS_PREVIOUS)
    nsteps = int(round(args.tmax / cs["dt"] / EVERY)) * EVERY
    res = run(prm, nsteps, progress=40)
    if args.out:
        np.savetxt(args.out, res["rows"], fmt="%20.12E")
    summary = {"case": args.case, "precision": args.precision, "solver": args.solver, "eps": args.eps,
               "steps": nsteps, "wall_s": round(res["wall_s"], 2),
               "ms_per_step": float(res["step_ms"].mean()),
               "poisson_iters_per_step": float(res["poisson_iters"].mean()),
               "poisson_warnings": res["poisson_warnings"]}
    if args.reference:
        summary["vs_reference"] = compare_with(res["rows"], np.loadtxt(args.reference))
    print(json.dumps(summary))


if __name__ == "__main__":
    main()
