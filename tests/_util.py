"""Helpers shared by the GPU parity tests: one configuration drives both the
oracle (oracle.Case) and the CUDA library (o3d.Params)."""
import math

import numpy as np

PI = math.pi


def rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| relative to max |b| (norm-wise relative error)."""
    scale = float(np.abs(b).max())
    return float(np.abs(a - b).max()) / (scale if scale > 0 else 1.0)


def params_of(o3d, case, **extra):
    """o3d.Params with the same grid, boundaries and physics as an oracle Case."""
    kw = dict(nx=case.nx, ny=case.ny, nz=case.nz, xlx=case.xlx, yly=case.yly, zlz=case.zlz,
              x0=case.x0, y0=case.y0, z0=case.z0,
              nbcx1=case.bcx, nbcxn=case.bcx, nbcy1=case.bcy, nbcyn=case.bcy,
              nbcz1=case.bcz, nbczn=case.bcz, sim2d=case.sim2d,
              itscheme=case.itscheme, dt=case.dt, re=case.re, sc=case.sc, iles=case.iles,
              cs=case.cs, nscr=case.nscr, omega=case.omega, eps=case.eps, kmax=case.kmax,
              idyn=case.idyn)
    kw.update(extra)
    return o3d.default_params(**kw)


def periodic_case(oracle, n, **kw):
    L = 2 * PI * (n - 1) / n
    base = dict(dt=0.2 * 2 * PI / n)
    base.update(kw)
    return oracle.Case(n, n, n, L, L, L, **base)


def open_x_case(oracle, n, **kw):
    """x open (inflow at x(1), outflow at x(nx)), y and z free-slip."""
    base = dict(bcx=2, bcy=1, bcz=1, dt=0.1 * PI / (n - 1))
    base.update(kw)
    return oracle.Case(n, n, n, PI, PI, PI, **base)


def free_slip_case(oracle, n, **kw):
    base = dict(bcx=1, bcy=1, bcz=1, dt=0.1 * PI / (n - 1))
    base.update(kw)
    return oracle.Case(n, n, n, PI, PI, PI, **base)


def _mode(n, kind, k, phase):
    """One smooth mode on n nodes: 'per' has period n points, 'even'/'odd' are
    symmetric/antisymmetric about both end nodes (the free-slip parities)."""
    i = np.arange(n)
    if kind == "per":
        return np.sin(2 * PI * k * i / n + phase)
    s = i / (n - 1)
    return np.cos(PI * k * s) if kind == "even" else np.sin(PI * k * s)


def perturbed(u, seed, amp=1e-2, kinds=("per", "per", "per")):
    """u plus a smooth seeded perturbation with the given parity per axis, so
    that it respects the closures of the field (periodic, even or odd)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = u.shape
    k = rng.integers(1, 4, 3)
    ph = rng.uniform(0, 2 * PI, 3)
    fx = _mode(nx, kinds[0], k[0], ph[0])[:, None, None]
    fy = _mode(ny, kinds[1], k[1], ph[1])[None, :, None]
    fz = _mode(nz, kinds[2], k[2], ph[2])[None, None, :]
    return np.asfortranarray(u + amp * fx * fy * fz)


def kinds_of(case, comp):
    """Parity of velocity component `comp` per axis: periodic axes stay
    periodic; on free-slip axes the component normal to the wall is odd; an
    open axis takes any smooth mode (even)."""
    bcs = (case.bcx, case.bcy, case.bcz)
    return tuple("per" if bcs[a] == 0 else ("even" if bcs[a] == 2 else ("odd" if a == comp else "even"))
                 for a in range(3))
