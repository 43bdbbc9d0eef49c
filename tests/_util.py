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


def free_slip_case(oracle, n, **kw):
    base = dict(bcx=1, bcy=1, bcz=1, dt=0.1 * PI / (n - 1))
    base.update(kw)
    return oracle.Case(n, n, n, PI, PI, PI, **base)


def perturbed(u, seed, amp=1e-2):
    """u plus a smooth seeded perturbation (keeps every field nonzero and generic)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = u.shape
    x = np.linspace(0, 1, nx)[:, None, None]
    y = np.linspace(0, 1, ny)[None, :, None]
    z = np.linspace(0, 1, nz)[None, None, :]
    a, b, c, d = rng.uniform(0.5, 3.0, 4)
    return np.asfortranarray(u + amp * np.sin(a * x + d) * np.cos(b * y + 0.3) * np.sin(c * z + 0.7))
