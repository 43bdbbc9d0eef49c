"""The FP64 oracle, pinned against the reference's own published numbers and
checked for the properties its kernels must have.  CPU only."""
import math
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden")
PI = 3.141592653589793


def test_golden_row0_re1600(oracle):
    """Row 0 of examples/tgv_re1600_dns/tgv_stats_re1600_dns.dat: free-slip
    [0,pi]^3 TGV on 185^3 nodes, statistics_calc at t = 0.  This pins the
    free-slip first/second derivative closures and the statistics formulas."""
    gold = np.loadtxt(os.path.join(GOLD, "tgv_re1600_dns_stats_head.txt"))[0]
    c = oracle.Case(185, 185, 185, PI, PI, PI, bcx=1, bcy=1, bcz=1, re=1600.0)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s, omp=True)
    st = oracle.statistics(c, s, 0.0, omp=True)
    nz = gold != 0
    rel = np.abs(st[nz] - gold[nz]) / np.abs(gold[nz])
    # the file keeps 13 significant digits
    assert rel.max() < 2e-12, rel
    assert np.all(st[~nz] == 0.0)


@pytest.mark.slow
def test_golden_re2500_les_25_steps(oracle):
    """Row 1 of examples/tgv_re2500_les/tgv_stats_re2500_les.dat (t = 0.0125,
    after 25 AB3 steps of LES with SOR eps = 1e-6) at 129^3.  The file was
    written by an earlier version of the code, so this is a loose pin of the
    whole step: E_k, dissipation and enstrophy agree to a few 1e-7."""
    gold = np.loadtxt(os.path.join(GOLD, "tgv_re2500_les_stats_head.txt"))[0]
    c = oracle.Case(129, 129, 129, PI, PI, PI, bcx=1, bcy=1, bcz=1, re=2500.0, dt=5e-4,
                    itscheme=3, iles=1, cs=0.17, omega=1.999, idyn=1, eps=1e-6, kmax=10000)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s, omp=True)
    r = oracle.Runner(c, s, omp=True)
    for it in range(1, 26):
        info = r.step(it)
        assert info.sor_status == oracle.SOR_CONVERGED
        assert info.diverged == 0
    st = oracle.statistics(c, s, 25 * 5e-4, omp=True)
    assert st[0] == pytest.approx(gold[0], rel=1e-12)
    for col in (1, 2, 4, 5, 6):  # E_k, eps, dzeta, <u^2>, <v^2>
        assert abs(st[col] - gold[col]) / abs(gold[col]) < 1e-6, (col, st[col], gold[col])
    assert abs(st[3] - gold[3]) / abs(gold[3]) < 1e-5  # eps2
    assert abs(st[7] - gold[7]) / abs(gold[7]) < 1e-4  # <w^2>, grows from zero


def _ghost_line(f, n, closure, odd_sign):
    """Reference line with ghost values: periodic wrap or mirror (sign for odd)."""
    out = np.empty(n + 6)
    for m in range(-3, n + 3):
        if 0 <= m < n:
            out[m + 3] = f[m]
        elif closure == 0:
            out[m + 3] = f[m % n]
        else:
            r = -m if m < 0 else 2 * (n - 1) - m
            out[m + 3] = odd_sign * f[r]
    return out


@pytest.mark.parametrize("n", [6, 7, 11, 16])
@pytest.mark.parametrize("closure", [0, 1, 2])
def test_explicit_closures_equal_ghost_form(oracle, n, closure):
    """The explicit boundary rows of src/derivation.f90 equal the interior
    stencil on ghost values, bit for bit; the CUDA kernels use the ghost form."""
    rng = np.random.default_rng(n + 10 * closure)
    f = rng.standard_normal(n)
    d = 0.37
    F = np.asfortranarray(f.reshape(n, 1, 1).repeat(1, 1))
    F3 = np.asfortranarray(np.tile(f.reshape(n, 1, 1), (1, 1, 1)))
    # oracle along x on an (n,1,1) grid
    d1 = oracle.der1(F3, 0, closure, d)[:, 0, 0]
    d2 = oracle.der2(F3, 0, closure, d)[:, 0, 0]
    sign = -1.0 if closure == 2 else 1.0
    g = _ghost_line(f, n, 0 if closure == 0 else 1, sign)
    s60 = 60.0 * d
    a, b, c = 1.0 / s60, 9.0 / s60, 45.0 / s60
    t12 = 12.0 * d * d
    a2, b2, c2 = 1.0 / t12, 16.0 / t12, 30.0 / t12
    for i in range(n):
        v = g[i:i + 7]
        e1 = a * (v[6] - v[0]) - b * (v[5] - v[1]) + c * (v[4] - v[2])
        e2 = -a2 * (v[1] + v[5]) + b2 * (v[2] + v[4]) - c2 * v[3]
        assert d1[i] == e1, (i, d1[i], e1)
        assert d2[i] == e2, (i, d2[i], e2)
    del F


@pytest.mark.parametrize("axis", [0, 1, 2])
def test_periodic_orders(oracle, axis):
    """6th order for the first derivative, 4th for the second (periodic)."""
    errs1, errs2 = [], []
    for n in (16, 32):
        h = 2 * PI / n
        x = np.arange(n) * h
        shape = [1, 1, 1]
        shape[axis] = n
        f = np.asfortranarray(np.broadcast_to(np.sin(x).reshape(shape), (n, n, n)).copy())
        ex1 = np.broadcast_to(np.cos(x).reshape(shape), (n, n, n))
        ex2 = np.broadcast_to(-np.sin(x).reshape(shape), (n, n, n))
        errs1.append(np.abs(oracle.der1(f, axis, oracle.PERIODIC, h) - ex1).max())
        errs2.append(np.abs(oracle.der2(f, axis, oracle.PERIODIC, h) - ex2).max())
    assert math.log2(errs1[0] / errs1[1]) > 5.8
    assert math.log2(errs2[0] / errs2[1]) > 3.8


def test_sor_manufactured(oracle):
    """Lexicographic SOR converges to the discrete solution of a manufactured
    periodic problem (the 7-point operator of src/poisson.f90)."""
    n = 16
    L = 2 * PI * (n - 1) / n
    c = oracle.Case(n, n, n, L, L, L)
    h = L / (n - 1)
    x = np.arange(n) * h
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    p_true = np.asfortranarray(np.sin(X) * np.cos(2 * Y) + 0.3 * np.cos(Z))
    lap = (np.roll(p_true, 1, 0) + np.roll(p_true, -1, 0) + np.roll(p_true, 1, 1) + np.roll(p_true, -1, 1)
           + np.roll(p_true, 1, 2) + np.roll(p_true, -1, 2) - 6 * p_true) / h ** 2
    rhs = np.asfortranarray(lap)
    pp = oracle.field3(c.shape)
    st, it, dm, om = oracle.poisson_sor(c, pp, rhs, 1.7, 1e-12, 20000)
    assert st == oracle.SOR_CONVERGED
    err = (pp - pp.mean()) - (p_true - p_true.mean())
    assert np.abs(err).max() < 1e-9


def test_rb_and_lexicographic_share_fixed_point(oracle):
    """Red-black and lexicographic SOR converge to the same pressure (up to
    the constant of the singular periodic problem)."""
    n = 12
    L = 2 * PI * (n - 1) / n
    c = oracle.Case(n, n, n, L, L, L, bcx=0, bcy=1, bcz=0)
    rng = np.random.default_rng(3)
    rhs = np.asfortranarray(rng.standard_normal(c.shape))
    # compatible rhs for the mirror operator: remove the trapezoid-weighted mean
    w = np.ones(n)
    w[0] = w[-1] = 0.5
    W = w.reshape(1, n, 1) * np.ones(c.shape)
    rhs -= (W * rhs).sum() / W.sum()
    rhs = np.asfortranarray(rhs)
    p1 = oracle.field3(c.shape)
    oracle.poisson_sor(c, p1, rhs, 1.6, 1e-13, 100000)
    p2 = oracle.field3(c.shape)
    for _ in range(20000):
        if oracle.rbsor_sweep(c, p2, rhs, 1.6) < 1e-13:
            break
    d = (p1 - p1.mean()) - (p2 - p2.mean())
    assert np.abs(d).max() < 1e-10


def test_mixing_layer_initial_state_matches_oracle(oracle, o3d):
    """The product's mixing-layer initial state (without noise) equals the
    oracle's restatement of src/initial_conditions.f90:329-394."""
    p = o3d.mixing_layer_params(16, 17, 8, ratio=0.5)
    ux, uy, uz, pp, phi = o3d.mixing_layer_fields(p, ratio=0.5, noise=0.0)
    c = oracle.Case(16, 17, 8, p.xlx, p.yly, p.zlz, bcx=0, bcy=1, bcz=0, dt=p.dt, y0=p.y0, nscr=1, ratio=0.5)
    s = oracle.State.zeros(c)
    oracle.init_mixing_layer(c, s)
    assert np.abs(ux - s.u[0]).max() < 1e-14
    assert np.abs(phi - s.phi).max() < 1e-14
    assert np.abs(pp - s.pp).max() == 0.0 and np.abs(uy).max() == 0.0


@pytest.mark.parametrize("n", [9, 16, 23])
def test_open_axis_closures_are_exact_on_polynomials(oracle, n):
    """The open x axis (this library's closure; the reference binds none):
    every row of the first derivative (2nd-order one-sided, 2nd/4th/6th
    central) is exact on quadratics, every row of the second derivative
    (2nd-order one-sided, 3-point and 5-point central) on cubics."""
    d = 0.37
    x = np.arange(n) * d
    shape = (n, 5, 4)
    quad = np.asfortranarray(np.broadcast_to((1.0 + 2.0 * x - 0.7 * x ** 2)[:, None, None], shape).copy())
    cub = np.asfortranarray(np.broadcast_to((1.0 + 2.0 * x - 0.7 * x ** 2 + 0.3 * x ** 3)[:, None, None],
                                            shape).copy())
    d1 = oracle.der1(quad, 0, oracle.OPEN, d)[:, 0, 0]
    d2 = oracle.der2(cub, 0, oracle.OPEN, d)[:, 0, 0]
    assert np.abs(d1 - (2.0 - 1.4 * x)).max() < 1e-12
    assert np.abs(d2 - (-1.4 + 1.8 * x)).max() < 1e-11


def test_coplanar_jet_initial_state_matches_oracle(oracle, o3d):
    """The product's co-planar jet initial state (without noise) equals the
    oracle's restatement of src/initial_conditions.f90:244-327."""
    p = o3d.coplanar_jet_params(17, 21, 9, ratio=0.5)
    ux, uy, uz, pp, phi = o3d.coplanar_jet_fields(p, ratio=0.5, noise=0.0)
    c = oracle.Case(17, 21, 9, p.xlx, p.yly, p.zlz, bcx=2, bcy=1, bcz=1, dt=p.dt, y0=p.y0, z0=p.z0, nscr=1,
                    ratio=0.5)
    s = oracle.State.zeros(c)
    oracle.init_coplanar_jet(c, s)
    assert np.abs(ux - s.u[0]).max() < 1e-14
    assert np.abs(phi - s.phi).max() < 1e-14
    assert np.abs(pp).max() == 0.0 and np.abs(uy).max() == 0.0 and np.abs(s.pp).max() == 0.0
    assert abs(ux.max() - 2.0) < 1e-3  # the inner jet, u0 / ratio
