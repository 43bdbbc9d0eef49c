"""GPU pressure solvers against the oracle's lexicographic SOR
(src/poisson.f90), through o3d_poisson_solve (the poi_type interface).

Red-black SOR and multigrid converge to the fixed point of the same 7-point
operator; they are compared with the oracle solved to eps * 1e-3, after
removing the free constant of the singular problem.  Tolerance: the
pressure error of an update-norm stop at eps is about eps * rho / (1 - rho)
with rho the sweep's contraction factor (near 0.98 on the 33^3 mirror grid
at omega = 1.8, measured on the oracle's red-black sweep: error 57 eps); the
tests allow 200 eps (SOR) and 5 eps (multigrid, whose stop test is on the
whole correction)."""
import numpy as np
import pytest

from _util import PI, params_of, rel_err

pytestmark = pytest.mark.gpu

VARIANTS = [
    # (nx, ny, nz), (bcx, bcy, bcz): 0000, 0011, 111111 solvers
    ((32, 32, 32), (0, 0, 0)),
    ((32, 33, 16), (0, 1, 0)),
    ((33, 33, 33), (1, 1, 1)),
]


def _case(oracle, shape, bcs, **kw):
    nx, ny, nz = shape
    L = [2 * PI * (n - 1) / n if b == 0 else PI for n, b in zip(shape, bcs)]
    return oracle.Case(nx, ny, nz, L[0], L[1], L[2], bcx=bcs[0], bcy=bcs[1], bcz=bcs[2], **kw)


def _compatible_rhs(c, seed):
    """Smooth seeded rhs with zero trapezoid-weighted mean on the Poisson grid."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = c.shape
    x = np.linspace(0, 1, nx)[:, None, None]
    y = np.linspace(0, 1, ny)[None, :, None]
    z = np.linspace(0, 1, nz)[None, None, :]
    r = np.zeros(c.shape)
    for _ in range(4):
        a, b, d = rng.integers(1, 4, 3)
        r += rng.standard_normal() * np.cos(2 * PI * a * x) * np.cos(2 * PI * b * y) * np.cos(2 * PI * d * z)
    r += 0.05 * rng.standard_normal(c.shape)
    mirror = [c.bcx, c.bcy, 1 if c.bcx == 1 else 0]  # the 0011 solver keeps z periodic
    W = np.ones(c.shape)
    for ax, m in enumerate(mirror):
        if m:
            w = np.ones(c.shape[ax])
            w[0] = w[-1] = 0.5
            sh = [1, 1, 1]
            sh[ax] = -1
            W = W * w.reshape(sh)
    r -= (W * r).sum() / W.sum()
    return np.asfortranarray(r)


def _demean(p):
    return p - p.mean()


@pytest.mark.parametrize("shape,bcs", VARIANTS)
def test_one_red_black_sweep(oracle, o3d, shape, bcs):
    """kmax = 1: exactly one red-black sweep, same values and same max
    |p_gs - p| as the oracle's red-black sweep."""
    c = _case(oracle, shape, bcs)
    rng = np.random.default_rng(1)
    p0 = np.asfortranarray(rng.standard_normal(c.shape))
    rhs = np.asfortranarray(rng.standard_normal(c.shape))
    for sweeps in (1, 3):
        ref = p0.copy(order="F")
        for _ in range(sweeps):
            dref = oracle.rbsor_sweep(c, ref, rhs, 1.37)
        with o3d.Context(params_of(o3d, c, solver=o3d.SOLVER_SOR)) as ctx:
            got = p0.copy(order="F")
            st, it, dm, om = ctx.poisson_solve(got, rhs, 1.37, 0.0, sweeps, 0)
        assert st == o3d.WARN_POISSON_MAXIT and it == sweeps
        assert rel_err(got, ref) < 1e-13
        assert dm == pytest.approx(dref, rel=1e-11)


@pytest.mark.parametrize("shape,bcs", VARIANTS)
@pytest.mark.parametrize("solver", ["sor", "mg"])
def test_fixed_point_matches_lexicographic_sor(oracle, o3d, shape, bcs, solver):
    eps = 1e-9
    c = _case(oracle, shape, bcs)
    rhs = _compatible_rhs(c, 5)
    ref = oracle.field3(c.shape)
    st, _, _, _ = oracle.poisson_sor(c, ref, rhs, 1.8, eps * 1e-3, 200000)
    assert st == oracle.SOR_CONVERGED
    kind = o3d.SOLVER_SOR if solver == "sor" else o3d.SOLVER_MG
    with o3d.Context(params_of(o3d, c, solver=kind)) as ctx:
        got = ctx.field()
        st, it, dm, om = ctx.poisson_solve(got, rhs, 1.8, eps, 100000 if solver == "sor" else 100, 0)
    assert st == o3d.OK, (st, it, dm)
    assert dm < eps
    err = np.abs(_demean(got) - _demean(ref)).max()
    assert err < (200 * eps if solver == "sor" else 5 * eps), (err, it)


@pytest.mark.parametrize("shape,bcs", [((15, 15, 15), (0, 0, 0)), ((17, 17, 9), (0, 1, 0))])
def test_odd_periodic_sor_fixed_point(oracle, o3d, shape, bcs):
    """Odd point counts on periodic axes: the red-black sweep adds seam-class
    passes (the wrap plane of each odd periodic axis) and still reaches the
    lexicographic SOR fixed point."""
    eps = 1e-9
    c = _case(oracle, shape, bcs)
    rhs = _compatible_rhs(c, 3)
    ref = oracle.field3(c.shape)
    st, _, _, _ = oracle.poisson_sor(c, ref, rhs, 1.6, eps * 1e-3, 200000)
    assert st == oracle.SOR_CONVERGED
    with o3d.Context(params_of(o3d, c, solver=o3d.SOLVER_SOR)) as ctx:
        got = ctx.field()
        st, it, dm, om = ctx.poisson_solve(got, rhs, 1.6, eps, 100000, 0)
    assert st == o3d.OK, (st, it, dm)
    err = np.abs(_demean(got) - _demean(ref)).max()
    assert err < 200 * eps, (err, it)


NON_NESTED = [
    # (shape, boundaries, the neighbouring shape whose axes all halve onto
    # every other node): an even free-slip axis, an odd periodic axis, and
    # the reference's mixing-layer layout (odd periodic x and z) with an even
    # free-slip y
    ((32, 32, 16), (0, 1, 0), (32, 33, 16)),
    ((33, 32, 32), (0, 0, 0), (32, 32, 32)),
    ((31, 32, 17), (0, 1, 0), (32, 33, 16)),
    # a non-nested transfer between the last two levels: y 19 -> 10 -> 5
    # (even free-slip at 16 x 10 x 16), z 36 -> 18 -> 9 -> 4 (odd periodic
    # at 8 x 8 x 9)
    ((32, 19, 32), (0, 1, 0), (32, 17, 32)),
    ((32, 32, 36), (0, 0, 0), (32, 32, 32)),
]


def _mg_solve(oracle, o3d, shape, bcs, eps, **kw):
    c = _case(oracle, shape, bcs)
    rhs = _compatible_rhs(c, 5)
    with o3d.Context(params_of(o3d, c, solver=o3d.SOLVER_MG, **kw)) as ctx:
        got = ctx.field()
        st, it, dm, om = ctx.poisson_solve(got, rhs, 1.0, eps, 400, 0)
    assert st == o3d.OK, (st, it, dm)
    return c, rhs, got, it


@pytest.mark.parametrize("shape,bcs,nested", NON_NESTED)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_non_nested_coarsening_multigrid(oracle, o3d, shape, bcs, nested, precision):
    """An axis that cannot be halved onto every other node (even free-slip,
    odd periodic) is coarsened onto a non-nested grid of about half the
    nodes, with linear interpolation and its transpose: the multigrid reaches
    the lexicographic SOR fixed point, in about as many V-cycles as on the
    neighbouring size (keeping the axis instead, semi-coarsening, takes 5 to
    20 more at these sizes)."""
    eps = 1e-9
    kw = {} if precision == "fp64" else {"precision": o3d.PREC_MIXED}
    c, rhs, got, it = _mg_solve(oracle, o3d, shape, bcs, eps, **kw)
    ref = oracle.field3(c.shape)
    st, _, _, _ = oracle.poisson_sor(c, ref, rhs, 1.8, eps * 1e-3, 200000)
    assert st == oracle.SOR_CONVERGED
    err = np.abs(_demean(got) - _demean(ref)).max()
    tol = 5 * eps if precision == "fp64" else 1e-6 * np.abs(ref).max() + 5 * eps
    assert err < tol, (err, it)
    _, _, _, it_nested = _mg_solve(oracle, o3d, nested, bcs, eps, **kw)
    assert it <= it_nested + 2, (it, it_nested)


@pytest.mark.parametrize("shape,bcs", VARIANTS)
def test_mixed_precision_multigrid(oracle, o3d, shape, bcs):
    """FP32 V-cycles inside the FP64 correction loop reach the FP64 fixed point."""
    eps = 1e-9
    c = _case(oracle, shape, bcs)
    rhs = _compatible_rhs(c, 9)
    ref = oracle.field3(c.shape)
    oracle.poisson_sor(c, ref, rhs, 1.8, eps * 1e-3, 200000)
    with o3d.Context(params_of(o3d, c, solver=o3d.SOLVER_MG, precision=o3d.PREC_MIXED)) as ctx:
        got = ctx.field()
        st, it, dm, om = ctx.poisson_solve(got, rhs, 1.0, eps, 100, 0)
    assert st == o3d.OK, (st, it, dm)
    err = np.abs(_demean(got) - _demean(ref)).max()
    assert err < 1e-6 * np.abs(ref).max() + 5 * eps, err


FUSED_CASES = [
    # shape, boundaries, multigrid options, the mg_kernels mode compared with
    # one kernel per pass (1): 2 fuses every level the kernels can serve (at
    # these sizes all but the coarsest, with partial tiles), 0 only the levels
    # of at least 152 blocks, and on a level of 2^22 points or more it runs
    # the pre-smoothing of a V(1, *) cycle from zero, the residual and the
    # restriction as 2.5D one-pass kernels before the fused k_mg_up.  The
    # zero-start and from-correction kernels, V(2,1), V(1,1) and V(1,2), odd
    # free-slip sizes, and fused levels below a non-nested one.
    ((64, 64, 64), (0, 0, 0), {"mg_pre": 2, "mg_post": 1}, 2),
    ((64, 65, 32), (0, 1, 0), {"mg_cycles": 2}, 2),
    ((33, 33, 33), (1, 1, 1), {"mg_pre": 1, "mg_post": 2}, 2),
    ((64, 64, 32), (0, 1, 0), {}, 2),
    ((256, 256, 64), (0, 0, 0), {}, 0),
    ((256, 256, 64), (0, 0, 0), {"mg_cycles": 2}, 0),  # the second cycle starts from its correction
    ((256, 256, 64), (0, 0, 0), {}, 2),
    # a large level with a non-nested y axis: its 2.5D one-pass smoothing
    # and residual against the plain kernels
    ((256, 256, 64), (0, 1, 0), {"mg_pre": 2, "mg_post": 1}, 0),
]


@pytest.mark.parametrize("shape,bcs,kw,mode", FUSED_CASES)
def test_fused_level_kernels_match_unfused(oracle, o3d, shape, bcs, kw, mode):
    """The fused level kernels (pre-smoothing + residual + restriction, and
    prolongation + post-smoothing + update) evaluate the expressions of the
    one-pass kernels in the same order: both solves agree bit for bit."""
    c = _case(oracle, shape, bcs)
    rhs = _compatible_rhs(c, 13)
    out = []
    for mk in (mode, 1):
        prm = params_of(o3d, c, solver=o3d.SOLVER_MG, precision=o3d.PREC_MIXED, mg_kernels=mk, **kw)
        with o3d.Context(prm) as ctx:
            got = ctx.field()
            n0 = ctx.launches
            st, it, dm, om = ctx.poisson_solve(got, rhs, 1.0, 1e-9, 100, 0)
            per_cycle = (ctx.launches - n0) / it
        out.append((st, it, dm, got, per_cycle))
    assert out[0][0] == o3d.OK
    assert out[0][:3] == out[1][:3]
    np.testing.assert_array_equal(out[0][3], out[1][3])
    # the fused levels ran: fewer launches per outer iteration (a grid whose
    # levels all have a non-nested axis fuses none, with as many launches)
    if bcs != (0, 1, 0) or shape[0] < 256:
        assert out[0][4] < out[1][4], (out[0][4], out[1][4])


OMEGA_CASES = [
    # shape, boundaries (solver variant and its factor), initial omega, rhs:
    # 0000 and 111111 use factor 1.05 (src/poisson.f90:35,288), 0011 1.01
    # (:162); the constant rhs on the all-mirror grid has no solution and
    # ends on the stagnation test
    ((32, 32, 32), (0, 0, 0), 1.8, "smooth"),
    ((32, 33, 16), (0, 1, 0), 1.8, "smooth"),
    ((33, 33, 33), (1, 1, 1), 1.8, "smooth"),
    ((32, 32, 32), (0, 0, 0), 1.5, "smooth"),
    ((17, 17, 17), (1, 1, 1), 1.9, "constant"),
]


@pytest.mark.parametrize("shape,bcs,om0,kind", OMEGA_CASES)
def test_dynamic_omega_trajectory_and_exit_match_oracle(oracle, o3d, shape, bcs, om0, kind):
    """idyn = 1: the GPU red-black SOR applies src/poisson.f90:110-122 after
    every sweep.  The oracle drives its red-black sweep with the same rule
    (orc_poisson_rbsor); omega after k sweeps (a solve capped at kmax = k),
    the exit iteration, the exit status and the final omega are identical,
    and the last update norm agrees to rounding."""
    c = _case(oracle, shape, bcs)
    rhs = _compatible_rhs(c, 11) if kind == "smooth" else np.asfortranarray(np.ones(c.shape))
    eps = 1e-8
    st_ref, it_ref, dm_ref, om_ref, otr, dtr = oracle.poisson_rbsor(c, oracle.field3(c.shape), rhs, om0, eps,
                                                                    20000, 1)
    want = oracle.SOR_CONVERGED if kind == "smooth" else oracle.SOR_STAGNATED
    assert st_ref == want
    assert np.count_nonzero(np.diff(otr)) >= 1  # the rule changed omega at least once
    code = {oracle.SOR_CONVERGED: o3d.OK, oracle.SOR_STAGNATED: o3d.WARN_STAGNATION}[st_ref]
    with o3d.Context(params_of(o3d, c)) as ctx:
        got = ctx.field()
        st, it, dm, om = ctx.poisson_solve(got, rhs, om0, eps, 20000, 1)
        assert (st, it) == (code, it_ref)
        assert om == om_ref  # bit-identical: same factors applied in the same order
        assert dm == pytest.approx(dm_ref, rel=1e-6)
        # the trajectory: every sweep where omega changed, its neighbours, and
        # points across the 16-sweep batches
        ks = {1, 2, 3, 15, 16, 17, 31, 32, 33, it_ref - 1}
        for q in np.flatnonzero(np.diff(otr)):
            ks |= {int(q) + 1, int(q) + 2, int(q) + 3}
        for k in sorted(x for x in ks if 1 <= x < it_ref):
            got = ctx.field()
            st_k, it_k, dm_k, om_k = ctx.poisson_solve(got, rhs, om0, eps, k, 1)
            assert (st_k, it_k) == (o3d.WARN_POISSON_MAXIT, k), k
            assert om_k == otr[k - 1], (k, om_k, otr[k - 1])
            assert dm_k == pytest.approx(dtr[k - 1], rel=1e-6), k


def test_incompatible_rhs_stagnates_like_reference(oracle, o3d):
    """A constant rhs on the all-mirror grid has no solution; the reference's
    SOR ends on its stagnation test (src/poisson.f90:111-114) and so does the
    GPU red-black SOR."""
    c = _case(oracle, (17, 17, 17), (1, 1, 1))
    rhs = np.asfortranarray(np.ones(c.shape))
    ref = oracle.field3(c.shape)
    st_ref, _, _, _ = oracle.poisson_sor(c, ref, rhs, 1.5, 1e-8, 20000)
    with o3d.Context(params_of(o3d, c)) as ctx:
        got = ctx.field()
        st, it, dm, om = ctx.poisson_solve(got, rhs, 1.5, 1e-8, 20000, 0)
    assert st_ref == oracle.SOR_STAGNATED
    assert st == o3d.WARN_STAGNATION


def test_two_point_residual_matches_one_point(oracle, o3d):
    """Mixed multigrid steps with the FP32 rhs on a grid whose nx is a
    multiple of 64 take the residual with two points per thread; with one
    plain kernel per pass (mg_kernels = 1) they take the one-point residual.
    The velocity and the pressure after three steps agree bit for bit."""
    c = _case(oracle, (128, 32, 32), (0, 0, 0))
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    out = []
    for mk in (0, 1):
        prm = params_of(o3d, c, solver=o3d.SOLVER_MG, precision=o3d.PREC_MIXED, eps=1e-9, kmax=100,
                        guess=o3d.GUESS_EXTRAPOLATED2, mg_kernels=mk)
        with o3d.Context(prm) as ctx:
            for nm, f in zip(("ux", "uy", "uz", "pp"), (s.u[0], s.u[1], s.u[2], s.pp)):
                ctx.upload(nm, f)
            for it in range(1, 4):
                assert ctx.step(it).poisson_status == o3d.OK
            out.append([ctx.download(nm) for nm in ("ux", "uy", "uz", "pp")])
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)
