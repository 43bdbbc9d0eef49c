"""GPU parity of the stencil kernels against the FP64 oracle, through the C ABI.

Tolerance: 1e-12 relative (max |gpu - oracle| / max |oracle|) in FP64; the
kernels contract a*b+c into fused multiply-adds, the oracle does not."""
import numpy as np
import pytest

from _util import PI, free_slip_case, open_x_case, params_of, perturbed, periodic_case, rel_err

pytestmark = pytest.mark.gpu

TOL = 1e-12

SHAPES = [
    # shape, (bcx, bcy, bcz)
    ((16, 12, 10), (0, 0, 0)),
    ((13, 17, 11), (1, 1, 1)),
    ((16, 9, 12), (0, 1, 0)),
    ((20, 33, 8), (0, 1, 1)),
    ((17, 13, 11), (2, 1, 1)),  # open x: one-sided closures at inflow and outflow
]


def _case(oracle, shape, bcs):
    nx, ny, nz = shape
    return oracle.Case(nx, ny, nz, 1.3, 0.9, 1.7, bcx=bcs[0], bcy=bcs[1], bcz=bcs[2])


@pytest.mark.parametrize("shape,bcs", SHAPES)
def test_all_derivative_operators(oracle, o3d, shape, bcs):
    """The 18 der* routines of src/derivation.f90 (3 axes x order 1/2 x even/odd
    closure, plus the periodic ones) on seeded random fields, odd sizes included."""
    c = _case(oracle, shape, bcs)
    rng = np.random.default_rng(sum(shape))
    f = np.asfortranarray(rng.standard_normal(shape))
    h = [c.xlx / (c.nx - 1), c.yly / (c.ny - 1), c.zlz / (c.nz - 1)]
    with o3d.Context(params_of(o3d, c)) as ctx:
        for axis in range(3):
            for order in (1, 2):
                for odd in (0, 1):
                    closure = (oracle.PERIODIC if bcs[axis] == 0 else oracle.OPEN if bcs[axis] == 2
                               else (oracle.ODD if odd else oracle.EVEN))
                    ref = (oracle.der1 if order == 1 else oracle.der2)(f, axis, closure, h[axis])
                    got = ctx.der(f, axis, order, bool(odd))
                    assert rel_err(got, ref) < TOL, (axis, order, odd)


def test_2d_mode_z_derivatives_vanish(oracle, o3d):
    c = oracle.Case(16, 16, 8, 1.0, 1.0, 1.0, sim2d=1)
    f = np.asfortranarray(np.random.default_rng(1).standard_normal(c.shape))
    with o3d.Context(params_of(o3d, c)) as ctx:
        assert np.all(ctx.der(f, 2, 1, False) == 0.0)
        assert np.all(ctx.der(f, 2, 2, True) == 0.0)


@pytest.mark.parametrize("shape,bcs", SHAPES)
def test_divergence(oracle, o3d, shape, bcs):
    c = _case(oracle, shape, bcs)
    rng = np.random.default_rng(7)
    fx, fy, fz = (np.asfortranarray(rng.standard_normal(shape)) for _ in range(3))
    with o3d.Context(params_of(o3d, c)) as ctx:
        for odd in (0, 1):
            ref = oracle.divergence(c, fx, fy, fz, odd)
            assert rel_err(ctx.divergence(fx, fy, fz, odd), ref) < TOL


@pytest.mark.parametrize("maker,n", [(free_slip_case, 17), (periodic_case, 16), (open_x_case, 15)])
def test_nu_t(oracle, o3d, maker, n):
    c = maker(oracle, n, iles=1, cs=0.17)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    u = [perturbed(s.u[a], a) for a in range(3)]
    ref = oracle.nu_t(c, *u)
    with o3d.Context(params_of(o3d, c)) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, u[a])
        assert rel_err(ctx.calculate_nu_t(), ref) < TOL


@pytest.mark.parametrize("iles", [0, 1])
@pytest.mark.parametrize("itscheme", [1, 2, 3])
@pytest.mark.parametrize("maker,n", [(free_slip_case, 17), (periodic_case, 16), (open_x_case, 15)])
def test_predictor_and_history(oracle, o3d, maker, n, itscheme, iles):
    """predict_velocity over itime = 1..4 (Euler / AB2 start-up, then the
    scheme), including the flux-history shift."""
    c = maker(oracle, n, iles=iles, itscheme=itscheme)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    s.u = [perturbed(s.u[a], 10 + a) for a in range(3)]
    with o3d.Context(params_of(o3d, c)) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        for itime in range(1, 5):
            oracle.predict_velocity(c, s, itime)
            ctx.predict_velocity(itime)
            for a, name in enumerate(("ux_pred", "uy_pred", "uz_pred")):
                assert rel_err(ctx.download(name), s.upred[a]) < TOL, (itime, name)
            for a in range(3):
                # newest flux = the reference's fux(:,:,:,1)
                assert rel_err(ctx.flux(a, 0), s.fu[3 * a]) < TOL
            if iles:
                assert rel_err(ctx.download("nu_t"), s.nu_t) < TOL


@pytest.mark.parametrize("maker,n", [(free_slip_case, 33), (periodic_case, 32), (open_x_case, 25)])
def test_statistics(oracle, o3d, maker, n):
    """statistics_calc (src/utils.f90:243-375): all 16 moments."""
    c = maker(oracle, n, re=1600.0)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    u = [perturbed(s.u[a], 20 + a) for a in range(3)]
    ref = oracle.statistics_of(c, u, 0.5)
    with o3d.Context(params_of(o3d, c)) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, u[a])
        got = ctx.statistics_calc(0.5)
    assert got[0] == 0.5
    for q in range(1, 17):
        assert abs(got[q] - ref[q]) <= 1e-12 * max(abs(ref[q]), 1e-30), (q, got[q], ref[q])


def test_golden_row0_on_gpu(oracle, o3d):
    """The reference's own t = 0 statistics row (185^3 free-slip TGV), computed
    by the GPU statistics kernel."""
    import os
    gold = np.loadtxt(os.path.join(os.path.dirname(__file__), "golden", "tgv_re1600_dns_stats_head.txt"))[0]
    c = oracle.Case(185, 185, 185, PI, PI, PI, bcx=1, bcy=1, bcz=1, re=1600.0)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s, omp=True)
    with o3d.Context(params_of(o3d, c)) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        got = ctx.statistics_calc(0.0)
    nz = gold != 0
    assert (np.abs(got[nz] - gold[nz]) / np.abs(gold[nz])).max() < 2e-12


def test_integer_pipe_conversions_are_bit_exact(o3d):
    """The FP64 <-> FP32 conversions the kernels do with integer arithmetic
    (round to nearest even) equal the conversion instructions bit for bit,
    over raw patterns, widened-and-nudged binary32 values, exact ties and the
    edges of the binary32 normal range."""
    assert o3d.check_conversions(1 << 24, seed=7) == 0


@pytest.mark.parametrize("maker,n", [("periodic", 16), ("free_slip", 13), ("open_x", 14)])
def test_vorticity_and_q_criterion(oracle, o3d, maker, n):
    """rotational and calculate_Q_criterion (src/differential_operators.f90:
    40-108) against the oracle, FP64, 1e-12."""
    c = {"periodic": periodic_case, "free_slip": free_slip_case, "open_x": open_x_case}[maker](oracle, n)
    rng = np.random.default_rng(21)
    u = [perturbed(np.asfortranarray(rng.standard_normal(c.shape)), 60 + a) for a in range(3)]
    rot = oracle.rotational(c, u)
    q = oracle.q_criterion(c, u)
    with o3d.Context(params_of(o3d, c)) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, u[a])
        got = ctx.vorticity()
    for a in range(3):
        assert rel_err(got[a], rot[a]) < 1e-12, a
    assert rel_err(got[3], q) < 1e-12


def test_velocity_residuals(oracle, o3d):
    """calculate_residuals (src/utils.f90:93-163) of a step against the kept
    old velocity: rms, max and the max's location equal the oracle's."""
    c = periodic_case(oracle, 16, omega=1.6, eps=1e-11, kmax=100000)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    with o3d.Context(params_of(o3d, c)) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        ctx.upload("pp", s.pp)
        ctx.save_old_velocity()
        old = [ctx.download(nm) for nm in ("ux", "uy", "uz")]
        ctx.step(1)
        got = ctx.velocity_residuals(t_ref=2.0, u_ref=0.5)
        new = [ctx.download(nm) for nm in ("ux", "uy", "uz")]
    ref = oracle.residuals(c, new, old, c.dt, 2.0, 0.5)
    assert np.abs(got[:6] - ref[:6]).max() < 1e-12 * np.abs(ref[:6]).max()
    assert (got[6:] == ref[6:]).all(), (got[6:], ref[6:])
