"""Whole time steps on the GPU (src/osinco3d_main.f90:104-128) against the
oracle's time loop: velocity, pressure, flux history, scalar and the per-step
diagnostics after N steps.

Both sides solve the pressure to eps = 1e-11 so that the red-black versus
lexicographic iterate order leaves differences far below the tolerance:
velocity 1e-9 relative; pressure (mean removed) 1e-8 of max |p| plus
100 eps for the update-norm stop test."""
import numpy as np
import pytest

from _util import PI, free_slip_case, kinds_of, params_of, periodic_case, perturbed, rel_err

pytestmark = pytest.mark.gpu

EPS = 1e-11


def _run_both(oracle, o3d, c, nsteps, init="tgv", **extra):
    s = oracle.State.zeros(c)
    if init == "tgv":
        oracle.init_tgv(c, s)
    elif init == "jet":
        oracle.init_coplanar_jet(c, s)
    else:
        oracle.init_mixing_layer(c, s)
    # a smooth seeded perturbation (with each component's free-slip parity)
    # breaks the symmetries of the analytic states
    for a in range(3):
        s.u[a][...] = perturbed(s.u[a], 30 + a, kinds=kinds_of(c, a))
    runner = oracle.Runner(c, s)
    ctx = o3d.Context(params_of(o3d, c, **extra))
    for a, name in enumerate(("ux", "uy", "uz")):
        ctx.upload(name, s.u[a])
    ctx.upload("pp", s.pp)
    if c.nscr:
        ctx.upload("phi", s.phi)
        ctx.upload("src", s.src)
    infos = []
    for it in range(1, nsteps + 1):
        ri = runner.step(it)
        gi = ctx.step(it)
        # a compatible right-hand side: the reference's SOR converges
        assert ri.sor_status == oracle.SOR_CONVERGED, (it, ri.sor_status)
        infos.append((ri, gi))
    return s, ctx, infos


def _check_fields(s, ctx, c, tol_u=1e-9, tol_p=1e-8):
    for a, name in enumerate(("ux", "uy", "uz")):
        ref = s.u[a]
        if np.abs(ref).max() == 0:
            assert np.abs(ctx.download(name)).max() < 1e-12
        else:
            assert rel_err(ctx.download(name), ref) < tol_u, name
    # pressure up to its free constant: relative to max |p|, plus the SOR
    # stop-test error (about 50 eps on the mirror grids)
    p = ctx.download("pp")
    dp = np.abs((p - p.mean()) - (s.pp - s.pp.mean())).max()
    assert dp <= tol_p * np.abs(s.pp).max() + 100 * c.eps, dp
    if c.nscr:
        assert rel_err(ctx.download("phi"), s.phi) < tol_u


@pytest.mark.parametrize("itscheme", [2, 3])
def test_tgv_periodic_steps(oracle, o3d, itscheme):
    c = periodic_case(oracle, 32, itscheme=itscheme, omega=1.6, eps=EPS, kmax=100000)
    s, ctx, infos = _run_both(oracle, o3d, c, 6)
    _check_fields(s, ctx, c)
    for ri, gi in infos:
        assert gi.poisson_status == 0 and ri.sor_status == 0
        assert gi.diverged == 0
        # per-step diagnostics the driver prints
        for q in range(3):
            assert gi.divu_pred_stats[q] == pytest.approx(ri.divu_pred_stats[q], rel=1e-7, abs=1e-9)
            assert gi.divu_stats[q] == pytest.approx(ri.divu_stats[q], rel=1e-6, abs=1e-8)
        for q in range(3):
            assert gi.cfl[q] == pytest.approx(ri.cfl[q], rel=1e-8, abs=1e-14)
    ctx.close()


def test_free_slip_les_scalar_steps(oracle, o3d):
    """Free-slip box (poisson_solver_111111), Smagorinsky LES and the passive
    scalar with its conservative clipping."""
    c = free_slip_case(oracle, 33, iles=1, cs=0.17, nscr=1, sc=0.7, omega=1.7, eps=EPS, kmax=100000,
                       re=1600.0)
    s, ctx, infos = _run_both(oracle, o3d, c, 5)
    _check_fields(s, ctx, c)
    assert rel_err(ctx.download("nu_t"), s.nu_t) < 1e-9
    ctx.close()


def test_mixing_layer_0011_steps(oracle, o3d):
    """x/z periodic, y free-slip (poisson_solver_0011), mixing-layer initial
    state of src/initial_conditions.f90:364-389, LES and scalar."""
    nx, ny, nz = 32, 33, 16
    c = oracle.Case(nx, ny, nz, 12.0 * (nx - 1) / nx, 12.0, 4.0 * (nz - 1) / nz, bcx=0, bcy=1, bcz=0,
                    y0=-6.0, z0=-2.0, ratio=0.5, re=3000.0, iles=1, cs=0.17, nscr=1, sc=1.0,
                    dt=0.01, omega=1.7, eps=EPS, kmax=100000)
    s, ctx, infos = _run_both(oracle, o3d, c, 4, init="ml")
    _check_fields(s, ctx, c)
    ctx.close()


def _jet_case(oracle, **kw):
    # Neumann on every face: SOR contracts slowly, so both sides solve to
    # 1e-13 to keep the oracle's update-norm stop error below the tolerance
    nx, ny, nz = 33, 33, 17
    base = dict(bcx=2, bcy=1, bcz=1, y0=-2.0, z0=-1.0, ratio=0.5, re=2200.0, iles=1, cs=0.17, nscr=1,
                sc=0.7, dt=0.02, omega=1.7, eps=1e-13, kmax=200000)
    base.update(kw)
    return oracle.Case(nx, ny, nz, 8.0, 4.0, 2.0, **base)


@pytest.mark.parametrize("solver", [0, 1])
def test_coplanar_jet_open_x_steps(oracle, o3d, solver):
    """Open x axis (inflow held at x(1), outflow at x(nx), dery1D-style
    one-sided closures, Neumann pressure), y/z free-slip, the co-planar jet
    of src/initial_conditions.f90:244-327 with LES and scalar: SOR and
    multigrid steps against the oracle's."""
    c = _jet_case(oracle)
    s, ctx, infos = _run_both(oracle, o3d, c, 4, init="jet", solver=solver)
    _check_fields(s, ctx, c)
    # the inflow plane kept its initial values
    for a, name in enumerate(("ux", "uy", "uz")):
        assert np.array_equal(ctx.download(name)[0], s.u[a][0])
    for ri, gi in infos:
        assert gi.diverged == 0
    ctx.close()


@pytest.mark.parametrize("solver", ["sor", "mg"])
def test_mixing_layer_odd_periodic_steps(oracle, o3d, solver):
    """The layout of the reference's mixing-layer example (odd point counts
    on the periodic x and z axes, src/../examples/mixing_layer_re3000_les:
    241 x 241 x 81), scaled down: red-black SOR with the seam classes of the
    odd periodic axes, and the multigrid with those axes coarsened onto
    non-nested grids, reach the lexicographic solver's fixed point."""
    nx, ny, nz = 31, 33, 17
    c = oracle.Case(nx, ny, nz, 12.0 * (nx - 1) / nx, 12.0, 4.0 * (nz - 1) / nz, bcx=0, bcy=1, bcz=0,
                    y0=-6.0, z0=-2.0, ratio=0.5, re=3000.0, iles=1, cs=0.17, nscr=1, sc=1.0,
                    dt=0.01, omega=1.7, eps=EPS, kmax=100000)
    kw = {} if solver == "sor" else {"solver": o3d.SOLVER_MG, "kmax": 200}
    s, ctx, infos = _run_both(oracle, o3d, c, 3, init="ml", **kw)
    _check_fields(s, ctx, c)
    ctx.close()


@pytest.mark.parametrize("guess,cycles", [(0, 1), (0, 2), (3, 1), (4, 1), (1, 1)])
def test_multigrid_step_matches(oracle, o3d, guess, cycles):
    """The multigrid solver inside the step gives the same velocity, whatever
    the initial guess (previous, linear or quadratic extrapolation in time,
    zero) and the number of V-cycles per FP64 residual."""
    c = periodic_case(oracle, 32, omega=1.6, eps=EPS, kmax=100000)
    s, ctx, infos = _run_both(oracle, o3d, c, 4, solver=o3d.SOLVER_MG, kmax=200, guess=guess,
                              mg_cycles=cycles)
    _check_fields(s, ctx, c)
    for ri, gi in infos:
        assert gi.poisson_status == 0
        assert gi.poisson_cycles == cycles * gi.poisson_iters
    ctx.close()


def test_mixed_precision_step_error(oracle, o3d):
    """FP32 stencils + FP32 V-cycles in FP64 defect correction: error against
    the FP64 oracle after 10 steps stays at FP32 rounding level."""
    c = periodic_case(oracle, 32, omega=1.6, eps=1e-10, kmax=100000)
    s, ctx, infos = _run_both(oracle, o3d, c, 10, solver=o3d.SOLVER_MG, precision=o3d.PREC_MIXED,
                              kmax=200, eps=1e-8)
    for a, name in enumerate(("ux", "uy", "uz")):
        assert rel_err(ctx.download(name), s.u[a]) < 1e-5, name
    ctx.close()


def test_mixed_precision_open_x_jet(oracle, o3d):
    """The mixed method on the open-x co-planar jet (FP32 stencils with the
    one-sided closures, FP32 V-cycles in FP64 defect correction): error
    against the FP64 oracle after 6 steps at FP32 rounding level of the jet
    velocity (the cross-stream components start at the 1e-2 perturbation),
    and the inflow plane held to FP32 rounding."""
    c = _jet_case(oracle)
    s, ctx, infos = _run_both(oracle, o3d, c, 6, init="jet", solver=o3d.SOLVER_MG,
                              precision=o3d.PREC_MIXED, kmax=200, eps=1e-8)
    U = np.abs(s.u[0]).max()
    for a, name in enumerate(("ux", "uy", "uz")):
        got = ctx.download(name)
        assert np.abs(got - s.u[a]).max() < 1e-5 * U, name
        assert np.abs(got[0] - s.u[a][0]).max() <= 1e-7 * U
    assert rel_err(ctx.download("phi"), s.phi) < 1e-5
    ctx.close()


def test_step_host_equals_step(oracle, o3d):
    """o3d_step_host (driver arrays copied in and out) = o3d_step."""
    c = periodic_case(oracle, 16, omega=1.6, eps=1e-10, kmax=100000)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    p = params_of(o3d, c)
    with o3d.Context(p) as a, o3d.Context(p) as b:
        u = [x.copy(order="F") for x in s.u]
        pp = s.pp.copy(order="F")
        for name, f in zip(("ux", "uy", "uz", "pp"), u + [pp]):
            a.upload(name, f)
        for it in (1, 2, 3):
            a.step(it)
            b.step_host(it, u[0], u[1], u[2], pp)
        for q, name in enumerate(("ux", "uy", "uz")):
            assert np.array_equal(a.download(name), u[q])
        assert np.array_equal(a.download("pp"), pp)


def test_fault_nan_velocity_reports_nonfinite(oracle, o3d):
    """A NaN planted in the input makes the step return O3D_ERR_NONFINITE
    where the reference stops (src/integration.f90:309-325); the context
    remains usable."""
    c = periodic_case(oracle, 16, omega=1.6, eps=1e-8, kmax=50)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    with o3d.Context(params_of(o3d, c)) as ctx:
        u = s.u[0].copy(order="F")
        u[3, 4, 5] = np.nan
        ctx.upload("ux", u)
        ctx.upload("uy", s.u[1])
        with pytest.raises(o3d.O3DError) as ei:
            ctx.step(1)
        assert ei.value.code == o3d.ERR_NONFINITE
        # recover: fresh finite state, the next step succeeds
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        ctx.upload("pp", s.pp)
        ctx.step(1)


def test_fault_kmax_reports_maxit(oracle, o3d):
    c = periodic_case(oracle, 16, omega=1.6, eps=1e-14, kmax=3)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    with o3d.Context(params_of(o3d, c)) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        info = ctx.step(1)
        assert ctx.last_status == o3d.WARN_POISSON_MAXIT
        assert info.poisson_iters == 3
