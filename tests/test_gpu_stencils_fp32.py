"""The mixed method's FP32 stencil kernels against the FP64 oracle.

On grids with nx a multiple of 4 the mixed method runs the two-point
kernels of csrc/k_stencil25v.cu (two x-adjacent points per thread, 64 x 8
tiles, rows copied in 16-byte chunks); other grids run the one-point
kernels.  The cases cover a partial tile whose chunks lie past the x end
(nx = 40: per-cell ghost copies), mirrored axes with odd ny and nz (sign
flips of the odd components), the open x axis, LES, the 2D mode and the
Euler / AB2 start-up followed by AB3 over itime = 1..4, on both kernel
families.

Tolerance: the inputs are rounded to FP32 and every operation runs in
FP32, so u* is compared at 2e-6 of max |u*| and the new flux at 1e-5 of max
|F| (a unit roundoff of 6e-8 amplified by the stencil coefficients and the
cancellation in the derivatives), nu_t at 1e-5.
"""
import numpy as np
import pytest

from _util import PI, kinds_of, params_of, perturbed, rel_err

pytestmark = pytest.mark.gpu

CASES = [
    # shape, boundaries (x, y, z), extra case parameters
    ((64, 24, 40), (0, 0, 0), {}),
    ((40, 16, 30), (0, 0, 0), {}),           # partial x tile: chunks past nx
    ((36, 33, 29), (1, 1, 1), {}),           # mirror flips, odd ny and nz
    ((128, 17, 19), (0, 1, 0), {}),          # two x tiles, mixing-layer boundaries
    ((44, 25, 21), (2, 1, 1), {}),           # open x axis
    ((64, 24, 16), (0, 0, 0), {"sim2d": 1}),  # 2D mode: no z derivatives
    ((33, 20, 24), (0, 1, 0), {}),           # nx not a multiple of 4: one-point kernel
    ((132, 24, 16), (0, 1, 0), {}),          # a tile with no ghost-mapped halo
]


def _case(oracle, shape, bcs, **kw):
    lens = [2 * PI * (n - 1) / n if b == 0 else PI for n, b in zip(shape, bcs)]
    dt = 0.1 * min(L / (n - 1) for L, n in zip(lens, shape))
    return oracle.Case(shape[0], shape[1], shape[2], lens[0], lens[1], lens[2], bcx=bcs[0], bcy=bcs[1],
                       bcz=bcs[2], dt=dt, **kw)


@pytest.mark.parametrize("iles", [0, 1])
@pytest.mark.parametrize("shape,bcs,kw", CASES)
def test_fp32_predictor_matches_oracle(oracle, o3d, shape, bcs, kw, iles):
    c = _case(oracle, shape, bcs, iles=iles, cs=0.17, itscheme=3, **kw)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    s.u = [perturbed(s.u[a], 40 + a, amp=0.05, kinds=kinds_of(c, a)) for a in range(3)]
    if c.sim2d:
        s.u[2][...] = 0.0
    with o3d.Context(params_of(o3d, c, precision=o3d.PREC_MIXED, solver=o3d.SOLVER_MG)) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        for itime in range(1, 5):
            oracle.predict_velocity(c, s, itime)
            ctx.predict_velocity(itime)
            for a, name in enumerate(("ux_pred", "uy_pred", "uz_pred")):
                if np.abs(s.upred[a]).max() == 0:
                    assert np.abs(ctx.download(name)).max() == 0
                    continue
                assert rel_err(ctx.download(name), s.upred[a]) < 2e-6, (itime, name)
            for a in range(3):
                ref = s.fu[3 * a]
                if np.abs(ref).max() == 0:
                    continue
                assert rel_err(ctx.flux(a, 0), ref) < 1e-5, (itime, a)
            if iles:
                assert rel_err(ctx.download("nu_t"), s.nu_t) < 1e-5, itime
            # the predictor's output becomes the next step's input, as after
            # a correction, so the history ring turns with new data
            for a, name in enumerate(("ux", "uy", "uz")):
                s.u[a][...] = s.upred[a]
                ctx.upload(name, s.u[a])


@pytest.mark.parametrize("shape,bcs,kw", [c for c in CASES if not c[2]])
def test_fp32_kernels_in_mixed_steps_match_oracle(oracle, o3d, shape, bcs, kw):
    """Three whole mixed-method steps (predictor, divergence -> FP64 rhs with
    its weighted sum, multigrid in the FP64 defect correction, correction
    with its extrema, diagnostic divergence) against the oracle's FP64 steps
    with its SOR solved to 1e-12.  Velocity within 2e-5 of max |u|; pressure
    (mean removed) within 1e-5 of max |u|^2: the FP32 rounding of u* sets its
    absolute error, of order eps32 |u|^2 / CFL at CFL 0.1 (1.5e-6 |u|^2
    measured on the 128 x 17 x 19 grid); the printed diagnostics: extrema
    within 2e-5, the divergence statistics of u* within 1e-4 of their scale,
    CFL within 2e-5."""
    c = _case(oracle, shape, bcs, itscheme=3, eps=1e-12, kmax=400000, omega=1.6)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    for a in range(3):
        s.u[a][...] = perturbed(s.u[a], 50 + a, amp=0.05, kinds=kinds_of(c, a))
    runner = oracle.Runner(c, s)
    prm = params_of(o3d, c, precision=o3d.PREC_MIXED, solver=o3d.SOLVER_MG, eps=1e-9, kmax=200)
    with o3d.Context(prm) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        ctx.upload("pp", s.pp)
        for it in range(1, 4):
            ri = runner.step(it)
            gi = ctx.step(it)
            assert gi.poisson_status == o3d.OK and gi.diverged == 0
            umax = max(np.abs(x).max() for x in s.u)
            for a in range(3):
                assert gi.umin[a] == pytest.approx(s.u[a].min(), abs=2e-5 * umax), (it, a)
                assert gi.umax[a] == pytest.approx(s.u[a].max(), abs=2e-5 * umax), (it, a)
                assert gi.cfl[a] == pytest.approx(ri.cfl[a], rel=2e-5, abs=1e-12), (it, a)
            dscale = max(abs(ri.divu_pred_stats[0]), abs(ri.divu_pred_stats[1]))
            for q in range(3):
                assert abs(gi.divu_pred_stats[q] - ri.divu_pred_stats[q]) < 1e-4 * dscale, (it, q)
        umax = max(np.abs(x).max() for x in s.u)
        for a, name in enumerate(("ux", "uy", "uz")):
            assert np.abs(ctx.download(name) - s.u[a]).max() < 2e-5 * umax, name
        p = ctx.download("pp")
        dp = np.abs((p - p.mean()) - (s.pp - s.pp.mean())).max()
        assert dp < 1e-5 * umax ** 2, dp


SCALAR_CASES = [
    ((64, 24, 40), (0, 0, 0), 0),
    ((36, 33, 29), (1, 1, 1), 1),
    ((128, 17, 19), (0, 1, 0), 1),
    ((44, 25, 21), (2, 1, 1), 1),   # open x: the inflow plane holds its scalar
    ((33, 20, 24), (0, 1, 0), 1),   # one-point kernels
]


@pytest.mark.parametrize("shape,bcs,iles", SCALAR_CASES)
def test_fp32_scalar_transport_in_mixed_steps(oracle, o3d, shape, bcs, iles):
    """transeq with its conservative clipping (src/integration.f90:405-450) in
    three mixed-method steps against the oracle's FP64 steps.  The scalar
    starts as a smooth field that overshoots [0, 1] by up to 0.2, so the
    clipping and the redistribution of the excess act at every step.  The
    scalar is compared within 5e-5 (FP32 transport of values of order 1 over
    three steps), and its mean, which the redistribution conserves, within
    1e-6."""
    c = _case(oracle, shape, bcs, itscheme=3, eps=1e-12, kmax=400000, omega=1.6, nscr=1, sc=0.7, iles=iles,
              cs=0.17)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    for a in range(3):
        s.u[a][...] = perturbed(s.u[a], 70 + a, amp=0.05, kinds=kinds_of(c, a))
    nx, ny, nz = shape
    x = np.linspace(0, 1, nx)[:, None, None]
    y = np.linspace(0, 1, ny)[None, :, None]
    z = np.linspace(0, 1, nz)[None, None, :]
    s.phi[...] = 0.5 + 0.7 * np.cos(PI * x) * np.cos(PI * y) * np.cos(PI * z)
    runner = oracle.Runner(c, s)
    prm = params_of(o3d, c, precision=o3d.PREC_MIXED, solver=o3d.SOLVER_MG, eps=1e-9, kmax=200)
    with o3d.Context(prm) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        ctx.upload("pp", s.pp)
        ctx.upload("phi", s.phi)
        ctx.upload("src", s.src)
        for it in range(1, 4):
            runner.step(it)
            gi = ctx.step(it)
            assert gi.poisson_status == o3d.OK and gi.diverged == 0
        got = ctx.download("phi")
    assert got.min() >= 0.0 and got.max() <= 1.0
    assert np.abs(got - s.phi).max() < 5e-5
    assert abs(got.mean() - s.phi.mean()) < 1e-6
