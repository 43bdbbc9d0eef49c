"""Checkpoint and restart: the reference's flow-state file
(save_fields / read_fields, src/IOfunctions.f90:360-470) plus the history
file, and the exact continuation of a run from them."""
import numpy as np
import pytest

from _util import params_of, periodic_case

pytestmark = pytest.mark.gpu


def _read_reference_layout(path):
    """The reader of bin/fields_analyser.py:20-31, restated: time, int32 dims,
    coordinates, then column-major FP64 fields."""
    with open(path, "rb") as f:
        t = np.fromfile(f, dtype=np.float64, count=1)[0]
        nx, ny, nz = np.fromfile(f, dtype=np.int32, count=3)
        xyz = [np.fromfile(f, dtype=np.float64, count=m) for m in (nx, ny, nz)]
        n = nx * ny * nz
        fields = [np.fromfile(f, dtype=np.float64, count=n).reshape((nx, ny, nz), order="F") for _ in range(5)]
    return t, (nx, ny, nz), xyz, fields


def _mixing_case(oracle):
    nx, ny, nz = 32, 33, 16
    return oracle.Case(nx, ny, nz, 12.0 * (nx - 1) / nx, 12.0, 4.0 * (nz - 1) / nz, bcx=0, bcy=1, bcz=0,
                       y0=-6.0, z0=-2.0, ratio=0.5, re=3000.0, iles=1, cs=0.17, nscr=1, sc=1.0,
                       dt=0.01, omega=1.7, eps=1e-9, kmax=100000, idyn=1)


def test_fields_file_has_the_reference_layout(oracle, o3d, tmp_path):
    c = _mixing_case(oracle)
    s = oracle.State.zeros(c)
    oracle.init_mixing_layer(c, s)
    with o3d.Context(params_of(o3d, c)) as ctx:
        for a, nm in enumerate(("ux", "uy", "uz")):
            ctx.upload(nm, s.u[a])
        ctx.upload("pp", s.pp)
        ctx.upload("phi", s.phi)
        ctx.step(1)
        path = str(tmp_path / "fields_000001.bin")
        ctx.save_fields(path, 0.01)
        got = [ctx.download(nm) for nm in ("ux", "uy", "uz", "pp", "phi")]
    t, dims, xyz, fields = _read_reference_layout(path)
    assert t == 0.01 and dims == c.shape
    assert np.allclose(xyz[1], -6.0 + np.arange(33) * 12.0 / 32, rtol=0, atol=1e-14)
    for a, b in zip(fields, got):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("mode", ["fp64_sor_scalar", "mixed_mg_extrapolated", "mixed_mg_extrapolated2"])
def test_restart_continues_bit_for_bit(oracle, o3d, tmp_path, mode):
    """N steps in one go equal k steps, save_fields + save_history, a new
    context, load_fields + load_history and N - k more steps, bit for bit."""
    if mode == "fp64_sor_scalar":
        c = _mixing_case(oracle)
        s = oracle.State.zeros(c)
        oracle.init_mixing_layer(c, s)
        kw = {}
        names = ("ux", "uy", "uz", "pp", "phi")
        init = [s.u[0], s.u[1], s.u[2], s.pp, s.phi]
    else:
        c = periodic_case(oracle, 32, omega=1.6, eps=1e-9, kmax=100000)
        s = oracle.State.zeros(c)
        oracle.init_tgv(c, s)
        # the quadratic guess keeps two previous pressures: the history file
        # carries both
        guess = o3d.GUESS_EXTRAPOLATED2 if mode == "mixed_mg_extrapolated2" else o3d.GUESS_EXTRAPOLATED
        kw = dict(solver=o3d.SOLVER_MG, precision=o3d.PREC_MIXED, guess=guess, kmax=200)
        names = ("ux", "uy", "uz", "pp")
        init = [s.u[0], s.u[1], s.u[2], s.pp]
    N, k = 6, 3
    with o3d.Context(params_of(o3d, c, **kw)) as ctx:
        for nm, f in zip(names, init):
            ctx.upload(nm, f)
        for it in range(1, N + 1):
            ctx.step(it)
        ref = [ctx.download(nm) for nm in names]
    fpath, hpath = str(tmp_path / "fields.bin"), str(tmp_path / "hist.bin")
    with o3d.Context(params_of(o3d, c, **kw)) as ctx:
        for nm, f in zip(names, init):
            ctx.upload(nm, f)
        for it in range(1, k + 1):
            ctx.step(it)
        ctx.save_fields(fpath, k * c.dt)
        ctx.save_history(hpath)
    with o3d.Context(params_of(o3d, c, **kw)) as ctx:
        t = ctx.load_fields(fpath)
        ctx.load_history(hpath)
        assert t == k * c.dt
        for it in range(k + 1, N + 1):
            ctx.step(it)
        got = [ctx.download(nm) for nm in names]
    for nm, a, b in zip(names, got, ref):
        assert np.array_equal(a, b), nm
