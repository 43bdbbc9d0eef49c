"""The output-cadence writer (write_all_data + write_xdmf,
src/visualization.f90:242-354) through o3d_write_output: the raw FP64 files
and the XDMF description, written asynchronously while the next step runs.

Checked: every file is nx*ny*nz little-endian FP64 in column-major order
with no record markers; ux, uy, uz, pp, phi and nu_t are the fields at the
time of the call (a step taken before the writer finishes does not leak
into them); vort = |curl u| and qcrit match the oracle's rotational and
calculate_Q_criterion at 1e-12 in FP64 (1e-5 of their maxima for the FP32
fields of the mixed method); the XDMF text is the reference's, line for
line, with its Fortran number formats (I5 dimensions, F25.12 reals)."""
import numpy as np
import pytest

from _util import free_slip_case, kinds_of, params_of, perturbed, rel_err

pytestmark = pytest.mark.gpu


def _expected_xdmf(num, shape, h, origin, time, names):
    nx, ny, nz = shape
    lines = ['<?xml version="1.0" ?>', '<!DOCTYPE Xdmf SYSTEM "Xdmf.dtd" []>',
             '<Xdmf xmlns:xi="http://www.w3.org/2001/XInclude" Version="2.0">', '<Domain>',
             f'<Topology name="topo" TopologyType="3DRectMesh" Dimensions="{nz:5d}{ny:5d}{nx:5d}"/>',
             '<Geometry name="geo" GeometryType="ORIGIN_DXDYDZ">', '<DataItem Dimensions="3" Format="XML">',
             "".join(f"{v:25.12f}" for v in origin), "</DataItem>", '<DataItem Dimensions="3" Format="XML">',
             "".join(f"{v:25.12f}" for v in h), "</DataItem>", "</Geometry>",
             f'<Grid Name="{num}" GridType="Uniform">', f'<Time Value="{time:25.12f}"/>',
             '<Topology Reference="/Xdmf/Domain/Topology[1]"/>', '<Geometry Reference="/Xdmf/Domain/Geometry[1]"/>']
    for nm in names:
        lines += [f'<Attribute Name="{nm}" Center="Node">',
                  '<DataItem Format="Binary" DataType="Float" Precision="8" Endian="little" Seek="0" '
                  f'Dimensions="{nz:5d}{ny:5d}{nx:5d}">', f"{nm}_{num}.bin", "</DataItem>", "</Attribute>"]
    lines += ["</Grid>", "</Domain>", "</Xdmf>"]
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("mixed", [False, True])
def test_write_output_files_and_xdmf(oracle, o3d, tmp_path, mixed):
    c = free_slip_case(oracle, 33, iles=1, cs=0.17, nscr=1, sc=0.7, omega=1.7, eps=1e-10, kmax=100000)
    s = oracle.State.zeros(c)
    oracle.init_tgv(c, s)
    for a in range(3):
        s.u[a][...] = perturbed(s.u[a], 60 + a, kinds=kinds_of(c, a))
    extra = dict(precision=o3d.PREC_MIXED, solver=o3d.SOLVER_MG, eps=1e-8, kmax=200) if mixed else {}
    with o3d.Context(params_of(o3d, c, **extra)) as ctx:
        for a, name in enumerate(("ux", "uy", "uz")):
            ctx.upload(name, s.u[a])
        ctx.upload("pp", s.pp)
        ctx.upload("phi", s.phi + 0.25)
        ctx.upload("src", s.src)
        ctx.step(1)  # a step so that p, phi and nu_t are the solver's
        want = {nm: ctx.download(nm) for nm in ("ux", "uy", "uz", "pp", "phi", "nu_t")}
        ctx.write_output(str(tmp_path), 7, 0.125)
        ctx.step(2)  # runs while the files are written
        ctx.output_wait()
        moved = rel_err(ctx.download("ux"), want["ux"])
    assert moved > 1e-6  # the step changed the velocity after the snapshot
    shape = c.shape
    names = ["ux", "uy", "uz", "pp", "vort", "qcrit", "phi", "nu_t"]
    got = {}
    for nm in names:
        raw = np.fromfile(tmp_path / f"{nm}_7.bin", dtype="<f8")
        assert raw.size == np.prod(shape), nm
        got[nm] = raw.reshape(shape, order="F")
    for nm in ("ux", "uy", "uz", "pp", "phi", "nu_t"):
        assert np.array_equal(got[nm], want[nm]), nm
    u = [np.asfortranarray(want[nm]) for nm in ("ux", "uy", "uz")]
    rot = oracle.rotational(c, u)
    vort = np.sqrt(rot[0] ** 2 + rot[1] ** 2 + rot[2] ** 2)
    q = oracle.q_criterion(c, u)
    tol = 1e-5 if mixed else 1e-12
    assert rel_err(got["vort"], vort) < tol
    assert rel_err(got["qcrit"], q) < tol
    h = [L / (n - 1) for L, n in zip((c.xlx, c.yly, c.zlz), shape)]
    text = (tmp_path / "output_7.xdmf").read_text()
    assert text == _expected_xdmf(7, shape, h, (c.x0, c.y0, c.z0), 0.125, names)


def test_write_output_reports_an_unwritable_directory(oracle, o3d, tmp_path):
    c = free_slip_case(oracle, 17)
    with o3d.Context(params_of(o3d, c)) as ctx:
        ctx.write_output(str(tmp_path / "missing" / "dir"), 0, 0.0)
        with pytest.raises(o3d.O3DError) as ei:
            ctx.output_wait()
        assert ei.value.code == o3d.ERR_BADARG
        assert "cannot write" in str(ei.value)
        ctx.output_wait()  # the error was reported once; the writer is usable again
        ctx.write_output(str(tmp_path), 1, 0.0)
        ctx.output_wait()
    assert (tmp_path / "output_1.xdmf").exists()
