"""The C-ABI library builds, loads and exports what include/o3d.h declares;
the struct layouts seen by ctypes match the C compiler's; parameter checks
reject what the reference rejects.  No kernel runs here (CPU only)."""
import ctypes as C
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_every_declared_symbol_is_exported(o3d):
    L = o3d.lib()
    names = o3d.declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", o3d.library_path()], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    assert set(names) <= exported
    # nothing else of ours leaks out of the library
    assert {e for e in exported if e.startswith("o3d")} == set(names)


def test_struct_layouts_match_c(o3d, tmp_path):
    src = tmp_path / "sz.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "o3d.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu\\n\", sizeof(o3d_params), sizeof(o3d_step_info),"
        " offsetof(o3d_params, precision), offsetof(o3d_step_info, cfl), offsetof(o3d_params, dt));return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == C.sizeof(o3d.Params)
    assert vals[1] == C.sizeof(o3d.StepInfo)
    assert vals[2] == o3d.Params.precision.offset
    assert vals[3] == o3d.StepInfo.cfl.offset
    assert vals[4] == o3d.Params.dt.offset


def test_default_params(o3d):
    p = o3d.default_params()
    assert (p.nx, p.ny, p.nz) == (64, 64, 64)
    assert p.itscheme == 3 and p.eps == 1e-8 and p.kmax == 2000
    assert p.omega == pytest.approx(2.0 / (1.0 + __import__("math").sin(__import__("math").pi * 2 * __import__("math").pi / 64)))


@pytest.mark.parametrize("kw,msg", [
    (dict(nbcx1=0, nbcxn=1), "x boundary"),        # src/initialization.f90:238-242
    (dict(nbcy1=1, nbcyn=0), "y boundary"),
    (dict(nbcx1=1, nbcxn=1), "no Poisson solver"),  # x free-slip, y periodic: no poisson_solver bound
    (dict(itscheme=4), "itscheme"),               # src/integration.f90:99-104
    (dict(nx=5), "too small"),
    (dict(solver=7), "solver"),
    (dict(mg_kernels=3), "mg_kernels"),
])
def test_bad_params_rejected_before_any_device_work(o3d, kw, msg):
    p = o3d.default_params(**kw)
    with pytest.raises(o3d.O3DError) as ei:
        o3d.Context(p)
    assert ei.value.code == o3d.ERR_BADARG
    assert msg in str(ei.value)
