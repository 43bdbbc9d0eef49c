"""The divergence-with-statistics entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc: a driver whose device memory
is all held by its own pool allocator, a time loop that must not take the
device-wide synchronisation of cudaMalloc/cudaFree, or code where allocation
is forbidden.  Its output is checked against the existing entry point
o3d_divergence (through a context) and the oracle's function_stats of that
result, twice in a row so that the shared scratch array is exercised across
calls.  This file is collected last."""
import ctypes as C

import numpy as np
import pytest

from _util import PI, params_of, rel_err


def _fields(shape, seed):
    rng = np.random.default_rng(seed)
    return [np.asfortranarray(rng.standard_normal(shape)) for _ in range(3)]


@pytest.mark.gpu
@pytest.mark.parametrize("shape,bcs", [((32, 24, 40), (0, 0, 0)), ((33, 17, 21), (1, 1, 1)), ((48, 33, 16), (0, 1, 0))])
def test_noalloc_divergence_matches_context_entry_point(oracle, o3d, shape, bcs):
    torch = pytest.importorskip("torch")
    nx, ny, nz = shape
    lens = [2 * PI * (n - 1) / n if b == 0 else PI for n, b in zip(shape, bcs)]
    case = oracle.Case(nx, ny, nz, lens[0], lens[1], lens[2], bcx=bcs[0], bcy=bcs[1], bcz=bcs[2])
    h = [L / (n - 1) for L, n in zip(lens, shape)]
    with o3d.Context(params_of(o3d, case)) as ctx:
        for call, seed in enumerate((11, 12)):  # two calls in a row, different data
            fx, fy, fz = _fields(shape, seed + 10 * sum(bcs))
            ref = ctx.divergence(fx, fy, fz, 1)
            ref_stats = (C.c_double * 6)()
            oracle.lib().orc_function_stats(oracle.ptr(ref), nx, ny, nz, ref_stats)
            # device copies in the column-major layout of the fields
            dev = [torch.from_numpy(np.ravel(a, order="F")).cuda() for a in (fx, fy, fz)]
            d_div = torch.full((nx * ny * nz,), float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            st, stats = o3d.divergence_stats_noalloc(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(),
                                                     d_div.data_ptr(), shape, h, bcs, odd=1)
            assert st == o3d.OK
            got = d_div.cpu().numpy().reshape(shape, order="F")
            assert rel_err(got, ref) < 1e-12, call
            assert stats[0] == pytest.approx(ref_stats[0], rel=1e-12)
            assert stats[1] == pytest.approx(ref_stats[1], rel=1e-12)
            assert stats[2] == pytest.approx(ref_stats[2], rel=1e-9, abs=1e-12 * np.abs(ref).max())
            assert list(stats[3:]) == list(ref_stats[3:6]), call


def test_noalloc_rejects_grids_beyond_its_scratch(o3d):
    """A grid needing more reduction records than the fixed scratch holds is
    refused with O3D_ERR_BADARG before any device work (the pointers are never
    touched on that path)."""
    with pytest.raises(o3d.O3DError) as ei:
        o3d.divergence_stats_noalloc(16, 16, 16, None, (1024, 1024, 1024), (1.0, 1.0, 1.0), (0, 0, 0))
    assert ei.value.code == o3d.ERR_BADARG
    assert "reduction records" in str(ei.value)
