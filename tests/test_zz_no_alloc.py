"""The divergence-with-statistics entry point that allocates no device memory.

It serves callers that cannot call cudaMalloc: a driver whose device memory
is all held by its own pool allocator, a time loop that must not take the
device-wide synchronisation of cudaMalloc/cudaFree, or code where allocation
is forbidden.  Its output is checked against the oracle's divergence and
function_stats and against the context entry point o3d_divergence, twice in
a row so that the shared scratch array is exercised across calls, and on a
grid that needs exactly as many block records as the scratch holds.  This
file is collected last."""
import ctypes as C

import numpy as np
import pytest

from _util import PI, params_of, rel_err


def _fields(shape, seed):
    rng = np.random.default_rng(seed)
    return [np.asfortranarray(rng.standard_normal(shape)) for _ in range(3)]


def _case(oracle, shape, bcs):
    lens = [2 * PI * (n - 1) / n if b == 0 else PI for n, b in zip(shape, bcs)]
    case = oracle.Case(shape[0], shape[1], shape[2], lens[0], lens[1], lens[2], bcx=bcs[0], bcy=bcs[1], bcz=bcs[2])
    h = [L / (n - 1) for L, n in zip(lens, shape)]
    return case, h


def _noalloc(o3d, torch, fields, shape, h, bcs):
    """One call on device copies of the fields; returns (div on the host, stats)."""
    nx, ny, nz = shape
    dev = [torch.from_numpy(np.ravel(a, order="F")).cuda() for a in fields]
    d_div = torch.full((nx * ny * nz,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st, stats = o3d.divergence_stats_noalloc(dev[0].data_ptr(), dev[1].data_ptr(), dev[2].data_ptr(),
                                             d_div.data_ptr(), shape, h, bcs, odd=1)
    assert st == o3d.OK
    return d_div.cpu().numpy().reshape(shape, order="F"), stats


def _check_stats(stats, ref_stats, div_scale):
    assert stats[0] == pytest.approx(ref_stats[0], rel=1e-12)
    assert stats[1] == pytest.approx(ref_stats[1], rel=1e-12)
    assert stats[2] == pytest.approx(ref_stats[2], rel=1e-9, abs=1e-12 * div_scale)
    assert list(stats[3:]) == list(ref_stats[3:6])


@pytest.mark.gpu
@pytest.mark.parametrize("shape,bcs", [((32, 24, 40), (0, 0, 0)), ((33, 17, 21), (1, 1, 1)), ((48, 33, 16), (0, 1, 0))])
def test_noalloc_divergence_matches_oracle_and_context(oracle, o3d, shape, bcs):
    torch = pytest.importorskip("torch")
    nx, ny, nz = shape
    case, h = _case(oracle, shape, bcs)
    with o3d.Context(params_of(o3d, case)) as ctx:
        for call, seed in enumerate((11, 12)):  # two calls in a row, different data
            fx, fy, fz = _fields(shape, seed + 10 * sum(bcs))
            ref = oracle.divergence(case, fx, fy, fz, 1)
            ref_stats = (C.c_double * 6)()
            oracle.lib().orc_function_stats(oracle.ptr(ref), nx, ny, nz, ref_stats)
            got, stats = _noalloc(o3d, torch, (fx, fy, fz), shape, h, bcs)
            assert rel_err(got, ref) < 1e-12, call
            _check_stats(stats, ref_stats, np.abs(ref).max())
            # the context entry point gives the same divergence
            assert rel_err(got, ctx.divergence(fx, fy, fz, 1)) < 1e-12, call


@pytest.mark.gpu
def test_noalloc_serves_a_grid_at_its_record_limit(oracle, o3d):
    """8 x 768 x 7168 points (352 MB per field) need 1 * 96 * 256 = 24576
    block records, exactly what the scratch holds; the call is served and
    agrees with the oracle, twice in a row."""
    torch = pytest.importorskip("torch")
    shape, bcs = (8, 768, 7168), (0, 1, 0)
    assert o3d.noalloc_records(shape) == o3d.NOALLOC_MAX_RECORDS
    case, h = _case(oracle, shape, bcs)
    for seed in (3, 4):
        fields = _fields(shape, seed)
        ref = oracle.divergence(case, *fields, 1)
        ref_stats = (C.c_double * 6)()
        oracle.lib().orc_function_stats(oracle.ptr(ref), *shape, ref_stats)
        got, stats = _noalloc(o3d, torch, fields, shape, h, bcs)
        assert rel_err(got, ref) < 1e-12, seed
        _check_stats(stats, ref_stats, np.abs(ref).max())
        del fields, ref, got
        torch.cuda.empty_cache()


@pytest.mark.parametrize("shape", [(8, 56, 98308), (1024, 1024, 1024)])
def test_noalloc_rejects_grids_beyond_its_scratch(o3d, shape):
    """A grid needing more block records than the fixed scratch holds (one
    more than the limit, and far more) is refused with O3D_ERR_BADARG before
    any device work: the pointers are never touched on that path."""
    assert o3d.noalloc_records(shape) > o3d.NOALLOC_MAX_RECORDS
    if shape == (8, 56, 98308):
        assert o3d.noalloc_records(shape) == o3d.NOALLOC_MAX_RECORDS + 1
    with pytest.raises(o3d.O3DError) as ei:
        o3d.divergence_stats_noalloc(16, 16, 16, None, shape, (1.0, 1.0, 1.0), (0, 0, 0))
    assert ei.value.code == o3d.ERR_BADARG
    assert "reduction records" in str(ei.value)
