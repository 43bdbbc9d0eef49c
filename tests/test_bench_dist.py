"""Host logic of bench.py's multi-rank mode (replicas only: no data exchange,
a barrier around the timed region and the max-over-ranks time), run as two
gloo ranks on CPU, and the clock-record parser."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    r, w, local = bench.dist_setup()
    assert (r, w, local) == (rank, world, rank)
    assert dist.get_backend() == "gloo"
    bench.barrier(w)
    t = bench.max_over_ranks(1.5 + rank, w)
    ref = bench.reference_arm(type("A", (), {"warmup": 0, "steps": 0})(), r, w) if r != 0 else "rank0"
    out.put((rank, t, ref))
    bench.barrier(w)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [t for _, t, _ in res] == [2.5, 2.5]
    # the reference arm runs on rank 0 only; other ranks return nothing
    assert res[1][2] is None


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(3.25, 1) == 3.25
    bench.barrier(1)


def test_clock_record_summary(tmp_path):
    sys.path.insert(0, ROOT)
    import bench

    p = tmp_path / "clk.csv"
    p.write_text("0, 1965, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n"
                 "0, 1980, 2070, 1100.0, 0x4, Not Active, Not Active, Not Active, Active\n"
                 "0, 1995, 2070, 1150.0, 0x4, Not Active, Not Active, Not Active, Active\n")
    c = bench.ClockSampler(0)
    c.path = str(p)
    s = c.summary()
    assert s["sm_mhz"] == 1980 and s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["sw_power_cap"] and s["samples"] == 3


def test_roofline_tables_name_timed_kernels():
    """Every kernel bench.py reports a roofline for has a timing id in the
    library's o3d_time_kernel, the roofline kernel is one of them, and every
    DRAM traffic figure belongs to a reported kernel."""
    sys.path.insert(0, ROOT)
    import bench
    from osinco3d_gb300 import o3d

    ids = o3d.Context.KERNELS
    assert set(bench.KERNEL_BYTES) <= set(ids)
    assert bench.ROOF_KERNEL in bench.KERNEL_BYTES
    assert set(bench.TRAFFIC_PER_LAUNCH) <= set(bench.KERNEL_BYTES)
    assert sorted(ids.values()) == list(range(len(ids)))  # 0 .. 11, the ids o3d_time_kernel accepts
    src = open(os.path.join(ROOT, "osinco3d_gb300", "csrc", "o3d_api.cu")).read()
    assert f"kernel > {len(ids) - 1})" in src
