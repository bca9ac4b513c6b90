"""bench.py's host-side arithmetic on the CPU.  Its multi-GPU form is
replicas only: each rank solves the same case and the job's rate is world
solves per the slowest rank's step; the rank plumbing (process group,
barrier, max over ranks) runs here as two gloo ranks.  And the roofline of
the fused PCG iteration from per-kernel times."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import bench
    w, r, local, dist = bench.dist_init()
    assert (w, r, local) == (world, rank, rank) and dist is not None
    # rank 1 is the slow replica: 200 ms steps against 100 and 120 ms
    steps = [100.0, 120.0] if rank == 0 else [200.0, 200.0]
    bench.barrier(dist)
    value, ms = bench.whole_job_rate(dist, w, steps)
    with open(os.path.join(out_dir, f"rank{rank}"), "w") as f:
        f.write(f"{value!r} {ms!r}")
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank(tmp_path):
    world, port = 2, _free_port()
    mp.spawn(_rank, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    for rank in range(world):
        value, ms = (float(v) for v in (tmp_path / f"rank{rank}").read_text().split())
        assert ms == 200.0 and value == pytest.approx(2 * 1000.0 / 200.0)


def test_one_process_is_its_own_job():
    import bench
    value, ms = bench.whole_job_rate(None, 1, [250.0, 250.0])
    assert ms == 250.0 and value == 4.0


def test_iteration_roofline_of_the_fused_pcg():
    """bench.py's roofline of the fused PCG iteration: both kernels'
    algorithmic bytes over their summed launch times (the 128^3 figures of
    a solve: 121.6 us and 78.0 us per launch)."""
    import bench
    N, F, B = 2097152, 6242304, 98304
    tot_n = {"loc_precond": 10, "loc_spmv": 10, "rhs": 1}
    tot_ms = {"loc_precond": 1.216, "loc_spmv": 0.780, "rhs": 1.25}
    it = bench.iteration_roofline(tot_ms, tot_n, N, F, B, 4, 6 * N, False, True, 6778.0)
    b = (bench.algorithmic_bytes("loc_precond", N, F, B, 4, 6 * N, False, True)
         + bench.algorithmic_bytes("loc_spmv", N, F, B, 4, 6 * N, False, True))
    assert it["algorithmic_bytes"] == b and it["us"] == pytest.approx(199.6)
    assert it["frac"] == pytest.approx(b / 199.6e-6 / 1e9 / 6778.0)
    assert bench.iteration_roofline({"rhs": 1.0}, {"rhs": 1}, N, F, B, 4, 0, False, False,
                                    6778.0) is None
