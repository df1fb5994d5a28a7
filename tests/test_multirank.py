"""The N > 1 path of the benchmark on CPU: world_size 2 over gloo (no GPU).

Every rank runs its own replica of the workload (weak scaling, no data-path
collective); the job's time is the maximum over the ranks and the job's
throughput counts the units of all ranks.  The ranks here report different
local times, and both must see the same maximum and the same throughput.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = [40.0, 65.0][rank]
    ms = bench.job_max(local_ms, world)
    out[rank] = (ms, bench.job_value(world, 13824, ms))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_job_time_is_the_maximum_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(100)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        res = dict(out)
    assert res[0] == res[1]
    ms, value = res[0]
    assert ms == 65.0
    assert value == pytest.approx(2 * 13824 / 0.065)


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.job_max(12.5, 1) == 12.5
    assert bench.job_value(1, 1000, 500.0) == pytest.approx(2000.0)


def test_roofline_traffic_figures_are_read_from_the_profiles():
    """The bench's roofline traffic comes from the committed ncu figures of
    small cases of the contraction; sizes without a capture give None."""
    import bench
    t12, unit = bench.measured_traffic("galerkin_poisson_hexa_12^3_p5_integration1", "k_ozaki_gemm")
    assert unit == "per_launch" and t12 > 1e9
    t16, _ = bench.measured_traffic("galerkin_poisson_hexa_16^3_p5_integration1", "k_ozaki_gemm")
    assert t16 > t12
    assert bench.measured_traffic("galerkin_poisson_hexa_24^3_p5_integration1", "k_ozaki_gemm") is None
    assert bench.measured_traffic("ultraweak_dpg_maxwell_hexa_10^3_p3_impedance", "k_zupd") is None
