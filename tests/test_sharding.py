"""Multi-process decomposition on CPU (gloo, two ranks): each rank correlates
its share of a job's timeslices (with the C restatement standing in for a
GPU), rank 0 gathers and merges the outputs, and the result is byte for byte
the single-process correlation of the whole job; the ranks' timings reduce to
their maximum.  No GPU and no GPU collective is involved."""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "sfxc-1_gb300"))
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    from oracle import jobs
    from sfxc_gpu import correlator, scenario, sharding
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sc = scenario.c1_plain(integration_us=15625, n_integrations=5, seed=3)
        job = scenario.build_job(sc, correlator.delay_list, correlator.write_protocol, fast_random=True)
        mine = sharding.jobs_for_rank(job["n_integrations"], world, rank)
        parts, tparts = [], []
        for it in mine:
            r = jobs.correlate(sharding.slice_job(job, it), impl="oracle")
            parts.append((it, r["cor"]))
            tparts.append((it, r["tsys"]))
        got = sharding.gather_outputs(parts)
        gott = sharding.gather_outputs(tparts)
        wall = sharding.max_over_ranks([1.0 + rank, 10.0 - rank])
        if rank == 0:
            full = jobs.correlate(job, impl="oracle")
            ok = (sharding.merge_outputs(got) == full["cor"] and sharding.merge_outputs(gott) == full["tsys"]
                  and sorted(i for i, _ in got) == list(range(job["n_integrations"])) and wall == [2.0, 10.0])
            open(os.path.join(outdir, "result"), "w").write("ok" if ok else "mismatch")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_reproduce_single_process_output(tmp_path, oracle_exe):
    import torch.multiprocessing as mp
    mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    assert (tmp_path / "result").read_text() == "ok"


def test_jobs_for_rank_partition():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "sfxc-1_gb300"))
    from sfxc_gpu import sharding
    for n in (1, 7, 8, 33):
        for world in (1, 2, 3, 8):
            shares = [sharding.jobs_for_rank(n, world, r) for r in range(world)]
            flat = sorted(i for s in shares for i in s)
            assert flat == list(range(n))
            assert max(map(len, shares)) - min(map(len, shares)) <= 1
    with pytest.raises(ValueError):
        sharding.jobs_for_rank(4, 2, 2)


def _gpu_rank_main(rank, world, port, outdir):
    """As _rank_main with the library on the GPU as each rank's worker (both
    ranks' contexts on one GPU here: independent jobs, no kernel of one rank
    waits on the other; the collectives are gloo on the host)."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "sfxc-1_gb300"))
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist
    from sfxc_gpu import correlator, lib, scenario, sharding
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        sc = scenario.c1_plain(integration_us=15625, n_integrations=5, seed=3)
        job = scenario.build_job(sc, correlator.delay_list, correlator.write_protocol, fast_random=True)
        node = correlator.CorrelatorNode(0, lib.X_TC_HILO)
        mine = sharding.jobs_for_rank(job["n_integrations"], world, rank)
        parts, tparts = [], []
        for it in mine:
            cor, tsys = node.correlate(sharding.slice_job(job, it))
            parts.append((it, cor))
            tparts.append((it, tsys))
        got = sharding.gather_outputs(parts)
        gott = sharding.gather_outputs(tparts)
        if rank == 0:
            full_cor, full_tsys = node.correlate(job)
            ok = (sharding.merge_outputs(got) == full_cor and sharding.merge_outputs(gott) == full_tsys
                  and sorted(i for i, _ in got) == list(range(job["n_integrations"])))
            open(os.path.join(outdir, "result"), "w").write("ok" if ok else "mismatch")
        node.close()
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_two_ranks_on_the_library_reproduce_single_process_output(tmp_path, sfxc_lib):
    """The library under torch.distributed (gloo, two spawned ranks): each
    rank correlates its timeslices on its own context, rank 0 merges, and the
    bytes equal one context correlating the whole job."""
    import torch.multiprocessing as mp
    mp.start_processes(_gpu_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    assert (tmp_path / "result").read_text() == "ok"
