"""Replica runs on several ranks, on the CPU with the gloo backend.

The single-model path does not shard: under torchrun every rank runs its own
model, and bench.py reports the steps all ranks made over the slowest rank's
time.  Two gloo ranks check that aggregation, that the reference arm prints
from rank 0 only, and that replicas of the reference algorithm on different
ranks give identical fields (no state is shared between them).
"""
import json
import os
import socket
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp
from conftest import ROOT, golden_input

WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(WORLD), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist

    import bench
    from oracle_port import Oracle
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)
    try:
        # rank r made 3 + r steps in (r + 1) seconds
        v = bench.job_throughput(dist, 3 + rank, float(rank + 1))
        o = Oracle(golden_input("cfg1_l5"))
        o.step()
        np.save(os.path.join(out_dir, f"T{rank}.npy"), o.get("T"))
        o.close()
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as fh:
            json.dump({"value": v, "max": bench.rmax(dist, rank + 0.5), "sum": bench.rsum(dist, rank + 1)}, fh)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregation_and_independent_replicas(tmp_path):
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, str(tmp_path))) for r in range(WORLD)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(WORLD)]
    for r in res:
        assert r["value"] == pytest.approx((3 + 4) / 2.0)   # 7 steps, slowest rank took 2 s
        assert r["max"] == 1.5 and r["sum"] == 3.0
    np.testing.assert_array_equal(np.load(tmp_path / "T0.npy"), np.load(tmp_path / "T1.npy"))


def _ref_arm(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(WORLD), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import contextlib
    import io

    import bench

    class A:
        steps, warmup, workload = 1, 0, "cfg1_plain_64"
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        rc = bench.run_reference(A, bench.WORKLOADS["cfg1_plain_64"])
    with open(os.path.join(out_dir, f"ref{rank}.txt"), "w") as fh:
        fh.write(f"{rc}\n{buf.getvalue()}")


def test_reference_arm_prints_on_rank0_only(tmp_path):
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_ref_arm, args=(r, port, str(tmp_path))) for r in range(WORLD)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs)
    r0 = (tmp_path / "ref0.txt").read_text().splitlines()
    r1 = (tmp_path / "ref1.txt").read_text().splitlines()
    assert r0[0] == "0" and r1 == ["0"]
    line = json.loads(r0[1])
    assert line["impl"] == "reference" and line["n_gpus"] == WORLD and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


# ---- configuration 4: members sharded over ranks, gathered on the host -----------
ENS_N, ENS_SIZES = 6, (8, 16)


def _member_fields(i):
    """Member i of a small drawn ensemble, one step of the reference algorithm
    (the CPU oracle stands in for the device here): its T after the step."""
    from mantle_convection_lab_gb300 import ensemble
    from oracle_port import Oracle
    p = ensemble.draw(ENS_N, 4, ENS_SIZES)[i]
    cfg = ensemble.member_config(*p)
    cfg.max_citcom_cycle, cfg.max_cg_cycle = 20, 50
    o = Oracle(cfg)
    o.step()
    T = o.get("T")
    o.close()
    return T


def _shard_rank(rank, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(WORLD), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import torch.distributed as dist

    import bench
    from mantle_convection_lab_gb300 import ensemble
    dist.init_process_group("gloo", rank=rank, world_size=WORLD)
    try:
        mine = ensemble.shard(ENS_N, rank, WORLD)
        done = bench.gather_members(dist, {i: _member_fields(i) for i in mine})
        if rank == 0:
            np.savez(os.path.join(out_dir, "gathered.npz"), **{str(k): v for k, v in done.items()},
                     mine=np.array(mine))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_ensemble_members_sharded_and_gathered(tmp_path):
    """Two ranks each step their share of the members (rank r: r, r+2, ...);
    the host gather puts every member on rank 0 once, and each equals the same
    member stepped in a one-rank run, bit for bit."""
    from mantle_convection_lab_gb300 import ensemble
    assert ensemble.shard(ENS_N, 0, WORLD) == [0, 2, 4] and ensemble.shard(ENS_N, 1, WORLD) == [1, 3, 5]
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_shard_rank, args=(r, port, str(tmp_path))) for r in range(WORLD)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=240)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    g = np.load(tmp_path / "gathered.npz")
    assert sorted(int(k) for k in g.files if k != "mine") == list(range(ENS_N))
    assert list(g["mine"]) == [0, 2, 4]
    for i in range(ENS_N):
        np.testing.assert_array_equal(g[str(i)], _member_fields(i))
