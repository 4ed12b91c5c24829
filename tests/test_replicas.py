"""Multi-rank host logic of the benchmark on CPU ranks (gloo, world size 2):
the slowest rank's time is what every rank reports, the whole-job value counts
every rank's vertices, and the condensate shards are what the two scaling modes
promise (weak: 64 per rank, equal sizes, distinct condensates; strong: the
single-GPU batch split disjointly and evenly by size).  No GPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    pg = bench._init_pg(world, "gloo")
    ws, r, _ = bench._dist()
    ms = 10.0 + 5.0 * r                       # rank 1 is slower
    ms_max = bench._max_over_ranks(pg, ms)
    value = bench.replica_value(1000, ws, 100, ms_max)
    out[r] = (ws, ms_max, value)
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_slowest_rank():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    assert res[0] == res[1]
    ws, ms_max, value = res[0]
    assert ws == 2 and ms_max == 15.0
    assert value == pytest.approx(1000 * 2 * 100 / 15e-3)


def _shard_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    pg = bench._init_pg(world, "gloo")
    res = {}
    for scaling in ("weak", "strong"):
        conds = bench.build_batch(rank, world, scaling)
        verts = sum(c.inst.nx * c.inst.ny * c.inst.nz * 2 for c in conds)
        res[scaling] = ([(c.inst.nx, c.inst.g, c.inst.trap, float(abs(c.psi).sum())) for c in conds], verts,
                        bench._sum_over_ranks(pg, verts))
    out[rank] = res
    dist.barrier()
    dist.destroy_process_group()


def test_condensate_shards_over_two_ranks():
    from vaikkari_gb300 import workloads
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.start_processes(_shard_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
        res = dict(out)
    single = workloads.config4()
    key = [(c.inst.nx, c.inst.g, c.inst.trap, float(abs(c.psi).sum())) for c in single]
    # weak: rank 0 is the single-GPU batch; rank 1 has the same sizes, other condensates
    w0, w1 = res[0]["weak"], res[1]["weak"]
    assert w0[0] == key
    assert [x[0] for x in w1[0]] == [x[0] for x in key] and w1[1] == w0[1]
    assert not set(x[1] for x in w1[0]) & set(x[1] for x in key)
    assert w0[2] == w1[2] == 2 * w0[1]
    # strong: a disjoint split of the single-GPU batch, loads within one condensate
    s0, s1 = res[0]["strong"], res[1]["strong"]
    assert sorted(s0[0] + s1[0], key=key.index) == key
    assert s0[1] + s1[1] == w0[1] and s0[2] == s1[2] == w0[1]
    assert abs(s0[1] - s1[1]) <= 2 * max(c.inst.nx * c.inst.ny * c.inst.nz for c in single)


def test_shard_by_size_balance():
    from vaikkari_gb300.gpe import Instance
    from vaikkari_gb300.workloads import shard_by_size
    insts = [Instance(n, n, n, 0.25, 1e-4, 1.0) for n in (96, 24, 64, 32, 96, 48, 24, 64, 32, 48)]
    for world in (1, 2, 3, 4, 8, 12):
        parts = shard_by_size(insts, world)
        assert len(parts) == world and sorted(i for p in parts for i in p) == list(range(len(insts)))
        loads = [sum(insts[i].nx ** 3 for i in p) for p in parts]
        if world <= len(insts):
            assert max(loads) - min(loads) <= 96 ** 3


def _tune_writer(rank, path, n):
    import json
    os.environ["GPE_AUTOTUNE_CACHE"] = path
    import importlib
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import vaikkari_gb300.autotune as at
    importlib.reload(at)
    for k in range(n):
        db = at._load()
        db[f"rank{rank}-{k}"] = {"tile": k}
        at._store(db)
    json.load(open(path))  # the file is always complete


def test_autotune_cache_survives_concurrent_writers(tmp_path):
    """Ranks of one job store autotune results at the same time: every write
    leaves a complete file (no shared temporary file)."""
    import json
    path = str(tmp_path / "cache.json")
    mp.start_processes(_tune_writer, args=(path, 20), nprocs=4, join=True, start_method="spawn")
    db = json.load(open(path))
    assert len(db) >= 20 and all(k.startswith("rank") for k in db)


def test_autotune_refuses_other_lattices():
    """The autotuner's variants are the BCC2 fused kernel's: a TETRA12 batch is
    refused before anything is timed or cached."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import pytest
    from vaikkari_gb300.autotune import autotune
    from vaikkari_gb300.gpe import Instance, Lattice
    with pytest.raises(ValueError):
        autotune([Instance(4, 4, 4, 0.1, 1e-3, 1.0)], lattice=Lattice.TETRA12, cache=False)
