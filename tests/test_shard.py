"""Sharding of a batch of independent systems over ranks (the multi-GPU form of the batched solver).

The host logic runs here on CPU: the partition itself, and a world_size-2 run over the gloo
backend in which each rank solves its shard (with the oracle standing in for the GPU batch call)
and the results are gathered and compared with the whole batch solved in one process.  The data
path has no collective: only the final gather, which a caller needs only to collect results.
"""
import os
import socket

import numpy as np
import pytest

import shard as S


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_partition_covers_every_system_once_and_is_balanced(oracle):
    sizes = oracle.batch_sizes(2000, seed=21, lo=4, hi=256)
    for ws in (1, 2, 3, 8):
        parts = S.partition(sizes, ws)
        allidx = np.sort(np.concatenate(parts))
        assert np.array_equal(allidx, np.arange(len(sizes)))
        ld = S.loads(sizes, parts)
        cost = S.system_cost(sizes)
        # LPT makespan bound: at most the average load plus the largest single system
        assert ld.max() <= cost.sum() / ws + cost.max() + 1e-6
        # deterministic: every rank computes the same partition without communicating
        assert all(np.array_equal(x, y) for x, y in zip(parts, S.partition(sizes, ws)))


def test_partition_more_ranks_than_systems():
    parts = S.partition([5, 3], 4)
    assert [len(p) for p in parts] == [1, 1, 0, 0]
    with pytest.raises(ValueError):
        S.partition([1], 0)


def test_pack_unpack_round_trip(oracle):
    sizes = [3, 1, 4, 0, 2]
    a = np.arange(sum(n * n for n in sizes), dtype=np.float64)
    b = -np.arange(sum(sizes), dtype=np.float64)
    parts = S.partition(sizes, 2)
    a2, b2 = np.full_like(a, np.nan), np.full_like(b, np.nan)
    for p in parts:
        pa, pb = S.pack(sizes, p, a, b)
        S.unpack_into(sizes, p, pa, pb, a2, b2)
    assert np.array_equal(a, a2) and np.array_equal(b, b2)


def _rank_main(rank, ws, port, sizes, a, b, out_path):
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    for sub in ("oracle", "eigen-git-mirror_gb300"):
        sys.path.insert(0, str(root / sub))
    import torch.distributed as dist

    import oracle as O
    import shard as SH

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    idx = SH.partition(sizes, ws)[rank]
    pa, pb = SH.pack(sizes, idx, a, b)
    info = O.batched_posv(np.asarray(sizes)[idx], pa, pb) if len(idx) else np.zeros(0, np.int64)
    got = [None] * ws
    dist.all_gather_object(got, (idx, pa, pb, np.asarray(info)))
    if rank == 0:
        a_out, b_out = np.full_like(a, np.nan), np.full_like(b, np.nan)
        info_out = np.full(len(sizes), -9, dtype=np.int64)
        for gidx, ga, gb, ginfo in got:
            SH.unpack_into(sizes, gidx, ga, gb, a_out, b_out)
            info_out[gidx] = ginfo
        np.savez(out_path, a=a_out, b=b_out, info=info_out)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("ws", [2])
def test_sharded_batch_over_gloo_matches_single_process(oracle, tmp_path, ws):
    mp = pytest.importorskip("torch.multiprocessing")
    sizes = list(oracle.batch_sizes(60, seed=41, lo=1, hi=90)) + [0, 130]
    mats = [oracle.gen_gram(n, seed=50 + i) if n else np.zeros((0, 0)) for i, n in enumerate(sizes)]
    mats[5][2, 2] = -1.0  # one failing system: its info must come back from the rank that owned it
    a = np.concatenate([m.ravel(order="F") for m in mats])
    b = np.concatenate([oracle.normal(70 + i, n) for i, n in enumerate(sizes)])
    out = tmp_path / "gathered.npz"
    mp.start_processes(_rank_main, args=(ws, _free_port(), sizes, a, b, str(out)), nprocs=ws, join=True,
                       start_method="spawn")
    g = np.load(out)
    a_ref, b_ref = a.copy(), b.copy()
    info_ref = oracle.batched_posv(np.asarray(sizes), a_ref, b_ref)
    assert np.array_equal(g["info"], np.asarray(info_ref))
    ok = np.asarray(info_ref) == 0
    assert g["info"][5] == 3 and not ok[5]
    # identical arithmetic per system, so the gathered results are bit-identical where solved
    aoff = np.concatenate([[0], np.cumsum(np.asarray(sizes) ** 2)])
    boff = np.concatenate([[0], np.cumsum(sizes)])
    for i, n in enumerate(sizes):
        if ok[i]:
            assert np.array_equal(g["a"][aoff[i]:aoff[i + 1]], a_ref[aoff[i]:aoff[i + 1]])
            assert np.array_equal(g["b"][boff[i]:boff[i + 1]], b_ref[boff[i]:boff[i + 1]])
