"""Row-range sharding (the multi-GPU form of the search): two gloo ranks on
the CPU each hold half of the store, compute their local exact top-k (the
oracle stands in for each rank's GPU search), gather and merge with the
library's svdb_merge_topk; the result must equal the global top-k, ties to
the lowest global index."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, result_dir):
    sys.path[:0] = [os.path.join(ROOT, "simple-vector-db_gb300"), os.path.join(ROOT, "oracle")]
    import torch.distributed as dist

    import oracle as O
    from svdb_gb300 import shard

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(77)
    X = rng.normal(size=(3001, 24))
    X[2000] = X[10]  # a duplicate across the two shards: tie to the lower global index
    Q = np.concatenate([rng.normal(size=(7, 24)), X[[10, 2999]]])
    lo, hi = shard.shard_bounds(X.shape[0], world, rank)
    o = O.Oracle()
    for metric in range(3):
        for k in (1, 10, 50):
            lid, lval = o.topk(metric, X[lo:hi], Q, k, threads=1)
            gid, gval = shard.gather_topk(metric, lid, lval, lo)
            np.save(os.path.join(result_dir, f"r{rank}_m{metric}_k{k}_ids.npy"), gid)
            np.save(os.path.join(result_dir, f"r{rank}_m{metric}_k{k}_vals.npy"), gval)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_merge_equals_global_topk(tmp_path, oracle, svdb):
    import torch.multiprocessing as mp

    port = 29500 + (os.getpid() % 2000)
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    rng = np.random.default_rng(77)
    X = rng.normal(size=(3001, 24))
    X[2000] = X[10]
    Q = np.concatenate([rng.normal(size=(7, 24)), X[[10, 2999]]])
    for metric in range(3):
        for k in (1, 10, 50):
            wid, wval = oracle.topk(metric, X, Q, k)
            for rank in range(2):
                gid = np.load(tmp_path / f"r{rank}_m{metric}_k{k}_ids.npy")
                gval = np.load(tmp_path / f"r{rank}_m{metric}_k{k}_vals.npy")
                assert np.array_equal(gid, wid), (metric, k, rank)
                assert np.array_equal(gval, wval), (metric, k, rank)


def test_merge_topk_missing_entries_and_nan(svdb):
    ids = np.array([[[0, 1, -1]], [[5, -1, -1]]], np.int64)
    vals = np.array([[[3.0, np.nan, np.nan]], [[3.0, np.nan, np.nan]]])
    oi, ov = svdb.merge_topk(1, ids, vals)  # Euclidean: ascending, NaN last, tie -> lower id
    assert list(oi[0]) == [0, 5, 1] and ov[0, 0] == 3.0 and np.isnan(ov[0, 2])
    oi, ov = svdb.merge_topk(0, ids[:, :, :1], vals[:, :, :1])
    assert list(oi[0]) == [0]


@pytest.mark.gpu
@pytest.mark.parametrize("metric", [0, 1, 2])
def test_gpu_shards_merge_equals_single_store(oracle, svdb, metric):
    """Three row-range shards as three stores on one GPU: local BF16-screened
    top-k per shard, merged, equals the whole store's exact top-k."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from svdb_gb300 import shard
    rng = np.random.default_rng(90 + metric)
    C = rng.normal(size=(16, 96))
    X = C[rng.integers(0, 16, 9000)] + 0.05 * rng.normal(size=(9000, 96))
    X[7000] = X[12]
    Q = np.concatenate([C[rng.integers(0, 16, 20)] + 0.05 * rng.normal(size=(20, 96)), X[[12]]])
    k = 10
    ids, vals = [], []
    for r in range(3):
        lo, hi = shard.shard_bounds(X.shape[0], 3, r)
        db = svdb.VectorDatabase(0, 3)
        db.insert_batch(X[lo:hi])
        li, lv = db.search(Q, k, metric, svdb.PREC_BF16)
        db.close()
        ids.append(np.where(li >= 0, li + lo, -1))
        vals.append(lv)
    gid, gval = svdb.merge_topk(metric, np.stack(ids), np.stack(vals))
    wid, wval = oracle.topk(metric, X, Q, k)
    assert np.array_equal(gid, wid) and np.array_equal(gval, wval)
