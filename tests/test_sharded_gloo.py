"""Row-sharded calls across ranks (world_size 2, gloo, CPU).

The exchange logic of wildboar_gb300.distance.sharded runs on CPU ranks with
the oracle as the per-rank compute (the GPU call has the same contract); the
gathered result must equal the oracle's single-process answer bit for bit.
"""

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from wildboar_gb300.distance.sharded import shard_bounds  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _ts(x):
    x = np.asarray(x, dtype=float)
    return x.reshape(x.shape[0], 1, x.shape[1]) if x.ndim == 2 else x


def _o_pairwise(x, y, dim=0, metric="euclidean", metric_params=None):
    from oracle import oracle as O
    return O.pairwise(_ts(x), _ts(y), dim=dim, metric=metric, metric_params=metric_params)


def _o_argmin(x, y, k=1, return_distance=True, metric="euclidean", metric_params=None):
    from oracle import oracle as O
    return O.argmin(x, y, k=k, metric=metric, metric_params=metric_params)


def _o_subseq(y, x, metric="euclidean", metric_params=None, return_index=False):
    from oracle import oracle as O
    d, i = O.subsequence(y, x, metric=metric, metric_params=metric_params)
    return (d, i) if return_index else d


def _data():
    rng = np.random.default_rng(3)
    X = np.cumsum(rng.standard_normal((23, 40)), axis=1)
    Y = np.cumsum(rng.standard_normal((9, 40)), axis=1)
    shp = [np.cumsum(rng.standard_normal(L)) for L in (5, 12, 7)]
    return X, Y, shp


def _worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from wildboar_gb300.distance import sharded as S

        X, Y, shp = _data()
        d = S.pairwise_distance(X, Y, compute=_o_pairwise, metric="dtw",
                                metric_params={"r": 0.3})
        i, a = S.argmin_distance(X, Y, k=3, compute=_o_argmin, metric="msm")
        sd, si = S.pairwise_subsequence_distance(shp, X, compute=_o_subseq,
                                                 return_index=True)
        t = S.max_over_ranks(1.5 + rank)
        np.savez(os.path.join(out_dir, f"r{rank}.npz"), d=d, i=i, a=a, sd=sd, si=si, t=t)
    finally:
        dist.destroy_process_group()


def test_shard_bounds_tile_rows():
    for n in (0, 1, 5, 23, 100):
        for world in (1, 2, 3, 8):
            blocks = [shard_bounds(n, r, world) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            for (a0, a1), (b0, b1) in zip(blocks, blocks[1:]):
                assert a1 == b0
            sizes = [b - a for a, b in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_bounds(4, 2, 2)


def test_world2_gloo_gather_equals_single_process(tmp_path):
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    X, Y, shp = _data()
    want_d = _o_pairwise(X, Y, metric="dtw", metric_params={"r": 0.3})
    want_i, want_a = _o_argmin(X, Y, k=3, metric="msm")
    want_sd, want_si = _o_subseq(shp, X, return_index=True)
    for rank in (0, 1):
        got = np.load(tmp_path / f"r{rank}.npz")
        np.testing.assert_array_equal(got["d"], want_d)
        np.testing.assert_array_equal(got["i"], want_i)
        np.testing.assert_array_equal(got["a"], want_a)
        np.testing.assert_array_equal(got["sd"], want_sd)
        np.testing.assert_array_equal(got["si"], want_si)
        assert float(got["t"]) == 2.5
