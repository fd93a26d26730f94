"""Replica exchange on CPU ranks (gloo, world size 2): the batch-sharded
backward_kernel with the rank-ordered sum equals the full-batch oracle dW
and is identical on both ranks and across runs."""

import os
import socket

import numpy as np

from owl_gb300.replicas import shard


def test_shard_covers_the_batch():
    for n in (0, 1, 5, 64, 65):
        for world in (1, 2, 3, 4):
            parts = [shard(n, world, r) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import sys

    sys.path.insert(0, os.path.join(os.path.dirname(__file__), ".."))
    import torch.distributed as dist

    import oracle
    from owl_gb300.dense import NN
    from owl_gb300.replicas import conv2d_backward_kernel_dp

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        nn = NN(oracle.OracleBackend(threads=1))
        rng = np.random.default_rng(21)
        x = rng.uniform(-1, 1, (5, 9, 8, 6))
        w = rng.uniform(-1, 1, (3, 3, 6, 4))
        dy = rng.standard_normal((5, 9, 8, 4))
        a = conv2d_backward_kernel_dp(nn, x, w, [1, 1], dy)
        b = conv2d_backward_kernel_dp(nn, x, w, [1, 1], dy)
        np.save(os.path.join(out, f"dw{rank}_a.npy"), a)
        np.save(os.path.join(out, f"dw{rank}_b.npy"), b)
    finally:
        dist.destroy_process_group()


def test_sharded_weight_gradient_matches_full_batch(tmp_path, oracle_nn):
    import torch.multiprocessing as mp

    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn")
    rng = np.random.default_rng(21)
    x = rng.uniform(-1, 1, (5, 9, 8, 6))
    w = rng.uniform(-1, 1, (3, 3, 6, 4))
    dy = rng.standard_normal((5, 9, 8, 4))
    full = oracle_nn.conv2d_backward_kernel(x, w, [1, 1], dy)
    d0a, d0b = np.load(tmp_path / "dw0_a.npy"), np.load(tmp_path / "dw0_b.npy")
    d1a = np.load(tmp_path / "dw1_a.npy")
    assert np.array_equal(d0a, d1a)      # every replica holds the same dW
    assert np.array_equal(d0a, d0b)      # and the same on every run
    assert np.max(np.abs(d0a - full)) <= 1e-12 * np.max(np.abs(full))
