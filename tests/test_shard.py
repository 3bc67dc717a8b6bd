"""Shots split across processes (gpu-c_3dqmodeling_gb300/shard.py), on the CPU.

* the partition: contiguous blocks covering the list, balanced by cost;
* with 2 and 3 gloo ranks, the misfit gradient summed across ranks equals one
  process adding every shot's terms in shot order, bit for bit -- with terms
  whose magnitudes span 2^-30 .. 2^30 (where another order of the additions
  gives other bits) and with the oracle's FP64 adjoint of small shots;
* the records of every rank's block arrive on rank 0 in shot order.
"""
import multiprocessing as mp
import socket

import numpy as np
import pytest

import shard
import shard_case


def test_partition_covers_and_balances():
    costs = [5, 1, 1, 1, 9, 2, 2, 2, 3, 1]
    for world in range(1, 13):
        blocks = shard.partition(costs, world)
        assert len(blocks) == world
        assert blocks[0][0] == 0 and blocks[-1][1] == len(costs)
        for (a, b), (c, d) in zip(blocks, blocks[1:]):
            assert b == c and a <= b
        worst = max(sum(costs[a:b]) for a, b in blocks)
        # no contiguous split into `world` blocks has a smaller largest block
        best = _best_split(costs, world)
        assert worst == best, (world, blocks)
    assert shard.partition([], 3) == [(0, 0)] * 3
    with pytest.raises(ValueError):
        shard.partition([1, 2], 0)


def _best_split(costs, world):
    import functools

    @functools.lru_cache(None)
    def f(i, k):
        if i == len(costs):
            return 0
        if k == 1:
            return sum(costs[i:])
        return min(max(sum(costs[i:j]), f(j, k - 1)) for j in range(i + 1, len(costs) + 1))
    return f(0, world)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run(world, kind):
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=shard_case.worker, args=(r, world, port, kind, q))
             for r in range(world)]
    for p in procs:
        p.start()
    out = {}
    import queue
    import time
    t0 = time.time()
    while len(out) < world:
        try:
            rank, J, G, blk, recs = q.get(timeout=1)
            out[rank] = (J, G, blk, recs)
        except queue.Empty:
            failed = [p.exitcode for p in procs if p.exitcode not in (None, 0)]
            if failed or time.time() - t0 > 300:
                for p in procs:
                    p.kill()
                raise AssertionError("a rank failed: exit codes %s" % failed)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return out


def _one_process(shots, fn):
    J, G = 0.0, [np.zeros(shots[0].N, np.float64) for _ in range(3)]
    for i, s in enumerate(shots):
        j, g = fn(i, s)
        J += j
        for q in range(3):
            G[q] += g[q]
    return J, G


@pytest.mark.parametrize("world,kind", [(2, "fake"), (3, "fake"), (2, "fake2")])
def test_gradient_sum_bit_equal_to_one_process(world, kind):
    shots = [shard_case.FakeShot(i) for i in range(7)]
    J1, G1 = _one_process(shots, lambda i, s: shard_case.fake_terms(i))
    # the stand-in terms do depend on the order of the additions
    rev = np.zeros_like(G1[0])
    for i in reversed(range(7)):
        rev += shard_case.fake_terms(i)[1][0]
    assert not np.array_equal(rev, G1[0])
    out = _run(world, kind)
    for rank in range(world):
        J, G, blk, recs = out[rank]
        assert J == J1
        for q in range(3):
            assert np.array_equal(G[q].view(np.uint64), G1[q].view(np.uint64))
    # records: rank 0 holds all of them in shot order
    J, G, blk, recs = out[0]
    assert blk == (0, 7) and len(recs) == 7
    for s, r in zip(shots, recs):
        assert np.array_equal(r, shard_case.fake_record(s))
    blocks = shard.partition([shard.shot_cost(s) for s in shots], world)
    for rank in range(1, world):
        assert out[rank][2] == blocks[rank]


def test_oracle_gradient_across_two_ranks():
    import synthetic
    try:
        shots = shard_case.oracle_shots()
        J1, G1 = _one_process(shots, shard_case.oracle_terms)
    finally:
        synthetic.set_backend("qp3d")
    assert all(np.linalg.norm(g) > 0 for g in G1)
    out = _run(2, "oracle")
    for rank in range(2):
        J, G, _, _ = out[rank]
        assert J == J1
        for q in range(3):
            assert np.array_equal(G[q].view(np.uint64), G1[q].view(np.uint64))


def test_concurrent_contexts_in_one_process():
    """Several grad functions (library contexts on one GPU) run shots at once;
    the terms are still added in shot order: the same bits as one function."""
    import threading
    shots = [shard_case.FakeShot(i) for i in range(9)]
    J1, G1 = _one_process(shots, lambda i, s: shard_case.fake_terms(i))
    lock = threading.Lock()
    busy = []

    def fn(i, s, out):
        with lock:
            busy.append(i)
        J, g = shard_case.fake_terms(i)
        for q in range(3):
            out[q] += g[q]
        return J

    J, G = shard.gradient(shots, [fn, fn, fn], group=shard.Group())
    assert J == J1 and sorted(busy) == list(range(9))
    for q in range(3):
        assert np.array_equal(G[q].view(np.uint64), G1[q].view(np.uint64))


def test_partition_of_the_batched_workload_is_balanced():
    """The 64 uneven shots of the batched workload (padded cells x steps):
    for 2 to 8 ranks the largest block exceeds the mean by at most one
    shot's cost, and the blocks cover the list in order."""
    import synthetic
    pml, nt = 20, 2000
    costs = [float((hx + 2 * pml) * (hy + 2 * pml) * (nz0 + 2 * pml) * nt)
             for _, _, hx, hy, nz0, _ in synthetic.batch_windows(64)]
    for world in range(2, 9):
        blocks = shard.partition(costs, world)
        assert blocks[0][0] == 0 and blocks[-1][1] == 64
        loads = [sum(costs[a:b]) for a, b in blocks]
        assert max(loads) <= sum(costs) / world + max(costs), (world, loads)
        print("%d ranks: largest block %.3f x the mean" % (world, max(loads) * world / sum(costs)))
