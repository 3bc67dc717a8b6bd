"""Shots across processes: the data-parallel axis of the modeling loop.

The reference runs its shots one after another in one process
(3dPureqPModeling1.0.c:225-277, Main.c:181-231).  Shots are independent --
each owns its model window, wavefields and record -- so N processes, one GPU
each, take contiguous blocks of the shot list and run them with no exchange
during the time loop (qp3d_batch or qp3d_adjoint per process).  Two
host-side exchanges follow, carried by torch.distributed on the CPU (gloo);
there is no device-to-device traffic and no collective inside a step:

* records: gathered to rank 0 in shot order, for the ordered appends of the
  modeling program's record files (read_write.c:66-77);
* the misfit gradient: the FP64 sum over shots.  One process adds the shots'
  terms left to right into its FP64 arrays (qp3d_adjoint adds each shot's
  gradient with +=), so the rounding of the sum depends on its order.  Here
  each rank keeps the terms of its own shots, receives the running sum of
  all lower ranks, adds its terms to it in shot order and passes it on; the
  last rank broadcasts the total.  The result equals one process's sum bit
  for bit for any number of ranks.

Blocks are contiguous and balanced by a per-shot cost (padded cells x time
steps by default).
"""
import numpy as np


def shot_cost(shot):
    """Work of one shot for the partition: padded cells x time steps."""
    return float(shot.nx) * float(shot.ny) * float(shot.nz) * float(shot.nt)


def partition(costs, world):
    """Contiguous blocks [(start, stop)] of len(costs) items for world ranks,
    the largest block cost as small as a contiguous split allows (binary
    search over the block-cost bound, greedy fill).  Ranks beyond the number
    of items get empty blocks."""
    costs = [float(c) for c in costs]
    if world < 1:
        raise ValueError("world must be >= 1")
    if any(c < 0 for c in costs):
        raise ValueError("costs must be >= 0")
    n = len(costs)

    def split(bound):
        blocks, start, acc = [], 0, 0.0
        for i, c in enumerate(costs):
            if i > start and acc + c > bound:
                blocks.append((start, i))
                start, acc = i, 0.0
            acc += c
        blocks.append((start, n))
        return blocks

    if n == 0:
        return [(0, 0)] * world
    lo, hi = max(costs), sum(costs)
    for _ in range(100):   # the bound converges to a block sum in few steps
        if hi - lo <= 1e-9 * max(hi, 1.0):
            break
        mid = 0.5 * (lo + hi)
        if len(split(mid)) <= world:
            hi = mid
        else:
            lo = mid
    blocks = split(hi)
    while len(blocks) < world:
        blocks.append((n, n))
    return blocks


def my_block(costs, rank, world):
    return partition(costs, world)[rank]


class Group:
    """Rank, world size and the host-side transport of the exchanges: a
    torch.distributed process group (gloo), or one process alone."""

    def __init__(self, rank=0, world=1, pg=None, dist=False):
        """pg: a torch.distributed group (None: the default group when dist)."""
        self.rank, self.world, self.pg = rank, world, pg
        if world > 1 and not dist:
            raise ValueError("a process group is needed for more than one rank")

    @classmethod
    def from_torch(cls, group=None):
        import torch.distributed as dist
        if not dist.is_available() or not dist.is_initialized():
            return cls()
        return cls(dist.get_rank(group), dist.get_world_size(group), group, dist=True)

    def _t(self, a):
        import torch
        return torch.from_numpy(a)

    def send(self, a, dst):
        import torch.distributed as dist
        dist.send(self._t(np.ascontiguousarray(a)), dst, group=self.pg)

    def recv(self, a, src):
        import torch.distributed as dist
        dist.recv(self._t(a), src, group=self.pg)

    def bcast(self, a, src):
        import torch.distributed as dist
        dist.broadcast(self._t(a), src, group=self.pg)


def ordered_sum(terms, group, length=None):
    """Sum over all ranks' terms in rank order, then term order within a rank,
    left to right from zero: the sum one process forms by adding the terms
    of every shot in shot order.  terms: this rank's list of float64 arrays
    (or scalars) of one common length; length is needed when this rank has
    none.  Returns the total on every rank."""
    arrs = [np.ascontiguousarray(np.asarray(t, np.float64).reshape(-1)) for t in terms]
    if length is None:
        if not arrs:
            raise ValueError("length is needed on a rank without terms")
        length = arrs[0].size
    if any(a.size != length for a in arrs):
        raise ValueError("terms differ in length")
    acc = np.zeros(length, np.float64)
    if group.rank > 0:
        group.recv(acc, group.rank - 1)
    for a in arrs:
        acc += a
    if group.rank + 1 < group.world:
        group.send(acc, group.rank + 1)
    if group.world > 1:
        group.bcast(acc, group.world - 1)
    return acc


def gradient(shots, grad_fn, group=None, costs=None, n=None):
    """Misfit gradient over a shot list split across ranks.

    grad_fn(i, shot, out) -> J_i: adds shot i's float64 gradient terms to the
    three arrays out (+=, as qp3d_adjoint adds to the caller's arrays) and
    returns its misfit.  Each rank calls it for its own block only: rank 0
    passes its running sums (it starts from zero, as one process does), the
    other ranks a zeroed set per shot (0 + t equals t exactly), whose terms
    they add to the running sum of the lower ranks once it arrives.  A list
    of such functions (one per library context, each with its own stream on
    the rank's GPU) runs that many shots of the block at once on host
    threads; their terms land in zeroed arrays and are added in shot order.
    n: cells per array (default shots[0].N).  Returns (J, [G_vp, G_eps,
    G_delta]) on every rank, equal bit for bit to one process calling
    grad_fn for every shot in shot order on one set of zeroed arrays."""
    group = group or Group.from_torch()
    costs = [shot_cost(s) for s in shots] if costs is None else costs
    a, b = my_block(costs, group.rank, group.world)
    n = shots[0].N if n is None else n
    fns = list(grad_fn) if isinstance(grad_fn, (list, tuple)) else [grad_fn]
    Js, gs = [], [[], [], []]

    def keep(J, out):
        if group.rank == 0:
            if not Js:
                Js.append(0.0)
                for q in range(3):
                    gs[q].append(np.zeros(n, np.float64))
            Js[0] += J
            for q in range(3):
                gs[q][0] += out[q]
        else:
            Js.append(J)
            for q in range(3):
                gs[q].append(out[q])

    if len(fns) == 1 and group.rank == 0:
        acc = [np.zeros(n, np.float64) for _ in range(3)]
        J0 = 0.0
        for i in range(a, b):
            J0 += fns[0](i, shots[i], acc)
        Js, gs = [J0], [[acc[q]] for q in range(3)]
    elif len(fns) == 1:
        for i in range(a, b):
            out = [np.zeros(n, np.float64) for _ in range(3)]
            keep(fns[0](i, shots[i], out), out)
    else:
        import queue
        from collections import deque
        from concurrent.futures import ThreadPoolExecutor
        free = queue.Queue()
        for f in fns:
            free.put(f)

        def task(i, out):
            for t in out:      # recycled arrays: zeroed in place
                t.fill(0.0)
            f = free.get()
            try:
                return f(i, shots[i], out), out
            finally:
                free.put(f)

        # at most one shot more in flight than there are contexts; the main
        # thread adds the terms in shot order and recycles rank 0's arrays
        pending, spare = deque(), []

        def consume():
            J, out = pending.popleft().result()
            keep(J, out)
            if group.rank == 0:
                spare.append(out)

        with ThreadPoolExecutor(len(fns)) as ex:
            for i in range(a, b):
                if len(pending) > len(fns):
                    consume()
                out = spare.pop() if spare else [np.empty(n, np.float64) for _ in range(3)]
                pending.append(ex.submit(task, i, out))
            while pending:
                consume()
    J = float(ordered_sum([np.array([v]) for v in Js], group, 1)[0])
    G = [ordered_sum(gs[q], group, n) for q in range(3)]
    return J, G


def records(shots, run_fn, group=None, costs=None, gather=True):
    """Records of a shot list split across ranks.  run_fn(shots_block) ->
    list of float32 records [nt][hx][hy] of those shots (e.g.
    Context.batch).  Returns (block, records): on rank 0 with gather, every
    shot's record in shot order; elsewhere this rank's own."""
    group = group or Group.from_torch()
    costs = [shot_cost(s) for s in shots] if costs is None else costs
    blocks = partition(costs, group.world)
    a, b = blocks[group.rank]
    mine = list(run_fn(shots[a:b])) if b > a else []
    if not gather or group.world == 1:
        return (a, b), mine
    if group.rank == 0:
        out = mine[:]
        for r in range(1, group.world):
            ra, rb = blocks[r]
            for i in range(ra, rb):
                s = shots[i]
                buf = np.empty((s.nt, s.hx, s.hy), np.float32)
                group.recv(buf, r)
                out.append(buf)
        return (0, len(shots)), out
    for rec in mine:
        group.send(np.ascontiguousarray(rec, np.float32), 0)
    return (a, b), mine
