"""Work split across ranks (one process per GPU): independent grids of a batch, and one grid split into
Morton ranges with a halo exchange.

Batches: grids share no nodes, so each rank builds a batch from its own grids with no exchange on the data
path. assign_by_size packs them by size (largest grid first, onto the rank with the fewest nodes so far; ties
to the lower rank), the same on every rank without communication.

One grid: nodes are numbered in (tree, Morton) order, so contiguous node ranges are compact pieces of the
domain, as p4est partitions them (src/my_p4est_nodes.c:606-627). Each rank owns one range and keeps a ghost
layer: the nodes its owned nodes' stencils reach. On one rank of an MPI run the reference sweeps its layer and
local node lists and updates the ghosts of phi after every stage and of the second derivatives after every
derivative sweep (src/my_p4est_level_set.cpp:376-401, 450-464; src/my_p4est_node_neighbors.cpp:1552-1627);
reinitialize_sharded runs the same schedule: per RK stage one exchange of the D second-derivative planes and one
of phi, point to point between the ranks that share ghosts (torch.distributed isend/irecv: NCCL for CUDA
tensors, gloo for host tensors), and the band check is one all-reduce of a double. Every rank holds
full-length arrays and the full node tables (each sweep launches over its own range only), so a rank's
memory does not shrink with the rank count; the work and the bytes each rank streams do.
"""
from __future__ import annotations

import heapq

import numpy as np


def assign_by_size(sizes, world):
    """sizes: node count per grid; returns one sorted list of grid indices per rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k))
    heap = [(0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        parts[r].append(k)
        heapq.heappush(heap, (load + int(sizes[k]), r))
    return [sorted(p) for p in parts]


def rank_share(sizes, rank, world):
    return assign_by_size(sizes, world)[rank]


# ---- one grid in Morton ranges ----------------------------------------------------------------------
class MortonPartition:
    """Contiguous node ranges of equal size and the ghost lists of every rank.

    records: the node-neighbour records (qnnn_dtype, node order) of the whole grid; the stencil of a node is
    the set of nodes its record names. ghosts[r]: the nodes outside rank r's range that its stencils reach;
    recv[r][s] = send[s][r]: those of them rank s owns (sorted)."""

    def __init__(self, records, world):
        if world < 1:
            raise ValueError("world must be >= 1")
        N = len(records)
        self.N = N
        self.world = world
        self.bounds = [(N * r) // world for r in range(world + 1)]
        nb = np.asarray(records["nb"]).reshape(N, -1)
        self.ghosts, self.recv = [], []
        for r in range(world):
            b, e = self.bounds[r], self.bounds[r + 1]
            ref = np.unique(nb[b:e].ravel())
            ref = ref[ref >= 0]
            g = ref[(ref < b) | (ref >= e)]
            self.ghosts.append(g)
            owner = np.searchsorted(self.bounds, g, side="right") - 1
            self.recv.append({s: g[owner == s] for s in range(world) if s != r and np.any(owner == s)})
        self.send = [{r: self.recv[r][s] for r in range(world) if s in self.recv[r]} for s in range(world)]

    def range_of(self, rank):
        return self.bounds[rank], self.bounds[rank + 1] - self.bounds[rank]

    def halo_bytes(self, rank, planes=1, itemsize=8):
        """Bytes rank receives in one exchange of `planes` node-sampled planes."""
        return int(sum(len(v) for v in self.recv[rank].values())) * planes * itemsize


class HaloExchange:
    """Point-to-point ghost update for one rank over torch.distributed: owned values at send[rank][peer]
    go to peer, the values at recv[rank][peer] come from peer. Arrays are 1-D tensors of planes * N values
    (host tensors with gloo, CUDA tensors with NCCL)."""

    def __init__(self, part: MortonPartition, rank: int, device=None):
        import torch
        self.part = part
        self.rank = rank
        self.N = part.N
        dev = device if device is not None else "cpu"
        self.send_idx = {p: torch.as_tensor(v, dtype=torch.int64, device=dev) for p, v in part.send[rank].items()}
        self.recv_idx = {p: torch.as_tensor(v, dtype=torch.int64, device=dev) for p, v in part.recv[rank].items()}

    def __call__(self, arr, planes=1):
        import torch
        import torch.distributed as dist
        if not self.send_idx and not self.recv_idx:
            return
        view = arr.view(planes, self.N)
        ops, inbox = [], {}
        for peer, idx in self.send_idx.items():
            ops.append(dist.P2POp(dist.isend, view[:, idx].contiguous(), peer))
        for peer, idx in self.recv_idx.items():
            buf = torch.empty((planes, len(idx)), dtype=arr.dtype, device=arr.device)
            inbox[peer] = buf
            ops.append(dist.P2POp(dist.irecv, buf, peer))
        for req in dist.batch_isend_irecv(ops):
            req.wait()
        for peer, buf in inbox.items():
            view[:, self.recv_idx[peer]] = buf


def reinit_schedule(order_space, order_pseudotime, iterations):
    """The sweeps and ghost updates of reinitialize_within_range_of_phi_0 (src/my_p4est_level_set.cpp:290-557)
    for one rank: ("dd", src, dst), ("exchange", name, planes), ("prep",), ("stage", src, dst, avg_with).
    The second derivatives are swept at every order: the quadratic neighbour values of a node
    (ngbd_with_quadratic_interpolation) need its own; second order in space also reads them at the
    neighbours, so only then are their ghosts updated."""
    ops = []
    second = order_space > 1
    ops.append(("dd", "phi0", "dd0"))
    if second:
        ops.append(("exchange", "dd0", True))
    ops.append(("prep",))
    for _ in range(iterations):
        ops.append(("dd", "phi", "ddc"))
        if second:
            ops.append(("exchange", "ddc", True))
        if order_pseudotime > 1:
            ops += [("stage", "phi", "phi1", None), ("exchange", "phi1", False), ("dd", "phi1", "ddc")]
            if second:
                ops.append(("exchange", "ddc", True))
            ops += [("stage", "phi1", "phi", "phi"), ("exchange", "phi", False)]
        else:
            ops += [("stage", "phi", "phi", None), ("exchange", "phi", False)]
    return ops


def run_schedule(ops, backend, arrays, first, count, exchange, dim, order_space, limit_high, limit_low):
    """Run a rank's schedule: backend sweeps over [first, first + count), exchange(arr, planes) for ghosts."""
    for op in ops:
        kind = op[0]
        if kind == "dd":
            backend.dd(arrays[op[1]], arrays[op[2]], first, count)
        elif kind == "exchange":
            exchange(arrays[op[1]], dim if op[2] else 1)
        elif kind == "prep":
            backend.prep(arrays["phi0"], arrays["dd0"], order_space, limit_high, limit_low, first, count)
        else:
            src, dst, avg = op[1], op[2], op[3]
            if dst == src and avg is None:  # first order in pseudo-time: phi_n+1 replaces phi_n after the stage
                backend.stage(order_space, arrays["phi0"], arrays[src], arrays["ddc"], arrays["phi1"], None, first, count)
                backend.copy(arrays["phi1"], arrays[dst], first, count)
            else:
                backend.stage(order_space, arrays["phi0"], arrays[src], arrays["ddc"], arrays[dst],
                              arrays[avg] if avg else None, first, count)


def reinitialize_sharded(part: MortonPartition, rank: int, phi, backend, exchange, iterations=50, order_space=2,
                         order_pseudotime=2, limit_high=np.finfo(np.float64).max, limit_low=-np.finfo(np.float64).max):
    """reinitialize_within_range_of_phi_0 on one rank of a Morton-range split. phi: a full-length float64 torch
    tensor whose owned entries hold this rank's values (others are filled by the exchange); updated in place
    at the owned range (and its ghosts). backend: the rank's sweeps (ShardBackend on a GPU)."""
    import torch
    N = part.N
    dim = backend.dim
    exchange(phi, 1)
    arrays = {"phi": phi, "phi0": phi.clone(), "phi1": torch.empty_like(phi),
              "dd0": torch.zeros(dim * N, dtype=phi.dtype, device=phi.device),
              "ddc": torch.zeros(dim * N, dtype=phi.dtype, device=phi.device)}
    first, count = part.range_of(rank)
    run_schedule(reinit_schedule(order_space, order_pseudotime, iterations), backend, arrays, first, count, exchange, dim, order_space,
                 limit_high, limit_low)
    return phi


def band_linf_sharded(part: MortonPartition, rank: int, a, b, band):
    """max |a - b| over the owned nodes with |b| < band, reduced over the ranks with one all-reduce(max)."""
    import torch
    import torch.distributed as dist
    first, count = part.range_of(rank)
    aa, bb = a[first:first + count], b[first:first + count]
    m = bb.abs() < band
    local = (aa[m] - bb[m]).abs().max() if bool(m.any()) else torch.zeros((), dtype=a.dtype, device=a.device)
    t = local.reshape(1).to(torch.float64)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ShardBackend:
    """A rank's FP64 sweeps on its GPU: my_p4est_level_set_t's node-range kernels (lsg_*_range_device)."""

    def __init__(self, ls):
        import torch
        from . import _lib as L
        self.L = L
        self.ls = ls
        self.dim = ls.ngbd.dim
        ls.set_stream(torch.cuda.current_stream().cuda_stream)  # ordered with the exchange's torch operations

    @staticmethod
    def _p(t):
        import ctypes as C
        return None if t is None else C.c_void_p(t.data_ptr())

    def dd(self, f, out, first, count):
        self.L.check(self.L.load().lsg_second_derivatives_range_device(self.ls.handle, self._p(f), self._p(out), first, count))

    def prep(self, phi0, dd0, order_space, limit_high, limit_low, first, count):
        self.L.check(self.L.load().lsg_reinit_prep_range_device(self.ls.handle, self._p(phi0), self._p(dd0), int(order_space),
                                                                float(limit_high), float(limit_low), first, count))

    def stage(self, order_space, phi0, phin, dd, out, avg_with, first, count):
        self.L.check(self.L.load().lsg_reinit_stage_range_device(self.ls.handle, int(order_space), self._p(phi0), self._p(phin),
                                                                 self._p(dd), self._p(out), self._p(avg_with), first, count))

    def copy(self, src, dst, first, count):
        dst[first:first + count] = src[first:first + count]
