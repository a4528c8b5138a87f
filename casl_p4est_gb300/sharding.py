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

Interpolation at arbitrary points (the semi-Lagrangian step): leaves are split into Morton ranges too, and a point
is interpolated by the rank that owns the leaf containing it, as my_p4est_interpolation_t forwards remote points
to their owners and returns the values (src/my_p4est_interpolation.cpp:341-467): per rank pair one message with
the point count, one with the points and one with the values. The owner reads the field and its second
derivatives at its leaves' corner nodes only, so it needs its node range plus the corner ghosts that
LeafPartition lists, filled by the same HaloExchange.
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
    the set of nodes its record names. ghosts[r]: the nodes outside rank r's range that its stencils reach
    (rings=2: also the nodes the stencils of those reach, which the mixed path reads: second neighbours and the
    stencils of the neighbours' second derivatives); recv[r][s] = send[s][r]: those of them rank s owns (sorted)."""

    def __init__(self, records, world, rings=1):
        if world < 1 or rings not in (1, 2):
            raise ValueError("world must be >= 1 and rings 1 or 2")
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
            if rings == 2:
                ref = np.unique(np.concatenate([ref, nb[ref].ravel()]))
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


class LeafPartition:
    """Contiguous leaf ranges of equal size (leaves in tree-major Morton order, as p4est partitions quadrants)
    and, per rank, the corner nodes of its leaves that lie outside its node range (node_bounds, the node
    partition's ranges): ghosts[r], recv[r][s] = send[s][r] (the attributes HaloExchange reads, with N).

    local_nodes: (leaves, 2^dim) corner node indices per leaf (Forest.local_nodes)."""

    def __init__(self, local_nodes, node_bounds, world):
        if world < 1 or len(node_bounds) != world + 1:
            raise ValueError("need world >= 1 and world + 1 node bounds")
        ln = np.asarray(local_nodes)
        nl = len(ln)
        ln = ln.reshape(nl, -1)
        self.world = world
        self.N = int(node_bounds[-1])
        self.node_bounds = [int(b) for b in node_bounds]
        self.bounds = [(nl * r) // world for r in range(world + 1)]
        self.ghosts, self.recv = [], []
        for r in range(world):
            b, e = self.node_bounds[r], self.node_bounds[r + 1]
            corners = np.unique(ln[self.bounds[r]:self.bounds[r + 1]].ravel())
            g = corners[(corners < b) | (corners >= e)]
            self.ghosts.append(g)
            owner = np.searchsorted(self.node_bounds, g, side="right") - 1
            self.recv.append({s: g[owner == s] for s in range(world) if s != r and np.any(owner == s)})
        self.send = [{r: self.recv[r][s] for r in range(world) if s in self.recv[r]} for s in range(world)]

    def owner_of_leaves(self, leaf):
        """Rank owning each leaf index (a torch tensor or a numpy array of leaf indices)."""
        if isinstance(leaf, np.ndarray):
            return np.searchsorted(self.bounds, leaf, side="right") - 1
        import torch
        b = torch.as_tensor(self.bounds, dtype=torch.int64, device=leaf.device)
        return torch.searchsorted(b, leaf.to(torch.int64), right=True) - 1


def _exchange_sized(world, rank, outgoing, make_inbox):
    """One batch of point-to-point messages: outgoing[peer] is sent to peer, and inbox[peer] = make_inbox(peer)
    (or None: nothing expected) is filled by peer. Empty messages are not sent."""
    import torch.distributed as dist
    ops, inbox = [], {}
    for peer in range(world):
        if peer == rank:
            continue
        t = outgoing.get(peer)
        if t is not None and t.numel() > 0:
            ops.append(dist.P2POp(dist.isend, t.contiguous(), peer))
        buf = make_inbox(peer)
        if buf is not None and buf.numel() > 0:
            inbox[peer] = buf
            ops.append(dist.P2POp(dist.irecv, buf, peer))
    if ops:
        for req in dist.batch_isend_irecv(ops):
            req.wait()
    return inbox


def interpolate_sharded(lpart: LeafPartition, rank: int, xyz, backend, method, F, Fdd=None):
    """my_p4est_interpolation_nodes_t::interpolate on one rank of a Morton split (src/my_p4est_interpolation.cpp:
    341-467, the query/reply exchange; the evaluation at a point is the single-process one, so the values are
    the same bits as on one rank). xyz: (n, dim) float64 tensor of this rank's points; F: (nf, N) field tensor
    and Fdd: (nf, dim, N) second derivatives (None for the linear method), valid at this rank's node range and
    at lpart's ghosts; backend: locate(xyz) -> leaf indices, interpolate(method, F, Fdd, xyz) -> (nf, n).
    Returns (nf, n)."""
    import torch
    world = lpart.world
    dim = xyz.shape[1]
    nf = F.shape[0]
    owner = lpart.owner_of_leaves(backend.locate(xyz))
    sel = {p: torch.nonzero(owner == p).flatten() for p in range(world)}
    # the number of points each peer forwards here (the reduce-scatter of the reference's senders count); on the
    # points' device, as NCCL wants CUDA tensors
    counts_out = {p: torch.tensor([len(sel[p])], dtype=torch.int64, device=xyz.device) for p in range(world) if p != rank}
    counts_in = _exchange_sized(world, rank, counts_out, lambda p: torch.zeros(1, dtype=torch.int64, device=xyz.device))
    n_in = {p: int(counts_in[p].item()) for p in counts_in}
    # queries: the points themselves
    pts_in = _exchange_sized(world, rank, {p: xyz[sel[p]].to(torch.float64) for p in counts_out},
                             lambda p: torch.empty((n_in[p], dim), dtype=torch.float64, device=xyz.device) if n_in[p] else None)
    # every point this rank owns, its own first, then each peer's in rank order
    peers = [p for p in range(world) if p != rank and n_in.get(p, 0) > 0]
    mine = xyz[sel[rank]]
    local_pts = torch.cat([mine] + [pts_in[p] for p in peers]) if peers else mine
    vals = backend.interpolate(method, F, Fdd, local_pts) if len(local_pts) else torch.empty((nf, 0), dtype=torch.float64,
                                                                                              device=xyz.device)
    out = torch.empty((nf, len(xyz)), dtype=torch.float64, device=xyz.device)
    out[:, sel[rank]] = vals[:, :len(mine)]
    # replies: the values of the forwarded points, back to their ranks
    replies, at = {}, len(mine)
    for p in peers:
        replies[p] = vals[:, at:at + n_in[p]].contiguous()
        at += n_in[p]
    got = _exchange_sized(world, rank, replies,
                          lambda p: torch.empty((nf, len(sel[p])), dtype=torch.float64, device=xyz.device) if len(sel[p]) else None)
    for p, v in got.items():
        out[:, sel[p]] = v
    return out


def clip_in_domain(xyz, xyz_min, xyz_max):
    """clip_in_domain (src/my_p4est_utils.h:2177-2187), non-periodic: coordinates outside the domain are clamped."""
    import torch
    lo = torch.as_tensor(xyz_min, dtype=xyz.dtype, device=xyz.device)
    hi = torch.as_tensor(xyz_max, dtype=xyz.dtype, device=xyz.device)
    out = (xyz < lo) | (xyz > hi)
    return torch.where(out, torch.maximum(lo, torch.minimum(hi, xyz)), xyz)


def sl_advect_sharded(lpart: LeafPartition, rank: int, xyz_np1, dt, v, vdd, phi, phi_dd, backend, xyz_min, xyz_max,
                      velo_method=4, phi_method=4):
    """my_p4est_semi_lagrangian_t::advect_from_n_to_np1(dt, v, vxx, phi_n, phi_xx_n, phi_np1) for this rank's new
    nodes xyz_np1 (n, dim) (src/my_p4est_semi_lagrangian.cpp:148-223): v at the new nodes, the midpoint
    x* = x - dt/2 v (clipped), v at x*, the departure point x_d = x - dt v(x*) (clipped), phi_n at x_d; every
    interpolation through interpolate_sharded. v: (dim, N), vdd: (dim, dim, N), phi: (N,), phi_dd: (dim, N),
    valid at this rank's nodes and lpart's ghosts. Returns phi_np1 at xyz_np1."""
    vt = interpolate_sharded(lpart, rank, xyz_np1, backend, velo_method, v, vdd)
    xs = clip_in_domain(xyz_np1 - (0.5 * dt) * vt.T, xyz_min, xyz_max)
    vt = interpolate_sharded(lpart, rank, xs, backend, velo_method, v, vdd)
    xd = clip_in_domain(xyz_np1 - dt * vt.T, xyz_min, xyz_max)
    return interpolate_sharded(lpart, rank, xd, backend, phi_method, phi.reshape(1, -1),
                               None if phi_dd is None else phi_dd.reshape(1, *phi_dd.shape))[0]


class HaloExchange:
    """Point-to-point ghost update for one rank over torch.distributed: owned values at send[rank][peer]
    go to peer, the values at recv[rank][peer] come from peer. Arrays are 1-D tensors of planes * N values
    (host tensors with gloo, CUDA tensors with NCCL)."""

    def __init__(self, part: MortonPartition, rank: int, device=None, slots=None):
        """slots: the slot of every node when the arrays are in another order (the mixed path's device order)."""
        import torch
        self.part = part
        self.rank = rank
        self.N = part.N
        dev = device if device is not None else "cpu"
        s = None if slots is None else np.asarray(slots.cpu() if hasattr(slots, "cpu") else slots)
        remap = (lambda v: v) if s is None else (lambda v: s[v])
        self.send_idx = {p: torch.as_tensor(remap(v), dtype=torch.int64, device=dev) for p, v in part.send[rank].items()}
        self.recv_idx = {p: torch.as_tensor(remap(v), dtype=torch.int64, device=dev) for p, v in part.recv[rank].items()}

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


def advect_schedule(given_dd):
    """The sweeps and ghost updates of advect_in_normal_direction (src/my_p4est_level_set.cpp:656-725) for one rank:
    second derivatives of phi_n (its quadratic neighbour values read the node's own; the minmod terms read the
    caller's second derivatives when given, else these, at the neighbours too), the first stage into phi, the
    second derivatives of that, the second stage averaged with phi_n. Ops: ("dd", src, dst), ("exchange", name,
    planes), ("clone", src, dst), ("astage", phin, ddq, ddm, velocity, avg_with, out), ("copy", src, dst)."""
    ddm = "phi_dd" if given_dd else "ddq"
    dd2 = "phi_dd" if given_dd else "ddq"
    return [("dd", "phi", "ddq"), ("exchange", ddm, True), ("clone", "phi", "phi_n"),
            ("astage", "phi_n", "ddq", ddm, "vn", None, "phi"), ("exchange", "phi", False),
            ("dd", "phi", dd2), ("exchange", dd2, True),
            ("astage", "phi", dd2, dd2, "vn1", "phi_n", "tmp"), ("copy", "tmp", "phi"), ("exchange", "phi", False)]


def run_advect_schedule(ops, backend, arrays, first, count, exchange, dim, dt):
    """Run a rank's advection schedule: backend sweeps over [first, first + count), exchange(arr, planes) for ghosts."""
    for op in ops:
        kind = op[0]
        if kind == "dd":
            backend.dd(arrays[op[1]], arrays[op[2]], first, count)
        elif kind == "exchange":
            exchange(arrays[op[1]], dim if op[2] else 1)
        elif kind == "clone":
            arrays[op[2]] = arrays[op[1]].clone()
        elif kind == "copy":
            backend.copy(arrays[op[1]], arrays[op[2]], first, count)
        else:
            _, phin, ddq, ddm, vel, avg, out = op
            backend.advect_stage(arrays[phin], arrays[ddq], arrays[ddm], arrays[vel], dt, arrays[out], arrays[avg] if avg else None,
                                 first, count)


def advect_normal_sharded(part: MortonPartition, rank: int, phi, vn, dt, backend, exchange, vn_np1=None, phi_dd=None):
    """advect_in_normal_direction(vn[, vn_np1], phi, dt[, phi_dd]) on one rank of a Morton-range split. phi: a
    full-length float64 tensor whose owned entries hold this rank's values; vn (and vn_np1) valid at the owned
    range; phi_dd, when given, a (dim * N) tensor that ends holding the second derivatives of the intermediate phi
    (as the reference overwrites its caller's arrays). Updates phi in place at the owned range and its ghosts."""
    import torch
    N = part.N
    dim = backend.dim
    exchange(phi, 1)
    arrays = {"phi": phi, "vn": vn, "vn1": vn_np1 if vn_np1 is not None else vn, "tmp": torch.empty_like(phi),
              "ddq": torch.zeros(dim * N, dtype=phi.dtype, device=phi.device)}
    if phi_dd is not None:
        arrays["phi_dd"] = phi_dd
    first, count = part.range_of(rank)
    run_advect_schedule(advect_schedule(phi_dd is not None), backend, arrays, first, count, exchange, dim, dt)
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

    def advect_stage(self, phin, ddq, ddm, vn, dt, out, avg_with, first, count):
        self.L.check(self.L.load().lsg_advect_stage_range_device(self.ls.handle, self._p(phin), self._p(ddq), self._p(ddm), self._p(vn),
                                                                 float(dt), self._p(out), self._p(avg_with), first, count))


class ShardInterpBackend:
    """A rank's point location and node interpolation on its GPU (lsg_locate_points_device,
    lsg_interpolate_nodes_device). The second derivatives are required for the quadratic methods: computed
    from F inside the call they would read nodes this rank neither owns nor receives."""

    def __init__(self, ls):
        import torch
        from . import _lib as L
        self.L = L
        self.ls = ls
        self.dim = ls.ngbd.dim
        ls.set_stream(torch.cuda.current_stream().cuda_stream)

    @staticmethod
    def _p(t):
        import ctypes as C
        return None if t is None else C.c_void_p(t.data_ptr())

    def locate(self, xyz):
        import torch
        x = xyz.contiguous()
        leaf = torch.empty(len(x), dtype=torch.int32, device=x.device)
        if len(x):
            self.L.check(self.L.load().lsg_locate_points_device(self.ls.handle, self._p(x), len(x), self._p(leaf)))
        return leaf.to(torch.int64)

    def interpolate(self, method, F, Fdd, xyz):
        import torch
        if method != 0 and Fdd is None:
            raise ValueError("the quadratic methods need the second derivatives (Fdd) in a split run")
        x = xyz.contiguous()
        F = F.contiguous()
        out = torch.empty((F.shape[0], len(x)), dtype=torch.float64, device=x.device)
        if len(x):
            self.L.check(self.L.load().lsg_interpolate_nodes_device(self.ls.handle, self._p(x), len(x), self._p(F), int(F.shape[0]),
                                                                    self._p(None if method == 0 else Fdd.contiguous()), int(method),
                                                                    self._p(out)))
        return out


class ShardMixedBackend:
    """A rank's mixed-precision reinitialisation on its GPU, stage by stage (lsg_mixed_split_*_device): the level
    set keeps every node and leaves the ones the rank does not own out of the updates (mask 0)."""

    def __init__(self, ls):
        import torch
        from . import _lib as L
        self.L = L
        self.ls = ls
        self.N = ls.num_nodes
        ls.set_stream(torch.cuda.current_stream().cuda_stream)

    def begin(self, phi, mask, order_space, limit_high, limit_low):
        import ctypes as C
        self.L.check(self.L.load().lsg_mixed_split_begin_device(self.ls.handle, C.c_void_p(phi.data_ptr()), C.c_void_p(mask.data_ptr()),
                                                                int(order_space), float(limit_high), float(limit_low)))

    def stage(self, order_space, stage):
        self.L.check(self.L.load().lsg_mixed_split_stage_device(self.ls.handle, int(order_space), int(stage)))

    def field(self, which):
        """The FP32 phi_n (0) or phi_1 (1) of the level set, N values in slot order, as a tensor over its memory."""
        import ctypes as C
        import torch
        p = C.c_void_p()
        self.L.check(self.L.load().lsg_mixed_split_field_device(self.ls.handle, int(which), C.byref(p)))

        class _View:
            __cuda_array_interface__ = {"shape": (self.N,), "typestr": "<f4", "data": (p.value, False), "version": 3}
        return torch.as_tensor(_View(), device="cuda")

    def slots(self):
        import ctypes as C
        import torch
        out = torch.empty(self.N, dtype=torch.int32, device="cuda")
        self.L.check(self.L.load().lsg_mixed_split_slots_device(self.ls.handle, C.c_void_p(out.data_ptr())))
        return out

    def end(self, phi):
        import ctypes as C
        self.L.check(self.L.load().lsg_mixed_split_end_device(self.ls.handle, C.c_void_p(phi.data_ptr())))


def reinitialize_mixed_sharded(part: MortonPartition, rank: int, phi, backend, exchange, exchange32, iterations=50, order_space=2,
                               limit_high=np.finfo(np.float64).max, limit_low=-np.finfo(np.float64).max):
    """The mixed-precision reinitialize_within_range_of_phi_0 (second order in pseudo-time) on one rank of a Morton
    split with two rings of ghosts (MortonPartition(..., rings=2)): phi's ghosts are updated once (exchange, node
    order), the rank's level set prepares every node and leaves the ones it does not own out of the updates, and
    after every stage the FP32 field's ghosts are updated (exchange32, slot order: HaloExchange(..., slots=)).
    Updates phi (full-length float64 CUDA tensor) at the owned range."""
    import torch
    first, count = part.range_of(rank)
    exchange(phi, 1)
    mask = torch.zeros_like(phi)
    mask[first:first + count] = 1.0
    backend.begin(phi, mask, order_space, limit_high, limit_low)
    f0, f1 = backend.field(0), backend.field(1)
    for _ in range(iterations):
        backend.stage(order_space, 0)
        exchange32(f1, 1)
        backend.stage(order_space, 1)
        exchange32(f0, 1)
    backend.end(phi)
    return phi
