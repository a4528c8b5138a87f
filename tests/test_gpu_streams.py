"""Separate level-set objects run concurrently on separate CUDA streams: results equal the ones of the
same calls run one after the other (each object keeps its own tables and work buffers; calls on one
object are ordered on its stream)."""
import numpy as np
import pytest

import casl_p4est_gb300 as G
from grids import circle_2d, flower_3d, phi0_circle_2d, phi0_flower_3d

pytestmark = pytest.mark.gpu


def test_two_objects_on_two_streams():
    import torch
    grids = [(circle_2d(3, 8), phi0_circle_2d), (flower_3d(3, 6), phi0_flower_3d)]
    objs, fields, want = [], [], []
    for f, p0 in grids:
        ls = G.my_p4est_level_set_t(G.my_p4est_node_neighbors_t(f), precision="mixed")
        phi = p0(f)
        seq = phi.copy()
        ls.reinitialize_2nd_order(seq, 20)
        seq64 = phi.copy()
        ls.reinitialize_2nd_order(seq64, 5, precision="fp64")
        objs.append(ls)
        fields.append(phi)
        want.append((seq, seq64))
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    dev = []
    for ls, phi, s in zip(objs, fields, streams):
        ls.set_stream(s.cuda_stream)
        with torch.cuda.stream(s):
            a = torch.from_numpy(phi).to("cuda", non_blocking=False)
            b = a.clone()
        dev.append((a, b))
    torch.cuda.synchronize()
    for _ in range(3):  # launched back to back on both streams, no synchronisation in between
        for (ls, s), (a, b), phi in zip(zip(objs, streams), dev, fields):
            with torch.cuda.stream(s):
                a.copy_(torch.from_numpy(phi).cuda(), non_blocking=False)
                b.copy_(a)
            ls.reinitialize_2nd_order(a, 20)
            ls.reinitialize_2nd_order(b, 5, precision="fp64")
    torch.cuda.synchronize()
    for (a, b), (seq, seq64) in zip(dev, want):
        assert np.array_equal(a.cpu().numpy(), seq)
        assert np.array_equal(b.cpu().numpy(), seq64)
