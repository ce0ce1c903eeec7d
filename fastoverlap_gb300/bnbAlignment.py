"""Branch and bound over rotations with the upstream interface.

Drop-in for fastoverlap/bnbAlignment.py's `BranchandBoundMaster` (:23-104)
searching with `BranchNodeCluster` nodes (:204-277): the search runs in
libfastoverlap_gb300.so (fo_bnb_cluster_batch), the children of every step
evaluated on the GPU, many searches side by side in `bnb_align_clusters`.
"""
import ctypes

import numpy as np

from . import _lib


def _niter(niter):
    return 2 ** 62 if niter is None or not np.isfinite(niter) else int(niter)


def bnb_align_clusters(pos1, pos2, invert=True, niter=None, rtol=5e-2, atol=1e-3, ctx=None):
    """Branch-and-bound alignment of many cluster pairs at once.  Returns
    (dists, aligned list (pos2's order, on pos1's centroid), nodes)."""
    ctx = ctx or _lib.default_context("fp64")
    p1 = [np.asarray(p, float).reshape(-1, 3) for p in pos1]
    p2 = [np.asarray(p, float).reshape(-1, 3) for p in pos2]
    n = np.array([len(p) for p in p1], np.int32)
    if any(len(a) != len(b) for a, b in zip(p1, p2)):
        raise ValueError("pos1 and pos2 pairs must have the same atom counts")
    P1 = np.ascontiguousarray(np.concatenate(p1))
    P2 = np.ascontiguousarray(np.concatenate(p2))
    d = np.zeros(len(n))
    al = np.zeros_like(P1)
    nodes = np.zeros(len(n), np.int64)
    st = ctx.lib.fo_bnb_cluster_batch(ctx.h, len(n), _lib.i(n), _lib.d(P1), _lib.d(P2), int(bool(invert)),
                                      _niter(niter), float(rtol), float(atol), _lib.d(d), _lib.d(al),
                                      nodes.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)))
    ctx.check(st, "branch and bound")
    off = np.concatenate([[0], np.cumsum(n)]).tolist()
    return d, [al[off[k]:off[k + 1]] for k in range(len(n))], nodes


class BranchandBoundMaster(object):
    """BranchandBoundMaster(initialNodes=[], rtol=5e-2, atol=1e-3)

    __call__(pos1, pos2, invert=True, niter=np.inf) -> (distance, pos1,
    rotated pos2 on pos1's centroid), as bnbAlignment.py:68-104; `nodes`
    holds the number of nodes taken from the queue."""

    def __init__(self, initialNodes=(), rtol=5e-2, atol=1e-3, ctx=None):
        if len(initialNodes):
            raise NotImplementedError("initial nodes are built from the structures by __call__")
        self.rtol = rtol
        self.atol = atol
        self.nodes = 0
        self._ctx = ctx

    def __call__(self, pos1, pos2, invert=True, niter=np.inf, extra_inputs=None, force=False, iprint=0):
        if extra_inputs is not None or force:
            raise NotImplementedError("extra start nodes and forced bounds are not taken")
        pos1 = np.array(pos1, dtype=float).reshape(-1, 3)
        d, al, nodes = bnb_align_clusters([pos1], [pos2], invert, niter, self.rtol, self.atol, self._ctx)
        self.nodes = int(nodes[0])
        return float(d[0]), pos1, al[0]
