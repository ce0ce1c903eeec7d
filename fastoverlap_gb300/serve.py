"""Serving through the C ABI (fo_server_*): alignment requests of mixed kinds
and sizes admitted as they arrive, batched continuously on the GPU.

    srv = Server(precision="mixed")
    t = srv.submit_cluster(pos1, pos2, perm, Jmax=15, scale=0.3)
    t2 = srv.submit_periodic(pos1, pos2, box, perm, scale=0.2, nwave=7)
    r = srv.wait(t)          # dict: dist, rmat, perm, aligned, status, ...
    srv.stats()              # latency p50/p99, batches, ...
    srv.close()

The server owns its context: while it lives no other call may use it.
"""
import ctypes

import numpy as np

from . import _lib
from .batch import _groups

FO_KIND_CLUSTER = 0
FO_KIND_BULK = 1


class Server(object):
    def __init__(self, ctx=None, precision="mixed", max_batch=4096, max_queue=0, max_wait_ms=0.0,
                 hbm_budget_bytes=0, workers=2):
        self.ctx = ctx or _lib.Context(precision=precision, hbm_budget_bytes=hbm_budget_bytes)
        self.lib = self.ctx.lib
        opts = _lib.FoServerOpts(int(max_batch), int(max_queue), float(max_wait_ms), int(workers), 0)
        h = ctypes.c_void_p()
        self.ctx.check(self.lib.fo_server_create(self.ctx.h, ctypes.byref(opts), ctypes.byref(h)),
                       "server create")
        self.h = h
        self.natoms = {}
        _lib.track("servers", self)

    # -- submission ---------------------------------------------------------------
    def _submit(self, req, pos1, pos2, perm):
        p1 = np.ascontiguousarray(np.asarray(pos1, np.float64).reshape(-1))
        p2 = np.ascontiguousarray(np.asarray(pos2, np.float64).reshape(-1))
        n = len(p1) // 3
        if len(p2) != 3 * n:
            raise ValueError("pos1 and pos2 must hold the same number of atoms")
        flat, sizes = _groups(perm, n)
        req.natoms = n
        req.ngroups = len(sizes)
        req.pos1 = _lib.d(p1)
        req.pos2 = _lib.d(p2)
        req.perm = _lib.i(flat)
        req.group_sizes = _lib.i(sizes)
        t = ctypes.c_int64()
        self.ctx.check(self.lib.fo_server_submit(self.h, ctypes.byref(req), ctypes.byref(t)), "submit")
        self.natoms[t.value] = n
        return t.value

    def submit_cluster(self, pos1, pos2, perm=None, Jmax=15, scale=0.3, nrot=10, invert=True):
        """A SphericalAlign request; returns its ticket."""
        req = _lib.FoRequest()
        req.kind = FO_KIND_CLUSTER
        req.jmax = int(Jmax)
        req.nrot = int(nrot)
        req.invert = int(bool(invert))
        req.sigma = float(scale) if scale is not None else 0.0
        return self._submit(req, pos1, pos2, perm)

    def submit_periodic(self, pos1, pos2, box, perm=None, scale=0.0, nwave=0, nfspace=0, ndisps=10):
        """A PeriodicAlign request; returns its ticket."""
        req = _lib.FoRequest()
        req.kind = FO_KIND_BULK
        req.nrot = int(ndisps)
        req.nwave = int(nwave or 0)
        req.nfspace = int(nfspace or 0)
        req.sigma = float(scale) if scale else 0.0
        b = np.broadcast_to(np.asarray(box, np.float64).ravel(), (3,))
        for k in range(3):
            req.box[k] = float(b[k])
        return self._submit(req, pos1, pos2, perm)

    # -- completion ---------------------------------------------------------------
    def _collect(self, fn, ticket, *extra):
        n = self.natoms[ticket]
        res = _lib.FoPairResult()
        al = np.zeros(3 * n)
        pb = np.zeros(n, np.int32)
        st = fn(self.h, ctypes.c_int64(ticket), *extra, ctypes.byref(res), _lib.d(al), _lib.i(pb))
        if st == 9:   # not ready
            return None
        if st == 4 and extra:   # wait timed out
            return None
        del self.natoms[ticket]
        return {"status": int(st), "dist": res.dist, "rmat": np.array(res.rmat[:]).reshape(3, 3),
                "disp": np.array(res.disp[:]), "inverted": bool(res.inverted), "ncand": res.ncand,
                "niter": res.niter, "overlap_max": res.overlap_max, "sigma": res.sigma,
                "aligned": al.reshape(-1, 3), "perm": pb}

    def poll(self, ticket):
        """The result dict, or None while the request is in flight."""
        return self._collect(self.lib.fo_server_poll, ticket)

    def wait(self, ticket, timeout_ms=-1.0):
        """Block until the request completes (None if timeout_ms runs out)."""
        return self._collect(self.lib.fo_server_wait, ticket, ctypes.c_double(timeout_ms))

    def stats(self):
        st = _lib.FoServerStats()
        self.ctx.check(self.lib.fo_server_stats_get(self.h, ctypes.byref(st)), "server stats")
        return {k: getattr(st, k) for k, _ in _lib.FoServerStats._fields_}

    def close(self):
        """Complete every queued request and stop the worker."""
        if self.h is not None:
            self.lib.fo_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
