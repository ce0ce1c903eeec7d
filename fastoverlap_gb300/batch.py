"""Batched alignment through the C ABI: pack many pairs, run one pipeline.

`ClusterBatch` / `BulkBatch` pack a list of pairs into the flat arrays the C
ABI takes (fo_cluster_pair / fo_bulk_pair), and either run them once
(`run`) or keep them resident on the GPU as a plan (`plan`, then
`plan_run` / `plan_wait` / `plan_results`) so that the inputs stay in HBM
between runs.
"""
import ctypes

import numpy as np

from . import _lib


def _groups(perm, n):
    if perm is None:
        perm = [np.arange(n)]
    flat = np.concatenate([np.asarray(p, dtype=np.int32).ravel() for p in perm]).astype(np.int32)
    sizes = np.array([len(np.asarray(p).ravel()) for p in perm], np.int32)
    return flat, sizes


class _Packed(object):
    def __init__(self, pos1, pos2, perms):
        self.n = np.array([len(np.asarray(p).reshape(-1, 3)) for p in pos1], np.int64)
        self.off = np.zeros(len(pos1), np.int64)
        if len(pos1) > 1:
            self.off[1:] = np.cumsum(self.n)[:-1]
        self.pos1 = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1)
                                                         for p in pos1]))
        self.pos2 = np.ascontiguousarray(np.concatenate([np.asarray(p, np.float64).reshape(-1)
                                                         for p in pos2]))
        flats, sizes = [], []
        self.perm_off = np.zeros(len(pos1), np.int64)
        self.group_off = np.zeros(len(pos1), np.int64)
        self.ngroups = np.zeros(len(pos1), np.int32)
        po = go = 0
        for k, (n, perm) in enumerate(zip(self.n, perms)):
            f, s = _groups(perm, int(n))
            flats.append(f)
            sizes.append(s)
            self.perm_off[k] = po
            self.group_off[k] = go
            self.ngroups[k] = len(s)
            po += len(f)
            go += len(s)
        self.perm = np.ascontiguousarray(np.concatenate(flats), np.int32)
        self.sizes = np.ascontiguousarray(np.concatenate(sizes), np.int32)
        self.natoms_total = int(self.n.sum())

    @property
    def h2d_bytes(self):
        return self.pos1.nbytes + self.pos2.nbytes + self.perm.nbytes + self.sizes.nbytes


class _BatchBase(object):
    kind = None

    def __init__(self, ctx, pos1, pos2, perms=None):
        self.ctx = ctx
        if perms is None:
            perms = [None] * len(pos1)
        if not (len(pos1) == len(pos2) == len(perms)):
            raise ValueError("pos1, pos2 and perms must have the same length")
        self.pk = _Packed(pos1, pos2, perms)
        self.npairs = len(pos1)
        self.plan_h = None

    # -- page-locked host buffers -------------------------------------------
    def pin(self):
        """Page-lock the packed input arrays and keep page-locked output arrays
        for run(), so that a batch's host<->device copies go by DMA.  After
        pin(), the per-atom arrays run() returns are views into the batch's
        output buffers, valid until its next run()."""
        if getattr(self, "_pinned", None):
            return self
        lib, h = self.ctx.lib, self.ctx.h
        self._out = (np.zeros(3 * self.pk.natoms_total), np.zeros(self.pk.natoms_total, np.int32))
        bufs = [self.pk.pos1, self.pk.pos2, self.pk.perm, self.pk.sizes, *self._out]
        self._pinned = []
        for b in bufs:
            if b.nbytes:
                self.ctx.check(lib.fo_host_register(h, b.ctypes.data, b.nbytes), "host register")
                self._pinned.append(b)
        return self

    def unpin(self):
        for b in getattr(self, "_pinned", None) or []:
            self.ctx.lib.fo_host_unregister(self.ctx.h, b.ctypes.data)
        self._pinned = None
        self._out = None

    # -- one-shot ------------------------------------------------------------
    def run(self):
        lib = self.ctx.lib
        if getattr(self, "_out", None) is not None:
            aligned, permbest = self._out
        else:
            aligned = np.zeros(3 * self.pk.natoms_total)
            permbest = np.zeros(self.pk.natoms_total, np.int32)
        res = np.zeros(self.npairs, _lib.RESULT_DTYPE)
        args = (self.ctx.h, self.npairs, _lib.vp(self.desc), _lib.d(self.pk.pos1), _lib.d(self.pk.pos2),
                _lib.i(self.pk.perm), _lib.i(self.pk.sizes), 0)
        if self.kind == "harmonic":
            st = lib.fo_cluster_harm_align_batch(*args, int(self.nmax), float(self.harmscale), _lib.d(aligned),
                                                 _lib.i(permbest), _lib.vp(res))
        else:
            fn = lib.fo_cluster_align_batch if self.kind == "cluster" else lib.fo_bulk_align_batch
            st = fn(*args, _lib.d(aligned), _lib.i(permbest), _lib.vp(res))
        self.ctx.check(st, "align batch")
        return self._unpack(res, aligned, permbest)

    # -- resident plan ---------------------------------------------------------
    def plan(self):
        lib = self.ctx.lib
        h = ctypes.c_void_p()
        args = (self.ctx.h, self.npairs, _lib.vp(self.desc), _lib.d(self.pk.pos1), _lib.d(self.pk.pos2),
                _lib.i(self.pk.perm), _lib.i(self.pk.sizes), 0)
        if self.kind == "harmonic":
            st = lib.fo_cluster_harm_plan_create(*args, int(self.nmax), float(self.harmscale), ctypes.byref(h))
        else:
            fn = lib.fo_cluster_plan_create if self.kind == "cluster" else lib.fo_bulk_plan_create
            st = fn(*args, ctypes.byref(h))
        self.ctx.check(st, "plan create")
        self.plan_h = h
        _lib.track("plans", self)
        return self

    def plan_graph(self, on=True):
        """Replay the plan's runs as a captured CUDA graph (from the second run on)."""
        self.ctx.check(self.ctx.lib.fo_plan_set_graph(self.plan_h, int(bool(on))), "plan graph")
        return self

    def plan_run(self):
        self.ctx.check(self.ctx.lib.fo_plan_run(self.plan_h), "plan run")

    def plan_wait(self):
        self.ctx.check(self.ctx.lib.fo_plan_wait(self.plan_h), "plan wait")

    def plan_results(self, with_coords=True):
        aligned = np.zeros(3 * self.pk.natoms_total) if with_coords else None
        permbest = np.zeros(self.pk.natoms_total, np.int32) if with_coords else None
        res = np.zeros(self.npairs, _lib.RESULT_DTYPE)
        st = self.ctx.lib.fo_plan_results(self.plan_h,
                                          _lib.d(aligned) if aligned is not None else None,
                                          _lib.i(permbest) if permbest is not None else None,
                                          _lib.vp(res))
        self.ctx.check(st, "plan results")
        return self._unpack(res, aligned, permbest)

    def plan_device_bytes(self):
        return int(self.ctx.lib.fo_plan_device_bytes(self.plan_h))

    def plan_tile_shape(self):
        """(chunk, group) of the tensor-core stage ((0, 0) when not used)."""
        c, g = ctypes.c_int(0), ctypes.c_int(0)
        self.ctx.check(self.ctx.lib.fo_plan_tile_shape(self.plan_h, ctypes.byref(c), ctypes.byref(g)), "tile shape")
        return c.value, g.value

    def plan_launches(self):
        """Kernel launches one plan_run issues."""
        return int(self.ctx.lib.fo_plan_launches(self.plan_h))

    def close(self):
        if self.plan_h is not None:
            self.ctx.lib.fo_plan_destroy(self.plan_h)
            self.plan_h = None
        self.unpin()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _unpack(self, res, aligned, permbest):
        out = {"result": res, "dist": res["dist"].copy(), "status": res["status"].copy()}
        if aligned is not None:
            al = aligned.reshape(-1, 3)
            if not hasattr(self, "_spans"):   # Python ints slice faster than numpy scalars
                self._spans = list(zip(self.pk.off.tolist(), (self.pk.off + self.pk.n).tolist()))
            out["aligned"] = [al[a:b] for a, b in self._spans]
            out["perm"] = [permbest[a:b] for a, b in self._spans]
        return out


class ClusterBatch(_BatchBase):
    """Many spherical (cluster) pairs.  params: per-pair dicts or scalars for
    Jmax, scale (sigma), nrot, invert."""
    kind = "cluster"

    def __init__(self, ctx, pos1, pos2, perms=None, Jmax=15, scale=0.3, nrot=10, invert=True):
        super().__init__(ctx, pos1, pos2, perms)
        npairs = self.npairs
        J = np.broadcast_to(np.asarray(Jmax), (npairs,))
        S = np.broadcast_to(np.asarray(scale if scale is not None else 0.0, float), (npairs,))
        R = np.broadcast_to(np.asarray(nrot), (npairs,))
        I = np.broadcast_to(np.asarray(invert), (npairs,))
        desc = (_lib.FoClusterPair * npairs)()
        for k in range(npairs):
            dsc = desc[k]
            dsc.natoms = int(self.pk.n[k])
            dsc.ngroups = int(self.pk.ngroups[k])
            dsc.jmax = int(J[k])
            dsc.nrot = int(R[k])
            dsc.invert = int(bool(I[k]))
            dsc.sigma = float(S[k])
            dsc.coord_off = int(self.pk.off[k])
            dsc.perm_off = int(self.pk.perm_off[k])
            dsc.group_off = int(self.pk.group_off[k])
        self.desc = np.frombuffer(desc, dtype=np.uint8).copy()


class HarmonicClusterBatch(ClusterBatch):
    """Cluster pairs in the harmonic-oscillator basis (SphericalHarmonicAlign /
    ALIGNHARM): coefficients of the coordinates as given, orders n <= nmax at
    length scale harmscale; `scale` is the kernel width (> 0)."""
    kind = "harmonic"

    def __init__(self, ctx, pos1, pos2, perms=None, Jmax=15, scale=0.3, nrot=10, invert=True, nmax=20,
                 harmscale=1.0):
        super().__init__(ctx, pos1, pos2, perms, Jmax=Jmax, scale=scale, nrot=nrot, invert=invert)
        self.nmax = int(nmax)
        self.harmscale = float(harmscale)


class BulkBatch(_BatchBase):
    """Many periodic (bulk) pairs with per-pair box, width, K, M, ndisps."""
    kind = "bulk"

    def __init__(self, ctx, pos1, pos2, boxes, perms=None, scale=0.0, nwave=0, nfspace=0,
                 ndisps=10, ohcell=False):
        super().__init__(ctx, pos1, pos2, perms)
        npairs = self.npairs
        boxes = np.broadcast_to(np.asarray(boxes, float).reshape(-1, 3), (npairs, 3))
        S = np.broadcast_to(np.asarray(scale if scale is not None else 0.0, float), (npairs,))
        K = np.broadcast_to(np.asarray(nwave if nwave is not None else 0), (npairs,))
        M = np.broadcast_to(np.asarray(nfspace if nfspace is not None else 0), (npairs,))
        D = np.broadcast_to(np.asarray(ndisps), (npairs,))
        O = np.broadcast_to(np.asarray(ohcell), (npairs,))
        desc = (_lib.FoBulkPair * npairs)()
        for k in range(npairs):
            dsc = desc[k]
            dsc.natoms = int(self.pk.n[k])
            dsc.ngroups = int(self.pk.ngroups[k])
            dsc.nwave = int(K[k])
            dsc.nfspace = int(M[k])
            dsc.ndisps = int(D[k])
            dsc.ohcell = int(bool(O[k]))
            dsc.sigma = float(S[k])
            for c in range(3):
                dsc.box[c] = float(boxes[k, c])
            dsc.coord_off = int(self.pk.off[k])
            dsc.perm_off = int(self.pk.perm_off[k])
            dsc.group_off = int(self.pk.group_off[k])
        self.desc = np.frombuffer(desc, dtype=np.uint8).copy()


def align_clusters(pos1, pos2, perms=None, Jmax=15, scale=0.3, nrot=10, invert=True,
                   precision="fp64", ctx=None):
    """Align many cluster pairs in one GPU pipeline; returns dict of arrays."""
    ctx = ctx or _lib.default_context(precision)
    return ClusterBatch(ctx, pos1, pos2, perms, Jmax, scale, nrot, invert).run()


def align_periodic(pos1, pos2, boxes, perms=None, scale=0.0, nwave=0, nfspace=0, ndisps=10,
                   precision="fp64", ctx=None):
    """Align many periodic pairs in one GPU pipeline; returns dict of arrays."""
    ctx = ctx or _lib.default_context(precision)
    return BulkBatch(ctx, pos1, pos2, boxes, perms, scale, nwave, nfspace, ndisps).run()


def cluster_overlap(pos1, pos2, perm=None, Jmax=15, scale=0.3, precision="fp64", ctx=None):
    """SO(3) coefficients [l, m1, m2] and the overlap grid [alpha, beta, gamma]
    of one pair (the non-inverted orientation), computed on the GPU."""
    ctx = ctx or _lib.default_context(precision)
    b = ClusterBatch(ctx, [pos1], [pos2], [perm], Jmax=Jmax, scale=scale, nrot=1, invert=False)
    L = int(Jmax)
    W, G = 2 * L + 1, 2 * (L + 1)
    coef = np.zeros(2 * (L + 1) * W * W)
    grid = np.zeros(G ** 3)
    st = ctx.lib.fo_cluster_overlap(ctx.h, _lib.vp(b.desc), _lib.d(b.pk.pos1), _lib.d(b.pk.pos2),
                                    _lib.i(b.pk.perm), _lib.i(b.pk.sizes), 0, _lib.d(coef),
                                    _lib.d(grid))
    ctx.check(st, "cluster overlap")
    c = (coef[0::2] + 1j * coef[1::2]).reshape(L + 1, W, W)
    return c, grid.reshape(G, G, G).transpose(2, 1, 0)


def bulk_overlap(pos1, pos2, box, perm=None, scale=0.0, nwave=0, nfspace=0, precision="fp64",
                 ctx=None):
    """Translation overlap grid |F| [x, y, z] of one periodic pair on the GPU."""
    ctx = ctx or _lib.default_context(precision)
    b = BulkBatch(ctx, [pos1], [pos2], box, [perm], scale=scale, nwave=nwave, nfspace=nfspace,
                  ndisps=1)
    n = len(np.asarray(pos1).reshape(-1, 3))
    K = nwave if nwave else int(np.ceil(1.3 * n ** (1.0 / 3.0)))
    M = nfspace if nfspace else _fastlen(4 * K + 3)
    grid = np.zeros(M ** 3)
    st = ctx.lib.fo_bulk_overlap(ctx.h, _lib.vp(b.desc), _lib.d(b.pk.pos1), _lib.d(b.pk.pos2),
                                 _lib.i(b.pk.perm), _lib.i(b.pk.sizes), 0, _lib.d(grid))
    ctx.check(st, "bulk overlap")
    return grid.reshape(M, M, M).transpose(2, 1, 0)


def findpeaks(grid, npeaks=10, width=2, precision="fp64", ctx=None):
    """Peaks of a periodic cubic grid indexed [i1, i2, i3] on the GPU, as the
    Fortran FINDPEAKS returns them (fastoverlap/f90/fastutils.f90:475-548):
    (peaks (k, 3) as 1-based fractional grid coordinates, amplitudes (k,)).
    Raises FoError when no peak is found (where FINDPEAKS stops)."""
    ctx = ctx or _lib.default_context(precision)
    g = np.asarray(grid, dtype=np.float64)
    n = g.shape[0]
    if g.shape != (n, n, n):
        raise ValueError("grid must be cubic, got shape %s" % (g.shape,))
    flat = np.ascontiguousarray(g.transpose(2, 1, 0)).ravel()   # i1 fastest
    pk = np.zeros(3 * npeaks)
    am = np.zeros(npeaks)
    nf = np.zeros(1, np.int32)
    st = ctx.lib.fo_findpeaks(ctx.h, _lib.d(flat), n, int(npeaks), int(width), _lib.d(pk), _lib.d(am),
                              _lib.i(nf))
    ctx.check(st, "findpeaks")
    k = int(nf[0])
    return pk[:3 * k].reshape(k, 3), am[:k]


def _fastlen(n):
    m = max(1, int(n))
    while True:
        k = m
        for f in (2, 3, 5):
            while k % f == 0:
                k //= f
        if k == 1:
            return m
        m += 1
