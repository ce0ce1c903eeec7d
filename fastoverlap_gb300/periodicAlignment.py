"""Periodic (bulk) alignment classes with the upstream signatures.

Drop-in for fastoverlap/periodicAlignment.py's `PeriodicAlign` (:341-479)
and `PeriodicAlignFortran` (:482-605), group alignment included
(`alignGroup`, :462-479 and :570-605 / fastbulk.f90 ALIGNGROUP :336-412).  Both run the GPU pipeline of the
Fortran bulk path (fastbulk.f90 ALIGN/ALIGN1): structure factors, damped
cross product, 3-D FFT, peak fits, iterative permutation/displacement
refinement from every peak.
"""
import ctypes

import numpy as np

from . import _lib
from .batch import BulkBatch


class PeriodicAlign(object):
    """PeriodicAlign(Natoms, boxvec, permlist=None, dim=3, scale=None, n=None)

    scale : Gaussian width, default (V/N)^(1/3)/3.
    n : wave vectors per axis K, default ceil(1.3 N^(1/3)); the translation
        grid has FASTLEN(4K+3)^3 points.
    """

    def __init__(self, Natoms, boxvec, permlist=None, dim=3, scale=None, n=None,
                 precision="fp64", ctx=None):
        if dim != 3:
            raise NotImplementedError("only dim=3 is supported")
        self.Natoms = Natoms
        self.boxvec = np.array(boxvec, dtype=float)
        self.dim = dim
        self.perm = [np.arange(Natoms)] if permlist is None else [np.asarray(p) for p in permlist]
        if scale is None:
            scale = (np.prod(self.boxvec) / self.Natoms) ** (1. / self.dim) / 3.
        self.scale = scale
        self.n = int(np.ceil(1.3 * Natoms ** (1. / 3.))) if n is None else n
        self.precision = precision
        self._ctx = ctx

    @property
    def ctx(self):
        if self._ctx is None:
            self._ctx = _lib.default_context(self.precision)
        return self._ctx

    def periodic(self, x, copy=False):
        if copy:
            x = x.copy()
        x -= np.round(x / self.boxvec) * self.boxvec
        return x

    def get_dist(self, X1, X2):
        return np.linalg.norm(self.periodic(X1 - X2, True))

    def align(self, pos1, pos2, Cs=None, npeaks=1, width=2):
        """Returns (distance, X1 wrapped pos1, X2 aligned pos2, perm, disp) with
        X2 = periodic(pos2[perm] - disp) as upstream (periodicAlignment.py:27-80)."""
        if Cs is not None:
            raise NotImplementedError("precomputed coefficients are not taken by the GPU path")
        pos1 = np.asarray(pos1, float).reshape(-1, 3)
        pos2 = np.asarray(pos2, float).reshape(-1, 3)
        b = BulkBatch(self.ctx, [pos1], [pos2], self.boxvec, [self.perm], scale=self.scale,
                      nwave=self.n, nfspace=0, ndisps=max(1, int(npeaks)))
        out = b.run()
        r = out["result"][0]
        if r["status"] != 0:
            raise _lib.FoError(int(r["status"]), "periodic alignment failed")
        perm = out["perm"][0].copy()
        disp = -np.asarray(r["disp"], float)
        X1 = self.periodic(pos1, True)
        X2 = self.periodic(pos2[perm] - disp[None, :], True)
        return float(r["dist"]), X1, X2, perm, disp

    def alignGroup(self, coords, keepCoords=False, npeaks=1, width=2, chunk=4096):
        """Every structure of `coords` aligned onto every other, as
        periodicAlignment.py:462-479: dists[i, j] = align(coords[i],
        coords[j])[0]; with keepCoords also aligned[0, i, j] = X1 and
        aligned[1, i, j] = X2.  All pairs run as periodic batches of at most
        `chunk` pairs; `width` is taken as align takes it (the peak search
        starts at half-width 2 and widens)."""
        coords = [np.asarray(p, float).reshape(-1, 3) for p in coords]
        n = len(coords)
        dists = np.zeros((n, n))
        aligned = np.empty((2, n, n) + coords[0].shape) if keepCoords else None
        pairs = [(i, j) for i in range(n) for j in range(n)]
        for c0 in range(0, len(pairs), chunk):
            part = pairs[c0:c0 + chunk]
            b = BulkBatch(self.ctx, [coords[i] for i, _ in part], [coords[j] for _, j in part],
                          self.boxvec, [self.perm] * len(part), scale=self.scale, nwave=self.n,
                          nfspace=0, ndisps=max(1, int(npeaks)))
            out = b.run()
            for k, (i, j) in enumerate(part):
                r = out["result"][k]
                if r["status"] != 0:
                    raise _lib.FoError(int(r["status"]), "periodic alignment of (%d, %d) failed" % (i, j))
                dists[i, j] = r["dist"]
                if keepCoords:
                    disp = -np.asarray(r["disp"], float)
                    aligned[0, i, j] = self.periodic(coords[i], True)
                    aligned[1, i, j] = self.periodic(coords[j][out["perm"][k]] - disp[None, :], True)
        if keepCoords:
            return dists, aligned
        return dists

    def __call__(self, pos1, pos2, *args, **kwargs):
        return self.align(pos1, pos2, *args, **kwargs)


class PeriodicAlignFortran(object):
    """PeriodicAlignFortran(Natoms, boxVec=None, scale=0, perm=None)

    align(pos1, pos2, ndisps=10, perm=None, ohcell=False, debug=False)
        -> (distance, X1 copy of pos1, X2 aligned pos2, perm)
    """

    def __init__(self, Natoms, boxVec=None, scale=0, perm=None, precision="fp64", ctx=None):
        self.Natoms = 1 if Natoms is None else Natoms
        self.boxvec = np.array(boxVec, dtype=float)
        self.scale = scale
        self.precision = precision
        self._ctx = ctx
        self.setPerm([np.arange(self.Natoms)] if perm is None else perm)

    @property
    def ctx(self):
        if self._ctx is None:
            self._ctx = _lib.default_context(self.precision)
        return self._ctx

    def setPerm(self, perm):
        if len(perm):
            self.perm = [np.asarray(p) for p in perm]
            self.nperm = len(perm)
            self.npermsize = [len(p) for p in perm]
            self.permgroup = np.concatenate([np.asarray(p) + 1 for p in perm])
            self.Natoms = len(self.permgroup)
        else:
            self.nperm = 1
            self.npermsize = [self.Natoms]
            self.permgroup = np.arange(self.Natoms) + 1
            self.perm = [self.permgroup - 1]

    def align(self, pos1, pos2, ndisps=10, perm=None, ohcell=False, debug=False):
        """With ohcell, pos2 is also tried under the 48 operations of the cubic
        point group (COMMONS OHCELLT); X2 is then the transformed, aligned pos2
        and self.ohop the winning operation (row-major 3x3)."""
        pos1 = np.asarray(pos1, float).reshape(-1, 3)
        pos2 = np.asarray(pos2, float).reshape(-1, 3)
        if perm is not None:
            self.setPerm(perm)
        if len(pos2) != self.Natoms:
            self.setPerm([np.arange(len(pos2))])
        b = BulkBatch(self.ctx, [pos1], [pos2], self.boxvec, [self.perm],
                      scale=self.scale if self.scale else 0.0, nwave=0, nfspace=0, ndisps=ndisps,
                      ohcell=bool(ohcell))
        out = b.run()
        r = out["result"][0]
        if r["status"] != 0:
            raise _lib.FoError(int(r["status"]), "periodic alignment failed")
        self.ohop = np.asarray(r["rmat"], float).reshape(3, 3).copy()
        return float(r["dist"]), pos1.copy(), out["aligned"][0].copy(), out["perm"][0].copy()

    def alignGroup(self, coords, ndisps=1):
        """Aligns a list of coordinates with themselves through
        fo_bulk_align_group (BULKFASTOVERLAP::ALIGNGROUP with SYM, as
        periodicAlignment.py:570-605 calls it).  The Gaussian width, K and M
        come from CALCDEFAULTS whatever `scale` is, as there.

        Returns dists (nlist, nlist): [i, j] for i >= j is structure j aligned
        onto structure i, the other entries 0; and aligned
        (Natoms, 3, nlist, nlist)."""
        coordslist = np.asarray(coords, dtype=float)
        nlist, natoms, dim = coordslist.shape
        assert dim == 3
        assert natoms == self.Natoms
        lib = self.ctx.lib
        kw, nw, nf = ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
        bx, by, bz = (float(v) for v in self.boxvec)
        self.ctx.check(lib.fo_bulk_calcdefaults(natoms, bx, by, bz, ctypes.byref(kw), ctypes.byref(nw),
                                                ctypes.byref(nf)), "calcdefaults")
        pg = np.ascontiguousarray(self.permgroup, dtype=np.int32)
        ns = np.ascontiguousarray(self.npermsize, dtype=np.int32)
        self.ctx.check(lib.fo_setperm(self.ctx.h, natoms, _lib.i(pg), _lib.i(ns), len(ns)), "setperm")
        flat = np.ascontiguousarray(coordslist.reshape(nlist, 3 * natoms))   # (3N, nlist) column-major
        dist = np.zeros(nlist * nlist)
        al = np.zeros(nlist * nlist * 3 * natoms)
        st = lib.fo_bulk_align_group(self.ctx.h, _lib.d(flat), nlist, _lib.d(flat), nlist, natoms, 0,
                                     bx, by, bz, kw.value, int(ndisps), nw.value, nf.value,
                                     _lib.d(dist), _lib.d(al), 1)
        self.ctx.check(st, "align group")
        dists = dist.reshape(nlist, nlist, order="F")
        aligned = al.reshape(3 * natoms, nlist, nlist, order="F").reshape(natoms, 3, nlist, nlist)
        return dists, aligned

    def __call__(self, pos1, pos2, *args, **kwargs):
        return self.align(pos1, pos2, *args, **kwargs)
