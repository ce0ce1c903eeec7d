"""Cluster (spherical) alignment classes with the upstream signatures.

Drop-in for fastoverlap/sphericalAlignment.py's `SphericalAlign`
(:250-273, call path :160-247) and `SphericalAlignFortran` (:441-533), and
for the harmonic-oscillator basis classes `SphericalHarmonicAlign`
(:276-414) and `SphericalHarmonicAlignFortran` (:535-663).  All run the GPU
pipeline of the Fortran cluster path (fastclusters.f90 ALIGN / ALIGNHARM):
SO(3) coefficients, inverse SO(3) transform, peak fits, iterative
permutation/rotation refinement from every peak, inversion check.
"""
import numpy as np

from . import _lib
from .batch import ClusterBatch


def _perm_or_all(perm, default, n):
    if perm is not None:
        return [np.asarray(p) for p in perm]
    if default is not None:
        return [np.asarray(p) for p in default]
    return [np.arange(n)]


class SphericalAlign(object):
    """SphericalAlign(scale=None, Jmax=15, perm=None)

    scale : Gaussian width; None picks 1/3 of the mean nearest-neighbour
        separation of the two structures (CHOOSE_KWIDTH).
    Jmax : maximum angular degree (SO(3) grid (2 Jmax + 2)^3).
    perm : list of index arrays, the permutable groups ("species").
    precision : "fp64" (plain form) or "mixed".
    """

    def __init__(self, scale=None, Jmax=15, perm=None, precision="fp64", ctx=None, cutoff=True):
        self.scale = scale
        self.calcScale = scale is None
        self.Jmax = Jmax
        self.perm = perm
        self.precision = precision
        self.cutoff = cutoff
        self._ctx = ctx

    @property
    def ctx(self):
        if self._ctx is None:
            self._ctx = _lib.default_context(self.precision, cutoff=self.cutoff)
        return self._ctx

    def _run(self, pos1, pos2, perm, invert, nrot):
        pos1 = np.asarray(pos1, float).reshape(-1, 3)
        pos2 = np.asarray(pos2, float).reshape(-1, 3)
        if pos1.shape != pos2.shape:
            raise ValueError("pos1 and pos2 must have the same shape")
        groups = _perm_or_all(perm, self.perm, len(pos1))
        b = ClusterBatch(self.ctx, [pos1], [pos2], [groups], Jmax=self.Jmax,
                         scale=(0.0 if self.calcScale else self.scale), nrot=nrot, invert=invert)
        out = b.run()
        r = out["result"][0]
        if r["status"] != 0:
            raise _lib.FoError(int(r["status"]), "cluster alignment failed")
        if self.calcScale:
            self.scale = float(r["sigma"])
        X1 = pos1 - pos1.mean(0)
        return float(r["dist"]), X1, out["aligned"][0].copy(), r, out["perm"][0].copy()

    def align(self, pos1, pos2, perm=None, invert=True, calcCoeffs=None):
        """Single best peak; returns (distance, X1 centred pos1, X2 aligned pos2)."""
        if calcCoeffs is not None:
            raise NotImplementedError("precomputed coefficients are not taken by the GPU path")
        d, X1, X2, _, _ = self._run(pos1, pos2, perm, invert, 1)
        return d, X1, X2

    def malign(self, pos1, pos2, perm=None, invert=True, calcCoeffs=None, nrot=10):
        if calcCoeffs is not None:
            raise NotImplementedError("precomputed coefficients are not taken by the GPU path")
        d, X1, X2, _, _ = self._run(pos1, pos2, perm, invert, nrot)
        return d, X1, X2

    def __call__(self, pos1, pos2, perm=None, invert=True, calcCoeffs=None, nrot=10, niter=None):
        """Refines the best `nrot` peaks of each orientation; returns
        (distance, X1, X2) like the upstream __call__ (sphericalAlignment.py:237-247).
        `niter` is accepted and unused, as upstream: that __call__ never reads
        it either."""
        return self.malign(pos1, pos2, perm, invert, calcCoeffs, nrot)

    def align_full(self, pos1, pos2, perm=None, invert=True, nrot=10):
        """As __call__, plus rotation matrix, permutation and diagnostics."""
        d, X1, X2, r, pb = self._run(pos1, pos2, perm, invert, nrot)
        return dict(dist=d, X1=X1, X2=X2, rmat=np.asarray(r["rmat"]).reshape(3, 3), perm=pb,
                    inverted=bool(r["inverted"]), ncand=int(r["ncand"]),
                    overlap_max=float(r["overlap_max"]), niter=int(r["niter"]),
                    sigma=float(r["sigma"]))


class SphericalAlignFortran(object):
    """SphericalAlignFortran(scale=0.3, Jmax=15, perm=None, Natoms=None)

    __call__(pos1, pos2, perm=None, invert=True, nrot=10, debug=False)
        -> (distance, X1 centred pos1, X2 aligned pos2, rmatbest)
    """

    def __init__(self, scale=0.3, Jmax=15, perm=None, Natoms=None, precision="fp64", ctx=None,
                 cutoff=True):
        self.scale = scale
        self.Jmax = Jmax
        self.Natoms = Natoms
        self.perm = perm
        if perm is not None:
            self.setPerm(perm)
        self._sa = SphericalAlign(scale if scale and scale > 0 else None, Jmax, perm, precision,
                                  ctx, cutoff)
        self.malign = self.__call__

    def setPerm(self, perm):
        self.Natoms = int(sum(len(p) for p in perm))
        self.perm = perm
        self.nperm = len(perm)
        self.npermsize = [len(p) for p in perm]
        self.permgroup = np.concatenate([np.asarray(p) + 1 for p in perm])

    def align(self, pos1, pos2, perm=None, invert=True, debug=False):
        return self(pos1, pos2, perm, invert, 1, debug)

    def __call__(self, pos1, pos2, perm=None, invert=True, nrot=10, debug=False):
        pos1 = np.asarray(pos1, float).reshape(-1, 3)
        if perm is not None:
            self.setPerm(perm)
        elif self.perm is None or len(pos1) != self.Natoms:
            self.setPerm([np.arange(len(pos1))])
        self._sa.perm = self.perm
        d, X1, X2, r, _ = self._sa._run(pos1, pos2, self.perm, invert, nrot)
        return d, X1, X2, np.asarray(r["rmat"]).reshape(3, 3).copy()


def _average_separation(pos):
    """Mean nearest-neighbour distance (averageSeparation, sphericalAlignment.py:35-41)."""
    d = np.linalg.norm(pos[:, None, :] - pos[None, :, :], axis=-1)
    np.fill_diagonal(d, np.inf)
    return float(d.min(1).mean())


class SphericalHarmonicAlign(object):
    """SphericalHarmonicAlign(scale=None, harmscale=1.0, nmax=15, Jmax=15, perm=None)

    The cluster alignment with the SO(3) coefficients expanded in the
    isotropic harmonic-oscillator basis (sphericalAlignment.py:276-414): both
    structures are centred (COM_shift) and the coefficients c_nlm of orders
    n <= nmax at length scale harmscale are contracted over n.  scale is the
    Gaussian kernel width; None takes (s1 + s2) / 6 from the mean
    nearest-neighbour separations.
    """

    def __init__(self, scale=None, harmscale=1.0, nmax=15, Jmax=15, perm=None, precision="fp64", ctx=None):
        self.scale = scale
        self.calcScale = scale is None
        self.harmscale = harmscale
        self.nmax = nmax
        self.Jmax = Jmax
        self.perm = perm
        self.precision = precision
        self._ctx = ctx

    @property
    def ctx(self):
        if self._ctx is None:
            self._ctx = _lib.default_context(self.precision)
        return self._ctx

    def _batch(self, pos1s, pos2s, perm, invert, nrot):
        from .batch import HarmonicClusterBatch
        X1s, X2s, groups = [], [], []
        for pos1, pos2 in zip(pos1s, pos2s):
            pos1 = np.asarray(pos1, float).reshape(-1, 3)
            pos2 = np.asarray(pos2, float).reshape(-1, 3)
            if pos1.shape != pos2.shape:
                raise ValueError("pos1 and pos2 must have the same shape")
            X1s.append(pos1 - pos1.mean(0))
            X2s.append(pos2 - pos2.mean(0))
            groups.append(_perm_or_all(perm, self.perm, len(pos1)))
        if self.calcScale:
            scales = [(_average_separation(a) + _average_separation(b)) / 6 for a, b in zip(X1s, X2s)]
            self.scale = scales[-1]
        else:
            scales = self.scale
        b = HarmonicClusterBatch(self.ctx, X1s, X2s, groups, Jmax=self.Jmax, scale=scales, nrot=nrot,
                                 invert=invert, nmax=self.nmax, harmscale=self.harmscale)
        out = b.run()
        for k, r in enumerate(out["result"]):
            if r["status"] != 0:
                raise _lib.FoError(int(r["status"]), "harmonic-basis alignment of pair %d failed" % k)
        return X1s, out

    def align(self, pos1, pos2, perm=None, invert=True, calcCoeffs=None):
        """Single best peak; returns (distance, X1 centred pos1, X2 aligned pos2)."""
        return self.malign(pos1, pos2, perm, invert, calcCoeffs, 1)

    def malign(self, pos1, pos2, perm=None, invert=True, calcCoeffs=None, nrot=10):
        if calcCoeffs is not None:
            raise NotImplementedError("precomputed coefficients are not taken by the GPU path")
        X1s, out = self._batch([pos1], [pos2], perm, invert, nrot)
        return float(out["result"][0]["dist"]), X1s[0], out["aligned"][0].copy()

    def __call__(self, pos1, pos2, perm=None, invert=True, calcCoeffs=None, nrot=10, niter=None):
        return self.malign(pos1, pos2, perm, invert, calcCoeffs, nrot)

    def alignGroup(self, coords, keepCoords=False):
        """align() of every ordered pair of `coords` (sphericalAlignment.py:397-414),
        all pairs in one batch: dists[i, j], and with keepCoords aligned[0, i, j]
        = X1, aligned[1, i, j] = X2."""
        coords = [np.asarray(p, float).reshape(-1, 3) for p in coords]
        n = len(coords)
        pairs = [(i, j) for i in range(n) for j in range(n)]
        X1s, out = self._batch([coords[i] for i, _ in pairs], [coords[j] for _, j in pairs], None, True, 1)
        dists = out["result"]["dist"].reshape(n, n).copy()
        if not keepCoords:
            return dists
        aligned = np.empty((2, n, n) + coords[0].shape)
        for k, (i, j) in enumerate(pairs):
            aligned[0, i, j] = X1s[k]
            aligned[1, i, j] = out["aligned"][k]
        return dists, aligned


class SphericalHarmonicAlignFortran(object):
    """SphericalHarmonicAlignFortran(scale=0.3, Jmax=15, harmscale=1.0, nmax=20, perm=None, Natoms=None)

    The harmonic-basis path of the Fortran module (sphericalAlignment.py:535-663)
    through fo_cluster_align_harm (ALIGNHARM: coordinates as given) and
    fo_calc_overlap_matrices (CALCOVERLAPMATRICES).

    __call__(pos1, pos2, perm=None, invert=True, nrot=10, debug=False)
        -> (distance, pos1 as given, X2 aligned pos2, rmatbest)
    compareList(poslist, perm=None) -> (avgoverlap, maxoverlap, navgoverlap, nmaxoverlap)
    """

    def __init__(self, scale=0.3, Jmax=15, harmscale=1.0, nmax=20, perm=None, Natoms=None, precision="fp64",
                 ctx=None):
        self.scale = scale
        self.Jmax = Jmax
        self.harmscale = harmscale
        self.nmax = nmax
        self.Natoms = Natoms
        self.precision = precision
        self._ctx = ctx
        self.perm = None
        if perm is not None:
            self.setPerm(perm)
        elif Natoms is not None:
            self.setPerm([np.arange(Natoms)])
        self.malign = self.__call__

    @property
    def ctx(self):
        if self._ctx is None:
            self._ctx = _lib.default_context(self.precision)
        return self._ctx

    def setPerm(self, perm):
        self.Natoms = int(sum(len(p) for p in perm))
        self.perm = perm
        self.nperm = len(perm)
        self.npermsize = [len(p) for p in perm]
        self.permgroup = np.concatenate([np.asarray(p) + 1 for p in perm])

    def _setperm(self):
        pg = np.ascontiguousarray(self.permgroup, dtype=np.int32)
        ns = np.ascontiguousarray(self.npermsize, dtype=np.int32)
        self.ctx.check(self.ctx.lib.fo_setperm(self.ctx.h, int(self.Natoms), _lib.i(pg), _lib.i(ns), len(ns)),
                       "setperm")

    def align(self, pos1, pos2, perm=None, invert=True, debug=False):
        return self(pos1, pos2, perm, invert, 1, debug)

    def __call__(self, pos1, pos2, perm=None, invert=True, nrot=10, debug=False):
        import ctypes
        if perm is not None:
            self.setPerm(perm)
        elif self.perm is None or len(pos1) != self.Natoms:
            self.setPerm([np.arange(len(pos1))])
        self._setperm()
        coordsb = np.ascontiguousarray(pos1, dtype=float).flatten()
        coordsa = np.ascontiguousarray(pos2, dtype=float).flatten()
        dist, dist2 = ctypes.c_double(), ctypes.c_double()
        rmat = np.zeros(9)
        st = self.ctx.lib.fo_cluster_align_harm(self.ctx.h, _lib.d(coordsb), _lib.d(coordsa), int(self.Natoms),
                                                int(bool(debug)), int(self.nmax), int(self.Jmax),
                                                float(self.harmscale), float(self.scale), ctypes.byref(dist),
                                                ctypes.byref(dist2), _lib.d(rmat), int(nrot), int(bool(invert)))
        self.ctx.check(st, "align harm")
        return (dist.value, coordsb.reshape(self.Natoms, 3), coordsa.reshape(self.Natoms, 3),
                rmat.reshape(3, 3, order="F"))

    def compareList(self, poslist, perm=None):
        """Average (squared-norm) and maximum overlaps of every pair of a list of
        structures, and both normalised by the geometric mean of the diagonals
        (sphericalAlignment.py:622-663).  The structures are centred first."""
        coords = np.array(poslist, dtype=float)
        nlist, natoms, dim = coords.shape
        assert dim == 3
        if perm is None:
            if natoms != self.Natoms or self.perm is None:
                self.Natoms = natoms
                self.setPerm([np.arange(self.Natoms)])
        else:
            self.setPerm(perm)
        self._setperm()
        coords -= coords.mean(1)[:, None, :]
        flat = np.ascontiguousarray(coords.reshape(nlist, -1))   # (3N, nlist) column-major
        avg = np.zeros(nlist * nlist)
        mx = np.zeros(nlist * nlist)
        st = self.ctx.lib.fo_calc_overlap_matrices(self.ctx.h, _lib.d(flat), natoms, nlist, int(self.nmax),
                                                   int(self.Jmax), float(self.harmscale), float(self.scale),
                                                   _lib.d(avg), _lib.d(mx))
        self.ctx.check(st, "overlap matrices")
        avg = avg.reshape(nlist, nlist, order="F")
        mx = mx.reshape(nlist, nlist, order="F")
        da, dm = avg.diagonal(), mx.diagonal()
        return avg, mx, avg / np.sqrt(da[:, None] * da[None, :]), mx / np.sqrt(dm[:, None] * dm[None, :])
