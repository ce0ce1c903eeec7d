"""Cluster (spherical) alignment classes with the upstream signatures.

Drop-in for fastoverlap/sphericalAlignment.py's `SphericalAlign`
(:250-273, call path :160-247) and `SphericalAlignFortran` (:441-533).  Both
run the GPU pipeline of the Fortran cluster path (fastclusters.f90 ALIGN):
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
        (distance, X1, X2) like the upstream __call__ (sphericalAlignment.py:237-247)."""
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
