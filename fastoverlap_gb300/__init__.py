"""fastoverlap_gb300 -- GB300 (sm_103a) implementation of the FASTOVERLAP
alignment path.

Public classes keep the upstream names and signatures:
    SphericalAlign, SphericalAlignFortran   (cluster alignment)
    SphericalHarmonicAlign, SphericalHarmonicAlignFortran
                                            (cluster alignment, harmonic-oscillator basis)
    PeriodicAlign, PeriodicAlignFortran     (periodic alignment)
Batched and resident forms:
    align_clusters, align_periodic, ClusterBatch, BulkBatch
Peak search on an overlap grid (the Fortran FINDPEAKS):
    findpeaks
Serving (requests admitted as they arrive, continuous batching):
    Server
All compute runs in libfastoverlap_gb300.so (CUDA); there is no CPU path.
"""
from ._lib import Context, FoError, default_context, load  # noqa: F401
from .batch import (BulkBatch, ClusterBatch, HarmonicClusterBatch, align_clusters, align_periodic,  # noqa: F401
                    findpeaks)
from .serve import Server  # noqa: F401
from .periodicAlignment import PeriodicAlign, PeriodicAlignFortran  # noqa: F401
from .bnbAlignment import BranchandBoundMaster, bnb_align_clusters  # noqa: F401
from .sphericalAlignment import (SphericalAlign, SphericalAlignFortran, SphericalHarmonicAlign,  # noqa: F401
                                 SphericalHarmonicAlignFortran)

__all__ = ["SphericalAlign", "SphericalAlignFortran", "SphericalHarmonicAlign", "SphericalHarmonicAlignFortran",
           "HarmonicClusterBatch", "PeriodicAlign", "PeriodicAlignFortran", "BranchandBoundMaster",
           "bnb_align_clusters",
           "align_clusters", "align_periodic", "ClusterBatch", "BulkBatch", "findpeaks", "Server", "Context",
           "FoError", "default_context", "load"]
