"""Import the upstream fastoverlap Python package in place, for fixture generation.

The upstream code targets older numpy/scipy/munkres APIs.  This module installs
small in-memory compatibility shims (no file of the upstream tree is modified)
and imports the package from a read-only checkout whose path the environment
variable ``FO_REF_ROOT`` must give (there is no default).  It is used
only by ``make_golden.py`` to produce the committed fixtures; nothing in the
library or in the GPU tests imports it.

Shims installed:
  * ``scipy.special.sph_harm(m, n, az, pol)`` -> ``sph_harm_y(n, m, pol, az)``
  * ``scipy.median`` -> ``numpy.median``
  * ``scipy.special.orthogonal`` / ``scipy.special.basic`` aliases
  * ``numpy.NaN`` -> ``numpy.nan``
  * a ``munkres`` module whose ``Munkres().compute`` wraps
    ``scipy.optimize.linear_sum_assignment`` (exact for the dense costs used)
"""
import os
import sys
import types

import numpy as np
import scipy
import scipy.special
import scipy.optimize


def install_shims():
    if not hasattr(scipy.special, "sph_harm"):
        def sph_harm(m, n, az, pol):
            return scipy.special.sph_harm_y(n, m, pol, az)
        scipy.special.sph_harm = sph_harm
    if not hasattr(scipy, "median"):
        scipy.median = np.median
    if not hasattr(np, "NaN"):
        np.NaN = np.nan
    orth = types.ModuleType("scipy.special.orthogonal")
    orth.genlaguerre = scipy.special.genlaguerre
    orth.eval_genlaguerre = scipy.special.eval_genlaguerre
    sys.modules["scipy.special.orthogonal"] = orth
    scipy.special.orthogonal = orth
    basic = types.ModuleType("scipy.special.basic")
    basic.factorial = scipy.special.factorial
    basic.comb = scipy.special.comb
    sys.modules["scipy.special.basic"] = basic
    scipy.special.basic = basic
    munk = types.ModuleType("munkres")

    class Munkres(object):
        def compute(self, cost):
            r, c = scipy.optimize.linear_sum_assignment(np.asarray(cost))
            return list(zip(r.tolist(), c.tolist()))
    munk.Munkres = Munkres
    sys.modules["munkres"] = munk


def reference_root():
    """The upstream checkout named by FO_REF_ROOT (required)."""
    root = os.environ.get("FO_REF_ROOT")
    if not root:
        raise RuntimeError("set FO_REF_ROOT to the upstream fastoverlap checkout")
    return root


def import_reference(root=None):
    root = root or reference_root()
    install_shims()
    sys.dont_write_bytecode = True
    if root not in sys.path:
        sys.path.insert(0, root)
    import fastoverlap  # noqa: F401
    from fastoverlap import sphericalAlignment, periodicAlignment, soft, utils
    return types.SimpleNamespace(pkg=fastoverlap, sph=sphericalAlignment,
                                 per=periodicAlignment, soft=soft, utils=utils)
