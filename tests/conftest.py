import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    return load


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def fo():
    import fastoverlap_gb300 as F
    F.load()
    return F


def _peak_agreement(ours, ref, nref, G):
    """Peaks (k, 3) of one grid against the upstream findPeaks fixture.
    ours: 1-based fractional grid coordinates (FINDPEAKS convention); ref:
    upstream 0-based coordinates (nref valid rows).  Returns the first peak's
    largest coordinate difference and the fraction of upstream peaks that have
    one of ours within 0.05 cells (periodic distance on the G grid)."""
    ours = np.asarray(ours, float) - 1.0
    ref = np.asarray(ref, float)[:nref]
    def pdist(a, b):
        d = np.abs(a - b) % G
        return np.minimum(d, G - d)
    first = float(pdist(ours[0], ref[0]).max())
    d = pdist(ref[:, None, :], ours[None, :, :]).max(2)
    return first, float((d.min(1) < 0.05).mean())


@pytest.fixture(scope="session")
def peak_agreement():
    return _peak_agreement
