"""Upstream known answers through the CUDA library (C ABI via ctypes)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("L", [7, 14])
def test_lj38(fo, oracle_mod, golden, prec, L):
    g = golden("lj38")
    r = fo.SphericalAlign(0.3, L, precision=prec).align_full(g["pos1"], g["pos2"])
    ref = float(g["dist_j7"] if L == 7 else g["dist_j14"])
    tol = 1e-8 if prec == "fp64" else 1e-5
    assert abs(r["dist"] - ref) <= tol * ref
    o = oracle_mod.cluster_align(g["pos1"], g["pos2"], Jmax=L, sigma=0.3, nrot=10)
    assert np.array_equal(r["perm"], o["perm"]) and r["inverted"] == o["inverted"]
    # the returned pieces are consistent: X2 = R (+-centred pos2)[perm]
    X2c = g["pos2"] - g["pos2"].mean(0)
    s = -1.0 if r["inverted"] else 1.0
    rebuilt = (s * X2c[r["perm"]]) @ r["rmat"].T
    assert np.abs(rebuilt - r["X2"]).max() < 1e-9
    assert abs(np.linalg.norm(r["X1"] - r["X2"]) - r["dist"]) < 1e-9


def test_lj38_inverted_input(fo, golden):
    g = golden("lj38")
    d = fo.SphericalAlign(0.3, 7)(g["pos1"], -g["pos2"])[0]
    assert abs(d - float(g["dist_j7_inverted"])) <= 1e-8 * d


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_blj256(fo, golden, prec):
    g = golden("blj256")
    n = int(g["ntypeA"])
    pl = [np.arange(n), np.arange(n, 256)]
    d, X1, X2, perm = fo.PeriodicAlignFortran(256, g["box"], perm=pl, precision=prec).align(
        g["pos1"], g["pos2"])
    tol = 1e-8 if prec == "fp64" else 1e-5
    assert abs(d - float(g["dist"])) <= tol * d
    assert sorted(perm[:n]) == list(range(n)) and sorted(perm[n:]) == list(range(n, 256))


def test_blj256_python_class(fo, golden):
    g = golden("blj256")
    n = int(g["ntypeA"])
    pa = fo.PeriodicAlign(256, g["box"], [np.arange(n), np.arange(n, 256)], scale=0.2, n=7)
    d, X1, X2, perm, disp = pa.align(g["pos1"], g["pos2"], npeaks=10)
    assert abs(d - float(g["dist_s02_n7"])) <= 1e-8 * d
    assert abs(pa.get_dist(X1, X2) - d) < 1e-9


def test_fortran_style_entry_points(fo, golden):
    """fo_setperm + fo_cluster_align as a Fortran caller would use them."""
    from fastoverlap_gb300 import _lib
    g = golden("lj38")
    ctx = fo.default_context("fp64")
    lib = ctx.lib
    pg = np.arange(1, 39, dtype=np.int32)
    ctx.check(lib.fo_setperm(ctx.h, 38, _lib.i(pg), _lib.i(np.array([38], np.int32)), 1))
    cb = np.ascontiguousarray(g["pos1"].ravel().copy())
    ca = np.ascontiguousarray(g["pos2"].ravel().copy())
    kw = ctypes.c_double(0.3)
    dist, d2 = ctypes.c_double(), ctypes.c_double()
    rm = np.zeros(9)
    ctx.check(lib.fo_cluster_align(ctx.h, _lib.d(cb), _lib.d(ca), 38, 0, 7, ctypes.byref(kw), 10,
                                   1, ctypes.byref(dist), ctypes.byref(d2), _lib.d(rm)))
    assert abs(dist.value - float(g["dist_j7"])) <= 1e-8 * dist.value
    assert abs(d2.value - dist.value ** 2) < 1e-12
    assert np.abs(cb.reshape(-1, 3).mean(0)).max() < 1e-12       # COORDSB centred in place
    assert abs(np.linalg.norm(cb - ca) - dist.value) < 1e-9      # COORDSA aligned in place
    R = rm.reshape(3, 3, order="F")                              # Fortran RMATBEST(3,3)
    assert np.abs(R @ R.T - np.eye(3)).max() < 1e-12
    bp = np.zeros(38, np.int32)
    ctx.check(lib.fo_get_bestperm(ctx.h, _lib.i(bp)))
    assert sorted(bp) == list(range(1, 39))


def test_bulk_fortran_entry_and_defaults(fo, golden):
    from fastoverlap_gb300 import _lib
    g = golden("blj256")
    ctx = fo.default_context("fp64")
    lib = ctx.lib
    n = int(g["ntypeA"])
    pg = np.arange(1, 257, dtype=np.int32)
    ctx.check(lib.fo_setperm(ctx.h, 256, _lib.i(pg), _lib.i(np.array([n, 256 - n], np.int32)), 2))
    cb = np.ascontiguousarray(g["pos1"].ravel().copy())
    ca = np.ascontiguousarray(g["pos2"].ravel().copy())
    dist, d2 = ctypes.c_double(), ctypes.c_double()
    L = float(g["box"][0])
    ctx.check(lib.fo_bulk_align(ctx.h, _lib.d(cb), _lib.d(ca), 256, 0, L, L, L, 0.0, 10, 0, 0,
                                ctypes.byref(dist), ctypes.byref(d2)))
    assert abs(dist.value - float(g["dist"])) <= 1e-8 * dist.value
    kw = ctypes.c_double()
    nw, nf = ctypes.c_int(), ctypes.c_int()
    ctx.check(lib.fo_bulk_calcdefaults(256, L, L, L, ctypes.byref(kw), ctypes.byref(nw), ctypes.byref(nf)))
    w = (L ** 3 / 256) ** (1 / 3) / 3
    assert abs(kw.value - w) < 1e-15
    assert nw.value == int(np.ceil(2 * 3.14159265359 / L * 1.5 / w))
    assert nf.value >= 4 * nw.value + 3
