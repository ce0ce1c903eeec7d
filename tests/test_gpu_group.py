"""Group alignment (BULKFASTOVERLAP::ALIGNGROUP and the alignGroup methods of
PeriodicAlign / PeriodicAlignFortran) against single-pair alignments and the
CPU oracle."""
import ctypes

import numpy as np
import pytest

from fastoverlap_gb300 import synth

pytestmark = pytest.mark.gpu


def _structures():
    """Four 64-atom structures in one box: two aligned pairs (a structure and
    its translated, permuted, noisy copy) and the pairs between them."""
    a, b = synth.periodic_pair(3, n=64, sizes=(52, 12)), synth.periodic_pair(4, n=64, sizes=(52, 12))
    assert np.allclose(a["box"], b["box"])
    return [a["pos1"], a["pos2"], b["pos1"], b["pos2"]], a["box"], a["perm"]


def _min_image_dist(x, y, box):
    d = x - y
    d -= np.round(d / box) * box
    return np.linalg.norm(d)


def test_fortran_align_group_against_oracle(fo, oracle_mod):
    coords, box, perm = _structures()
    n = len(coords)
    ctx = fo.Context(precision="fp64")
    al = fo.PeriodicAlignFortran(64, box, perm=perm, ctx=ctx)
    dists, aligned = al.alignGroup(coords, ndisps=2)
    assert dists.shape == (n, n) and aligned.shape == (64, 3, n, n)
    kw, nw, nf = ctypes.c_double(), ctypes.c_int(), ctypes.c_int()
    ctx.check(ctx.lib.fo_bulk_calcdefaults(64, *map(float, box), ctypes.byref(kw), ctypes.byref(nw),
                                           ctypes.byref(nf)))
    for j in range(n):
        for i in range(n):
            if i < j:   # the triangular loop skips these
                assert dists[i, j] == 0.0 and not aligned[:, :, i, j].any()
                continue
            o = oracle_mod.bulk_align(coords[i], coords[j], box, perm=perm, sigma=kw.value,
                                      nwave=nw.value, nfspace=nf.value, ndisps=2)
            assert o["status"] == 0
            assert abs(dists[i, j] - o["dist"]) <= 1e-8 * o["dist"] + 1e-12   # + self-alignment zeros
            dd = aligned[:, :, i, j] - o["aligned"]
            dd -= np.round(dd / box) * box   # the same positions up to periodic images
            assert np.max(np.abs(dd)) <= 1e-8 * box[0]
            assert abs(_min_image_dist(coords[i], aligned[:, :, i, j], box) - dists[i, j]) \
                <= 1e-8 * dists[i, j] + 1e-12
    assert dists[1, 0] < 0.2 * dists[2, 0] and dists[3, 2] < 0.2 * dists[2, 0]


def test_align_group_c_abi_full_and_sym(fo):
    """sym = 0 aligns every (i, j) of two lists; its i >= j entries equal the
    sym run's, and pair (i, j) equals fo_bulk_align of the same pair."""
    coords, box, perm = _structures()
    ctx = fo.Context(precision="mixed")
    lib = ctx.lib
    pg = np.concatenate([np.asarray(p) + 1 for p in perm]).astype(np.int32)
    ns = np.array([len(p) for p in perm], np.int32)
    ctx.check(lib.fo_setperm(ctx.h, 64, fo._lib.i(pg), fo._lib.i(ns), len(ns)))
    l1 = np.ascontiguousarray(np.stack(coords[:3]).reshape(3, -1))
    l2 = np.ascontiguousarray(np.stack(coords[:2]).reshape(2, -1))
    bx, by, bz = map(float, box)
    full = np.zeros(3 * 2)
    alf = np.zeros(3 * 2 * 192)
    ctx.check(lib.fo_bulk_align_group(ctx.h, fo._lib.d(l1), 3, fo._lib.d(l2), 2, 64, 0, bx, by, bz, 0.3, 3, 6,
                                      0, fo._lib.d(full), fo._lib.d(alf), 0))
    full = full.reshape(3, 2, order="F")
    sym = np.zeros(3 * 2)
    ctx.check(lib.fo_bulk_align_group(ctx.h, fo._lib.d(l1), 3, fo._lib.d(l2), 2, 64, 0, bx, by, bz, 0.3, 3, 6,
                                      0, fo._lib.d(sym), None, 1))
    sym = sym.reshape(3, 2, order="F")
    for i in range(3):
        for j in range(2):
            ca = coords[j].ravel().copy()
            d = ctypes.c_double()
            ctx.check(lib.fo_bulk_align(ctx.h, fo._lib.d(coords[i].ravel().copy()), fo._lib.d(ca), 64, 0,
                                        bx, by, bz, 0.3, 3, 6, 0, ctypes.byref(d), None))
            assert full[i, j] == d.value
            np.testing.assert_array_equal(alf.reshape(192, 3, 2, order="F")[:, i, j], ca)
            assert sym[i, j] == (full[i, j] if i >= j else 0.0)


def test_align_group_bad_arguments(fo):
    ctx = fo.Context(precision="fp64")
    x = np.zeros(3 * 8)
    out = np.zeros(4)
    st = ctx.lib.fo_bulk_align_group(ctx.h, fo._lib.d(x), 1, fo._lib.d(x), 2, 8, 0, 2.0, 2.0, 2.0, 0.3, 1, 0,
                                     0, fo._lib.d(out), None, 1)
    assert st == 1   # sym with a longer second list
    st = ctx.lib.fo_bulk_align_group(ctx.h, fo._lib.d(x), 0, fo._lib.d(x), 1, 8, 0, 2.0, 2.0, 2.0, 0.3, 1, 0,
                                     0, fo._lib.d(out), None, 0)
    assert st == 1


def test_python_align_group_equals_align(fo):
    coords, box, perm = _structures()
    coords = coords[:3]
    ctx = fo.Context(precision="fp64")
    al = fo.PeriodicAlign(64, box, perm, scale=0.25, n=5, ctx=ctx)
    dists, aligned = al.alignGroup(coords, keepCoords=True, npeaks=2, chunk=4)
    assert dists.shape == (3, 3) and aligned.shape == (2, 3, 3, 64, 3)
    for i in range(3):
        for j in range(3):
            d, X1, X2, _, _ = al.align(coords[i], coords[j], npeaks=2)
            assert dists[i, j] == d
            np.testing.assert_array_equal(aligned[0, i, j], X1)
            np.testing.assert_array_equal(aligned[1, i, j], X2)
    assert np.all(np.diag(dists) < 1e-6)
    np.testing.assert_array_equal(al.alignGroup(coords, npeaks=2), dists)
