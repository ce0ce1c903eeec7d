"""OHCELL: the 48 cubic-cell operations of the periodic alignment (ALIGN1
with OHCELLT) against the CPU oracle."""
import ctypes

import numpy as np
import pytest

from fastoverlap_gb300 import synth

pytestmark = pytest.mark.gpu


def _pair(op):
    """A 64-atom cubic-box pair whose second structure is also transformed by
    cubic operation `op`."""
    import oracle
    p = synth.periodic_pair(11, n=64, sizes=(52, 12))
    return p, p["pos2"] @ oracle.oh_operation(op).T


@pytest.mark.parametrize("op", [19, 42])
def test_ohcell_against_oracle(fo, oracle_mod, op):
    p, pos2 = _pair(op)
    ctx = fo.Context(precision="fp64")
    al = fo.PeriodicAlignFortran(64, p["box"], scale=0.3, perm=p["perm"], ctx=ctx)
    d_plain = al.align(p["pos1"], pos2, ndisps=4)[0]
    d, X1, X2, perm = al.align(p["pos1"], pos2, ndisps=4, ohcell=True)
    kw, nw, nf = 0.3, int(np.ceil(1.3 * 64 ** (1 / 3))), 0
    o = oracle_mod.bulk_align_ohcell(p["pos1"], pos2, p["box"], p["perm"], sigma=kw, nwave=nw, nfspace=nf,
                                     ndisps=4)
    assert abs(d - o["dist"]) <= 1e-8 * o["dist"]
    np.testing.assert_array_equal(perm, o["perm"])
    np.testing.assert_array_equal(al.ohop, o["M"])
    # the operation found undoes the one applied, and beats the plain alignment
    np.testing.assert_array_equal(al.ohop @ oracle_mod.oh_operation(op), np.eye(3))
    assert d < 0.5 * d_plain


def test_ohcell_batch_mixed_with_plain_pairs(fo):
    p, pos2 = _pair(19)
    q = synth.periodic_pair(12, n=64, sizes=(52, 12))
    ctx = fo.Context(precision="mixed")
    mk = lambda oh: fo.BulkBatch(ctx, [p["pos1"], q["pos1"]], [pos2, q["pos2"]], p["box"], [p["perm"], q["perm"]],
                                 scale=0.3, ndisps=3, ohcell=oh)
    both = mk([True, False]).run()
    plain = mk(False).run()
    single = fo.BulkBatch(ctx, [p["pos1"]], [pos2], p["box"], [p["perm"]], scale=0.3, ndisps=3, ohcell=True).run()
    assert both["dist"][1] == plain["dist"][1]
    np.testing.assert_array_equal(both["perm"][1], plain["perm"][1])
    assert both["dist"][0] == single["dist"][0]
    np.testing.assert_array_equal(both["aligned"][0], single["aligned"][0])
    assert both["result"]["ncand"][0] > 40 * plain["result"]["ncand"][0] // 2
    with pytest.raises(fo.FoError) as e:
        mk([True, False]).plan()
    assert e.value.status == 1


def test_set_ohcell_c_abi(fo):
    p, pos2 = _pair(42)
    ctx = fo.Context(precision="fp64")
    lib = ctx.lib
    pg = np.concatenate([np.asarray(g) + 1 for g in p["perm"]]).astype(np.int32)
    ns = np.array([len(g) for g in p["perm"]], np.int32)
    ctx.check(lib.fo_setperm(ctx.h, 64, fo._lib.i(pg), fo._lib.i(ns), len(ns)))
    bx, by, bz = map(float, p["box"])
    out = {}
    for oh in (0, 1):
        ctx.check(lib.fo_set_ohcell(ctx.h, oh))
        ca = pos2.ravel().copy()
        d = ctypes.c_double()
        ctx.check(lib.fo_bulk_align(ctx.h, fo._lib.d(p["pos1"].ravel().copy()), fo._lib.d(ca), 64, 0, bx, by, bz,
                                    0.3, 4, 0, 0, ctypes.byref(d), None))
        out[oh] = d.value
    al = fo.PeriodicAlignFortran(64, p["box"], scale=0.3, perm=p["perm"], ctx=ctx)
    assert out[1] == al.align(p["pos1"], pos2, ndisps=4, ohcell=True)[0]
    assert out[0] == al.align(p["pos1"], pos2, ndisps=4)[0]
    assert out[1] < 0.5 * out[0]
