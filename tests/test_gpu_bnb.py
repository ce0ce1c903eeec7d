"""Branch and bound over rotations on the GPU against the oracle and the
upstream Python fixtures (same expanded nodes, distance and coordinates)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pairs(g):
    off, out = 0, []
    for n in g["natoms"]:
        sl = slice(off, off + int(n))
        out.append((g["pos1"][sl], g["pos2"][sl], sl))
        off += int(n)
    return out


def test_matches_upstream_python(fo, golden):
    g = golden("bnb")
    ctx = fo.Context(precision="fp64")
    for k, (p1, p2, sl) in enumerate(_pairs(g)):
        m = fo.BranchandBoundMaster(ctx=ctx)
        d, X1, X2 = m(p1, p2)
        assert m.nodes == int(g["nodes"][k])
        assert abs(d - g["dist"][k]) <= 1e-10 * g["dist"][k]
        assert np.max(np.abs(X2 - g["aligned"][sl])) <= 1e-10


def test_batch_equals_single_searches(fo, golden):
    g = golden("bnb")
    ctx = fo.Context(precision="fp64")
    P = _pairs(g)
    d, al, nodes = fo.bnb_align_clusters([p[0] for p in P], [p[1] for p in P], ctx=ctx)
    for k, (p1, p2, _) in enumerate(P):
        d1, al1, n1 = fo.bnb_align_clusters([p1], [p2], ctx=ctx)
        assert d[k] == d1[0] and nodes[k] == n1[0]
        np.testing.assert_array_equal(al[k], al1[0])


def test_node_limit_against_oracle(fo, oracle_mod, golden):
    g = golden("bnb")
    ctx = fo.Context(precision="fp64")
    for p1, p2, _ in _pairs(g)[:2]:
        d, _, nodes = fo.bnb_align_clusters([p1], [p2], niter=200, ctx=ctx)
        o = oracle_mod.bnb_cluster(p1, p2, niter=200)
        assert nodes[0] == o["nodes"]
        assert abs(d[0] - o["dist"]) <= 1e-10 * o["dist"]


def test_bad_arguments(fo):
    ctx = fo.Context(precision="fp64")
    x = np.random.default_rng(0).normal(size=(300, 3))
    with pytest.raises(fo.FoError) as e:
        fo.bnb_align_clusters([x], [x], ctx=ctx)
    assert e.value.status == 1
