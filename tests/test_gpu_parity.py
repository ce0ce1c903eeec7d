"""GPU against the CPU oracle on seeded inputs: stages, single pairs, batches."""
import numpy as np
import pytest

from fastoverlap_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cutoff", [True, False])
@pytest.mark.parametrize("L", [3, 7, 12])
def test_coefficients_and_grid_fp64(fo, oracle_mod, cutoff, L):
    from fastoverlap_gb300.batch import cluster_overlap
    p = synth.cluster_pair(31 + L, n=29)
    A = p["pos1"] - p["pos1"].mean(0)
    B = p["pos2"] - p["pos2"].mean(0)
    ctx = fo.Context(precision="fp64", cutoff=cutoff)
    c, grid = cluster_overlap(p["pos1"], p["pos2"], Jmax=L, scale=0.35, ctx=ctx)
    ref = oracle_mod.cluster_coeffs(A, B, L, 0.35, cutoff=cutoff)
    assert np.max(np.abs(c - ref)) <= 1e-12 * np.max(np.abs(ref))
    gref = oracle_mod.isoft(ref)
    assert np.max(np.abs(grid - gref)) <= 1e-12 * np.max(np.abs(gref))


def test_coefficients_against_upstream_fixture(fo, golden):
    from fastoverlap_gb300.batch import cluster_overlap
    g = golden("stages")
    ctx = fo.Context(precision="fp64", cutoff=False)
    c, grid = cluster_overlap(g["A"], g["B"], Jmax=int(g["L"]), scale=float(g["sigma"]), ctx=ctx)
    assert np.max(np.abs(c - g["coeffs"])) <= 1e-12 * np.max(np.abs(g["coeffs"]))
    assert np.max(np.abs(grid - g["grid"])) <= 1e-12 * np.max(np.abs(g["grid"]))


def test_coefficients_mixed_precision(fo, oracle_mod):
    """FP32 coefficients: relative error vs FP64 stated and bounded (1e-5)."""
    from fastoverlap_gb300.batch import cluster_overlap
    p = synth.cluster_pair(5, n=60)
    A = p["pos1"] - p["pos1"].mean(0)
    B = p["pos2"] - p["pos2"].mean(0)
    ctx = fo.Context(precision="mixed")
    c, grid = cluster_overlap(p["pos1"], p["pos2"], Jmax=11, scale=0.3, ctx=ctx)
    ref = oracle_mod.cluster_coeffs(A, B, 11, 0.3, cutoff=True)
    assert np.max(np.abs(c - ref)) <= 1e-5 * np.max(np.abs(ref))


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_periodic_grid(fo, oracle_mod, golden, prec):
    from fastoverlap_gb300.batch import bulk_overlap
    g = golden("stages")
    s = g["per_sizes"]
    perm = [np.arange(s[0]), np.arange(s[0], s[0] + s[1])]
    grid = bulk_overlap(g["per_pos1"], g["per_pos2"], g["per_box"], perm=perm,
                        scale=float(g["per_sigma"]), nwave=int(g["per_n"]), precision=prec)
    ref = g["per_fabs"]
    tol = 1e-12 if prec == "fp64" else 1e-5
    assert np.max(np.abs(grid - ref)) <= tol * ref.max()


def test_periodic_grid_config1_size(fo, oracle_mod):
    from fastoverlap_gb300.batch import bulk_overlap
    p = synth.config1(3)
    grid = bulk_overlap(p["pos1"], p["pos2"], p["box"], perm=p["perm"], scale=0.2, nwave=7)
    ref = oracle_mod.bulk_fspace(p["pos1"], p["pos2"], p["box"], perm=p["perm"], sigma=0.2, nwave=7)
    assert grid.shape == (32, 32, 32)
    assert np.max(np.abs(grid - ref)) <= 1e-12 * ref.max()


@pytest.mark.parametrize("k", range(8))
def test_config0_pairs(fo, oracle_mod, golden, k):
    g = golden("e2e")
    p = synth.config0(k)
    r = fo.SphericalAlign(0.3, 7).align_full(p["pos1"], p["pos2"], perm=p["perm"])
    o = oracle_mod.cluster_align(p["pos1"], p["pos2"], perm=p["perm"], Jmax=7, sigma=0.3, nrot=10)
    assert abs(r["dist"] - o["dist"]) <= 1e-8 * o["dist"]
    assert np.array_equal(r["perm"], o["perm"])
    assert abs(r["dist"] - float(g["c0_dist"][k])) <= 1e-8 * r["dist"]   # upstream Python


@pytest.mark.parametrize("k", range(2))
def test_config1_pairs(fo, oracle_mod, golden, k):
    g = golden("e2e")
    p = synth.config1(k)
    d, X1, X2, perm, disp = fo.PeriodicAlign(256, p["box"], p["perm"], scale=0.2, n=7)(
        p["pos1"], p["pos2"], npeaks=10)
    o = oracle_mod.bulk_align(p["pos1"], p["pos2"], p["box"], perm=p["perm"], sigma=0.2, nwave=7,
                              ndisps=10)
    assert abs(d - o["dist"]) <= 1e-8 * o["dist"]
    assert np.array_equal(perm, o["perm"])
    assert abs(d - float(g["c1_dist"][k])) <= 1e-8 * d                  # upstream Python


def _batch(fo, ps, prec, **kw):
    ctx = fo.Context(precision=prec)
    b = fo.ClusterBatch(ctx, [p["pos1"] for p in ps], [p["pos2"] for p in ps],
                        [p["perm"] for p in ps], Jmax=[p["Jmax"] for p in ps], scale=0.3,
                        nrot=10, invert=True, **kw)
    return b.run()


def test_config2_batch_fp64(fo, oracle_mod):
    ps = synth.config2(48)
    out = _batch(fo, ps, "fp64")
    od = oracle_mod.cluster_align_many(ps)
    assert np.all(out["status"] == 0)
    rel = np.abs(out["dist"] - od) / od
    assert rel.max() <= 1e-8
    for p, perm in zip(ps[:8], out["perm"][:8]):
        o = oracle_mod.cluster_align(p["pos1"], p["pos2"], perm=p["perm"], Jmax=p["Jmax"],
                                     sigma=0.3, nrot=10)
        assert np.array_equal(perm, o["perm"])


def test_config2_batch_mixed(fo, oracle_mod):
    """Mixed precision: final distance within 1e-5 relative of the FP64 oracle
    and identical permutations on >= 99.9% of pairs (all, at this size)."""
    ps = synth.config2(48, seed_offset=500)
    out = _batch(fo, ps, "mixed")
    od, operm = oracle_mod.cluster_align_many(ps, with_perm=True)
    rel = np.abs(out["dist"] - od) / od
    assert np.all(out["status"] == 0)
    assert rel.max() <= 1e-5
    same = [np.array_equal(a, b) for a, b in zip(out["perm"], operm)]
    assert np.mean(same) >= 0.999


def test_batch_equals_single_pairs(fo):
    """Each result is the same alone and in the mix."""
    ps = synth.config2(6, seed_offset=900)
    out = _batch(fo, ps, "fp64")
    for k, p in enumerate(ps):
        one = _batch(fo, [p], "fp64")
        assert one["dist"][0] == out["dist"][k]
        assert np.array_equal(one["perm"][0], out["perm"][k])


def test_deterministic(fo):
    ps = synth.config2(8, seed_offset=77)
    a = _batch(fo, ps, "mixed")
    b = _batch(fo, ps, "mixed")
    assert np.array_equal(a["dist"], b["dist"])


def test_large_cluster_sparse_assignment(fo, oracle_mod):
    """Groups above 60 atoms use the 60-nearest sparse cost lists."""
    p = synth.cluster_pair(11, n=150, radius=1.9 * (150 / 38.0) ** (1 / 3), sizes=[120, 30])
    r = fo.SphericalAlign(0.3, 7).align_full(p["pos1"], p["pos2"], perm=p["perm"], nrot=4)
    o = oracle_mod.cluster_align(p["pos1"], p["pos2"], perm=p["perm"], Jmax=7, sigma=0.3, nrot=4)
    assert abs(r["dist"] - o["dist"]) <= 1e-8 * o["dist"]
    assert np.array_equal(r["perm"], o["perm"])


@pytest.mark.parametrize("prec,n", [("fp64", 300), ("mixed", 1000)])
def test_large_bandwidth_properties(fo, prec, n):
    """Jmax 31, two species: size-independent checks of the outputs."""
    na = int(0.8 * n)
    p = synth.cluster_pair(4000 + n, n=n, radius=1.9 * (n / 38.0) ** (1 / 3), sizes=[na, n - na])
    r = fo.SphericalAlign(0.25, 31, precision=prec).align_full(p["pos1"], p["pos2"],
                                                                perm=p["perm"], nrot=4)
    R = r["rmat"]
    assert np.abs(R @ R.T - np.eye(3)).max() < 1e-10
    assert sorted(r["perm"][:na]) == list(range(na))
    assert sorted(r["perm"][na:]) == list(range(na, n))
    assert abs(np.linalg.norm(r["X1"] - r["X2"]) - r["dist"]) < 1e-8
    assert r["dist"] < 0.05 * np.sqrt(3 * n) * 1.5   # noise level of the generator


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_plan_graph_replay_equals_eager(fo, prec):
    """A plan replayed as a captured CUDA graph gives the eager results, bit for bit."""
    ps = synth.config2(24)
    ctx = fo.Context(precision=prec)
    mk = lambda: fo.ClusterBatch(ctx, [p["pos1"] for p in ps], [p["pos2"] for p in ps],
                                 [p["perm"] for p in ps], Jmax=[p["Jmax"] for p in ps], scale=0.3,
                                 nrot=10).plan()
    eager = mk()
    eager.plan_run()
    eager.plan_wait()
    ref = eager.plan_results(True)
    eager.close()
    g = mk().plan_graph()
    for _ in range(3):   # eager + capture, then two replays
        g.plan_run()
        g.plan_wait()
        out = g.plan_results(True)
        np.testing.assert_array_equal(out["dist"], ref["dist"])
        for a, b in zip(out["aligned"], ref["aligned"]):
            np.testing.assert_array_equal(a, b)
    g.plan_graph(False)
    g.plan_run()
    g.plan_wait()
    np.testing.assert_array_equal(g.plan_results(False)["dist"], ref["dist"])
    g.close()
