"""Edge cases and argument errors through the C ABI."""
import numpy as np
import pytest

from fastoverlap_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_tiny_clusters(fo, oracle_mod, n):
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, 3))
    B = A @ synth.haar_rotation(rng).T
    o = oracle_mod.cluster_align(A, B, Jmax=4, sigma=0.3, nrot=3)
    if o["status"] != 0:
        # a flat overlap grid has no peak to fit; the upstream code stops there
        with pytest.raises(fo.FoError):
            fo.SphericalAlign(0.3, 4).align_full(A, B, nrot=3)
        return
    r = fo.SphericalAlign(0.3, 4).align_full(A, B, nrot=3)
    assert r["dist"] == pytest.approx(o["dist"], rel=1e-8, abs=1e-10)


def test_atom_at_centroid(fo):
    X = synth.cluster_pair(3, n=10)["pos1"]
    A = np.vstack([X, -X, np.zeros((1, 3))])    # centroid at the origin, one atom on it
    r = fo.SphericalAlign(0.3, 5).align_full(A + 1.0, A + 1.0, nrot=3)
    assert np.isfinite(r["dist"]) and r["dist"] < 1e-6


def test_identical_structures_give_zero(fo):
    p = synth.config0(2)
    r = fo.SphericalAlign(0.3, 7).align_full(p["pos1"], p["pos1"])
    assert r["dist"] < 1e-8


def test_one_atom_species_and_no_inversion(fo, oracle_mod):
    p = synth.cluster_pair(8, n=30, sizes=[1, 20, 9])
    r = fo.SphericalAlign(0.3, 6).align_full(p["pos1"], p["pos2"], perm=p["perm"], invert=False)
    o = oracle_mod.cluster_align(p["pos1"], p["pos2"], perm=p["perm"], Jmax=6, sigma=0.3, nrot=10,
                                 invert=False)
    assert abs(r["dist"] - o["dist"]) <= 1e-8 * o["dist"]
    assert not r["inverted"]


@pytest.mark.parametrize("L", [0, 1, 2])
def test_small_bandwidth(fo, oracle_mod, L):
    p = synth.config0(4)
    r = fo.SphericalAlign(0.3, L).align_full(p["pos1"], p["pos2"], nrot=2)
    o = oracle_mod.cluster_align(p["pos1"], p["pos2"], Jmax=L, sigma=0.3, nrot=2)
    assert abs(r["dist"] - o["dist"]) <= 1e-8 * o["dist"]


def test_auto_width(fo, oracle_mod, golden):
    g = golden("lj38")
    sa = fo.SphericalAlign(None, 7)
    r = sa.align_full(g["pos1"], g["pos2"])
    o = oracle_mod.cluster_align(g["pos1"], g["pos2"], Jmax=7, sigma=None, nrot=10)
    assert abs(r["sigma"] - o["sigma"]) < 1e-14
    assert abs(r["dist"] - o["dist"]) <= 1e-8 * o["dist"]


def test_periodic_single_displacement_and_defaults(fo, oracle_mod):
    p = synth.periodic_pair(9, n=100, sizes=(80, 20))
    d, X1, X2, perm = fo.PeriodicAlignFortran(100, p["box"], perm=p["perm"]).align(
        p["pos1"], p["pos2"], ndisps=1)
    o = oracle_mod.bulk_align(p["pos1"], p["pos2"], p["box"], perm=p["perm"], ndisps=1)
    assert abs(d - o["dist"]) <= 1e-8 * o["dist"]


def test_bad_arguments_raise(fo):
    A = np.random.default_rng(0).normal(size=(10, 3))
    with pytest.raises(fo.FoError):
        fo.SphericalAlign(0.3, 7, perm=[np.arange(5)]).align_full(A, A)       # groups miss atoms
    with pytest.raises(fo.FoError):
        fo.SphericalAlign(0.3, 7, perm=[np.arange(10), np.array([3])]).align_full(A, A)
    with pytest.raises(fo.FoError):
        fo.SphericalAlign(0.3, 40).align_full(A, A)                           # Jmax above 31
    B = A.copy()
    B[2, 1] = np.nan
    with pytest.raises(fo.FoError):
        fo.SphericalAlign(0.3, 7).align_full(A, B)
    with pytest.raises(fo.FoError):
        fo.PeriodicAlignFortran(10, [0.0, 1.0, 1.0]).align(A, A)              # zero box length


def test_plan_runs_after_l2_flush_and_events(fo):
    """Benchmark helpers (L2 flush, event timing) leave the context usable."""
    ps = synth.config2(6, seed_offset=31)
    ctx = fo.Context(precision="mixed", profile=True)
    b = fo.ClusterBatch(ctx, [p["pos1"] for p in ps], [p["pos2"] for p in ps],
                        [p["perm"] for p in ps], Jmax=[p["Jmax"] for p in ps], scale=0.3,
                        nrot=10).plan()
    b.plan_run()
    b.plan_wait()
    first = b.plan_results(False)["dist"]
    for _ in range(2):
        ctx.flush_l2(64 << 20)
        ctx.record(0)
        b.plan_run()
        ctx.record(1)
        b.plan_wait()
        assert ctx.elapsed_ms(0, 1) > 0
    assert np.array_equal(b.plan_results(False)["dist"], first)
    assert "refine" in ctx.profile()
    b.close()


def test_exit_with_open_objects(fo):
    """A process that exits with a server, a plan and contexts still open
    exits cleanly (they are closed before the interpreter is torn down)."""
    import subprocess
    import sys
    import os
    code = ("import sys; sys.path.insert(0, %r)\n"
            "import fastoverlap_gb300 as F\n"
            "from fastoverlap_gb300 import synth\n"
            "ps = synth.config2(4, seed_offset=31)\n"
            "ctx = F.Context(precision='mixed')\n"
            "b = F.ClusterBatch(ctx, [p['pos1'] for p in ps], [p['pos2'] for p in ps], [p['perm'] for p in ps],"
            " Jmax=[p['Jmax'] for p in ps], scale=0.3).plan()\n"
            "b.plan_run(); b.plan_wait()\n"
            "srv = F.Server(precision='mixed')\n"
            "t = srv.submit_cluster(ps[0]['pos1'], ps[0]['pos2'], ps[0]['perm'], Jmax=7)\n"
            "print('ok', srv.wait(t)['status'])\n") % os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "ok 0" in r.stdout
