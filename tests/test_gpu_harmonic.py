"""Harmonic-oscillator basis (SphericalHarmonicAlign / ALIGNHARM /
CALCOVERLAPMATRICES) on the GPU against the CPU oracle and the upstream
Python fixtures."""
import numpy as np
import pytest

from fastoverlap_gb300 import synth

pytestmark = pytest.mark.gpu


def test_alignment_matches_upstream_python(fo, oracle_mod, golden):
    g = golden("harm")
    ctx = fo.Context(precision="fp64")
    for k in range(len(g["dist_nmax10_j7"])):
        al = fo.SphericalHarmonicAlign(scale=0.3, harmscale=1.0, nmax=10, Jmax=7, ctx=ctx)
        d, X1, X2 = al(g["pos1"][k], g["pos2"][k])
        assert abs(d - g["dist_nmax10_j7"][k]) <= 1e-8 * d
        o = oracle_mod.harm_align(g["pos1"][k], g["pos2"][k], None, nmax=10, Jmax=7, hwidth=1.0, kwidth=0.3)
        assert np.max(np.abs(X2 - o["aligned"])) <= 1e-8
        assert abs(np.linalg.norm(X1 - X2) - d) <= 1e-8 * d


@pytest.mark.parametrize("k", range(3))
def test_fortran_class_against_oracle(fo, oracle_mod, k):
    """Coordinates as given (not centred), two species, inversion on."""
    p = synth.cluster_pair(300 + k, n=30, sizes=[20, 10])
    shift1, shift2 = np.array([0.3, -0.2, 0.1]), np.array([-0.1, 0.25, 0.05])
    pos1, pos2 = p["pos1"] + shift1, p["pos2"] + shift2
    ctx = fo.Context(precision="fp64")
    al = fo.SphericalHarmonicAlignFortran(scale=0.3, Jmax=7, harmscale=1.1, nmax=8, perm=p["perm"], ctx=ctx)
    d, cb, ca, R = al(pos1, pos2)
    o = oracle_mod.harm_align(pos1, pos2, p["perm"], nmax=8, Jmax=7, hwidth=1.1, kwidth=0.3, nrot=10,
                              invert=True)
    assert o["status"] == 0
    assert abs(d - o["dist"]) <= 1e-8 * o["dist"]
    np.testing.assert_array_equal(cb, pos1)          # ALIGNHARM leaves COORDSB as given
    assert np.max(np.abs(ca - o["aligned"])) <= 1e-8
    assert np.max(np.abs(R - o["rmat"])) <= 1e-8
    assert abs(np.linalg.norm(pos1 - ca) - d) <= 1e-8 * d


def test_mixed_precision_against_fp64(fo):
    ps = [synth.cluster_pair(400 + k, n=24 + 3 * k) for k in range(6)]
    out = {}
    for prec in ("fp64", "mixed"):
        ctx = fo.Context(precision=prec)
        b = fo.HarmonicClusterBatch(ctx, [p["pos1"] for p in ps], [p["pos2"] for p in ps],
                                    [p["perm"] for p in ps], Jmax=7, scale=0.3, nrot=10, nmax=10,
                                    harmscale=1.0)
        out[prec] = b.run()
    a, m = out["fp64"], out["mixed"]
    assert np.all(a["status"] == 0) and np.all(m["status"] == 0)
    assert np.max(np.abs(a["dist"] - m["dist"]) / a["dist"]) <= 1e-5
    for x, y in zip(a["perm"], m["perm"]):
        np.testing.assert_array_equal(x, y)


def test_resident_plan_equals_run(fo):
    ps = [synth.cluster_pair(500 + k, n=20) for k in range(4)]
    ctx = fo.Context(precision="fp64")
    mk = lambda: fo.HarmonicClusterBatch(ctx, [p["pos1"] for p in ps], [p["pos2"] for p in ps],
                                         [p["perm"] for p in ps], Jmax=6, scale=0.35, nrot=5, nmax=6)
    r0 = mk().run()
    b = mk().plan()
    b.plan_run()
    b.plan_wait()
    r1 = b.plan_results(True)
    np.testing.assert_array_equal(r0["dist"], r1["dist"])
    b.close()


def test_compare_list_against_oracle_and_upstream(fo, oracle_mod, golden):
    g = golden("harm")
    nmax, L, hw, kw = int(g["nmax"]), int(g["L"]), float(g["hwidth"]), float(g["kwidth"])
    rng = np.random.default_rng(3)
    Z = g["X"] + rng.normal(scale=0.2, size=g["X"].shape)
    lst = [g["X"], g["Y"], Z]
    al = fo.SphericalHarmonicAlignFortran(scale=kw, Jmax=L, harmscale=hw, nmax=nmax, ctx=fo.Context(precision="fp64"))
    avg, mx, navg, nmx = al.compareList(lst)
    cent = [x - x.mean(0) for x in lst]
    norms, maxs = oracle_mod.overlap_matrices(cent, None, nmax, L, hw, kw)
    assert np.max(np.abs(avg - norms) / norms) <= 1e-10
    assert np.max(np.abs(mx - maxs) / np.abs(maxs)) <= 1e-10
    assert abs(avg[0, 1] - float(g["norm"])) <= 1e-10 * float(g["norm"])       # upstream Python
    assert abs(mx[0, 1] - float(g["maxover"])) <= 1e-10 * abs(float(g["maxover"]))
    np.testing.assert_allclose(np.diag(navg), 1.0, rtol=1e-14)
    np.testing.assert_allclose(np.diag(nmx), 1.0, rtol=1e-14)
    np.testing.assert_array_equal(avg, avg.T)


def test_bad_arguments(fo):
    p = synth.cluster_pair(1, n=12)
    ctx = fo.Context(precision="fp64")
    with pytest.raises(fo.FoError) as e:
        fo.HarmonicClusterBatch(ctx, [p["pos1"]], [p["pos2"]], [p["perm"]], Jmax=5, scale=0.3, nmax=41).run()
    assert e.value.status == 1
    with pytest.raises(fo.FoError) as e:
        fo.HarmonicClusterBatch(ctx, [p["pos1"]], [p["pos2"]], [p["perm"]], Jmax=5, scale=0.0, nmax=4).run()
    assert e.value.status == 1
    with pytest.raises(fo.FoError) as e:
        fo.HarmonicClusterBatch(ctx, [p["pos1"]], [p["pos2"]], [p["perm"]], Jmax=5, scale=0.3, nmax=4,
                                harmscale=0.0).run()
    assert e.value.status == 1
