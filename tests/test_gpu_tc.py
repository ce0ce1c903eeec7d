"""The tensor-core (tcgen05, split TF32) Wigner contraction of the mixed form
against the FP64 oracle and against the same form on the FP32 CUDA cores.

Bounds: grids within 1e-5 of their largest value (FP32-like accuracy of the
3xTF32 split); alignments within 1e-5 relative of the FP64 oracle with
identical permutations (the mixed form's bar).
"""
import numpy as np
import pytest

from fastoverlap_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("L", [0, 1, 3, 7, 11, 15, 31])
def test_tensor_core_grid(fo, oracle_mod, L):
    from fastoverlap_gb300.batch import cluster_overlap
    n = 60 if L < 31 else 150
    p = synth.cluster_pair(700 + L, n=n, radius=1.9 * (n / 38.0) ** (1 / 3))
    A = p["pos1"] - p["pos1"].mean(0)
    B = p["pos2"] - p["pos2"].mean(0)
    sig = 0.3 if L < 31 else 0.25
    ref = oracle_mod.isoft(oracle_mod.cluster_coeffs(A, B, L, sig, cutoff=True))
    tc = fo.Context(precision="mixed")
    cc = fo.Context(precision="mixed", tensor_cores=False)
    _, g_tc = cluster_overlap(p["pos1"], p["pos2"], Jmax=L, scale=sig, ctx=tc)
    _, g_cc = cluster_overlap(p["pos1"], p["pos2"], Jmax=L, scale=sig, ctx=cc)
    scale = np.abs(ref).max()
    assert np.abs(g_tc - ref).max() <= 1e-5 * scale
    assert np.abs(g_tc - g_cc).max() <= 1e-5 * scale
    tc.close()
    cc.close()


def _align(fo, ps, ctx, invert=True):
    return fo.ClusterBatch(ctx, [p["pos1"] for p in ps], [p["pos2"] for p in ps], [p["perm"] for p in ps],
                           Jmax=[p["Jmax"] for p in ps], scale=0.3, nrot=10, invert=invert).run()


def test_tensor_core_batch_many_tiles(fo, oracle_mod):
    """150 pairs over three bandwidths: full and partial tiles of 64."""
    ps = synth.config2(150, seed_offset=3100)
    ctx = fo.Context(precision="mixed")
    out = _align(fo, ps, ctx)
    ctx.close()
    od, operm = oracle_mod.cluster_align_many(ps, with_perm=True)
    assert np.all(out["status"] == 0)
    assert np.max(np.abs(out["dist"] - od) / od) <= 1e-5
    assert np.mean([np.array_equal(a, b) for a, b in zip(out["perm"], operm)]) >= 0.99


def test_tensor_core_many_bandwidths_and_no_inversion(fo):
    """Thirteen bandwidths in one plan (two launch groups of at most eight
    tables) and pairs without the inverted orientation: the tensor-core
    results equal the CUDA-core ones.  Jmax 0 and 1 are left out here: their
    4^3 and smaller grids are too coarse for the peak search to be stable
    under FP32-level differences (their grids are compared above)."""
    ps = []
    for k, L in enumerate(range(2, 15)):
        p = synth.cluster_pair(8800 + k, n=24 + k)
        p.update(Jmax=L)
        ps.append(p)
    for invert in (True, False):
        a = fo.Context(precision="mixed")
        b = fo.Context(precision="mixed", tensor_cores=False)
        ra, rb = _align(fo, ps, a, invert), _align(fo, ps, b, invert)
        a.close()
        b.close()
        assert np.all(ra["status"] == 0)
        assert np.max(np.abs(ra["dist"] - rb["dist"]) / rb["dist"]) <= 1e-5
        assert all(np.array_equal(x, y) for x, y in zip(ra["perm"], rb["perm"]))


def _coef_oracle(oracle_mod, p, L, sig, groups):
    """FP64 coefficients of a pair with permutation groups: the per-group
    sums of the oracle's single-group contraction (structures centred as a
    whole, as the GPU path does)."""
    A = p["pos1"] - p["pos1"].mean(0)
    B = p["pos2"] - p["pos2"].mean(0)
    return sum(oracle_mod.cluster_coeffs(A[g], B[g], L, sig, cutoff=True) for g in groups)


@pytest.mark.parametrize("L,sizes,sig", [(0, [5], 0.3), (7, [40, 29, 1], 0.3), (11, [33, 31], 0.3),
                                         (15, [100, 47], 0.3), (31, [240, 60], 0.25)])
def test_tensor_core_coefficients(fo, oracle_mod, L, sizes, sig):
    """The tcgen05 coefficient contraction (3xTF32, FP32 accumulators in tensor
    memory) against the FP64 oracle and against the FP32 CUDA-core kernel:
    several permutation groups, groups spanning several 32-atom tiles and K
    stages, a 1-atom group, Jmax 0 to 31.  Bound: 1e-5 of the largest
    coefficient.  (The FP32 CUDA-core kernel is near 1e-7; the split-TF32
    products carry about 2^-22 of relative error each, so the tensor-core
    sums land near 1e-6.)"""
    from fastoverlap_gb300.batch import cluster_overlap
    n = sum(sizes)
    p = synth.cluster_pair(4400 + L, n=n, radius=1.9 * (n / 38.0) ** (1 / 3), sizes=sizes)
    groups = [np.asarray(g) for g in p["perm"]]
    ref = _coef_oracle(oracle_mod, p, L, sig, groups)
    tc = fo.Context(precision="mixed")
    cc = fo.Context(precision="mixed", tensor_cores=False)
    c_tc, _ = cluster_overlap(p["pos1"], p["pos2"], perm=groups, Jmax=L, scale=sig, ctx=tc)
    c_cc, _ = cluster_overlap(p["pos1"], p["pos2"], perm=groups, Jmax=L, scale=sig, ctx=cc)
    tc.close()
    cc.close()
    scale = np.abs(ref).max()
    e_tc, e_cc = np.abs(c_tc - ref).max(), np.abs(c_cc - ref).max()
    assert e_tc <= 1e-5 * scale, (e_tc / scale, e_cc / scale)
    assert e_cc <= 1e-5 * scale, (e_tc / scale, e_cc / scale)


def test_tensor_core_coefficients_1000_atoms(fo):
    """A 1000-atom Jmax-31 pair (800:200, the large-bandwidth workload): the
    tensor-core coefficients equal the FP32 CUDA-core ones within 1e-5 of the
    largest coefficient (25 tiles x 25 K stages for the 800-atom group)."""
    from fastoverlap_gb300.batch import cluster_overlap
    p = synth.config3(1, seed_offset=7)[0]
    groups = [np.asarray(g) for g in p["perm"]]
    tc = fo.Context(precision="mixed")
    cc = fo.Context(precision="mixed", tensor_cores=False)
    c_tc, g_tc = cluster_overlap(p["pos1"], p["pos2"], perm=groups, Jmax=31, scale=0.25, ctx=tc)
    c_cc, g_cc = cluster_overlap(p["pos1"], p["pos2"], perm=groups, Jmax=31, scale=0.25, ctx=cc)
    tc.close()
    cc.close()
    assert np.abs(c_tc - c_cc).max() <= 1e-5 * np.abs(c_cc).max()
    assert np.abs(g_tc - g_cc).max() <= 1e-5 * np.abs(g_cc).max()
