"""Generate the golden fixtures in this directory from the upstream Python code.

Run in a container that has the upstream checkout (FO_REF_ROOT, read-only);
the GPU test machine only reads the .npz files this writes.

  python tests/golden/make_golden.py

Fixtures:
  lj38.npz    the upstream example pair examples/LJ38/{coords,finish} and the
              SphericalAlign distances at Jmax 7 and 14 (published: 1.4767,
              fastoverlap/sphericalAlignment.py:692)
  blj256.npz  examples/BLJ256/{coords,finish}, box 5.975206329, 204:52, and
              the PeriodicAlign distance (published 1.559,
              fastoverlap/periodicAlignment.py:609).  The upstream periodic
              cost matrix is transposed relative to what
              find_best_permutation expects (periodicAlignment.py:100 vs
              utils.py:161-165); the fixture uses a subclass that transposes
              it, which reproduces the published value.
  stages.npz  stage vectors from the upstream functions on seeded inputs:
              SO(3) coefficients (calcSO3Coeffs), Wigner-d tables (SOFT.Ds),
              inverse SOFT grid (SOFT.iSOFT), periodic overlap grid
              (PeriodicAlign.setPos fabs), Kearsley rotation (findrotation),
              linear assignment (the scipy solver behind the munkres shim).
  e2e.npz     SphericalAlign / PeriodicAlign distances on seeded synthetic
              pairs of the 38-atom and 256-atom configurations.
  e2e_perm.npz  the same classes on 32 seeded 38-atom pairs and 8 seeded
              256-atom periodic pairs: distance, aligned coordinates,
              permutation and overlap maxima (both orientations of the
              spherical pair; the periodic |F| maximum).
  peaks.npz   upstream findPeaks (fastoverlap/utils.py:366-396) on seeded
              overlap grids: 12 inverse-SOFT grids of 38-atom pairs (16^3) and
              4 periodic |F| grids of 256-atom pairs (32^3); the grids are
              recomputed by the tests.
  bessel_c3.npz  upstream calcSO3Coeffs (no cutoff) of a 100-atom pair in a
              ball of radius 5.65 at sigma 0.25, Jmax 31: the large-argument
              regime of i_l (x up to about 280) of the 1000-atom study
              (slices l = 0, 1, 15, 30, 31).

  python tests/golden/make_golden.py [harm|bnb|more]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "..", ".."))

import ref_shim  # noqa: E402
from fastoverlap_gb300 import synth  # noqa: E402


def main():
    root = ref_shim.reference_root()
    R = ref_shim.import_reference(root)
    ex = os.path.join(root, "examples")

    p1 = np.loadtxt(os.path.join(ex, "LJ38", "coords"))
    p2 = np.loadtxt(os.path.join(ex, "LJ38", "finish"))
    d14 = float(np.real(R.sph.SphericalAlign(0.3, 14)(p1, p2)[0]))
    d7 = float(np.real(R.sph.SphericalAlign(0.3, 7)(p1, p2)[0]))
    d7i = float(np.real(R.sph.SphericalAlign(0.3, 7)(p1, -p2)[0]))
    np.savez(os.path.join(HERE, "lj38.npz"), pos1=p1, pos2=p2, dist_j14=d14, dist_j7=d7,
             dist_j7_inverted=d7i, published=1.4767)

    q1 = np.loadtxt(os.path.join(ex, "BLJ256", "coords"))
    q2 = np.loadtxt(os.path.join(ex, "BLJ256", "finish"))
    box = np.ones(3) * 5.975206329
    pl = [np.arange(204), np.arange(204, 256)]

    class Fixed(R.per.PeriodicAlign):
        def cost_matrix(self, X1, X2):
            return R.per.PeriodicAlign.cost_matrix(self, X1, X2).T

    dper = float(Fixed(256, box, pl)(q1, q2)[0])
    dper7 = float(Fixed(256, box, pl, scale=0.2, n=7)(q1, q2, npeaks=10)[0])
    np.savez(os.path.join(HERE, "blj256.npz"), pos1=q1, pos2=q2, box=box, ntypeA=204, dist=dper,
             dist_s02_n7=dper7, published=1.559)

    rng = np.random.default_rng(20170212)
    A = rng.normal(size=(20, 3)) * 1.5
    A -= A.mean(0)
    B = A @ synth.haar_rotation(rng).T + rng.normal(size=A.shape) * 0.05
    B -= B.mean(0)
    sa = R.sph.SphericalAlign(0.4, 7)
    coeffs = sa.calcSO3Coeffs(A, B)               # [l, m1, m2], pos1 = A
    grid = sa.soft.iSOFT(coeffs).real             # [alpha, beta, gamma]
    ds4 = R.soft.SOFT(4).Ds
    dkab, Rkab = R.utils.findrotation(A, B)
    cost = rng.integers(0, 10 ** 7, size=(40, 40))
    from scipy.optimize import linear_sum_assignment
    _, lsa = linear_sum_assignment(cost)
    bq1 = synth.periodic_pair(77, n=64, sizes=(48, 16))
    pa = Fixed(64, bq1["box"], bq1["perm"], scale=0.3, n=3)
    pa.setPos(bq1["pos1"], bq1["pos2"])
    np.savez(os.path.join(HERE, "stages.npz"), A=A, B=B, sigma=0.4, L=7, coeffs=coeffs,
             grid=grid, wigner_bw4=ds4, kabsch_dist=float(np.real(dkab)), kabsch_R=Rkab,
             lap_cost=cost, lap_cols=lsa, per_pos1=bq1["pos1"], per_pos2=bq1["pos2"],
             per_box=bq1["box"], per_sizes=np.array([48, 16]), per_sigma=0.3, per_n=3,
             per_fabs=pa.fabs)

    sph_d, sph_inv = [], []
    for k in range(8):
        p = synth.config0(seed_offset=k)
        sph_d.append(float(np.real(R.sph.SphericalAlign(0.3, 7)(p["pos1"], p["pos2"])[0])))
        sph_inv.append(p["inverted"])
    per_d = []
    for k in range(2):
        p = synth.config1(seed_offset=k)
        per_d.append(float(Fixed(256, p["box"], p["perm"], scale=0.2, n=7)(p["pos1"], p["pos2"], npeaks=10)[0]))
    np.savez(os.path.join(HERE, "e2e.npz"), c0_seed_offsets=np.arange(8), c0_dist=np.array(sph_d),
             c0_inverted=np.array(sph_inv), c1_seed_offsets=np.arange(2), c1_dist=np.array(per_d))
    print("LJ38", d7, d14, d7i, "BLJ256", dper, dper7)
    print("c0", np.round(sph_d, 6), "c1", np.round(per_d, 6))


def harm(R=None):
    """harm.npz: the harmonic-basis path (SphericalHarmonicAlign) on centred
    structures -- coefficients, the SO(3) coefficients of a pair with their
    norm and overlap maximum (CALCSIMILARITY's two numbers), and end-to-end
    distances of four seeded 38-atom pairs (nmax 10, Jmax 7)."""
    R = R or ref_shim.import_reference(ref_shim.reference_root())
    nmax, L, hw, kw = 6, 5, 1.0, 0.3
    p = synth.cluster_pair(7, n=20)
    X = p["pos1"] - p["pos1"].mean(0)
    Y = p["pos2"] - p["pos2"].mean(0)
    a = R.sph.SphericalHarmonicAlign(scale=kw, harmscale=hw, nmax=nmax, Jmax=L)
    cX = a.calcHarmCoeff(X)                      # [n, l, m mod (2L+1)]
    so3 = a.calcSO3Coeffs(X, Y)                  # [l, m1, m2], pos1 = X
    grid = a.soft.iSOFT(so3).real
    norm = float(np.sum(np.abs(so3) ** 2))
    dists, pairs1, pairs2 = [], [], []
    for k in range(4):
        q = synth.cluster_pair(100 + k, n=38)
        X1, X2 = q["pos1"] - q["pos1"].mean(0), q["pos2"] - q["pos2"].mean(0)
        b = R.sph.SphericalHarmonicAlign(scale=0.3, harmscale=1.0, nmax=10, Jmax=7)
        dists.append(float(np.real(b(X1, X2)[0])))
        pairs1.append(X1)
        pairs2.append(X2)
    np.savez(os.path.join(HERE, "harm.npz"), X=X, Y=Y, nmax=nmax, L=L, hwidth=hw, kwidth=kw, coeffs_X=cX,
             so3=so3, norm=norm, maxover=float(grid.max()), pos1=np.array(pairs1), pos2=np.array(pairs2),
             dist_nmax10_j7=np.array(dists))
    print("harm", np.round(dists, 9), norm, float(grid.max()))


def bnb(R=None):
    """bnb.npz: the upstream Python branch and bound over rotations
    (BranchandBoundMaster, default rtol/atol, to completion) on four seeded
    cluster pairs: distance, expanded node count and aligned coordinates."""
    R = R or ref_shim.import_reference(ref_shim.reference_root())
    from fastoverlap import bnbAlignment
    P1, P2, D, N, A = [], [], [], [], []
    for k, n in [(5, 13), (6, 16), (7, 20), (8, 13)]:
        q = synth.cluster_pair(k, n=n)
        m = bnbAlignment.BranchandBoundMaster()
        d, _, x2 = m(q["pos1"], q["pos2"])
        P1.append(q["pos1"]); P2.append(q["pos2"]); D.append(float(d)); N.append(m.nodes); A.append(x2)
    np.savez(os.path.join(HERE, "bnb.npz"), natoms=np.array([len(x) for x in P1]), pos1=np.concatenate(P1),
             pos2=np.concatenate(P2), dist=np.array(D), nodes=np.array(N), aligned=np.concatenate(A))
    print("bnb", D, N)


def _fixed_periodic(R):
    class Fixed(R.per.PeriodicAlign):
        """The upstream periodic class with its cost matrix transposed to the
        orientation find_best_permutation expects (see blj256.npz)."""
        def cost_matrix(self, X1, X2):
            return R.per.PeriodicAlign.cost_matrix(self, X1, X2).T
    return Fixed


def _perm_from_radii(X2, Y):
    """Atom order of an aligned copy of Y: an alignment moves Y rigidly about
    its centroid (rotation, maybe inversion), which keeps each atom's distance
    to the centroid, so row i of X2 came from the atom of Y with the same
    radius (the radii of a random structure differ)."""
    ry = np.linalg.norm(Y - Y.mean(0), axis=1)
    rx = np.linalg.norm(X2 - X2.mean(0), axis=1)
    d = np.abs(rx[:, None] - ry[None, :])
    perm = d.argmin(1)
    srt = np.sort(d, axis=1)
    return perm, float(srt[:, 0].max()), float(srt[:, 1].min())


def e2e_perm(R=None):
    R = R or ref_shim.import_reference(ref_shim.reference_root())
    Fixed = _fixed_periodic(R)
    c0 = dict(dist=[], aligned=[], perm=[], omax=[], omax_inv=[])
    for k in range(32):
        p = synth.config0(seed_offset=k)
        sa = R.sph.SphericalAlign(0.3, 7)
        d, X1, X2 = sa(p["pos1"], p["pos2"])
        perm, err, gap = _perm_from_radii(X2, p["pos2"])
        assert err < 1e-8 < gap, (k, err, gap)
        Y1, Y2 = sa.COM_shift(p["pos1"], p["pos2"])
        om = sa.soft.iSOFT(sa.calcSO3Coeffs(Y1, Y2)).real.max()
        omi = sa.soft.iSOFT(sa.calcSO3Coeffs(Y1, -Y2)).real.max()
        c0["dist"].append(float(np.real(d)))
        c0["aligned"].append(np.real(X2))
        c0["perm"].append(perm)
        c0["omax"].append(float(om))
        c0["omax_inv"].append(float(omi))
    c1 = dict(dist=[], aligned=[], perm=[], omax=[], disp=[])
    for k in range(8):
        p = synth.config1(seed_offset=k)
        pa = Fixed(256, p["box"], p["perm"], scale=0.2, n=7)
        d, X1, X2, perm, disp = pa(p["pos1"], p["pos2"], npeaks=10)
        c1["dist"].append(float(d))
        c1["aligned"].append(X2)
        c1["perm"].append(np.asarray(perm))
        c1["omax"].append(float(pa.fabs.max()))
        c1["disp"].append(np.asarray(disp))
    np.savez(os.path.join(HERE, "e2e_perm.npz"), c0_seed_offsets=np.arange(32),
             **{"c0_" + k: np.array(v) for k, v in c0.items()},
             c1_seed_offsets=np.arange(8), **{"c1_" + k: np.array(v) for k, v in c1.items()})
    print("e2e_perm c0", np.round(c0["dist"], 4), "c1", np.round(c1["dist"], 4))


def peaks(R=None):
    """Upstream findPeaks on the overlap grids of seeded pairs.  The grids
    themselves are not stored: the tests recompute them (oracle or GPU), which
    agree with the upstream grids to 1e-12 (stages.npz pins that)."""
    R = R or ref_shim.import_reference(ref_shim.reference_root())
    Fixed = _fixed_periodic(R)
    kinds, seeds, pk, npk = [], [], [], []
    grids = []
    for k in range(12):
        p = synth.config0(seed_offset=k)
        sa = R.sph.SphericalAlign(0.3, 7)
        X1, X2 = sa.COM_shift(p["pos1"], p["pos2"])
        grids.append(sa.soft.iSOFT(sa.calcSO3Coeffs(X1, X2)).real)
        kinds.append(0)
        seeds.append(k)
    for k in range(4):
        p = synth.config1(seed_offset=k)
        pa = Fixed(256, p["box"], p["perm"], scale=0.2, n=7)
        pa.setPos(p["pos1"], p["pos2"])
        grids.append(pa.fabs.copy())
        kinds.append(1)
        seeds.append(k)
    for g in grids:
        q = np.asarray(R.utils.findPeaks(g, npeaks=10, width=2)[0]).reshape(-1, 3)
        npk.append(len(q))
        pk.append(np.vstack([q, np.full((10 - len(q), 3), np.nan)]))
    np.savez(os.path.join(HERE, "peaks.npz"), kind=np.array(kinds), seed_offset=np.array(seeds),
             peaks=np.array(pk), npeaks=np.array(npk))
    print("peaks found", npk)


def bessel_c3(R=None):
    """Upstream calcSO3Coeffs in the large-argument regime; the slices
    l = 0, 1, 15, 30, 31 of the coefficients are kept (the others are formed
    by the same code path)."""
    R = R or ref_shim.import_reference(ref_shim.reference_root())
    p = synth.cluster_pair(31, n=100, radius=5.65, dmin=0.75)
    X1 = p["pos1"] - p["pos1"].mean(0)
    X2 = p["pos2"] - p["pos2"].mean(0)
    sa = R.sph.SphericalAlign(0.25, 31)
    c = sa.calcSO3Coeffs(X1, X2)
    ls = np.array([0, 1, 15, 30, 31])
    r1, r2 = np.linalg.norm(X1, axis=1), np.linalg.norm(X2, axis=1)
    np.savez(os.path.join(HERE, "bessel_c3.npz"), A=X1, B=X2, sigma=0.25, L=31, ls=ls, coeffs=c[ls],
             xmax=float(r1.max() * r2.max() / (2 * 0.25 ** 2)))
    print("bessel_c3 x max", r1.max() * r2.max() / (2 * 0.25 ** 2))


if __name__ == "__main__":
    if sys.argv[1:] == ["harm"]:
        harm()
    elif sys.argv[1:] == ["bnb"]:
        bnb()
    elif sys.argv[1:] == ["more"]:
        R = ref_shim.import_reference(ref_shim.reference_root())
        e2e_perm(R)
        peaks(R)
        bessel_c3(R)
    else:
        main()
        harm()
        bnb()
        R = ref_shim.import_reference(ref_shim.reference_root())
        e2e_perm(R)
        peaks(R)
        bessel_c3(R)
