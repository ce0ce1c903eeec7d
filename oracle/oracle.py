"""ctypes wrapper of the CPU oracle (fo_oracle.c).

TEST INFRASTRUCTURE ONLY: the parity checker and the CPU baseline.  Only the
tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg import
this module; the product library never does.

All arrays are numpy; coordinates are (n, 3) float64; permutation groups are
lists of 0-based index arrays, as in the upstream Python classes.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_int64)


class OrcResult(ctypes.Structure):
    _fields_ = [("dist", ctypes.c_double), ("rmat", ctypes.c_double * 9),
                ("disp", ctypes.c_double * 3), ("inverted", ctypes.c_int),
                ("ncand", ctypes.c_int), ("status", ctypes.c_int),
                ("sigma", ctypes.c_double), ("overlap_max", ctypes.c_double)]


def build():
    """Compile libfo_oracle.so in place (gcc, a few seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "libfo_oracle.so")
        src = os.path.join(_HERE, "fo_oracle.c")
        if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
            build()
        _LIB = ctypes.CDLL(path)
        _LIB.orc_fastlen.restype = ctypes.c_int
        _LIB.orc_choose_kwidth.restype = ctypes.c_double
        _LIB.orc_findrotation.restype = ctypes.c_double
        _LIB.orc_iterative_align.restype = ctypes.c_double
        _LIB.orc_findpeaks.restype = ctypes.c_int
        _LIB.orc_findpeaks_w.restype = ctypes.c_int
        _LIB.orc_jv.restype = ctypes.c_int
        _LIB.orc_cluster_align.restype = ctypes.c_int
        _LIB.orc_bulk_align.restype = ctypes.c_int
        _LIB.orc_harm_align.restype = ctypes.c_int
    return _LIB


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _groups(perm, n):
    if perm is None:
        perm = [np.arange(n)]
    flat = np.ascontiguousarray(np.concatenate([np.asarray(p, dtype=np.int32) for p in perm]),
                                dtype=np.int32)
    sizes = np.ascontiguousarray([len(p) for p in perm], dtype=np.int32)
    return flat, sizes


def fastlen(n):
    return lib().orc_fastlen(int(n))


def ylm(xyz, L):
    W = 2 * L + 1
    re = np.zeros((L + 1) * W)
    im = np.zeros((L + 1) * W)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    lib().orc_ylm(_d(xyz), int(L), _d(re), _d(im))
    return (re + 1j * im).reshape(L + 1, W)


def sphi(L, x):
    out = np.zeros(L + 1)
    lib().orc_sphi(int(L), ctypes.c_double(x), _d(out))
    return out


def cluster_coeffs(B, A, L, sigma, cutoff=True):
    """Coefficients in the upstream Python layout [l, m1 mod W, m2 mod W]."""
    B = np.ascontiguousarray(B, dtype=np.float64)
    A = np.ascontiguousarray(A, dtype=np.float64)
    W = 2 * L + 1
    out = np.zeros(2 * (L + 1) * W * W)
    lib().orc_cluster_coeffs(_d(B), _d(A), len(B), int(L), ctypes.c_double(sigma),
                             int(bool(cutoff)), _d(out))
    return (out[0::2] + 1j * out[1::2]).reshape(L + 1, W, W)


def wigner_d(bw):
    W, G = 2 * bw - 1, 2 * bw
    d = np.zeros(bw * W * W * G)
    lib().orc_wigner_d(int(bw), _d(d))
    return d.reshape(bw, W, W, G)


def isoft(ilmm):
    """Real overlap grid, returned in [alpha, beta, gamma] index order."""
    bw = ilmm.shape[0]
    G = 2 * bw
    c = np.zeros(2 * ilmm.size)
    c[0::2] = ilmm.real.ravel()
    c[1::2] = ilmm.imag.ravel()
    out = np.zeros(G ** 3)
    lib().orc_isoft(int(bw), _d(c), _d(out))
    return out.reshape(G, G, G).transpose(2, 1, 0)  # stored alpha fastest


def findpeaks(grid, npeaks, width=2):
    """grid indexed [i1, i2, i3]; returns (peaks (np,3) 1-based, amplitudes).
    width: starting window half-width."""
    n1, n2, n3 = grid.shape
    g = np.ascontiguousarray(np.asarray(grid, dtype=np.float64).transpose(2, 1, 0))
    pk = np.zeros(3 * npeaks)
    am = np.zeros(npeaks)
    nf = lib().orc_findpeaks_w(_d(g), n1, n2, n3, int(npeaks), int(width), _d(pk), _d(am))
    if nf < 0:
        raise RuntimeError("no peaks found")
    return pk[:3 * nf].reshape(nf, 3), am[:nf]


def jv(cost, kk=None, first=None):
    """Assignment on an int64 cost matrix (dense (n,n) or CSR)."""
    cost = np.asarray(cost, dtype=np.int64)
    if kk is None:
        n = cost.shape[0]
        cc = np.ascontiguousarray(cost.ravel())
        kk = np.ascontiguousarray(np.tile(np.arange(n, dtype=np.int32), n))
        first = np.ascontiguousarray(np.arange(n + 1, dtype=np.int32) * n)
    else:
        n = len(first) - 1
        cc = np.ascontiguousarray(cost)
        kk = np.ascontiguousarray(kk, dtype=np.int32)
        first = np.ascontiguousarray(first, dtype=np.int32)
    x = np.zeros(n, np.int32)
    y = np.zeros(n, np.int32)
    rc = lib().orc_jv(n, cc.ctypes.data_as(_lp), _i(kk), _i(first), _i(x), _i(y))
    return rc, x


def pairdists(p, q, bulk=False, box=(0., 0., 0.), maxnei=60):
    p = np.ascontiguousarray(p, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    n = len(p)
    m = min(n, maxnei)
    cc = np.zeros(n * m)
    kk = np.zeros(n * m, np.int32)
    bx = np.ascontiguousarray(box, dtype=np.float64)
    lib().orc_pairdists(n, _d(p), _d(q), int(bool(bulk)), _d(bx), int(maxnei), _d(cc), _i(kk))
    return cc.reshape(n, m), kk.reshape(n, m)


def findrotation(B, A):
    B = np.ascontiguousarray(B, dtype=np.float64)
    A = np.ascontiguousarray(A, dtype=np.float64)
    R = np.zeros(9)
    d = lib().orc_findrotation(_d(B), _d(A), len(B), _d(R))
    return d, R.reshape(3, 3)


def iterative_align(B, A, perm=None, bulk=False, box=(0., 0., 0.)):
    B = np.ascontiguousarray(B, dtype=np.float64)
    A = np.array(A, dtype=np.float64, order="C", copy=True)
    n = len(B)
    flat, sizes = _groups(perm, n)
    R = np.zeros(9)
    disp = np.zeros(3)
    pb = np.zeros(n, np.int32)
    it = ctypes.c_int(0)
    bx = np.ascontiguousarray(box, dtype=np.float64)
    d = lib().orc_iterative_align(_d(B), _d(A), n, _i(flat), _i(sizes), len(sizes),
                                  int(bool(bulk)), _d(bx), _d(R), _d(disp), _i(pb),
                                  ctypes.byref(it))
    return d, A, R.reshape(3, 3), disp, pb, it.value


def cluster_align(pos1, pos2, perm=None, Jmax=15, sigma=0.3, nrot=10, invert=True,
                  cutoff=True):
    """Fortran-semantics cluster alignment. Returns dict of outputs."""
    p1 = np.ascontiguousarray(pos1, dtype=np.float64).reshape(-1, 3)
    p2 = np.ascontiguousarray(pos2, dtype=np.float64).reshape(-1, 3)
    n = len(p1)
    flat, sizes = _groups(perm, n)
    al = np.zeros((n, 3))
    pb = np.zeros(n, np.int32)
    r = OrcResult()
    rc = lib().orc_cluster_align(_d(p1), _d(p2), n, _i(flat), _i(sizes), len(sizes), int(Jmax),
                                 ctypes.c_double(sigma if sigma is not None else 0.0),
                                 int(nrot), int(bool(invert)), int(bool(cutoff)), _d(al),
                                 _i(pb), ctypes.byref(r))
    return dict(status=rc, dist=r.dist, aligned=al, perm=pb,
                rmat=np.array(r.rmat).reshape(3, 3), inverted=bool(r.inverted),
                ncand=r.ncand, sigma=r.sigma, overlap_max=r.overlap_max)


def harmonic_nl(nmax, lmax, rj, sigma, r0):
    """HARMONICNL: (nmax+1, lmax+1) overlap integrals of one kernel."""
    out = np.zeros((nmax + 1) * (lmax + 1))
    lib().orc_harmonic_nl(int(nmax), int(lmax), ctypes.c_double(rj), ctypes.c_double(sigma),
                          ctypes.c_double(r0), _d(out))
    return out.reshape(nmax + 1, lmax + 1)


def harmonic_coeffs(X, nmax, L, hwidth, kwidth):
    """HARMONICCOEFFS of the coordinates as given: complex (nmax+1, L+1, 2L+1)
    indexed [n, l, m mod (2L+1)] (the upstream Python calcHarmCoeff layout)."""
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
    W = 2 * L + 1
    out = np.zeros(2 * (nmax + 1) * (L + 1) * W)
    lib().orc_harmonic_coeffs(_d(X), len(X), int(nmax), int(L), ctypes.c_double(hwidth),
                              ctypes.c_double(kwidth), _d(out))
    return (out[0::2] + 1j * out[1::2]).reshape(nmax + 1, L + 1, W)


def harm_align(pos1, pos2, perm=None, nmax=20, Jmax=15, hwidth=1.0, kwidth=0.3, nrot=10,
               invert=True):
    """ALIGNHARM semantics (coordinates as given).  Returns dict of outputs."""
    p1 = np.ascontiguousarray(pos1, dtype=np.float64).reshape(-1, 3)
    p2 = np.ascontiguousarray(pos2, dtype=np.float64).reshape(-1, 3)
    n = len(p1)
    flat, sizes = _groups(perm, n)
    al = np.zeros((n, 3))
    pb = np.zeros(n, np.int32)
    r = OrcResult()
    rc = lib().orc_harm_align(_d(p1), _d(p2), n, _i(flat), _i(sizes), len(sizes), int(nmax), int(Jmax),
                              ctypes.c_double(hwidth), ctypes.c_double(kwidth), int(nrot),
                              int(bool(invert)), _d(al), _i(pb), ctypes.byref(r))
    return dict(status=rc, dist=r.dist, aligned=al, perm=pb,
                rmat=np.array(r.rmat).reshape(3, 3), inverted=bool(r.inverted),
                ncand=r.ncand, overlap_max=r.overlap_max)


def overlap_matrices(coordslist, perm=None, nmax=20, Jmax=15, hwidth=1.0, kwidth=0.3):
    """CALCOVERLAPMATRICES: (norms, maxovers), each (nlist, nlist), from the
    per-group harmonic coefficients of each structure (coordinates as given)."""
    X = [np.asarray(x, dtype=np.float64).reshape(-1, 3) for x in coordslist]
    n = len(X[0])
    flat, sizes = _groups(perm, n)
    cs = []
    for x in X:
        off, parts = 0, []
        for sz in sizes:
            idx = flat[off:off + sz]
            c = harmonic_coeffs(x[idx], nmax, Jmax, hwidth, kwidth)
            parts.append(np.stack([c.real, c.imag], -1).ravel())
            off += sz
        cs.append(np.ascontiguousarray(np.concatenate(parts)))
    nl = len(X)
    norms, maxs = np.zeros((nl, nl)), np.zeros((nl, nl))
    for i in range(nl):
        for j in range(i, nl):
            a, b = ctypes.c_double(), ctypes.c_double()
            lib().orc_calc_similarity(_d(cs[i]), _d(cs[j]), len(sizes), int(nmax), int(Jmax),
                                      ctypes.byref(a), ctypes.byref(b))
            norms[i, j] = norms[j, i] = a.value
            maxs[i, j] = maxs[j, i] = b.value
    return norms, maxs


def bulk_fspace(pos1, pos2, box, perm=None, sigma=0.2, nwave=7, nf=None):
    p1 = np.ascontiguousarray(pos1, dtype=np.float64).reshape(-1, 3)
    p2 = np.ascontiguousarray(pos2, dtype=np.float64).reshape(-1, 3)
    n = len(p1)
    flat, sizes = _groups(perm, n)
    nf = nf or fastlen(4 * nwave + 3)
    out = np.zeros(nf ** 3)
    bx = np.ascontiguousarray(box, dtype=np.float64)
    lib().orc_bulk_fspace(_d(p1), _d(p2), n, _i(flat), _i(sizes), len(sizes), _d(bx),
                          ctypes.c_double(sigma), int(nwave), int(nf), _d(out))
    return out.reshape(nf, nf, nf).transpose(2, 1, 0)


def bulk_align(pos1, pos2, box, perm=None, sigma=0.0, nwave=0, nfspace=0, ndisps=10):
    p1 = np.ascontiguousarray(pos1, dtype=np.float64).reshape(-1, 3)
    p2 = np.ascontiguousarray(pos2, dtype=np.float64).reshape(-1, 3)
    n = len(p1)
    flat, sizes = _groups(perm, n)
    al = np.zeros((n, 3))
    pb = np.zeros(n, np.int32)
    r = OrcResult()
    bx = np.ascontiguousarray(box, dtype=np.float64)
    rc = lib().orc_bulk_align(_d(p1), _d(p2), n, _i(flat), _i(sizes), len(sizes), _d(bx),
                              ctypes.c_double(sigma or 0.0), int(nwave or 0), int(nfspace or 0),
                              int(ndisps), _d(al), _i(pb), ctypes.byref(r))
    return dict(status=rc, dist=r.dist, aligned=al, perm=pb, disp=np.array(r.disp),
                ncand=r.ncand, sigma=r.sigma, overlap_max=r.overlap_max)


def oh_operation(op):
    """Operation op (0..47) of the cubic point group as a signed axis
    permutation (row-major): output axis r takes input axis P[op // 8][r],
    negated when bit r of op % 8 is set.  Operation 0 is the identity."""
    P = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    M = np.zeros((3, 3))
    for r in range(3):
        M[r, P[op // 8][r]] = -1.0 if (op % 8) >> r & 1 else 1.0
    return M


def bulk_align_ohcell(pos1, pos2, box, perm=None, sigma=0.0, nwave=0, nfspace=0, ndisps=10):
    """ALIGN1 with OHCELLT (fastbulk.f90:458-481): the alignment of pos1 with
    op(pos2) for the 48 cubic operations, the smallest distance kept (the
    first operation on ties).  The overlap of each operation is formed from
    the transformed structure.  Returns the best dict with 'op' and 'M'."""
    p2 = np.asarray(pos2, dtype=np.float64).reshape(-1, 3)
    best = None
    for op in range(48):
        M = oh_operation(op)
        r = bulk_align(pos1, p2 @ M.T, box, perm, sigma, nwave, nfspace, ndisps)
        if r["status"] == 0 and (best is None or r["dist"] < best["dist"]):
            best = dict(r, op=op, M=M)
    return best


def bnb_cluster(pos1, pos2, invert=True, niter=None, rtol=5e-2, atol=1e-3):
    """Branch and bound over rotations (upstream BranchandBoundMaster).
    Returns dict(dist, aligned, nodes)."""
    p1 = np.ascontiguousarray(pos1, dtype=np.float64).reshape(-1, 3)
    p2 = np.ascontiguousarray(pos2, dtype=np.float64).reshape(-1, 3)
    al = np.zeros_like(p1)
    d = ctypes.c_double()
    nodes = ctypes.c_longlong()
    lib().orc_bnb_cluster(_d(p1), _d(p2), len(p1), int(bool(invert)),
                          ctypes.c_longlong(2 ** 62 if niter is None else int(niter)), ctypes.c_double(rtol),
                          ctypes.c_double(atol), ctypes.byref(d), _d(al), ctypes.byref(nodes))
    return dict(dist=d.value, aligned=al, nodes=nodes.value)


def cluster_align_many(pairs, nrot=10, invert=True, cutoff=True, nthreads=None, with_perm=False):
    """pairs: list of dicts(pos1, pos2, perm, Jmax, sigma). Returns distances,
    and with_perm the list of best permutations too."""
    nthreads = nthreads or os.cpu_count() or 1
    p1 = np.ascontiguousarray(np.concatenate([np.asarray(p["pos1"], float).ravel() for p in pairs]))
    p2 = np.ascontiguousarray(np.concatenate([np.asarray(p["pos2"], float).ravel() for p in pairs]))
    natoms = np.array([len(np.asarray(p["pos1"]).reshape(-1, 3)) for p in pairs], np.int32)
    coff = np.zeros(len(pairs), np.int64)
    coff[1:] = np.cumsum(3 * natoms)[:-1]
    flats, sizes, poff, goff, ng = [], [], [], [], []
    po = go = 0
    for p, n in zip(pairs, natoms):
        f, s = _groups(p.get("perm"), int(n))
        flats.append(f)
        sizes.append(s)
        poff.append(po)
        goff.append(go)
        ng.append(len(s))
        po += len(f)
        go += len(s)
    flat = np.ascontiguousarray(np.concatenate(flats), np.int32)
    gs = np.ascontiguousarray(np.concatenate(sizes), np.int32)
    poff = np.ascontiguousarray(poff, np.int64)
    goff = np.ascontiguousarray(goff, np.int32)
    ng = np.ascontiguousarray(ng, np.int32)
    L = np.ascontiguousarray([p["Jmax"] for p in pairs], np.int32)
    sg = np.ascontiguousarray([p["sigma"] for p in pairs], np.float64)
    out = np.zeros(len(pairs))
    pout = np.zeros(int(natoms.sum()), np.int32) if with_perm else None
    lib().orc_cluster_align_many(len(pairs), _d(p1), _d(p2), coff.ctypes.data_as(_lp),
                                 _i(natoms), _i(flat), poff.ctypes.data_as(_lp), _i(gs),
                                 _i(goff), _i(ng), _i(L), _d(sg), int(nrot), int(bool(invert)),
                                 int(bool(cutoff)), int(nthreads), _d(out),
                                 _i(pout) if with_perm else None)
    if with_perm:
        ao = np.concatenate([[0], np.cumsum(natoms)])
        return out, [pout[ao[k]:ao[k + 1]].copy() for k in range(len(pairs))]
    return out
