"""Seeded synthetic alignment workloads.

No public dataset is named for these benchmarks, so seeded generators with
the stated shapes and value distributions stand in:

  cluster_pair : points uniform in a ball of radius R by rejection with a
                 minimum pair distance; B = A under a Haar-random rotation, a
                 uniform random permutation within each species and
                 N(0, noise^2) coordinate noise, inverted for odd seeds when
                 asked.
  periodic_pair: points uniform by rejection (minimum-image distance) in a
                 cubic periodic box; B = (A + t) mod box under a random
                 within-species permutation and N(0, noise^2) noise.
  config_*     : the benchmark configurations (single pairs, the 4096-pair
                 batch, the 64-pair large-bandwidth study, the Poisson stream).
RNG: numpy PCG64, seed per pair = base seed + pair index.
"""
import numpy as np

BASE_SEED = {"c0": 1000, "c1": 2000, "c2": 3000, "c3": 4000, "c4": 5000}


def haar_rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def _rsa(rng, n, draw, dist2_to, dmin, stall_rounds=None, batch=1024):
    """Random sequential addition: candidates are drawn in batches and accepted
    in draw order when no accepted point lies within the current minimum
    distance.  At the densities of the larger configurations (packing
    fraction near 0.4 for 1000 atoms) addition at the nominal distance jams,
    so after `stall_rounds` batches of 1024 candidates without a new point the
    minimum distance is lowered by 5% (40 batches up to 40 atoms, which keeps
    the 38-atom configuration at its nominal distance; 8 above)."""
    if stall_rounds is None:
        stall_rounds = 40 if n <= 40 else 8
    pts = np.empty((n, 3))
    k = 0
    dcur = dmin
    stall = 0
    while k < n:
        cand = draw(batch)
        d2min = dcur * dcur
        if k:
            cand = cand[dist2_to(pts[:k], cand).min(axis=0) >= d2min]
        placed = 0
        if len(cand):
            # sequential acceptance in draw order against the accepted ones
            close = dist2_to(cand, cand) < d2min
            acc = np.zeros(len(cand), bool)
            for j in range(len(cand)):
                if placed == n - k:
                    break
                if not (close[j, :j] & acc[:j]).any():
                    acc[j] = True
                    placed += 1
            pts[k:k + placed] = cand[acc]
            k += placed
        stall = 0 if placed else stall + 1
        if stall >= stall_rounds:
            dcur *= 0.95
            stall = 0
    return pts


def ball_points(rng, n, radius, dmin):
    """Uniform in a ball of the given radius, minimum pair distance dmin."""
    def draw(m):
        p = rng.uniform(-radius, radius, size=(m, 3))
        return p[np.einsum("ij,ij->i", p, p) <= radius * radius]

    def d2(P, Q):
        return ((P[:, None, :] - Q[None, :, :]) ** 2).sum(-1)
    return _rsa(rng, n, draw, d2, dmin)


def box_points(rng, n, L, dmin):
    """Uniform in a periodic cube of side L, minimum-image distance dmin."""
    def draw(m):
        return rng.uniform(0, L, size=(m, 3))

    def d2(P, Q):
        d = P[:, None, :] - Q[None, :, :]
        d -= L * np.round(d / L)
        return (d ** 2).sum(-1)
    return _rsa(rng, n, draw, d2, dmin)


def species_split(rng, n, nspecies):
    """Random fractions (Dirichlet), every species at least one atom."""
    if nspecies == 1:
        return [n]
    frac = rng.dirichlet(np.ones(nspecies))
    sizes = np.maximum(1, np.floor(frac * n).astype(int))
    while sizes.sum() > n:
        sizes[np.argmax(sizes)] -= 1
    while sizes.sum() < n:
        sizes[rng.integers(nspecies)] += 1
    return [int(s) for s in sizes]


def _groups_from_sizes(sizes):
    out, o = [], 0
    for s in sizes:
        out.append(np.arange(o, o + s))
        o += s
    return out


def cluster_pair(seed, n=38, radius=1.9, dmin=0.9, noise=0.05, sizes=None, invert_odd=True):
    rng = np.random.Generator(np.random.PCG64(seed))
    A = ball_points(rng, n, radius, dmin)
    groups = _groups_from_sizes(sizes or [n])
    R = haar_rotation(rng)
    B = A @ R.T
    perm = np.arange(n)
    for g in groups:
        perm[g] = rng.permutation(g)
    B = B[perm] + rng.normal(scale=noise, size=B.shape)
    inverted = bool(invert_odd and (seed % 2 == 1))
    if inverted:
        B = -B
    return dict(pos1=A, pos2=B, perm=groups, rot=R, true_perm=perm, inverted=inverted)


def periodic_pair(seed, n=256, density=1.2, dmin=0.8, noise=0.05, sizes=(204, 52)):
    rng = np.random.Generator(np.random.PCG64(seed))
    L = (n / density) ** (1.0 / 3.0)
    A = box_points(rng, n, L, dmin)
    groups = _groups_from_sizes(list(sizes))
    t = rng.uniform(0, L, size=3)
    perm = np.arange(n)
    for g in groups:
        perm[g] = rng.permutation(g)
    B = np.mod(A + t, L)[perm] + rng.normal(scale=noise, size=(n, 3))
    return dict(pos1=A, pos2=B, perm=groups, box=np.array([L, L, L]), shift=t, true_perm=perm)


# -- benchmark configurations ---------------------------------------------------
def config0(seed_offset=0):
    """38 atoms, 1 species, ball R=1.9, dmin 0.9, sigma 0.3, Jmax 7, 10 peaks."""
    p = cluster_pair(BASE_SEED["c0"] + seed_offset)
    p.update(Jmax=7, sigma=0.3, nrot=10)
    return p


def config1(seed_offset=0):
    """256 atoms (204:52) in a periodic cube at density 1.2, sigma 0.2, K=7, 10 peaks."""
    p = periodic_pair(BASE_SEED["c1"] + seed_offset)
    p.update(sigma=0.2, nwave=7, ndisps=10)
    return p


def config2(npairs=4096, seed_offset=0):
    """Uneven batch: N ~ U{13..147}, 1-3 species, Jmax ~ {7,11,15}, R = 1.9 (N/38)^(1/3)."""
    pairs = []
    for k in range(npairs):
        seed = BASE_SEED["c2"] + seed_offset + k
        rng = np.random.Generator(np.random.PCG64(seed + 10 ** 7))
        n = int(rng.integers(13, 148))
        ns = int(rng.integers(1, 4))
        sizes = species_split(rng, n, ns)
        jmax = int(rng.choice([7, 11, 15]))
        p = cluster_pair(seed, n=n, radius=1.9 * (n / 38.0) ** (1.0 / 3.0), sizes=sizes)
        p.update(Jmax=jmax, sigma=0.3, nrot=10)
        pairs.append(p)
    return pairs


def config3(npairs=64, seed_offset=0):
    """1000-atom clusters (800:200), R = 1.9 (1000/38)^(1/3), sigma 0.25, Jmax 31, 20 peaks."""
    pairs = []
    for k in range(npairs):
        seed = BASE_SEED["c3"] + seed_offset + k
        p = cluster_pair(seed, n=1000, radius=1.9 * (1000 / 38.0) ** (1.0 / 3.0), sizes=[800, 200])
        p.update(Jmax=31, sigma=0.25, nrot=20)
        pairs.append(p)
    return pairs


def _c4_base(args):
    """One base structure of the served stream (kind, index)."""
    kind, k, seed_offset = args
    seed = BASE_SEED["c4"] + seed_offset + (0 if kind == "cluster" else 10 ** 5) + k
    rng = np.random.Generator(np.random.PCG64(seed + 10 ** 7))
    if kind == "cluster":
        n = int(rng.integers(13, 501))
        A = ball_points(rng, n, 1.9 * (n / 38.0) ** (1.0 / 3.0), 0.9)
        return dict(kind=kind, pos1=A, sizes=[n], Jmax=int(rng.choice([7, 15])))
    n = int(rng.integers(64, 1025))
    na = int(round(0.8 * n))
    L = (n / 1.2) ** (1.0 / 3.0)
    A = box_points(rng, n, L, 0.8)
    return dict(kind=kind, pos1=A, sizes=[na, n - na], box=np.array([L, L, L]),
                nwave=int(rng.choice([5, 7])))


def config4_pool(n_cluster=48, n_periodic=16, seed_offset=0, pool=None):
    """Base structures of the served stream: spherical N~U{13..500} in a ball of
    radius 1.9 (N/38)^(1/3) with minimum distance 0.9 (as config 0), periodic
    N~U{64..1024} at density 1.2, 80:20, minimum distance 0.8 (as config 1).
    pool: an optional multiprocessing pool (generation takes seconds per
    large structure)."""
    jobs = [("cluster", k, seed_offset) for k in range(n_cluster)] + \
           [("periodic", k, seed_offset) for k in range(n_periodic)]
    return list(pool.map(_c4_base, jobs)) if pool is not None else [_c4_base(a) for a in jobs]


def config4_requests(bases, rate=2000.0, duration=60.0, seed_offset=0, max_requests=None):
    """Poisson arrivals at `rate` per second: 70% spherical, 30% periodic, each
    drawn from the base structures.  A request's B is its base A under a fresh
    Haar rotation (spherical; inverted for half) or uniform translation mod box
    (periodic), a random within-species permutation and N(0, 0.05^2) noise.
    Yields (t_arrival, request dict)."""
    rng = np.random.Generator(np.random.PCG64(BASE_SEED["c4"] + seed_offset))
    cl = [b for b in bases if b["kind"] == "cluster"]
    pe = [b for b in bases if b["kind"] == "periodic"]
    t = 0.0
    k = 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration or (max_requests is not None and k >= max_requests):
            return
        b = cl[rng.integers(len(cl))] if rng.uniform() < 0.7 else pe[rng.integers(len(pe))]
        A = b["pos1"]
        n = len(A)
        groups = _groups_from_sizes(b["sizes"])
        perm = np.arange(n)
        for g in groups:
            perm[g] = rng.permutation(g)
        if b["kind"] == "cluster":
            B = (A @ haar_rotation(rng).T)[perm] + rng.normal(scale=0.05, size=A.shape)
            if rng.uniform() < 0.5:
                B = -B
            req = dict(kind="cluster", pos1=A, pos2=B, perm=groups, Jmax=b["Jmax"], sigma=0.3, nrot=10)
        else:
            L = b["box"]
            B = np.mod(A + rng.uniform(0, L[0], size=3), L)[perm] + rng.normal(scale=0.05, size=A.shape)
            req = dict(kind="periodic", pos1=A, pos2=B, perm=groups, box=L, sigma=0.0, nwave=b["nwave"],
                       ndisps=10)
        yield t, req
        k += 1
