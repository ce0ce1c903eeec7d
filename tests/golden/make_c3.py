"""Generate c3.npz: oracle (FP64 CPU restatement) alignments of large clusters.

The 1000-atom, Jmax-31 configuration (800:200 species, sigma 0.25, 20 peaks
per orientation, inversion) is too slow for the upstream Python path (its
coefficient einsum takes minutes per orientation), so its parity fixtures
come from the oracle, whose stages are pinned to the upstream code
separately (including bessel_c3.npz for the large-argument Bessel regime).
Four pairs of 1000 atoms (seed offsets 0-3 of the 1000-atom generator) and
four pairs of 300 atoms (240:60, ball radius scaled by N^(1/3), same width,
bandwidth and peak count) are aligned, one process per pair.

  python tests/golden/make_c3.py        (about 10 minutes on 8 cores)
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "..", "..")


def _pairs():
    sys.path.insert(0, ROOT)
    from fastoverlap_gb300 import synth
    out = [synth.config3(1, seed_offset=k)[0] for k in range(4)]
    for k in range(4):
        p = synth.cluster_pair(synth.BASE_SEED["c3"] + 500 + k, n=300,
                               radius=1.9 * (300 / 38.0) ** (1.0 / 3.0), sizes=[240, 60])
        p.update(Jmax=31, sigma=0.25, nrot=20)
        out.append(p)
    return out


def _align(p):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    r = O.cluster_align(p["pos1"], p["pos2"], perm=p["perm"], Jmax=p["Jmax"], sigma=p["sigma"],
                        nrot=p["nrot"], invert=True, cutoff=True)
    return r


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    pairs = _pairs()
    with mp.get_context("spawn").Pool(min(8, len(pairs))) as pool:
        res = pool.map(_align, pairs)
    assert all(r["status"] == 0 for r in res)
    natoms = np.array([len(p["pos1"]) for p in pairs])
    sizes = np.array([[len(g) for g in p["perm"]] for p in pairs])
    np.savez_compressed(os.path.join(HERE, "c3.npz"), natoms=natoms, sizes=sizes,
                        pos1=np.concatenate([p["pos1"] for p in pairs]),
                        pos2=np.concatenate([p["pos2"] for p in pairs]),
                        jmax=31, sigma=0.25, nrot=20,
                        dist=np.array([r["dist"] for r in res]),
                        perm=np.concatenate([r["perm"] for r in res]),
                        aligned=np.concatenate([r["aligned"] for r in res]),
                        rmat=np.array([r["rmat"] for r in res]),
                        inverted=np.array([r["inverted"] for r in res]),
                        overlap_max=np.array([r["overlap_max"] for r in res]))
    print("c3", [round(r["dist"], 6) for r in res], [r["inverted"] for r in res])


if __name__ == "__main__":
    main()
