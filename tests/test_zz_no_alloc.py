"""The allocation-free periodic overlap entry point (fo_bulk_overlap_noalloc).

Callers that own all device memory through their own pool, or that must not
allocate in the middle of a request, use this entry point: it takes device
pointers and keeps its scratch in a fixed device array.  It must give the
same grid as the allocating entry point (fo_bulk_overlap, FP64), including
on consecutive calls, which share and reuse that array.

Kept in a file of its own that is collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc_grid(lib, torch, p, sizes, scale, nwave, nfspace=0):
    from fastoverlap_gb300.batch import _fastlen
    M = nfspace if nfspace else _fastlen(4 * nwave + 3)
    d1 = torch.tensor(np.ascontiguousarray(p["pos1"].ravel()), dtype=torch.float64, device="cuda")
    d2 = torch.tensor(np.ascontiguousarray(p["pos2"].ravel()), dtype=torch.float64, device="cuda")
    out = torch.full((M ** 3,), -1.0, dtype=torch.float64, device="cuda")  # stale values
    gs = np.ascontiguousarray(sizes, dtype=np.int32)
    torch.cuda.synchronize()
    st = lib.fo_bulk_overlap_noalloc(ctypes.c_void_p(d1.data_ptr()), ctypes.c_void_p(d2.data_ptr()),
                                     len(p["pos1"]), gs.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                     len(gs), float(p["box"][0]), float(p["box"][1]),
                                     float(p["box"][2]), scale, nwave, nfspace,
                                     ctypes.c_void_p(out.data_ptr()), None)
    torch.cuda.synchronize()
    assert st == 0
    return out.cpu().numpy().reshape(M, M, M).transpose(2, 1, 0)


def _check(lib, torch, p, sizes, scale, nwave, nfspace=0):
    from fastoverlap_gb300.batch import bulk_overlap
    ref = bulk_overlap(p["pos1"], p["pos2"], p["box"], perm=p["perm"], scale=scale,
                       nwave=nwave, nfspace=nfspace, precision="fp64")
    got = _noalloc_grid(lib, torch, p, sizes, scale, nwave, nfspace)
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) <= 1e-12 * ref.max()


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(fo):
    torch = pytest.importorskip("torch")
    from fastoverlap_gb300 import _lib, synth
    lib = _lib.load()
    assert 0 < lib.fo_bulk_overlap_noalloc_scratch_bytes() <= 8 << 20
    # calls in a row that share the array: 24^3, then 32^3, then 24^3 again
    # (a smaller grid after a larger one must not see the larger call's data)
    cases = [(synth.periodic_pair(321, n=96, sizes=(72, 24)), (72, 24), 0.3, 5),
             (synth.periodic_pair(654, n=140, sizes=(100, 40)), (100, 40), 0.25, 7),
             (synth.periodic_pair(987, n=64, sizes=(51, 13)), (51, 13), 0.3, 5)]
    for p, sizes, scale, nwave in cases:
        _check(lib, torch, p, sizes, scale, nwave)


def test_noalloc_largest_grid(fo):
    """nfspace = 64 fills the whole fixed array; a smaller call follows it."""
    torch = pytest.importorskip("torch")
    from fastoverlap_gb300 import _lib, synth
    lib = _lib.load()
    big = synth.periodic_pair(2024, n=120, sizes=(96, 24))
    _check(lib, torch, big, (96, 24), 0.25, 9, nfspace=64)
    small = synth.periodic_pair(77, n=64, sizes=(51, 13))
    _check(lib, torch, small, (51, 13), 0.3, 5)


def test_noalloc_rejects_grid_above_limit(fo):
    from fastoverlap_gb300 import _lib
    lib = _lib.load()
    gs = np.array([10], np.int32)
    dummy = ctypes.c_void_p(16)   # never dereferenced: the size check comes first
    st = lib.fo_bulk_overlap_noalloc(dummy, dummy, 10, gs.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                     1, 5.0, 5.0, 5.0, 0.3, 20, 81, dummy, None)
    assert st == 1   # FO_ERR_BAD_ARGS: a 81^3 grid exceeds the fixed scratch
