"""Host-side checks that need no GPU: C ABI exports and struct layouts,
workload generators, batch packing, multi-process timing helpers."""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "fastoverlap_gb300.h")


def _declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fo_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(fo):
    from fastoverlap_gb300 import _lib
    lib = _lib.load()
    names = _declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
        assert name in _lib.EXPORTS, "ctypes signature missing for " + name


def test_struct_layouts_match_header(tmp_path, fo):
    from fastoverlap_gb300 import _lib
    src = tmp_path / "sz.c"
    src.write_text('#include "fastoverlap_gb300.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(fo_opts),'
                   ' sizeof(fo_cluster_pair), sizeof(fo_bulk_pair), sizeof(fo_pair_result),'
                   ' offsetof(fo_bulk_pair, box), offsetof(fo_pair_result, inverted),'
                   ' sizeof(fo_request), offsetof(fo_request, pos1), offsetof(fo_request, group_sizes),'
                   ' sizeof(fo_server_opts), sizeof(fo_server_stats));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = [ctypes.sizeof(_lib.FoOpts), ctypes.sizeof(_lib.FoClusterPair),
            ctypes.sizeof(_lib.FoBulkPair), ctypes.sizeof(_lib.FoPairResult),
            _lib.FoBulkPair.box.offset, _lib.FoPairResult.inverted.offset,
            ctypes.sizeof(_lib.FoRequest), _lib.FoRequest.pos1.offset,
            _lib.FoRequest.group_sizes.offset, ctypes.sizeof(_lib.FoServerOpts),
            ctypes.sizeof(_lib.FoServerStats)]
    assert got == want


def test_context_without_gpu_fails_cleanly(fo):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is visible")
    except ImportError:
        pass
    with pytest.raises(fo.FoError):
        fo.Context()


def test_config0_generator():
    from fastoverlap_gb300 import synth
    p = synth.config0()
    A, B = p["pos1"], p["pos2"]
    assert A.shape == (38, 3) and B.shape == (38, 3)
    assert np.all(np.linalg.norm(A, axis=1) <= 1.9 + 1e-12)
    d = np.sqrt(((A[:, None] - A[None]) ** 2).sum(-1)) + np.eye(38) * 10
    assert d.min() >= 0.9
    # B is A rotated, permuted, noised (and inverted for odd seeds)
    s = -1.0 if p["inverted"] else 1.0
    Bt = s * B
    back = np.empty_like(A)
    back[p["true_perm"]] = Bt
    Rb = back @ p["rot"]
    assert np.sqrt(((Rb - A) ** 2).sum(-1)).max() < 0.5


def test_config1_generator():
    from fastoverlap_gb300 import synth
    p = synth.config1()
    L = p["box"][0]
    assert abs(L - (256 / 1.2) ** (1 / 3)) < 1e-12
    A = p["pos1"]
    d = A[:, None] - A[None]
    d -= L * np.round(d / L)
    d = np.sqrt((d ** 2).sum(-1)) + np.eye(256) * 10
    assert d.min() >= 0.8
    assert [len(g) for g in p["perm"]] == [204, 52]


def test_config2_shapes():
    from fastoverlap_gb300 import synth
    ps = synth.config2(12)
    for p in ps:
        n = len(p["pos1"])
        assert 13 <= n <= 147 and p["Jmax"] in (7, 11, 15)
        assert 1 <= len(p["perm"]) <= 3 and sum(len(g) for g in p["perm"]) == n
        assert min(len(g) for g in p["perm"]) >= 1


def test_batch_packing_offsets():
    from fastoverlap_gb300.batch import _Packed
    rng = np.random.default_rng(0)
    p1 = [rng.normal(size=(n, 3)) for n in (3, 5, 2)]
    p2 = [rng.normal(size=(n, 3)) for n in (3, 5, 2)]
    perms = [None, [np.array([0, 2, 4]), np.array([1, 3])], None]
    pk = _Packed(p1, p2, perms)
    assert list(pk.off) == [0, 3, 8] and pk.natoms_total == 10
    assert list(pk.perm) == [0, 1, 2, 0, 2, 4, 1, 3, 0, 1]
    assert list(pk.sizes) == [3, 3, 2, 2] and list(pk.group_off) == [0, 1, 3]
    assert np.array_equal(pk.pos1[9:24], p1[1].ravel())


def _allmax_worker(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist = bench.init_dist(ws)
    bench.barrier(dist)
    q.put((rank, bench.allmax(dist, 10.0 + rank)))
    dist.destroy_process_group()


def test_bench_max_over_ranks_gloo():
    import multiprocessing as mp
    ctxm = mp.get_context("spawn")
    q = ctxm.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctxm.Process(target=_allmax_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert out == [(0, 11.0), (1, 11.0)]


def test_clock_sampler_parses_reasons():
    sys.path.insert(0, ROOT)
    import bench
    cs = bench.ClockSampler()
    cs.proc = type("P", (), {"terminate": lambda s: None, "wait": lambda s, timeout=None: 0})()
    cs.lines = ["0, 1980, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Active",
                "0, 1990, 2070, 910.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    r = cs.stop()
    assert r["sm_mhz"] == 1985 and r["sm_max_mhz"] == 2070 and r["reasons"] == ["sw_power_cap"]


def test_reference_arm_sampler_makes_at_least_one_call(oracle_mod):
    """The CPU sampler behind bench.py --impl reference and the cpu_baseline
    leg: a zero time budget (one call per reference-arm step) still aligns
    its pairs and reports a finite rate."""
    sys.path.insert(0, ROOT)
    import bench
    from fastoverlap_gb300 import synth
    pairs = [(p["pos1"], p["pos2"], [np.asarray(g) for g in p["perm"]], p["Jmax"])
             for p in synth.config2(2, seed_offset=77)]
    rate, done, dt, per_call = bench._oracle_sample(pairs, 1, 0.0, 2)
    assert done == 2 and per_call == 2 and dt > 0 and np.isfinite(rate) and rate > 0


def test_batch_result_unpacking_spans():
    """Per-pair views of the packed outputs (no GPU: the unpacking is host code)."""
    import numpy as np
    from fastoverlap_gb300 import batch, _lib

    class Pk(object):
        pass

    b = batch.ClusterBatch.__new__(batch.ClusterBatch)
    b.pk = Pk()
    b.pk.n = np.array([3, 5, 2])
    b.pk.off = np.array([0, 3, 8])
    b.pk.natoms_total = 10
    res = np.zeros(3, _lib.RESULT_DTYPE)
    out = b._unpack(res, np.arange(30.0), np.arange(10, dtype=np.int32))
    assert [x.shape for x in out["aligned"]] == [(3, 3), (5, 3), (2, 3)]
    assert [x.tolist() for x in out["perm"]] == [[0, 1, 2], [3, 4, 5, 6, 7], [8, 9]]
    assert out["aligned"][1][0].tolist() == [9.0, 10.0, 11.0]


def test_new_wrappers_refuse_unsupported_arguments_before_any_device_work():
    import numpy as np
    import pytest
    import fastoverlap_gb300 as F
    from fastoverlap_gb300.sphericalAlignment import _average_separation

    with pytest.raises(NotImplementedError):
        F.BranchandBoundMaster(initialNodes=[object()])
    with pytest.raises(NotImplementedError):
        F.BranchandBoundMaster()(np.zeros((3, 3)), np.zeros((3, 3)), extra_inputs=[1])
    with pytest.raises(NotImplementedError):
        F.SphericalHarmonicAlign(scale=0.3).align(np.zeros((3, 3)), np.zeros((3, 3)), calcCoeffs=lambda b: None)
    # averageSeparation (sphericalAlignment.py:35-41): mean nearest-neighbour distance
    x = np.array([[0.0, 0, 0], [1.0, 0, 0], [3.0, 0, 0]])
    assert abs(_average_separation(x) - (1.0 + 1.0 + 2.0) / 3) < 1e-15


def test_oracle_cubic_operations_are_the_48_signed_permutations(oracle_mod):
    import numpy as np
    Ms = [oracle_mod.oh_operation(k) for k in range(48)]
    assert np.array_equal(Ms[0], np.eye(3))
    assert len({tuple(M.ravel()) for M in Ms}) == 48
    for M in Ms:
        assert np.array_equal(M @ M.T, np.eye(3)) and set(np.abs(M).sum(0)) == {1.0}
