"""Batches whose host buffers are page-locked (fo_host_register): the same
results as with ordinary host memory, on repeated runs, and the buffers are
released again."""
import numpy as np
import pytest

from fastoverlap_gb300 import synth

pytestmark = pytest.mark.gpu


def test_pinned_batch_equals_pageable(fo):
    ps = synth.config2(48, seed_offset=5100)
    ctx = fo.Context(precision="mixed")
    args = ([p["pos1"] for p in ps], [p["pos2"] for p in ps], [p["perm"] for p in ps])
    ref = fo.ClusterBatch(ctx, *args, Jmax=[p["Jmax"] for p in ps], scale=0.3, nrot=10).run()
    b = fo.ClusterBatch(ctx, *args, Jmax=[p["Jmax"] for p in ps], scale=0.3, nrot=10).pin()
    for _ in range(2):
        out = b.run()
        assert np.array_equal(out["dist"], ref["dist"])
        assert all(np.array_equal(x, y) for x, y in zip(out["perm"], ref["perm"]))
        assert all(np.array_equal(x, y) for x, y in zip(out["aligned"], ref["aligned"]))
    b.close()
    assert b._pinned is None
    ctx.close()


def test_host_register_rejects_null(fo):
    ctx = fo.Context(precision="mixed")
    assert ctx.lib.fo_host_register(ctx.h, None, 16) != 0
    assert ctx.lib.fo_host_unregister(ctx.h, None) != 0
    ctx.close()
