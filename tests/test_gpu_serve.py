"""Serving (fo_server_*): requests of both kinds admitted as they arrive give
exactly the results of the same pairs run as one batch; plans split under an
HBM budget; a request that does not fit alone fails alone; bad requests are
refused at submission."""
import threading
import time

import numpy as np
import pytest

from fastoverlap_gb300 import synth

pytestmark = pytest.mark.gpu


def _pairs():
    cps = synth.config2(24, seed_offset=700)
    bps = [synth.config1(k) for k in range(4)]
    return cps, bps


def _submit_all(srv, cps, bps):
    tickets = []
    for i, p in enumerate(cps):
        tickets.append(("c", i, srv.submit_cluster(p["pos1"], p["pos2"], p["perm"], Jmax=p["Jmax"],
                                                   scale=0.3, nrot=10)))
        if i % 6 == 0 and i // 6 < len(bps):
            q = bps[i // 6]
            tickets.append(("b", i // 6, srv.submit_periodic(q["pos1"], q["pos2"], q["box"], q["perm"],
                                                             scale=0.2, nwave=7, ndisps=10)))
    return tickets


def _reference(fo, cps, bps, precision):
    ctx = fo.Context(precision=precision)
    rc = fo.ClusterBatch(ctx, [p["pos1"] for p in cps], [p["pos2"] for p in cps], [p["perm"] for p in cps],
                         Jmax=[p["Jmax"] for p in cps], scale=0.3, nrot=10).run()
    rb = fo.BulkBatch(ctx, [p["pos1"] for p in bps], [p["pos2"] for p in bps], [p["box"] for p in bps],
                      [p["perm"] for p in bps], scale=0.2, nwave=7, ndisps=10).run()
    return {"c": rc, "b": rb}


def _check_same(got, ref, kind, i):
    r = ref[kind]
    assert got["status"] == 0
    assert got["dist"] == r["dist"][i]
    assert np.array_equal(got["perm"], r["perm"][i])
    assert np.array_equal(got["aligned"], r["aligned"][i])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_server_mix_equals_batch(fo, precision):
    cps, bps = _pairs()
    srv = fo.Server(precision=precision)
    tickets = _submit_all(srv, cps, bps)
    got = {(k, i): srv.wait(t) for k, i, t in tickets}
    st = srv.stats()
    srv.close()
    ref = _reference(fo, cps, bps, precision)
    for (k, i), g in got.items():
        _check_same(g, ref, k, i)
    assert st["submitted"] == st["completed"] == len(tickets)
    assert st["failed"] == 0 and st["batches"] >= 1
    assert 0 < st["latency_p50_ms"] <= st["latency_p99_ms"] <= st["latency_max_ms"]


def test_server_threads_and_poll(fo):
    cps, bps = _pairs()
    srv = fo.Server(precision="mixed", max_wait_ms=2.0)
    out = {}

    def client(lo, hi):
        for i in range(lo, hi):
            p = cps[i]
            out[i] = srv.submit_cluster(p["pos1"], p["pos2"], p["perm"], Jmax=p["Jmax"], scale=0.3, nrot=10)

    th = [threading.Thread(target=client, args=(k, k + 6)) for k in range(0, 24, 6)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    got = {}
    while len(got) < len(out):
        for i, t in out.items():
            if i not in got:
                r = srv.poll(t)
                if r is not None:
                    got[i] = r
        time.sleep(0.001)
    srv.close()
    ref = _reference(fo, cps, bps[:1], "mixed")
    for i, g in got.items():
        _check_same(g, ref, "c", i)


def test_server_budget_splits_and_rejects(fo):
    cps, _ = _pairs()
    ctx = fo.Context(precision="mixed")
    plan = fo.ClusterBatch(ctx, [p["pos1"] for p in cps], [p["pos2"] for p in cps], [p["perm"] for p in cps],
                           Jmax=[p["Jmax"] for p in cps], scale=0.3, nrot=10).plan()
    whole = plan.plan_device_bytes()
    plan.close()
    # a budget of a third of the whole batch: the server must split it
    srv = fo.Server(ctx=fo.Context(precision="mixed", hbm_budget_bytes=whole // 3))
    tickets = [srv.submit_cluster(p["pos1"], p["pos2"], p["perm"], Jmax=p["Jmax"], scale=0.3, nrot=10)
               for p in cps]
    # one request far larger than the budget: 1000 atoms at Jmax 31
    big = synth.cluster_pair(77, n=1000, radius=1.9 * (1000 / 38.0) ** (1.0 / 3.0))
    tb = srv.submit_cluster(big["pos1"], big["pos2"], big["perm"], Jmax=31, scale=0.25, nrot=20)
    got = [srv.wait(t) for t in tickets]
    rbig = srv.wait(tb)
    st = srv.stats()
    srv.close()
    ref = _reference(fo, cps, [synth.config1(0)], "mixed")
    for i, g in enumerate(got):
        _check_same(g, ref, "c", i)
    assert rbig["status"] == 5          # FO_ERR_OOM_BUDGET, the others unaffected
    assert st["failed"] == 1


def test_server_refuses_bad_requests(fo):
    srv = fo.Server(precision="mixed")
    p = synth.config2(1, seed_offset=900)[0]
    bad_perm = [np.zeros(len(p["pos1"]), dtype=np.int32)]     # atom 0 repeated
    with pytest.raises(fo.FoError) as e:
        srv.submit_cluster(p["pos1"], p["pos2"], bad_perm, Jmax=7)
    assert e.value.status == 1
    with pytest.raises(fo.FoError):
        srv.submit_cluster(p["pos1"], p["pos2"], p["perm"], Jmax=40)
    with pytest.raises(fo.FoError):
        srv.submit_periodic(p["pos1"], p["pos2"], [0.0, 1.0, 1.0], p["perm"])
    assert srv.stats()["submitted"] == 0
    srv.close()
