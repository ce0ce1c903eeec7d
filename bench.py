"""Benchmark: aligned pairs/s on the 4096-pair batched spherical workload.

Workload (default): 4096 cluster pairs, N ~ U{13..147} atoms, 1-3 species,
Jmax ~ {7, 11, 15}, sigma 0.3, 10 peaks per orientation, inversion tested
(seeded synthetic data; see fastoverlap_gb300/synth.py).  One step = one
pass of the whole alignment pipeline over the batch.

  value : batched pairs/s with inputs resident in HBM (resident plan), the
          precision given by --precision (default mixed), device time from
          CUDA events on the library's stream, L2 flushed between steps.
  e2e   : the same batch through fo_cluster_align_batch with page-locked host buffers
          (upload, pipeline, download), wall time.
  config: also reports the plain FP64 GPU form (batched and one pair per
          call), the error of the mixed form against FP64, the large-bandwidth
          study (config.precision_study_c3: 64 pairs of 1000 atoms at Jmax 31,
          FP64 against mixed), and a served stream (config.serving, 2000
          req/s for 60 s): Poisson arrivals (70% spherical N 13..500, 30%
          periodic N 64..1024) through fo_server_* with p50/p99 latency and
          the median latency per 10 s window; config.serving_fp64 serves the
          same stream in plain FP64 at a rate near its capacity.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--npairs P] [--precision mixed|fp64]

For N > 1 (torchrun), every rank runs its own batch (weak scaling), timed
between barriers; rank 0 prints max-over-ranks timing.  --impl reference
times the CPU restatement of the reference algorithm (oracle/) on the host
cores over a bounded sample of the same workload.
"""
import argparse
import json
import multiprocessing as mp
import os
import queue
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "aligned pairs/s (batched+mixed vs plain FP64 GPU, RMSD-matched); p50/p99 ms"
# Warp instructions the refinement kernel issues per candidate on the 4096-pair
# workload (mixed form): smsp__inst_executed.sum over the bucket launches of
# one plan run (ncu), divided by the plan's candidates.
REFINE_INST_PER_CAND = 218932.0   # 17.86e9 over 81,574 candidates
WORKLOAD = ("c2: 4096 batched spherical pairs, N~U{13..147}, 1-3 species, Jmax~{7,11,15}, "
            "sigma 0.3, 10 peaks/orientation, inversion")


def _gen_chunk(args):
    lo, hi = args
    from fastoverlap_gb300 import synth
    out = []
    for k in range(lo, hi):
        p = synth.config2(1, seed_offset=k)[0]
        out.append((p["pos1"], p["pos2"], [np.asarray(g) for g in p["perm"]], p["Jmax"]))
    return out


def make_workload(npairs, seed_offset=0):
    cache = "/tmp/fo_bench_c2_%d_%d.npz" % (npairs, seed_offset)
    if os.path.exists(cache):
        z = np.load(cache, allow_pickle=True)
        return list(z["pairs"])
    nproc = min(16, os.cpu_count() or 1)
    chunks = [(seed_offset + i, seed_offset + min(i + 64, npairs)) for i in range(0, npairs, 64)]
    ctxm = mp.get_context("spawn")
    with ctxm.Pool(nproc) as pool:
        parts = pool.map(_gen_chunk, chunks)
    pairs = [x for part in parts for x in part]
    try:
        np.savez(cache, pairs=np.array(pairs, dtype=object))
    except Exception:
        pass
    return pairs


def _gen_c3(k):
    from fastoverlap_gb300 import synth
    p = synth.config3(1, seed_offset=k)[0]
    return (p["pos1"], p["pos2"], [np.asarray(g) for g in p["perm"]])


def c3_run(npairs):
    """Large-bandwidth precision study (config 3): 1000-atom clusters (800:200),
    Jmax 31, sigma 0.25, 20 peaks; the plain FP64 form against the mixed form."""
    from fastoverlap_gb300 import ClusterBatch, Context
    cache = "/tmp/fo_bench_c3_%d.npz" % npairs
    if os.path.exists(cache):
        pairs = list(np.load(cache, allow_pickle=True)["pairs"])
    else:
        with mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1)) as pool:
            pairs = pool.map(_gen_c3, range(npairs))
        try:
            np.savez(cache, pairs=np.array(pairs, dtype=object))
        except Exception:
            pass
    out, res = {"pairs": npairs, "atoms": 1000, "jmax": 31, "peaks": 20}, {}
    for prec in ("fp64", "mixed"):
        ctx = Context(precision=prec, profile=True)
        b = ClusterBatch(ctx, [p[0] for p in pairs], [p[1] for p in pairs], [p[2] for p in pairs],
                         Jmax=31, scale=0.25, nrot=20).plan()
        b.plan_run()
        b.plan_wait()
        ctx.profile_reset()
        ctx.flush_l2(512 << 20)
        ctx.record(0)
        b.plan_run()
        ctx.record(1)
        b.plan_wait()
        ms = ctx.elapsed_ms(0, 1)
        res[prec] = b.plan_results(with_coords=True)
        out["%s_pairs_per_s" % prec] = npairs / (ms / 1000.0)
        out["%s_kernel_ms" % prec] = {k: v[0] / max(1, v[1]) for k, v in ctx.profile().items()}
        b.close()
        ctx.close()
    out["mixed_over_fp64"] = out["mixed_pairs_per_s"] / out["fp64_pairs_per_s"]
    a, f = res["mixed"], res["fp64"]
    ok = (a["status"] == 0) & (f["status"] == 0)
    out["mixed_vs_fp64_max_rel_dist"] = float(np.max(np.abs(a["dist"][ok] - f["dist"][ok]) / f["dist"][ok]))
    out["mixed_vs_fp64_identical_perm_frac"] = float(np.mean([np.array_equal(x, y) for x, y, o in
                                                              zip(a["perm"], f["perm"], ok) if o]))
    om_a, om_f = a["result"]["overlap_max"][ok], f["result"]["overlap_max"][ok]
    out["mixed_vs_fp64_max_rel_overlap_max"] = float(np.max(np.abs(om_a - om_f) / np.abs(om_f)))
    out["pairs_failed"] = int((~ok).sum())
    return out


def _c4_pool(nproc):
    cache = "/tmp/fo_bench_c4_pool.npz"
    if os.path.exists(cache):
        z = np.load(cache, allow_pickle=True)
        return list(z["bases"])
    from fastoverlap_gb300 import synth
    ctxm = mp.get_context("spawn")
    with ctxm.Pool(nproc) as pool:
        bases = synth.config4_pool(pool=pool)
    try:
        np.savez(cache, bases=np.array(bases, dtype=object))
    except Exception:
        pass
    return bases


def serve_run(rate, duration, precision, workers=2):
    """Served stream: requests submitted at their Poisson arrival times from one
    host thread; returns latency percentiles (submit -> complete) and the
    completed requests per second of wall time."""
    from fastoverlap_gb300 import synth
    from fastoverlap_gb300.serve import Server
    bases = _c4_pool(min(16, os.cpu_count() or 1))
    reqs = list(synth.config4_requests(bases, rate=rate, duration=duration))
    srv = Server(precision=precision, workers=workers)
    # warm the kernels and the block pool with a few requests of each kind
    for _, q in reqs[:32]:
        _submit_req(srv, q)
    srv.close()
    srv = Server(precision=precision, workers=workers)
    # a second thread collects the tickets in submission order while the
    # stream runs; the time a ticket is collected bounds its completion from
    # above, which is enough to show whether latency grows over the run
    todo = queue.Queue()
    done = []

    def collect():
        while True:
            item = todo.get()
            if item is None:
                return
            t, ts = item
            srv.wait(t)
            done.append((ts, time.time() - t0 - ts))

    t0 = time.time()
    waiter = threading.Thread(target=collect)
    waiter.start()
    for ta, q in reqs:
        dt = t0 + ta - time.time()
        if dt > 0:
            time.sleep(dt)
        todo.put((_submit_req(srv, q), time.time() - t0))
    t_sub = time.time() - t0
    todo.put(None)
    waiter.join()
    wall = time.time() - t0
    st = srv.stats()
    srv.close()
    ncl = sum(1 for _, q in reqs if q["kind"] == "cluster")
    win = 10.0 if duration >= 20 else max(duration / 2.0, 1e-3)
    by_win = []
    for w0 in np.arange(0.0, t_sub, win):
        lat = [l for ts, l in done if w0 <= ts < w0 + win]
        if lat:
            by_win.append(round(1e3 * float(np.median(lat)), 1))
    return {"arrival_rate_per_s": rate, "duration_s": duration, "requests": len(reqs),
            "spherical": ncl, "periodic": len(reqs) - ncl, "submit_s": t_sub, "wall_s": wall,
            "workers": workers, "completed_per_s": st["completed"] / wall, "failed": int(st["failed"]),
            "latency_p50_ms": st["latency_p50_ms"], "latency_p99_ms": st["latency_p99_ms"],
            "latency_max_ms": st["latency_max_ms"], "batches": int(st["batches"]),
            "mean_batch": st["mean_batch"],
            "collected_p50_ms_by_window": by_win, "window_s": win,
            "stand_in": "requests drawn from 48 spherical + 16 periodic seeded base structures, "
                        "each with a fresh rotation/translation, permutation and noise"}


def _submit_req(srv, q):
    if q["kind"] == "cluster":
        return srv.submit_cluster(q["pos1"], q["pos2"], q["perm"], Jmax=q["Jmax"], scale=q["sigma"],
                                  nrot=q["nrot"])
    return srv.submit_periodic(q["pos1"], q["pos2"], q["box"], q["perm"], scale=q["sigma"],
                               nwave=q["nwave"], ndisps=q["ndisps"])


class ClockSampler(object):
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _oracle_sample(pairs, nthreads, budget_s, per_call=None):
    """The oracle (CPU restatement of the reference algorithm) over a bounded
    sample of the workload, in calls of per_call pairs (default 8 per thread,
    so that the threads' dynamic pair queue stays balanced): at least one call,
    then more until budget_s of CPU time has passed.  Returns (pairs/s, pairs
    done, seconds, per_call)."""
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as O
    sample = [dict(pos1=p[0], pos2=p[1], perm=p[2], Jmax=p[3], sigma=0.3) for p in pairs]
    per_call = per_call or 8 * nthreads
    done, dt = 0, 0.0
    while True:
        chunk = [sample[(done + i) % len(sample)] for i in range(per_call)]
        t0 = time.time()
        O.cluster_align_many(chunk, nrot=10, invert=True, cutoff=True, nthreads=nthreads)
        dt += time.time() - t0
        done += per_call
        if dt >= budget_s:
            break
    return done / dt, done, dt, per_call


def cpu_baseline_run(pairs, nthreads, budget_s=10.0):
    """CPU baseline of the oracle port beside the GPU line (same sampler as
    the reference arm)."""
    v, done, dt, _ = _oracle_sample(pairs, nthreads, budget_s)
    return v, done, dt


def run_reference(args, pairs):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    nthreads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import oracle as O
    O.build()
    sample = [dict(pos1=p[0], pos2=p[1], perm=p[2], Jmax=p[3], sigma=0.3) for p in pairs]
    for w in range(args.warmup):
        O.cluster_align_many(sample[:nthreads], nthreads=nthreads)
    # each step: one call of 8 pairs per thread (the same sampler as the
    # in-arm baseline), walking through the workload
    times = []
    per_step = 8 * nthreads
    for s in range(args.steps):
        v, done, dt, _ = _oracle_sample(pairs[(s * per_step) % len(pairs):] + pairs, nthreads, 0.0, per_step)
        times.append(dt)
    tot = sum(times)
    val = per_step * args.steps / tot
    line = {"metric": METRIC, "value": val, "unit": "pairs/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "sample_pairs_per_step": per_step,
                       "note": "CPU restatement of the reference Fortran cluster path (oracle/), "
                               "all host threads; the Fortran modules need gfortran/FFTW/LAPACK, "
                               "absent on this machine"},
            "cpu_baseline": {"value": val, "unit": "pairs/s", "cores": nthreads, "kind": "port",
                             "sample": "%d pairs per step of the same workload" % per_step},
            "e2e": {"value": val, "unit": "pairs/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--npairs", type=int, default=4096)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="time eager launches instead of graph replay")
    ap.add_argument("--no-tensor-cores", action="store_true",
                    help="mixed form: Wigner contraction on CUDA cores instead of tcgen05")
    ap.add_argument("--plain-sample", type=int, default=32)
    ap.add_argument("--c3-pairs", type=int, default=64, help="0 skips the large-bandwidth study")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-duration", type=float, default=60.0, help="0 skips the served stream")
    ap.add_argument("--serve-fp64-rate", type=float, default=200.0,
                    help="arrival rate of the plain FP64 served stream (its capacity is far lower)")
    ap.add_argument("--serve-fp64-duration", type=float, default=10.0, help="0 skips the FP64 served stream")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    ws, rank, local = dist_env()
    pairs = make_workload(args.npairs, seed_offset=rank * 1000003)
    if args.impl == "reference":
        run_reference(args, pairs)
        return
    dist = init_dist(ws)

    import fastoverlap_gb300 as F
    from fastoverlap_gb300.batch import ClusterBatch

    ctx = F.Context(device=local, precision=args.precision, profile=True,
                    tensor_cores=not args.no_tensor_cores)
    pos1 = [p[0] for p in pairs]
    pos2 = [p[1] for p in pairs]
    perms = [p[2] for p in pairs]
    jm = [p[3] for p in pairs]
    batch = ClusterBatch(ctx, pos1, pos2, perms, Jmax=jm, scale=0.3, nrot=10, invert=True).plan()

    for _ in range(args.warmup):
        batch.plan_run()
        batch.plan_wait()
    # per-kernel breakdown from one eager step (CUDA events between launches)
    ctx.profile_reset()
    ctx.flush_l2(512 << 20)
    batch.plan_run()
    batch.plan_wait()
    prof = ctx.profile()
    if not args.no_graph:
        # the timed steps replay the plan as one captured CUDA graph (this run
        # goes eagerly and captures it)
        batch.plan_graph(True)
        batch.plan_run()
        batch.plan_wait()
    clocks = ClockSampler(local)
    barrier(dist)
    ctx.synchronize()
    clocks.start()
    step_ms = []
    for s in range(args.steps):
        ctx.flush_l2(512 << 20)
        ctx.record(0)
        batch.plan_run()
        ctx.record(1)
        batch.plan_wait()
        step_ms.append(ctx.elapsed_ms(0, 1))
    ctx.synchronize()
    barrier(dist)
    clk = clocks.stop()
    res = batch.plan_results(with_coords=True)
    tot_ms = allmax(dist, sum(step_ms))
    value = args.npairs * ws * args.steps / (tot_ms / 1000.0)

    # end to end through the public batch API with host buffers: inputs and
    # outputs in page-locked host memory (the caller's arrays registered once)
    e2e_times = []
    eb = ClusterBatch(ctx, pos1, pos2, perms, Jmax=jm, scale=0.3, nrot=10, invert=True).pin()
    for s in range(max(2, min(args.steps, 3))):
        barrier(dist)
        t0 = time.time()
        eb.run()
        e2e_times.append(time.time() - t0)
    e2e_s = allmax(dist, statistics.median(e2e_times))
    h2d = eb.pk.h2d_bytes + len(eb.desc)
    d2h = res["result"].nbytes + 3 * 8 * eb.pk.natoms_total + 4 * eb.pk.natoms_total

    if rank != 0:
        barrier(dist)
        return

    # plain FP64 forms and accuracy of the mixed form
    cfg_extra = {}
    # the plain FP64 form batched, timed exactly as `value`: resident plan,
    # W warm-up runs, K timed runs by CUDA events, L2 flushed before each
    ctx64 = F.Context(device=local, precision="fp64", profile=True)
    b64 = ClusterBatch(ctx64, pos1, pos2, perms, Jmax=jm, scale=0.3, nrot=10, invert=True).plan()
    for _ in range(args.warmup):
        b64.plan_run()
        b64.plan_wait()
    ctx64.profile_reset()
    ms64 = []
    for _ in range(args.steps):
        ctx64.flush_l2(512 << 20)
        ctx64.record(0)
        b64.plan_run()
        ctx64.record(1)
        b64.plan_wait()
        ms64.append(ctx64.elapsed_ms(0, 1))
    r64 = b64.plan_results(with_coords=True)
    cfg_extra["fp64_batched_pairs_per_s"] = args.npairs * args.steps / (sum(ms64) / 1000.0)
    cfg_extra["fp64_batched_kernel_ms_per_step"] = {k: v[0] / max(1, v[1]) for k, v in ctx64.profile().items()}
    cfg_extra["mixed_over_fp64_batched"] = value / cfg_extra["fp64_batched_pairs_per_s"]
    ns = min(args.plain_sample, args.npairs)
    tp = time.time()
    for k in range(ns):
        ClusterBatch(ctx64, [pos1[k]], [pos2[k]], [perms[k]], Jmax=jm[k], scale=0.3, nrot=10,
                     invert=True).run()
    tp = time.time() - tp
    plain = ns / tp
    cfg_extra["plain_fp64_single_pair_pairs_per_s"] = plain
    cfg_extra["speedup_vs_plain_fp64"] = value / plain
    ok = (res["status"] == 0) & (r64["status"] == 0)
    rel = np.abs(res["dist"][ok] - r64["dist"][ok]) / np.maximum(r64["dist"][ok], 1e-300)
    same = [np.array_equal(a, b) for a, b, o in zip(res["perm"], r64["perm"], ok) if o]
    cfg_extra["mixed_vs_fp64_max_rel_dist"] = float(rel.max()) if len(rel) else None
    cfg_extra["mixed_vs_fp64_frac_rel_le_1e-5"] = float(np.mean(rel <= 1e-5)) if len(rel) else None
    cfg_extra["mixed_vs_fp64_identical_perm_frac"] = float(np.mean(same)) if same else None
    cfg_extra["pairs_failed"] = int((~ok).sum())
    per_pair_ms = sorted(step_ms)
    cfg_extra["step_ms_p50"] = float(np.percentile(per_pair_ms, 50))
    cfg_extra["step_ms_p99"] = float(np.percentile(per_pair_ms, 99))

    # roofline of the dominant kernel (live CUDA-event times of the timed steps)
    peaks_file = os.path.join(HERE, "MEASURED_PEAKS.json")
    try:
        pk = json.load(open(peaks_file))
        hbm = float(pk["hbm_gbs"])
        peak_src = "measured"
    except Exception:
        hbm = 6800.0
        peak_src = "fallback"
    kern = {k: v for k, v in prof.items() if k not in ("memset",)}
    top = max(kern, key=lambda k: kern[k][0])
    top_ms = kern[top][0] / max(1, kern[top][1])
    tsz = 4 if args.precision == "mixed" else 8
    r = res["result"]
    G = np.array([2 * (j + 1) for j in jm], dtype=np.float64)
    if top == "findpeaks":
        # per orientation: one initial read of the grid, then per fitted peak a
        # subtraction pass (read + write) and an argmax/sum pass (read)
        byts = float(np.sum((2 + 3 * r["ncand"]) * G ** 3 * tsz))
    elif top == "refine":
        # per candidate and iteration, 24 bytes per entry of each species'
        # distance matrix (all columns, or the 60 nearest), as the reference
        # forms it in FP64 with its column indices; the winner's iteration
        # count stands for every candidate of the pair
        nsz = [np.array([len(g) for g in p]) for p in perms]
        per_iter = np.array([float(np.sum(n * np.minimum(n, 60) * 24)) for n in nsz])
        byts = float(np.sum(per_iter * np.maximum(r["niter"], 1) * r["ncand"]))
    else:
        byts = float(np.sum(2 * 2 * G ** 3 * tsz))
    achieved = byts / (top_ms / 1000.0) / 1e9
    # DRAM bytes (read + write) the kernel moves, from an ncu capture of a
    # 256-pair case of this workload, scaled by the units of the step:
    # refinement 1.04 KB per candidate (its data stays on chip and in L2)
    traffic = None
    if top == "refine":
        traffic = 1.04e3 * float(np.sum(r["ncand"]))
    roof = {"kernel": top, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": traffic, "peak_source": peak_src,
            "kernel_ms_per_launch": top_ms,
            "kernel_share": kern[top][0] / sum(v[0] for v in kern.values())}
    cfg_extra["candidates_per_step"] = int(np.sum(r["ncand"]))
    if top == "refine" and REFINE_INST_PER_CAND:
        # The refinement is bound by issue latency along each warp's sequential
        # assignment steps (ncu: 0.2 eligible warps per scheduler cycle, `wait`
        # stalls first, 0.6 KB of DRAM traffic per candidate), so its roofline
        # is the issue-slot one: warp instructions issued per second against
        # one per scheduler per cycle.  Instructions of one run of this
        # workload's plan, from an ncu capture of its bucket launches
        # (smsp__inst_executed.sum), scaled by the step's candidates; the
        # HBM model above is kept as hbm_model.
        import torch
        sms = torch.cuda.get_device_properties(0).multi_processor_count
        mhz = float(pk.get("sm_max_mhz", 2070.0)) if peak_src == "measured" else 2070.0
        peak_i = sms * 4 * mhz * 1e6
        inst = REFINE_INST_PER_CAND * float(np.sum(r["ncand"]))
        ach_i = inst / (top_ms / 1000.0)
        hbm_model = {k: roof[k] for k in ("bound", "achieved", "peak", "unit", "frac")}
        roof.update({"bound": "issue", "achieved": ach_i / 1e9, "peak": peak_i / 1e9,
                     "unit": "G warp-instructions/s", "frac": ach_i / peak_i,
                     "peak_source": "%d SMs x 4 schedulers x %.0f MHz (one warp instruction per scheduler "
                                    "per cycle)" % (sms, mhz),
                     "hbm_model": hbm_model})
    launches = batch.plan_launches() * args.steps
    chunk, group = batch.plan_tile_shape()
    if chunk:
        cfg_extra["tc_tile_shape"] = {"wigner_mm_per_cta": chunk, "fft_pairs_per_block": group,
                                      "picked_by": "autotuner (timed per plan shape, cached per context)"}

    if args.c3_pairs > 0:
        try:
            cfg_extra["precision_study_c3"] = c3_run(args.c3_pairs)
        except Exception as e:   # reported, never required
            cfg_extra["precision_study_c3"] = {"error": str(e)}

    if args.serve_duration > 0:
        try:
            cfg_extra["serving"] = serve_run(args.serve_rate, args.serve_duration, args.precision)
        except Exception as e:   # reported, never required
            cfg_extra["serving"] = {"error": str(e)}
    if args.serve_fp64_duration > 0 and args.precision == "mixed":
        try:
            sv = serve_run(args.serve_fp64_rate, args.serve_fp64_duration, "fp64")
            cfg_extra["serving_fp64"] = sv
            if "completed_per_s" in cfg_extra.get("serving", {}):
                cfg_extra["serving_mixed_over_fp64_completed"] = (cfg_extra["serving"]["completed_per_s"] /
                                                                   sv["completed_per_s"])
        except Exception as e:   # reported, never required
            cfg_extra["serving_fp64"] = {"error": str(e)}

    cpu = None
    if not args.no_cpu_baseline:
        try:
            nth = os.cpu_count() or 1
            v, done, dt = cpu_baseline_run(pairs, nth)
            cpu = {"value": v, "unit": "pairs/s", "cores": nth, "kind": "port",
                   "sample": "%d pairs of the same workload in %.1f s" % (done, dt)}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "pairs/s", "cores": 0, "kind": "port",
                   "sample": "failed: %s" % e}

    line = {"metric": METRIC, "value": value, "unit": "pairs/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64 (mixed)" if args.precision == "mixed" else "f64",
            "data": "synthetic",
            "config": dict({"workload": WORKLOAD, "npairs_per_gpu": args.npairs,
                            "precision": args.precision, "l2": "flushed (512 MiB write) between steps",
                            "launch": ("eager launches" if args.no_graph else
                                       "one CUDA-graph replay of the plan per step (kernel breakdown from an "
                                       "eager step)"),
                            "kernel_ms_per_step": {k: v[0] / max(1, v[1]) for k, v in kern.items()}},
                           **cfg_extra),
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": args.npairs * ws / e2e_s, "unit": "pairs/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "clocks": clk, "gpu_launches": int(launches)}
    print(json.dumps(line), flush=True)
    barrier(dist)


if __name__ == "__main__":
    main()
