// fo_server.cu -- serving: alignment requests admitted as they arrive.
//
// Host code over the public C ABI.  Requests are copied into the server at
// submission (validated first, so a bad request never reaches a batch).
// Several worker threads each own a context (the caller's and contexts
// created with its options), so their plans run on separate streams: the
// long tail of one batch -- a few large pairs still refining -- overlaps the
// next batch.  A free worker takes the pending requests in arrival order
// (continuous batching, at most max_batch), splits them by kind, and runs each
// kind as one resident plan (upload, the whole pipeline, download).  Device
// memory comes from each context's block pool, so a steady stream allocates
// nothing.  The HBM budget is shared evenly by the workers; a plan larger than
// a worker's share is split in halves until it fits, and a request that does
// not fit alone completes with FO_ERR_OOM_BUDGET.  Latency is measured from
// submission to completion on the host's steady clock.
#include "../../include/fastoverlap_gb300.h"
#include "fo_kernels.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    int64_t ticket = 0;
    fo_request r{};
    std::vector<double> pos1, pos2;
    std::vector<int> perm, gsz;
    Clock::time_point t_submit;
    fo_status status = FO_OK;
    fo_pair_result res{};
    std::vector<double> aligned;
    std::vector<int> permbest;
};

using ReqP = std::unique_ptr<Req>;

// Latency percentiles from a histogram with bins 1% wide on a log scale
// (1 microsecond up to about 6 hours): bounded memory whatever the run
// length; a percentile is reported as its bin's geometric centre, within
// 0.5% of the exact value.
struct LatencyHist {
    static constexpr int kBins = 2200;
    static constexpr double kLo = 1e-3, kRatio = 1.01;
    std::vector<int64_t> bins = std::vector<int64_t>(kBins, 0);
    int64_t count = 0;
    double max_ms = 0.0;
    void add(double ms) {
        int b = ms > kLo ? (int)std::floor(std::log(ms / kLo) / std::log(kRatio)) : 0;
        b = std::min(std::max(b, 0), kBins - 1);
        ++bins[b];
        ++count;
        max_ms = std::max(max_ms, ms);
    }
    double pct(double q) const {   // nearest rank
        int64_t k = (int64_t)std::ceil(q * count), acc = 0;
        if (k < 1) k = 1;
        for (int b = 0; b < kBins; ++b) {
            acc += bins[b];
            if (acc >= k) return std::min(kLo * std::pow(kRatio, b + 0.5), max_ms);
        }
        return max_ms;
    }
};

// The checks the plan builders make, without a context (bounds as there).
fo_status validate(const fo_request &q) {
    if (q.kind != FO_KIND_CLUSTER && q.kind != FO_KIND_BULK) return FO_ERR_BAD_ARGS;
    if (q.natoms < 1 || q.natoms > 2000 || q.ngroups < 1) return FO_ERR_BAD_ARGS;
    if (!q.pos1 || !q.pos2 || !q.perm || !q.group_sizes) return FO_ERR_BAD_ARGS;
    long long tot = 0;
    for (int g = 0; g < q.ngroups; ++g) {
        if (q.group_sizes[g] < 0) return FO_ERR_BAD_ARGS;
        tot += q.group_sizes[g];
    }
    if (tot != q.natoms) return FO_ERR_BAD_ARGS;
    std::vector<char> seen(q.natoms, 0);
    for (int s = 0; s < q.natoms; ++s) {
        const int a = q.perm[s];
        if (a < 0 || a >= q.natoms || seen[a]) return FO_ERR_BAD_ARGS;
        seen[a] = 1;
    }
    for (int k = 0; k < 3 * q.natoms; ++k)
        if (!std::isfinite(q.pos1[k]) || !std::isfinite(q.pos2[k])) return FO_ERR_BAD_ARGS;
    if (q.kind == FO_KIND_CLUSTER) {
        if (q.jmax < 0 || q.jmax > 31 || q.nrot < 1 || q.nrot > 64) return FO_ERR_BAD_ARGS;
        if (std::isnan(q.sigma)) return FO_ERR_BAD_ARGS;
    } else {
        for (int k = 0; k < 3; ++k)
            if (!(q.box[k] > 0.0) || !std::isfinite(q.box[k])) return FO_ERR_BAD_ARGS;
        if (q.nrot > 64 || q.nfspace > 256) return FO_ERR_BAD_ARGS;
    }
    return FO_OK;
}

}  // namespace

struct fo_server {
    fo_ctx *user_ctx = nullptr;
    size_t user_budget = 0;
    std::vector<fo_ctx *> ctxs;   // one per worker; ctxs[0] is the caller's
    fo_server_opts o{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<ReqP> pending;
    std::unordered_map<int64_t, ReqP> finished;
    std::unordered_set<int64_t> outstanding;   // issued and not yet collected
    int64_t next_ticket = 1;
    bool stop = false;
    std::vector<std::thread> workers;
    // statistics
    int64_t n_sub = 0, n_done = 0, n_fail = 0, n_batches = 0, n_batched = 0;
    LatencyHist lat;
    double busy_ms = 0;

    void run_kind(fo_ctx *ctx, std::vector<Req *> &rs, int kind);
    void run_group(fo_ctx *ctx, Req **rs, int n, int kind);
    void loop(fo_ctx *ctx);
};

// One plan for n requests of one kind; halves on FO_ERR_OOM_BUDGET, and runs
// requests one by one when a plan is refused for a reason the submit-time
// checks did not catch (so that only the offending request fails).
void fo_server::run_group(fo_ctx *ctx, Req **rs, int n, int kind) {
    if (n <= 0) return;
    std::vector<double> p1, p2;
    std::vector<int> perm, gsz;
    std::vector<fo_cluster_pair> cd;
    std::vector<fo_bulk_pair> bd;
    int64_t atoms = 0, goff = 0;
    for (int i = 0; i < n; ++i) {
        const fo_request &q = rs[i]->r;
        if (kind == FO_KIND_CLUSTER) {
            fo_cluster_pair d{};
            d.natoms = q.natoms;
            d.ngroups = q.ngroups;
            d.jmax = q.jmax;
            d.nrot = q.nrot;
            d.invert = q.invert;
            d.sigma = q.sigma;
            d.coord_off = atoms;
            d.perm_off = atoms;
            d.group_off = goff;
            cd.push_back(d);
        } else {
            fo_bulk_pair d{};
            d.natoms = q.natoms;
            d.ngroups = q.ngroups;
            d.nwave = q.nwave;
            d.nfspace = q.nfspace;
            d.ndisps = q.nrot;
            d.sigma = q.sigma;
            for (int k = 0; k < 3; ++k) d.box[k] = q.box[k];
            d.coord_off = atoms;
            d.perm_off = atoms;
            d.group_off = goff;
            bd.push_back(d);
        }
        p1.insert(p1.end(), rs[i]->pos1.begin(), rs[i]->pos1.end());
        p2.insert(p2.end(), rs[i]->pos2.begin(), rs[i]->pos2.end());
        perm.insert(perm.end(), rs[i]->perm.begin(), rs[i]->perm.end());
        gsz.insert(gsz.end(), rs[i]->gsz.begin(), rs[i]->gsz.end());
        atoms += q.natoms;
        goff += q.ngroups;
    }
    fo_plan *pl = nullptr;
    fo_status s = kind == FO_KIND_CLUSTER
                      ? fo_cluster_plan_create(ctx, n, cd.data(), p1.data(), p2.data(), perm.data(), gsz.data(), 0, &pl)
                      : fo_bulk_plan_create(ctx, n, bd.data(), p1.data(), p2.data(), perm.data(), gsz.data(), 0, &pl);
    if (s != FO_OK) {
        if (n > 1) {
            if (s == FO_ERR_OOM_BUDGET) {
                run_group(ctx, rs, n / 2, kind);
                run_group(ctx, rs + n / 2, n - n / 2, kind);
            } else {
                for (int i = 0; i < n; ++i) run_group(ctx, rs + i, 1, kind);
            }
        } else {
            rs[0]->status = s;
            rs[0]->res.status = s;
        }
        return;
    }
    std::vector<fo_pair_result> res(n);
    std::vector<double> al(3 * (size_t)atoms);
    std::vector<int> pb((size_t)atoms);
    s = fo_plan_run(pl);
    if (s == FO_OK) s = fo_plan_wait(pl);
    if (s == FO_OK) s = fo_plan_results(pl, al.data(), pb.data(), res.data());
    fo_plan_destroy(pl);
    int64_t off = 0;
    for (int i = 0; i < n; ++i) {
        Req *r = rs[i];
        const int na = r->r.natoms;
        if (s == FO_OK) {
            r->res = res[i];
            r->status = (fo_status)res[i].status;
            r->aligned.assign(al.begin() + 3 * off, al.begin() + 3 * (off + na));
            r->permbest.assign(pb.begin() + off, pb.begin() + off + na);
        } else {
            r->status = s;
            r->res.status = s;
        }
        off += na;
    }
}

void fo_server::run_kind(fo_ctx *ctx, std::vector<Req *> &rs, int kind) {
    std::vector<Req *> sel;
    for (Req *r : rs)
        if (r->r.kind == kind) sel.push_back(r);
    run_group(ctx, sel.data(), (int)sel.size(), kind);
}

void fo_server::loop(fo_ctx *ctx) {
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv_work.wait(lk, [&] { return stop || !pending.empty(); });
        if (pending.empty() && stop) break;
        if (o.max_wait_ms > 0 && (int)pending.size() < o.max_batch && !stop)
            cv_work.wait_for(lk, std::chrono::duration<double, std::milli>(o.max_wait_ms),
                             [&] { return stop || (int)pending.size() >= o.max_batch; });
        std::vector<ReqP> batch;
        while (!pending.empty() && (int)batch.size() < o.max_batch) {
            batch.push_back(std::move(pending.front()));
            pending.pop_front();
        }
        lk.unlock();
        const Clock::time_point t0 = Clock::now();
        std::vector<Req *> rs;
        for (auto &b : batch) rs.push_back(b.get());
        run_kind(ctx, rs, FO_KIND_CLUSTER);
        run_kind(ctx, rs, FO_KIND_BULK);
        const Clock::time_point t1 = Clock::now();
        lk.lock();
        busy_ms += std::chrono::duration<double, std::milli>(t1 - t0).count();
        ++n_batches;
        n_batched += (int64_t)batch.size();
        for (auto &b : batch) {
            lat.add(std::chrono::duration<double, std::milli>(t1 - b->t_submit).count());
            ++n_done;
            if (b->status != FO_OK) ++n_fail;
            const int64_t t = b->ticket;
            finished[t] = std::move(b);
        }
        cv_done.notify_all();
    }
}

extern "C" {

fo_status fo_server_create(fo_ctx *ctx, const fo_server_opts *opts, fo_server **out) {
    if (!ctx || !out) return FO_ERR_BAD_ARGS;
    *out = nullptr;
    fo_server *s = new fo_server();
    if (opts) s->o = *opts;
    if (s->o.max_batch <= 0) s->o.max_batch = 4096;
    if (s->o.max_queue <= 0) s->o.max_queue = 1 << 20;
    if (s->o.max_wait_ms < 0) s->o.max_wait_ms = 0;
    if (s->o.workers <= 0) s->o.workers = 2;
    fo_opts co = fo::ctx_opts(ctx);
    s->user_ctx = ctx;
    s->user_budget = co.hbm_budget_bytes;
    const size_t share = co.hbm_budget_bytes / (size_t)s->o.workers;
    if (co.hbm_budget_bytes) co.hbm_budget_bytes = share ? share : 1;
    s->ctxs.push_back(ctx);
    for (int w = 1; w < s->o.workers; ++w) {
        fo_ctx *c = nullptr;
        if (fo_ctx_create(&co, &c) != FO_OK) {
            for (size_t k = 1; k < s->ctxs.size(); ++k) fo_ctx_destroy(s->ctxs[k]);
            delete s;
            return FO_ERR_CUDA;
        }
        s->ctxs.push_back(c);
    }
    for (fo_ctx *c : s->ctxs) fo::ctx_set_budget(c, co.hbm_budget_bytes);
    for (fo_ctx *c : s->ctxs) s->workers.emplace_back([s, c] { s->loop(c); });
    *out = s;
    return FO_OK;
}

fo_status fo_server_submit(fo_server *srv, const fo_request *req, int64_t *ticket) {
    if (!srv || !req || !ticket) return FO_ERR_BAD_ARGS;
    fo_status v = validate(*req);
    if (v) return v;
    ReqP r(new Req());
    r->r = *req;
    const int n = req->natoms;
    r->pos1.assign(req->pos1, req->pos1 + 3 * (size_t)n);
    r->pos2.assign(req->pos2, req->pos2 + 3 * (size_t)n);
    r->perm.assign(req->perm, req->perm + n);
    r->gsz.assign(req->group_sizes, req->group_sizes + req->ngroups);
    r->r.pos1 = r->r.pos2 = nullptr;
    r->r.perm = r->r.group_sizes = nullptr;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        if (srv->stop) return FO_ERR_BAD_ARGS;
        if ((int64_t)srv->pending.size() >= srv->o.max_queue) return FO_ERR_QUEUE_FULL;
        r->ticket = srv->next_ticket++;
        *ticket = r->ticket;
        srv->outstanding.insert(r->ticket);
        ++srv->n_sub;
        srv->pending.push_back(std::move(r));
    }
    srv->cv_work.notify_one();
    return FO_OK;
}

static fo_status take_result(fo_server *srv, int64_t ticket, fo_pair_result *result, double *aligned,
                             int *permbest) {
    // caller holds srv->mu
    auto it = srv->finished.find(ticket);
    if (it == srv->finished.end()) return FO_ERR_NOT_READY;
    Req *r = it->second.get();
    if (result) *result = r->res;
    if (aligned && !r->aligned.empty()) std::copy(r->aligned.begin(), r->aligned.end(), aligned);
    if (permbest && !r->permbest.empty()) std::copy(r->permbest.begin(), r->permbest.end(), permbest);
    const fo_status s = r->status;
    srv->finished.erase(it);
    srv->outstanding.erase(ticket);
    srv->cv_done.notify_all();   // a second waiter on this ticket returns FO_ERR_BAD_ARGS
    return s;
}

fo_status fo_server_poll(fo_server *srv, int64_t ticket, fo_pair_result *result, double *aligned,
                         int *permbest) {
    if (!srv || ticket <= 0) return FO_ERR_BAD_ARGS;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (!srv->outstanding.count(ticket)) return FO_ERR_BAD_ARGS;   // never issued, or collected
    return take_result(srv, ticket, result, aligned, permbest);
}

fo_status fo_server_wait(fo_server *srv, int64_t ticket, double timeout_ms, fo_pair_result *result,
                         double *aligned, int *permbest) {
    if (!srv || ticket <= 0) return FO_ERR_BAD_ARGS;
    std::unique_lock<std::mutex> lk(srv->mu);
    if (!srv->outstanding.count(ticket)) return FO_ERR_BAD_ARGS;   // never issued, or collected
    // ready once finished, or when another caller collected it meanwhile
    auto ready = [&] { return srv->finished.count(ticket) > 0 || !srv->outstanding.count(ticket); };
    if (timeout_ms < 0) {
        srv->cv_done.wait(lk, ready);
    } else if (!srv->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
        return FO_ERR_TIMEOUT;
    }
    if (!srv->outstanding.count(ticket)) return FO_ERR_BAD_ARGS;
    return take_result(srv, ticket, result, aligned, permbest);
}

fo_status fo_server_stats_get(fo_server *srv, fo_server_stats *st) {
    if (!srv || !st) return FO_ERR_BAD_ARGS;
    std::lock_guard<std::mutex> lk(srv->mu);
    *st = fo_server_stats{};
    st->submitted = srv->n_sub;
    st->completed = srv->n_done;
    st->failed = srv->n_fail;
    st->batches = srv->n_batches;
    st->mean_batch = srv->n_batches ? (double)srv->n_batched / srv->n_batches : 0.0;
    st->busy_ms = srv->busy_ms;
    if (srv->lat.count) {
        st->latency_p50_ms = srv->lat.pct(0.50);
        st->latency_p99_ms = srv->lat.pct(0.99);
        st->latency_max_ms = srv->lat.max_ms;
    }
    return FO_OK;
}

void fo_server_destroy(fo_server *srv) {
    if (!srv) return;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    for (auto &w : srv->workers)
        if (w.joinable()) w.join();
    for (size_t k = 1; k < srv->ctxs.size(); ++k) fo_ctx_destroy(srv->ctxs[k]);
    fo::ctx_set_budget(srv->user_ctx, srv->user_budget);   // the caller's context as it was
    delete srv;
}

}  // extern "C"
