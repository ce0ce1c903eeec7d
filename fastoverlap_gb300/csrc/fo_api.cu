// fo_api.cu -- the C ABI (include/fastoverlap_gb300.h): context, Wigner-table
// cache, batch plans (validation, device layout, upload), pipeline launch
// and result download, plus the Fortran-style single-pair entry points.
#include "../../include/fastoverlap_gb300.h"
#include "fo_common.cuh"
#include "fo_kernels.h"

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <numeric>
#include <tuple>
#include <string>
#include <thread>
#include <vector>

#include "fo_refine.cuh"

namespace {

constexpr int kMaxAtoms = 2000;  // refinement keeps two float4 copies + 3 index arrays on chip
constexpr int kMaxJmax = 31;     // SO(3) grid <= 64^3 (two 64x64 complex slices on chip)
constexpr int kMaxNrot = 64;
constexpr int kMaxM = 256;

int fastlen(int n) {
    if (n <= 1) return 1;
    for (int m = n;; ++m) {
        int k = m;
        while (k % 2 == 0) k /= 2;
        while (k % 3 == 0) k /= 3;
        while (k % 5 == 0) k /= 5;
        if (k == 1) return m;
    }
}

const int kNumKernels = 17;
const char *kKernelNames[kNumKernels] = {
    "sph_center", "sph_ylm",    "sph_radial", "sph_coeff", "isoft",      "findpeaks",
    "refine",     "select",     "bulk_prep",  "bulk_sf",   "bulk_fft",   "memset",
    "wigner",     "h2d",        "d2h",        "other",     "wigner_tc"};
enum KId { K_CENTER, K_YLM, K_RADIAL, K_COEFF, K_ISOFT, K_PEAKS, K_REFINE, K_SELECT, K_BPREP,
           K_BSF, K_BFFT, K_MEMSET, K_WIGNER, K_H2D, K_D2H, K_OTHER, K_WTC };

}  // namespace

struct fo_ctx {
    fo_opts opts;
    cudaStream_t stream = nullptr;
    std::string err;
    std::map<int, std::pair<double *, float *>> dtab;
    int tc = 1;   // mixed form: Wigner contraction on the tensor cores
    int autotune = 1;   // pick the tensor-core tile shape per plan shape by timing
    std::map<std::string, std::pair<int, int>> tc_shapes;   // plan shape -> (chunk, FFT group)
    std::map<int, std::pair<float *, CUtensorMap>> dtc;   // per bandwidth: its tables in the MMA layout
    double **d_dtab64 = nullptr;
    float **d_dtab32 = nullptr;
    std::vector<int> permgroup, npermsize;
    int perm_natoms = 0;
    std::vector<int> bestperm;
    int ohcell = 0;   // COMMONS OHCELLT for fo_bulk_align
    double prof_ms[kNumKernels] = {0};
    int prof_n[kNumKernels] = {0};
    cudaEvent_t ev[64] = {};
    static constexpr int kAux = 16;   // one per refinement footprint class
    cudaStream_t aux[kAux] = {};
    cudaEvent_t fork = nullptr, join[kAux] = {};
    void *flush_buf = nullptr;
    size_t flush_bytes = 0;
    // device blocks of destroyed plans (at most kPoolMax, the largest kept),
    // handed to later plans that fit: repeated batches allocate nothing
    static constexpr int kPoolMax = 4;
    std::vector<std::pair<unsigned char *, size_t>> pool;
};

struct fo_plan {
    fo_ctx *ctx = nullptr;
    bool bulk = false, fp32 = false;
    int npairs = 0, nslots = 0, ncand = 0, ngroups = 0;
    int maxL = 0, maxG = 0, maxgroup = 0, maxn = 0;
    int index_base = 0;
    bool use_graph = false;  // runs after the first replay a captured CUDA graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int harm_n = -1;         // >= 0: harmonic-oscillator basis of this order
    size_t harm_d = 0;       // doubles of its radial overlap buffer
    std::vector<fo::PairDev> hp;
    std::vector<fo::GroupDev> hg;
    std::vector<long long> caller_off;  // caller's atom offset per pair
    unsigned char *dmem = nullptr;
    size_t dbytes = 0, block_bytes = 0;
    fo::SphBuffers sb{};
    fo::BulkBuffers bb{};
    fo::RefineBuffers rb{};
    size_t coef_bytes = 0, fgrid_bytes = 0;
    int *d_pstatus = nullptr, *d_npeaks = nullptr;
    void *d_coef = nullptr, *d_fgrid = nullptr;
    std::vector<cudaEvent_t> evs;
    std::vector<int> ev_kid;
    std::vector<fo::RefineBucket> buckets;
    bool tc = false;         // Wigner contraction on the tensor cores
    fo::TcBuffers tcb;
    std::vector<unsigned char> tc_meta;         // tiles, items, pair map (host copy, uploaded once)
    size_t tc_off_items = 0, tc_off_groups = 0;   // their offsets in tc_meta (tiles at 0)
    unsigned char *tc_meta_dev = nullptr;        // device copy (capacity for every shape tried)
    std::vector<fo::TcTile> tc_tiles;            // host tiles; tc_tile_t0[t]: first of its pairs in tc_order
    std::vector<int> tc_tile_t0, tc_order;
    int tc_chunk = 0, tc_group = 0;              // the tile shape in use
};

namespace {

fo_status set_err(fo_ctx *ctx, fo_status s, const char *fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return s;
}

fo_status cuda_check(fo_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return FO_OK;
    return set_err(ctx, FO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// ensure Wigner tables exist for every bandwidth in [1, maxbw] that is used
fo_status ensure_dtabs(fo_ctx *ctx, const std::vector<int> &bws) {
    int maxbw = 0;
    for (int b : bws) maxbw = std::max(maxbw, b);
    for (int bw : bws) {
        if (ctx->dtab.count(bw)) continue;
        int W = 2 * bw - 1;
        size_t n = (size_t)2 * bw * W * W * bw;
        double *d64 = nullptr;
        float *d32 = nullptr;
        fo_status s = cuda_check(ctx, cudaMalloc(&d64, n * sizeof(double)), "cudaMalloc(wigner)");
        if (s) return s;
        s = cuda_check(ctx, cudaMalloc(&d32, n * sizeof(float)), "cudaMalloc(wigner32)");
        if (s) { cudaFree(d64); return s; }
        fo::launch_wigner_table(bw, d64, d32, ctx->stream);
        ctx->dtab[bw] = {d64, d32};
    }
    // rebuild the device pointer tables indexed by bandwidth
    int cap = 65;
    std::vector<double *> h64(cap, nullptr);
    std::vector<float *> h32(cap, nullptr);
    for (auto &kv : ctx->dtab)
        if (kv.first < cap) { h64[kv.first] = kv.second.first; h32[kv.first] = kv.second.second; }
    if (!ctx->d_dtab64) {
        fo_status s = cuda_check(ctx, cudaMalloc(&ctx->d_dtab64, cap * sizeof(double *)), "cudaMalloc");
        if (s) return s;
        s = cuda_check(ctx, cudaMalloc(&ctx->d_dtab32, cap * sizeof(float *)), "cudaMalloc");
        if (s) return s;
    }
    fo_status s = cuda_check(ctx, cudaMemcpyAsync(ctx->d_dtab64, h64.data(), cap * sizeof(double *),
                                                  cudaMemcpyHostToDevice, ctx->stream), "copy");
    if (s) return s;
    s = cuda_check(ctx, cudaMemcpyAsync(ctx->d_dtab32, h32.data(), cap * sizeof(float *),
                                        cudaMemcpyHostToDevice, ctx->stream), "copy");
    if (s) return s;
    return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "wigner tables");
}

// the tensor-core layout of the Wigner tables of these bandwidths (after
// ensure_dtabs: built from the FP64 tables) and their tensor maps
fo_status ensure_tc_tables(fo_ctx *ctx, const std::vector<int> &bws) {
    for (int bw : bws) {
        if (ctx->dtc.count(bw)) continue;
        float *t = nullptr;
        fo_status s = cuda_check(ctx, cudaMalloc(&t, fo::tc_table_floats(bw) * sizeof(float)), "cudaMalloc(tc table)");
        if (s) return s;
        CUtensorMap map;
        if (!fo::tc_make_table(bw, ctx->dtab[bw].first, t, &map, ctx->stream)) {
            cudaFree(t);
            return set_err(ctx, FO_ERR_CUDA, "tensor-map encoder unavailable (driver entry point)");
        }
        ctx->dtc.emplace(bw, std::make_pair(t, map));
    }
    return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "tensor-core Wigner tables");
}

// f(i) for i < n on host threads, in chunks of 16 (serially for small n)
template <typename F>
void host_parallel(int n, const F &f) {
    const int nt = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 16u);
    if (n < 256 || nt <= 1) {
        for (int i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<int> next(0);
    auto work = [&] {
        for (int i0; (i0 = next.fetch_add(16)) < n;)
            for (int i = i0; i < std::min(n, i0 + 16); ++i) f(i);
    };
    std::vector<std::thread> th;
    try {
        for (int t = 1; t < nt; ++t) th.emplace_back(work);
    } catch (...) {   // no more threads: the ones started and this one finish the work
    }
    work();
    for (auto &x : th) x.join();
}

double centred_radius(const double *X, int n);

// The O(natoms) host work of plan creation for every pair, on host threads:
// the permutation groups (slot2orig at the pair's atom offset), finite
// coordinates, and (dmax != nullptr) the sum of both structures' centred
// radii.  bad[i] = 1 marks a pair that fails either check; the caller reports
// the first failing pair in pair order with check_groups' or its own message.
template <typename PairT>
void host_pair_checks(int npairs, const PairT *pairs, const double *pos1, const double *pos2, const int *perm,
                      const int *gsizes, int base, std::vector<long long> &aoff, std::vector<int> &s2o,
                      std::vector<char> &bad, std::vector<double> *dmax);

// validate the permutation groups of one pair and fill slot2orig
fo_status check_groups(fo_ctx *ctx, int i, int n, int ngroups, const int *perm,
                       const int *gsizes, int base, int *slot2orig) {
    if (ngroups < 1) return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: ngroups < 1", i);
    long long tot = 0;
    for (int g = 0; g < ngroups; ++g) {
        if (gsizes[g] < 0) return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: negative group size", i);
        tot += gsizes[g];
    }
    if (tot != n)
        return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: groups hold %lld atoms, natoms = %d", i, tot, n);
    std::vector<char> seen(n, 0);
    for (int s = 0; s < n; ++s) {
        int a = perm[s] - base;
        if (a < 0 || a >= n) return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: atom index %d out of range", i, perm[s]);
        if (seen[a]) return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: atom %d in two groups", i, perm[s]);
        seen[a] = 1;
        slot2orig[s] = a;
    }
    return FO_OK;
}

template <typename PairT>
void host_pair_checks(int npairs, const PairT *pairs, const double *pos1, const double *pos2, const int *perm,
                      const int *gsizes, int base, std::vector<long long> &aoff, std::vector<int> &s2o,
                      std::vector<char> &bad, std::vector<double> *dmax) {
    aoff.assign(npairs + 1, 0);
    for (int i = 0; i < npairs; ++i) aoff[i + 1] = aoff[i] + std::max(0, std::min(pairs[i].natoms, kMaxAtoms));
    s2o.assign((size_t)aoff[npairs], 0);
    bad.assign(npairs, 0);
    if (dmax) dmax->assign(npairs, 0.0);
    host_parallel(npairs, [&](int i) {
        const PairT &q = pairs[i];
        const int n = q.natoms;
        if (n < 1 || n > kMaxAtoms) return;   // reported by the scalar checks
        int *so = s2o.data() + aoff[i];
        const int *pm = perm + q.perm_off, *gs = gsizes + q.group_off;
        long long tot = 0;
        for (int g = 0; g < q.ngroups; ++g) {
            if (gs[g] < 0) { bad[i] = 1; return; }
            tot += gs[g];
        }
        if (q.ngroups < 1 || tot != n) { bad[i] = 1; return; }
        std::vector<char> seen(n, 0);
        for (int t = 0; t < n; ++t) {
            const int a = pm[t] - base;
            if (a < 0 || a >= n || seen[a]) { bad[i] = 1; return; }
            seen[a] = 1;
            so[t] = a;
        }
        const double *x1 = pos1 + 3 * q.coord_off, *x2 = pos2 + 3 * q.coord_off;
        for (int k = 0; k < 3 * n; ++k)
            if (!std::isfinite(x1[k]) || !std::isfinite(x2[k])) { bad[i] = 1; return; }
        if (dmax) (*dmax)[i] = centred_radius(x1, n) + centred_radius(x2, n);
    });
}

struct Carve {
    size_t off = 0;
    template <typename T> size_t take(size_t count) {
        size_t o = off;
        off += align256(count * sizeof(T));
        return o;
    }
};

void rec_event(fo_plan *pl, int kid) {
    if (!pl->ctx->opts.profile) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, pl->ctx->stream);
    pl->evs.push_back(e);
    pl->ev_kid.push_back(kid);
}

fo_status finish_plan_alloc(fo_ctx *ctx, fo_plan *pl, size_t bytes) {
    // the caller's budget bounds every plan; the automatic one (80% of the
    // free memory) only what still has to be allocated
    const size_t user = ctx->opts.hbm_budget_bytes;
    if (user && bytes > user)
        return set_err(ctx, FO_ERR_OOM_BUDGET, "plan needs %zu bytes, budget %zu", bytes, user);
    int best = -1;   // smallest pooled block that fits
    for (int k = 0; k < (int)ctx->pool.size(); ++k)
        if (ctx->pool[k].second >= bytes && (best < 0 || ctx->pool[k].second < ctx->pool[best].second)) best = k;
    if (best >= 0) {
        pl->dmem = ctx->pool[best].first;
        pl->block_bytes = ctx->pool[best].second;
        pl->dbytes = bytes;
        ctx->pool.erase(ctx->pool.begin() + best);
        return FO_OK;
    }
    if (!user) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        if (bytes > (size_t)(0.8 * fr))
            return set_err(ctx, FO_ERR_OOM_BUDGET, "plan needs %zu bytes, 80%% of free memory is %zu", bytes,
                           (size_t)(0.8 * fr));
    }
    fo_status s = cuda_check(ctx, cudaMalloc(&pl->dmem, bytes), "cudaMalloc(plan)");
    if (s) return s;
    pl->dbytes = pl->block_bytes = bytes;
    return FO_OK;
}

// 1: buckets of the mixed form with groups of more than 256 atoms run
// multi-warp blocks (helper warps for the neighbour lists)
#ifndef FO_REFINE_MW
#define FO_REFINE_MW 1
#endif

constexpr size_t kRefSmemCap = 96 * 1024;     // assignment arrays kept on chip up to this size
constexpr size_t kRefSplitCap = 120 * 1024;   // above it: only the working arrays on chip, up to this

struct RefAssign {
    size_t smem;
    long long lapstride;
    int ct64;
    int split;   // working arrays on chip, costs / neighbour lists in global scratch
    int mw;      // mixed form with groups for the multi-warp neighbour lists
};

// Shared-memory footprint of one refinement warp for a pair, and whether its
// assignment arrays fit on chip.  dmax bounds every atom-atom distance the
// refinement can meet; costs INT(d^2 1e6) below 2e9 are held in 32 bits.
// recomp: costs recomputed from FP32 coordinates instead of stored.
RefAssign ref_assign(int n, int maxg, bool fp32, bool recomp, double dmax) {
    RefAssign r;
    r.ct64 = (dmax * dmax * fo::kPScale >= 2.0e9) ? 1 : 0;
    r.mw = (fp32 && recomp && fo::ref_multiwarp(maxg)) ? 1 : 0;
    fo::RefLayout L;
    fo::ref_layout(n, maxg, fp32, r.ct64 ? 8 : 4, recomp, L);
    // Footprint classes, one launch each: the largest dynamic shared memory
    // with which k one-warp blocks stay resident on an SM (233472 bytes per
    // SM, 1 KB reserved per block, up to 640 bytes of the kernel's static
    // arrays: 528 in the multi-warp forms), k = 16 (the register limit of the
    // kernel) down to 1.  A finer class would not fit more warps on an SM.
    auto up = [](size_t b) {
        for (int k = 16; k >= 1; --k) {
            const size_t c = ((size_t)233472 / k - 1024 - 640) & ~(size_t)127;
            if (b <= c) return c;
        }
        return (b + 127) & ~(size_t)127;
    };
    r.split = 0;
    if (L.coord_end + L.lap_end <= kRefSmemCap) {
        r.smem = up(L.coord_end + L.lap_end);
        r.lapstride = 0;
    } else if (recomp && L.coord_end + L.lap_small <= kRefSplitCap) {
        // mixed form: the assignment's random-access arrays and the
        // neighbour-selection scratch stay on chip; the row-major neighbour
        // lists (read a row at a time) go to the candidate's global scratch.
        // (The FP64 form keeps its stored costs and everything else in global
        // scratch: its small on-chip part lets 16 warps share an SM, which
        // measured faster than the split's 5.)
        r.smem = up(L.coord_end + L.lap_small);
        r.lapstride = (long long)((L.lap_end + 255) & ~(size_t)255);
        r.split = 1;
    } else {
        r.smem = up(L.coord_end);
        r.lapstride = (long long)((L.lap_end + 255) & ~(size_t)255);
    }
    return r;
}

void build_buckets(fo_plan *pl, const std::vector<RefAssign> &ra, std::vector<int> &cand_list) {
    // within a class, heavier (more atoms) candidates first so the tail of
    // each launch is short; pairs of equal size keep their order
    std::vector<int> order(pl->hp.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return pl->hp[a].n > pl->hp[b].n; });
    // key: (footprint, 64-bit costs, multi-warp neighbour lists)
    std::map<std::tuple<size_t, int, int>, std::vector<int>> by;
    for (int i : order) {
        const fo::PairDev &P = pl->hp[i];
        auto &v = by[{ra[i].smem, ra[i].ct64, ra[i].mw}];
        for (int c = 0; c < P.norient * P.nrot; ++c) v.push_back(P.cand0 + c);
    }
    pl->buckets.clear();
    cand_list.clear();
    // largest footprint (the heaviest candidates) first: each class has its
    // own stream, and the longest launches start at once
    for (auto it = by.rbegin(); it != by.rend(); ++it) {
        auto &kv = *it;
        fo::RefineBucket b;
        b.offset = (int)cand_list.size();
        b.count = (int)kv.second.size();
        b.smem = std::get<0>(kv.first);
        b.ct64 = std::get<1>(kv.first);
        b.nw = (std::get<2>(kv.first) && FO_REFINE_MW) ? fo::refine_block_warps(pl->bulk, b.ct64, b.smem) : 1;
        cand_list.insert(cand_list.end(), kv.second.begin(), kv.second.end());
        pl->buckets.push_back(b);
    }
}

double centred_radius(const double *X, int n) {
    double c[3] = {0, 0, 0};
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < 3; ++k) c[k] += X[3 * j + k];
    double r2 = 0;
    for (int j = 0; j < n; ++j) {
        double s = 0;
        for (int k = 0; k < 3; ++k) {
            double t = X[3 * j + k] - c[k] / n;
            s += t * t;
        }
        r2 = std::max(r2, s);
    }
    return std::sqrt(r2);
}

void widen(const void *src, double *dst, size_t n, bool fp32) {
    if (fp32) {
        const float *f = (const float *)src;
        for (size_t i = 0; i < n; ++i) dst[i] = f[i];
    } else {
        memcpy(dst, src, n * sizeof(double));
    }
}

}  // namespace

extern "C" {

const char *fo_status_string(fo_status s) {
    switch (s) {
        case FO_OK: return "ok";
        case FO_ERR_BAD_ARGS: return "bad arguments";
        case FO_ERR_NO_PEAKS: return "no peaks found";
        case FO_ERR_LAP_FAILED: return "assignment failed";
        case FO_ERR_TIMEOUT: return "timeout";
        case FO_ERR_OOM_BUDGET: return "HBM budget exceeded";
        case FO_ERR_CUDA: return "CUDA error";
        case FO_ERR_UNIMPLEMENTED: return "unimplemented";
        case FO_ERR_QUEUE_FULL: return "queue full";
        case FO_ERR_NOT_READY: return "not ready";
    }
    return "unknown";
}

const char *fo_last_error(const fo_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

fo_status fo_ctx_create(const fo_opts *opts, fo_ctx **out) {
    if (!out) return FO_ERR_BAD_ARGS;
    *out = nullptr;
    fo_ctx *c = new fo_ctx();
    if (opts) c->opts = *opts;
    else {
        memset(&c->opts, 0, sizeof c->opts);
        c->opts.cutoff = 1;
    }
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        delete c;
        return FO_ERR_CUDA;
    }
    if (c->opts.device < 0 || c->opts.device >= ndev) { delete c; return FO_ERR_BAD_ARGS; }
    if (cudaSetDevice(c->opts.device) != cudaSuccess) { delete c; return FO_ERR_CUDA; }
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return FO_ERR_CUDA;
    }
    for (int a = 0; a < fo_ctx::kAux; ++a) {
        if (cudaStreamCreateWithFlags(&c->aux[a], cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&c->join[a], cudaEventDisableTiming) != cudaSuccess) {
            delete c;
            return FO_ERR_CUDA;
        }
    }
    if (cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming) != cudaSuccess) {
        delete c;
        return FO_ERR_CUDA;
    }
    fo::init_sph_tables();   // constant tables of this device (idempotent)
    if (cudaGetLastError() != cudaSuccess) { delete c; return FO_ERR_CUDA; }
    *out = c;
    return FO_OK;
}

void fo_ctx_destroy(fo_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->opts.device);
    cudaStreamSynchronize(ctx->stream);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    cudaFree(ctx->flush_buf);
    for (auto &b : ctx->pool) cudaFree(b.first);
    for (int a = 0; a < fo_ctx::kAux; ++a) {
        if (ctx->aux[a]) cudaStreamDestroy(ctx->aux[a]);
        if (ctx->join[a]) cudaEventDestroy(ctx->join[a]);
    }
    if (ctx->fork) cudaEventDestroy(ctx->fork);
    for (auto &kv : ctx->dtab) { cudaFree(kv.second.first); cudaFree(kv.second.second); }
    for (auto &kv : ctx->dtc) cudaFree(kv.second.first);
    cudaFree(ctx->d_dtab64);
    cudaFree(ctx->d_dtab32);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

fo_status fo_set_tensor_cores(fo_ctx *ctx, int on) {
    if (!ctx) return FO_ERR_BAD_ARGS;
    ctx->tc = on ? 1 : 0;
    return FO_OK;
}

fo_status fo_set_autotune(fo_ctx *ctx, int on) {
    if (!ctx) return FO_ERR_BAD_ARGS;
    ctx->autotune = on ? 1 : 0;
    return FO_OK;
}

fo_status fo_host_register(fo_ctx *ctx, void *ptr, size_t bytes) {
    if (!ctx || !ptr || !bytes) return set_err(ctx, FO_ERR_BAD_ARGS, "null buffer or zero size");
    cudaSetDevice(ctx->opts.device);
    return cuda_check(ctx, cudaHostRegister(ptr, bytes, cudaHostRegisterDefault), "cudaHostRegister");
}

fo_status fo_host_unregister(fo_ctx *ctx, void *ptr) {
    if (!ctx || !ptr) return set_err(ctx, FO_ERR_BAD_ARGS, "null buffer");
    cudaSetDevice(ctx->opts.device);
    return cuda_check(ctx, cudaHostUnregister(ptr), "cudaHostUnregister");
}

fo_status fo_plan_tile_shape(const fo_plan *pl, int *chunk, int *group) {
    if (!pl || !chunk || !group) return FO_ERR_BAD_ARGS;
    *chunk = pl->tc ? pl->tc_chunk : 0;
    *group = pl->tc ? pl->tc_group : 0;
    return FO_OK;
}

fo_status fo_set_precision(fo_ctx *ctx, int precision) {
    if (!ctx || (precision != FO_PREC_FP64 && precision != FO_PREC_MIXED)) return FO_ERR_BAD_ARGS;
    ctx->opts.precision = precision;
    return FO_OK;
}

// ---------------------------------------------------------------------------
static fo_status plan_common_alloc(fo_ctx *ctx, fo_plan *pl, const double *pos1, const double *pos2,
                                   const std::vector<int> &slot2orig, const std::vector<int> &slot2pair,
                                   const std::vector<int> &cand2pair, const std::vector<int> &cand_list,
                                   size_t ylm_n, size_t w_n,
                                   size_t coef_n, size_t grid_n, size_t fgrid_n, long long lap_total,
                                   size_t tc_meta_bytes = 0, size_t tc_s_floats = 0) {
    const size_t T = pl->fp32 ? 4 : 8;
    const int np = pl->npairs, ns = pl->nslots, nc = pl->ncand;
    Carve cv;
    size_t o_pairs = cv.take<fo::PairDev>(np), o_groups = cv.take<fo::GroupDev>(pl->ngroups);
    size_t o_s2o = cv.take<int>(ns), o_s2p = cv.take<int>(ns), o_c2p = cv.take<int>(nc);
    size_t o_clist = cv.take<int>(nc);
    size_t o_pos1 = cv.take<double>(3 * (size_t)ns), o_pos2 = cv.take<double>(3 * (size_t)ns);
    size_t o_xa = cv.take<double>(3 * (size_t)ns), o_xb = cv.take<double>(3 * (size_t)ns);
    size_t o_ra = cv.take<double>(ns), o_rb = cv.take<double>(ns);
    size_t o_ylmA = cv.take<char>(ylm_n * 2 * T), o_ylmB = cv.take<char>(ylm_n * 2 * T);
    size_t o_W = cv.take<char>(w_n * T);
    size_t o_coef = cv.take<char>(coef_n * 2 * T);
    size_t o_grid = cv.take<char>(grid_n * T);
    size_t o_fgrid = cv.take<char>(fgrid_n * 2 * T);
    size_t o_omax = cv.take<double>(2 * (size_t)np), o_peaks = cv.take<double>(3 * (size_t)nc);
    size_t o_npk = cv.take<int>(2 * (size_t)np), o_pst = cv.take<int>(np);
    size_t o_lap = cv.take<unsigned char>((size_t)lap_total);
    size_t candatoms = 0;
    for (auto &P : pl->hp) candatoms += (size_t)P.norient * P.nrot * P.n;
    size_t o_cdist = cv.take<double>(nc), o_cR = cv.take<double>(9 * (size_t)nc),
           o_cdisp = cv.take<double>(3 * (size_t)nc);
    size_t o_cxyz = cv.take<double>(3 * candatoms), o_cperm = cv.take<int>(candatoms);
    size_t o_cthr = cv.take<float>(pl->fp32 ? candatoms : 0);
    size_t o_b4 = cv.take<float4>(pl->fp32 ? (size_t)ns : 0), o_cscr = cv.take<int>(pl->fp32 ? 3 * candatoms : 0);
    size_t o_cnit = cv.take<int>(nc), o_cst = cv.take<int>(nc);
    size_t o_res = cv.take<fo_pair_result>(np), o_al = cv.take<double>(3 * (size_t)ns),
           o_pb = cv.take<int>(ns);
    size_t o_hd = cv.take<double>(pl->harm_d);
    size_t o_tcm = cv.take<unsigned char>(tc_meta_bytes), o_tcs = cv.take<float>(tc_s_floats),
           o_tce = cv.take<int>(tc_meta_bytes ? 1 : 0);
    fo_status s = finish_plan_alloc(ctx, pl, cv.off);
    if (s) return s;
    unsigned char *m = pl->dmem;
    auto P = [&](size_t o) { return (void *)(m + o); };
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(P(o_pairs), pl->hp.data(), np * sizeof(fo::PairDev), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(P(o_groups), pl->hg.data(), pl->ngroups * sizeof(fo::GroupDev), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(P(o_s2o), slot2orig.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(P(o_s2p), slot2pair.data(), ns * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(P(o_c2p), cand2pair.data(), nc * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(P(o_clist), cand_list.data(), nc * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(P(o_pos1), pos1, 3 * (size_t)ns * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(P(o_pos2), pos2, 3 * (size_t)ns * sizeof(double), cudaMemcpyHostToDevice, st);
    if (tc_meta_bytes) cudaMemcpyAsync(P(o_tcm), pl->tc_meta.data(), tc_meta_bytes, cudaMemcpyHostToDevice, st);
    s = cuda_check(ctx, cudaStreamSynchronize(st), "plan upload");
    if (s) return s;

    pl->sb.pairs = (const fo::PairDev *)P(o_pairs);
    pl->sb.groups = (const fo::GroupDev *)P(o_groups);
    pl->sb.slot2orig = (const int *)P(o_s2o);
    pl->sb.slot2pair = (const int *)P(o_s2p);
    pl->sb.pos1 = (const double *)P(o_pos1);
    pl->sb.pos2 = (const double *)P(o_pos2);
    pl->sb.xa = (double *)P(o_xa);
    pl->sb.xb = (double *)P(o_xb);
    pl->sb.ra = (double *)P(o_ra);
    pl->sb.rb = (double *)P(o_rb);
    pl->sb.ylmA = P(o_ylmA);
    pl->sb.ylmB = P(o_ylmB);
    pl->sb.W = P(o_W);
    pl->sb.coef = P(o_coef);
    pl->sb.grid = P(o_grid);
    pl->sb.npairs = np;
    pl->sb.ngroups = pl->ngroups;
    pl->sb.nslots = ns;
    pl->sb.maxL = pl->maxL;
    pl->sb.maxG = pl->maxG;
    pl->sb.maxgroup = pl->maxgroup;
    pl->sb.harm_n = pl->harm_n;
    pl->sb.hd = pl->harm_d ? (double *)P(o_hd) : nullptr;
    pl->d_coef = P(o_coef);
    pl->coef_bytes = coef_n * 2 * T;
    pl->d_fgrid = P(o_fgrid);
    pl->fgrid_bytes = fgrid_n * 2 * T;

    pl->bb.pairs = pl->sb.pairs;
    pl->bb.groups = pl->sb.groups;
    pl->bb.slot2orig = pl->sb.slot2orig;
    pl->bb.pos1 = pl->sb.pos1;
    pl->bb.pos2 = pl->sb.pos2;
    pl->bb.xa = pl->sb.xa;
    pl->bb.xb = pl->sb.xb;
    pl->bb.fgrid = P(o_fgrid);
    pl->bb.grid = P(o_grid);
    pl->bb.npairs = np;
    pl->bb.maxK = pl->maxL;
    pl->bb.maxM = pl->maxG;

    fo::RefineBuffers &r = pl->rb;
    r.pairs = pl->sb.pairs;
    r.groups = pl->sb.groups;
    r.slot2orig = pl->sb.slot2orig;
    r.cand2pair = (const int *)P(o_c2p);
    r.xa = pl->sb.xa;
    r.xb = pl->sb.xb;
    r.grid = P(o_grid);
    r.overlap_max = (double *)P(o_omax);
    r.peaks = (double *)P(o_peaks);
    r.npeaks = (int *)P(o_npk);
    r.pstatus = (int *)P(o_pst);
    r.lap = (unsigned char *)P(o_lap);
    r.cdist = (double *)P(o_cdist);
    r.cR = (double *)P(o_cR);
    r.cdisp = (double *)P(o_cdisp);
    r.cxyz = (double *)P(o_cxyz);
    r.cthr = (float *)P(o_cthr);
    r.b4 = (float4 *)P(o_b4);
    r.cscr = (int *)P(o_cscr);
    r.cperm = (int *)P(o_cperm);
    r.cniter = (int *)P(o_cnit);
    r.cstat = (int *)P(o_cst);
    r.results = P(o_res);
    r.aligned = (double *)P(o_al);
    r.permbest = (int *)P(o_pb);
    r.npairs = np;
    r.ncand = nc;
    r.maxG = pl->maxG;
    r.maxn = pl->maxn;
    r.cand_list = (const int *)P(o_clist);
    r.buckets = pl->buckets.data();
    r.nbuckets = (int)pl->buckets.size();
    r.fp32 = pl->fp32;
    r.recomp = pl->fp32;
    r.bulk = pl->bulk;
    pl->d_pstatus = r.pstatus;
    pl->d_npeaks = r.npeaks;
    if (tc_meta_bytes) {
        fo::TcBuffers &t = pl->tcb;
        unsigned char *mb = (unsigned char *)P(o_tcm);
        pl->tc_meta_dev = mb;
        t.tiles = (const fo::TcTile *)mb;
        t.items = (const fo::TcItem *)(mb + pl->tc_off_items);
        t.groups = (const fo::TcFftGroup *)(mb + pl->tc_off_groups);
        t.pairs = pl->sb.pairs;
        t.coef = pl->sb.coef;
        t.grid = pl->sb.grid;
        t.S = (float *)P(o_tcs);
        t.err = (int *)P(o_tce);
        t.npairs = np;
        t.maxG = pl->maxG;
    }
    return FO_OK;
}

// True when pair i's atoms start where pair i-1's end (the packed order the
// plans use), so the caller's coordinate arrays can be uploaded as they are
// and results downloaded straight into the caller's arrays.
extern "C++" {
template <typename PairT>
static bool packed_in_order(const PairT *pairs, int npairs) {
    long long off = 0;
    for (int i = 0; i < npairs; ++i) {
        if (pairs[i].coord_off != off || pairs[i].natoms < 0) return false;
        off += pairs[i].natoms;
    }
    return true;
}
}

// Tile shapes the autotuner tries: (m1, m2) combinations per contraction
// CTA and pairs per FFT block.
constexpr int kTcChunks[] = {16, 32, 64, 128};
constexpr int kTcGroups[] = {1, 2, 4};
constexpr int kTcTuneMinPairs = 256;   // smaller plans take the default shape untimed
constexpr int kTcChunkDefault = 64, kTcGroupDefault = 1;

// Tiles of the tensor-core contraction: the plan's pairs sorted by Jmax
// (stable), 64 per tile (fixed for the plan).  Returns the floats of the sum
// buffer S.
static size_t tc_plan_tiles(fo_plan *pl) {
    const int np = pl->npairs;
    pl->tc_order.resize(np);
    std::iota(pl->tc_order.begin(), pl->tc_order.end(), 0);
    std::stable_sort(pl->tc_order.begin(), pl->tc_order.end(),
                     [&](int a, int b) { return pl->hp[a].L < pl->hp[b].L; });
    const std::vector<int> &order = pl->tc_order;
    pl->tc_tiles.clear();
    pl->tc_tile_t0.clear();
    size_t sfl = 0;
    for (int a = 0; a < np;) {
        const int L = pl->hp[order[a]].L;
        int b = a;
        while (b < np && pl->hp[order[b]].L == L) ++b;
        const int G = 2 * (L + 1), W2 = (2 * L + 1) * (2 * L + 1);
        for (int t0 = a; t0 < b; t0 += fo::kTcTile) {
            fo::TcTile T{};
            T.L = L;
            T.npairs = std::min(fo::kTcTile, b - t0);
            T.s0 = (long long)sfl;
            for (int i = 0; i < T.npairs; ++i) T.coef0[i] = pl->hp[order[t0 + i]].coef0;
            sfl += 2ull * G * W2 * 2 * T.npairs;
            pl->tc_tiles.push_back(T);
            pl->tc_tile_t0.push_back(t0);
        }
        a = b;
    }
    pl->tc = true;
    return sfl;
}

// The work of one tile shape: contraction work items of `chunk` (m1, m2)
// combinations (launch groups of at most kTcMaxBuckets bandwidths) and FFT
// blocks of up to `group` pairs.  Fills pl->tc_meta (tiles, items, FFT
// groups), pl->tcb.launches, ngroups and fft_smem.
static void tc_plan_shape(fo_ctx *ctx, fo_plan *pl, int chunk, int group) {
    std::vector<fo::TcTile> tiles = pl->tc_tiles;
    std::vector<fo::TcItem> items;
    std::vector<fo::TcFftGroup> fgroups;
    size_t fsm = 0;
    std::vector<int> Ls;
    for (const auto &T : tiles) Ls.push_back(T.L);
    Ls.erase(std::unique(Ls.begin(), Ls.end()), Ls.end());
    pl->tcb.launches.clear();
    for (size_t g0 = 0; g0 < Ls.size(); g0 += fo::kTcMaxBuckets) {
        fo::TcLaunch lg{};
        lg.item0 = (int)items.size();
        lg.nrmax = 0;
        const size_t g1 = std::min(Ls.size(), g0 + fo::kTcMaxBuckets);
        for (size_t bi = g0; bi < g1; ++bi) {
            const int bw = Ls[bi] + 1;
            lg.maps.map[bi - g0] = ctx->dtc[bw].second;
            lg.maps.nr[bi - g0] = fo::tc_rows(bw);
            lg.nrmax = std::max(lg.nrmax, fo::tc_rows(bw));
            for (size_t t = 0; t < tiles.size(); ++t) {
                if (tiles[t].L != Ls[bi]) continue;
                tiles[t].bucket = (int)(bi - g0);
                const int W2 = (2 * Ls[bi] + 1) * (2 * Ls[bi] + 1);
                for (int m0 = 0; m0 < W2; m0 += chunk)
                    items.push_back(fo::TcItem{(int)t, m0, std::min(W2, m0 + chunk), 0});
            }
        }
        lg.nitems = (int)items.size() - lg.item0;
        pl->tcb.launches.push_back(lg);
    }
    for (size_t t = 0; t < tiles.size(); ++t) {
        const fo::TcTile &T = tiles[t];
        const int G = 2 * (T.L + 1), npg = fo::tc_fft_group(G, group);
        for (int q0 = 0; q0 < T.npairs; q0 += npg) {
            fo::TcFftGroup fg{};
            fg.s0 = T.s0;
            fg.L = T.L;
            fg.ntile = T.npairs;
            fg.p0 = q0;
            fg.npg = std::min(npg, T.npairs - q0);
            for (int q = 0; q < fg.npg; ++q) fg.pair[q] = pl->tc_order[pl->tc_tile_t0[t] + q0 + q];
            fgroups.push_back(fg);
        }
        fsm = std::max(fsm, fo::tc_fft_smem(G, npg));
    }
    const size_t bt = tiles.size() * sizeof(fo::TcTile);
    pl->tc_off_items = align256(bt);
    pl->tc_off_groups = pl->tc_off_items + align256(items.size() * sizeof(fo::TcItem));
    pl->tc_meta.assign(pl->tc_off_groups + fgroups.size() * sizeof(fo::TcFftGroup), 0);
    memcpy(pl->tc_meta.data(), tiles.data(), bt);
    memcpy(pl->tc_meta.data() + pl->tc_off_items, items.data(), items.size() * sizeof(fo::TcItem));
    memcpy(pl->tc_meta.data() + pl->tc_off_groups, fgroups.data(), fgroups.size() * sizeof(fo::TcFftGroup));
    pl->tcb.ngroups = (int)fgroups.size();
    pl->tcb.fft_smem = fsm;
    pl->tc_chunk = chunk;
    pl->tc_group = group;
}

// Device bytes of the tile metadata for the largest shape the autotuner tries.
static size_t tc_meta_capacity(fo_ctx *ctx, fo_plan *pl) {
    tc_plan_shape(ctx, pl, kTcChunks[0], 1);   // most items, most FFT groups
    return pl->tc_meta.size();
}

static fo_status tc_status(fo_plan *pl);

// Upload the tile metadata of the current shape and point the kernels at it.
static fo_status tc_upload_meta(fo_plan *pl) {
    fo::TcBuffers &t = pl->tcb;
    unsigned char *mb = pl->tc_meta_dev;
    t.tiles = (const fo::TcTile *)mb;
    t.items = (const fo::TcItem *)(mb + pl->tc_off_items);
    t.groups = (const fo::TcFftGroup *)(mb + pl->tc_off_groups);
    cudaMemcpyAsync(mb, pl->tc_meta.data(), pl->tc_meta.size(), cudaMemcpyHostToDevice, pl->ctx->stream);
    return cuda_check(pl->ctx, cudaStreamSynchronize(pl->ctx->stream), "tile metadata");
}

// The plan-shape key of the autotuner: the plan's distinct Jmax values and its
// pair count rounded up to a power of two.
static std::string tc_shape_key(const fo_plan *pl) {
    std::string k;
    int last = -1;
    for (const auto &T : pl->tc_tiles)
        if (T.L != last) { k += std::to_string(T.L) + ","; last = T.L; }
    int p2 = 1;
    while (p2 < pl->npairs) p2 *= 2;
    return k + "n" + std::to_string(p2);
}

// Pick the tensor-core tile shape of a plan.  Autotuner: for a plan shape
// not seen before (at least kTcTuneMinPairs pairs), compute the plan's
// coefficients once, then time the contraction and the FFT stage for every
// (chunk, group) of kTcChunks x kTcGroups with CUDA events (best of two
// runs each) and keep the fastest for this context; later plans of the same
// shape reuse it.  Smaller plans, and contexts with autotuning off, take the
// default shape.
static fo_status tc_tune(fo_ctx *ctx, fo_plan *pl) {
    int chunk = kTcChunkDefault, group = kTcGroupDefault;
    const std::string key = tc_shape_key(pl);
    bool tune = ctx->autotune && pl->npairs >= kTcTuneMinPairs;
    auto it = ctx->tc_shapes.find(key);
    if (it != ctx->tc_shapes.end()) {
        chunk = it->second.first;
        group = it->second.second;
        tune = false;
    }
    if (tune) {
        cudaStream_t st = ctx->stream;
        cudaMemsetAsync(pl->d_coef, 0, pl->coef_bytes, st);
        fo::launch_sph_center(pl->sb, st);
        fo::launch_sph_ylm(pl->sb, pl->fp32, st);
        fo::launch_sph_radial(pl->sb, pl->fp32, ctx->opts.cutoff, st);
        cudaMemsetAsync(pl->tcb.err, 0, sizeof(int), st);
        fo::launch_coef_tc(pl->sb, pl->tcb.err, st);
        fo_status s = cuda_check(ctx, cudaStreamSynchronize(st), "coefficients");
        if (!s) s = tc_status(pl);
        if (s) return s;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best = 3.0e38f;
        for (int c : kTcChunks)
            for (int g : kTcGroups) {
                tc_plan_shape(ctx, pl, c, g);
                s = tc_upload_meta(pl);
                if (s) break;
                float t = 3.0e38f;
                for (int rep = 0; rep < 2; ++rep) {
                    cudaMemsetAsync(pl->tcb.err, 0, sizeof(int), st);
                    cudaEventRecord(e0, st);
                    fo::launch_wigner_tc(pl->tcb, st);
                    fo::launch_isoft_tc(pl->tcb, st);
                    cudaEventRecord(e1, st);
                    s = cuda_check(ctx, cudaEventSynchronize(e1), "tile-shape timing");
                    if (!s) s = tc_status(pl);
                    if (s) break;
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    t = std::min(t, ms);
                }
                if (s) break;
                if (t < best) { best = t; chunk = c; group = g; }
            }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (s) return s;
        ctx->tc_shapes[key] = {chunk, group};
    }
    tc_plan_shape(ctx, pl, chunk, group);
    return tc_upload_meta(pl);
}

// harm_n < 0: the Gaussian-kernel coefficients of ALIGN; harm_n >= 0: the
// harmonic-oscillator basis of ALIGNHARM (order harm_n, length scale harm_r0).
static fo_status cluster_plan_create(fo_ctx *ctx, int npairs, const fo_cluster_pair *pairs, const double *pos1,
                                     const double *pos2, const int *perm, const int *group_sizes, int index_base,
                                     int harm_n, double harm_r0, fo_plan **out) {
    if (!ctx || !out || npairs <= 0 || !pairs || !pos1 || !pos2 || !perm || !group_sizes)
        return set_err(ctx, FO_ERR_BAD_ARGS, "null argument or npairs <= 0");
    if (harm_n > fo::kMaxHarmN || (harm_n >= 0 && !(harm_r0 > 0.0)))
        return set_err(ctx, FO_ERR_BAD_ARGS, "harmonic basis: nmax %d outside [0,%d] or length scale <= 0", harm_n,
                       fo::kMaxHarmN);
    *out = nullptr;
    cudaSetDevice(ctx->opts.device);
    fo_plan *pl = new fo_plan();
    pl->ctx = ctx;
    pl->bulk = false;
    pl->fp32 = ctx->opts.precision == FO_PREC_MIXED;
    pl->npairs = npairs;
    pl->index_base = index_base;
    std::vector<int> slot2orig, slot2pair, cand2pair;
    std::vector<double> hpos1, hpos2;
    std::vector<int> bws;
    std::vector<RefAssign> rassign;
    std::vector<int> cand_list;
    long long ylm_n = 0, w_n = 0, coef_n = 0, grid_n = 0, lap_total = 0, candatom = 0;
    int atom0 = 0, cand0 = 0;
    const bool contig = packed_in_order(pairs, npairs);   // upload straight from the caller's arrays
    std::vector<long long> aoff;
    std::vector<int> s2o_all;
    std::vector<char> bad;
    std::vector<double> dmaxv;
    host_pair_checks(npairs, pairs, pos1, pos2, perm, group_sizes, index_base, aoff, s2o_all, bad, &dmaxv);
    for (int i = 0; i < npairs; ++i) {
        const fo_cluster_pair &q = pairs[i];
        const int n = q.natoms, L = q.jmax;
        if (n < 1 || n > kMaxAtoms) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: natoms %d outside [1,%d]", i, n, kMaxAtoms); }
        if (L < 0 || L > kMaxJmax) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: jmax %d outside [0,%d]", i, L, kMaxJmax); }
        if (q.nrot < 1 || q.nrot > kMaxNrot) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: nrot %d outside [1,%d]", i, q.nrot, kMaxNrot); }
        if (!(q.sigma == q.sigma)) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: sigma is NaN", i); }
        if (harm_n >= 0 && !(q.sigma > 0.0)) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: the harmonic basis needs sigma > 0", i); }
        const int *s2o = s2o_all.data() + aoff[i];
        if (bad[i]) {   // the same checks again, serially, for the message
            std::vector<int> tmp(n);
            fo_status s = check_groups(ctx, i, n, q.ngroups, perm + q.perm_off, group_sizes + q.group_off,
                                       index_base, tmp.data());
            delete pl;
            return s ? s : set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: non-finite coordinate", i);
        }
        fo::PairDev P{};
        P.n = n;
        P.ngroups = q.ngroups;
        P.group0 = (int)pl->hg.size();
        P.L = L;
        P.G = 2 * (L + 1);
        P.nrot = q.nrot;
        P.norient = q.invert ? 2 : 1;
        P.atom0 = atom0;
        P.cand0 = cand0;
        P.bulk = 0;
        P.ylm0 = ylm_n;
        P.coef0 = coef_n;
        P.grid0 = grid_n;
        P.candatom0 = candatom;
        P.sigma = q.sigma;
        P.harm = harm_n >= 0 ? 1 : 0;
        P.harm_n = harm_n >= 0 ? harm_n : 0;
        P.harm_r0 = harm_r0;
        int maxg = 0, off = 0;
        for (int g = 0; g < q.ngroups; ++g) {
            int gn = group_sizes[q.group_off + g];
            fo::GroupDev G{};
            G.pair = i;
            G.slot0 = atom0 + off;
            G.n = gn;
            G.m = std::min(gn, fo::kMaxNei);
            G.w0 = w_n;
            w_n += (long long)(L + 1) * gn * gn;
            off += gn;
            maxg = std::max(maxg, gn);
            pl->maxgroup = std::max(pl->maxgroup, gn);
            pl->hg.push_back(G);
        }
        {
            RefAssign ra = ref_assign(n, maxg, pl->fp32, pl->fp32, dmaxv[i]);
            P.lapstride = ra.lapstride;
            P.lapsplit = ra.split;
            P.lap0 = lap_total;
            lap_total += (long long)P.norient * P.nrot * P.lapstride;
            rassign.push_back(ra);
        }
        pl->hp.push_back(P);
        pl->caller_off.push_back(q.coord_off);
        for (int s = 0; s < n; ++s) {
            slot2orig.push_back(s2o[s]);
            slot2pair.push_back(i);
        }
        for (int c = 0; c < P.norient * P.nrot; ++c) cand2pair.push_back(i);
        if (!contig) {
            hpos1.insert(hpos1.end(), pos1 + 3 * q.coord_off, pos1 + 3 * (q.coord_off + n));
            hpos2.insert(hpos2.end(), pos2 + 3 * q.coord_off, pos2 + 3 * (q.coord_off + n));
        }
        ylm_n += (long long)n * (L + 1) * (L + 1);
        coef_n += (long long)(L + 1) * (2 * L + 1) * (2 * L + 1);
        grid_n += (long long)P.norient * P.G * P.G * P.G;
        candatom += (long long)P.norient * P.nrot * n;
        atom0 += n;
        cand0 += P.norient * P.nrot;
        pl->maxL = std::max(pl->maxL, L);
        pl->maxG = std::max(pl->maxG, P.G);
        pl->maxn = std::max(pl->maxn, n);
        bws.push_back(L + 1);
    }
    pl->nslots = atom0;
    pl->ncand = cand0;
    pl->ngroups = (int)pl->hg.size();
    std::sort(bws.begin(), bws.end());
    bws.erase(std::unique(bws.begin(), bws.end()), bws.end());
    fo_status s = ensure_dtabs(ctx, bws);
    if (s) { delete pl; return s; }
    size_t tc_s = 0, tc_meta_cap = 0;
    if (pl->fp32 && ctx->tc) {
        s = ensure_tc_tables(ctx, bws);
        if (s) { delete pl; return s; }
        tc_s = tc_plan_tiles(pl);
        tc_meta_cap = tc_meta_capacity(ctx, pl);
    }
    build_buckets(pl, rassign, cand_list);
    pl->harm_n = harm_n >= 0 ? harm_n : -1;
    pl->harm_d = harm_n >= 0 ? 2 * (size_t)pl->nslots * (harm_n + 1) * (pl->maxL + 1) : 0;
    s = plan_common_alloc(ctx, pl, contig ? pos1 : hpos1.data(), contig ? pos2 : hpos2.data(), slot2orig,
                          slot2pair, cand2pair, cand_list, ylm_n, w_n, coef_n, grid_n, 0, lap_total,
                          tc_meta_cap, tc_s);
    if (s) { fo_plan_destroy(pl); return s; }
    if (pl->tc) {
        pl->sb.dtab = (const void *const *)ctx->d_dtab32;
        pl->sb.tc_layout = true;
        s = tc_tune(ctx, pl);
        if (s) { fo_plan_destroy(pl); return s; }
    }
    pl->sb.dtab = pl->fp32 ? (const void *const *)ctx->d_dtab32 : (const void *const *)ctx->d_dtab64;
    *out = pl;
    return FO_OK;
}

fo_status fo_cluster_plan_create(fo_ctx *ctx, int npairs, const fo_cluster_pair *pairs, const double *pos1,
                                 const double *pos2, const int *perm, const int *group_sizes, int index_base,
                                 fo_plan **out) {
    return cluster_plan_create(ctx, npairs, pairs, pos1, pos2, perm, group_sizes, index_base, -1, 0.0, out);
}

fo_status fo_cluster_harm_plan_create(fo_ctx *ctx, int npairs, const fo_cluster_pair *pairs, const double *pos1,
                                      const double *pos2, const int *perm, const int *group_sizes, int index_base,
                                      int nmax, double hwidth, fo_plan **out) {
    if (nmax < 0) return set_err(ctx, FO_ERR_BAD_ARGS, "nmax %d < 0", nmax);
    return cluster_plan_create(ctx, npairs, pairs, pos1, pos2, perm, group_sizes, index_base, nmax, hwidth, out);
}

fo_status fo_bulk_plan_create(fo_ctx *ctx, int npairs, const fo_bulk_pair *pairs, const double *pos1,
                              const double *pos2, const int *perm, const int *group_sizes,
                              int index_base, fo_plan **out) {
    if (!ctx || !out || npairs <= 0 || !pairs || !pos1 || !pos2 || !perm || !group_sizes)
        return set_err(ctx, FO_ERR_BAD_ARGS, "null argument or npairs <= 0");
    *out = nullptr;
    cudaSetDevice(ctx->opts.device);
    fo_plan *pl = new fo_plan();
    pl->ctx = ctx;
    pl->bulk = true;
    pl->fp32 = ctx->opts.precision == FO_PREC_MIXED;
    pl->npairs = npairs;
    pl->index_base = index_base;
    std::vector<int> slot2orig, slot2pair, cand2pair;
    std::vector<double> hpos1, hpos2;
    std::vector<RefAssign> rassign;
    std::vector<int> cand_list;
    long long fgrid_n = 0, grid_n = 0, lap_total = 0, candatom = 0;
    int atom0 = 0, cand0 = 0;
    const bool contig = packed_in_order(pairs, npairs);   // upload straight from the caller's arrays
    std::vector<long long> aoff;
    std::vector<int> s2o_all;
    std::vector<char> bad;
    host_pair_checks(npairs, pairs, pos1, pos2, perm, group_sizes, index_base, aoff, s2o_all, bad, nullptr);
    for (int i = 0; i < npairs; ++i) {
        const fo_bulk_pair &q = pairs[i];
        const int n = q.natoms;
        if (n < 1 || n > kMaxAtoms) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: natoms %d outside [1,%d]", i, n, kMaxAtoms); }
        for (int k = 0; k < 3; ++k)
            if (!(q.box[k] > 0.0) || !std::isfinite(q.box[k])) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: box lengths must be positive", i); }
        int K = q.nwave > 0 ? q.nwave : (int)std::ceil(1.3 * std::cbrt((double)n));
        int M = q.nfspace > 0 ? q.nfspace : fastlen(4 * K + 3);
        int nd = q.ndisps > 0 ? q.ndisps : 10;
        double sg = q.sigma > 0 ? q.sigma : std::cbrt(q.box[0] * q.box[1] * q.box[2] / n) / 3.0;
        if (M < 2 * K + 1 || M > kMaxM) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: nfspace %d must lie in [2K+1, %d]", i, M, kMaxM); }
        if (nd > kMaxNrot) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: ndisps %d > %d", i, nd, kMaxNrot); }
        if (q.ohcell) { delete pl; return set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: ohcell pairs run through fo_bulk_align_batch, not plans", i); }
        const int *s2o = s2o_all.data() + aoff[i];
        if (bad[i]) {   // the same checks again, serially, for the message
            std::vector<int> tmp(n);
            fo_status s = check_groups(ctx, i, n, q.ngroups, perm + q.perm_off, group_sizes + q.group_off,
                                       index_base, tmp.data());
            delete pl;
            return s ? s : set_err(ctx, FO_ERR_BAD_ARGS, "pair %d: non-finite coordinate", i);
        }
        fo::PairDev P{};
        P.n = n;
        P.ngroups = q.ngroups;
        P.group0 = (int)pl->hg.size();
        P.L = K;
        P.G = M;
        P.nrot = nd;
        P.norient = 1;
        P.atom0 = atom0;
        P.cand0 = cand0;
        P.bulk = 1;
        P.coef0 = fgrid_n;
        P.grid0 = grid_n;
        P.candatom0 = candatom;
        P.sigma = sg;
        for (int k = 0; k < 3; ++k) P.box[k] = q.box[k];
        int maxg = 0, off = 0;
        for (int g = 0; g < q.ngroups; ++g) {
            int gn = group_sizes[q.group_off + g];
            fo::GroupDev G{};
            G.pair = i;
            G.slot0 = atom0 + off;
            G.n = gn;
            G.m = std::min(gn, fo::kMaxNei);
            off += gn;
            maxg = std::max(maxg, gn);
            pl->hg.push_back(G);
        }
        {
            double dmax = 0.5 * std::sqrt(q.box[0] * q.box[0] + q.box[1] * q.box[1] + q.box[2] * q.box[2]);
            RefAssign ra = ref_assign(n, maxg, pl->fp32, pl->fp32, dmax);
            P.lapstride = ra.lapstride;
            P.lapsplit = ra.split;
            P.lap0 = lap_total;
            lap_total += (long long)P.nrot * P.lapstride;
            rassign.push_back(ra);
        }
        pl->hp.push_back(P);
        pl->caller_off.push_back(q.coord_off);
        for (int s = 0; s < n; ++s) {
            slot2orig.push_back(s2o[s]);
            slot2pair.push_back(i);
        }
        for (int c = 0; c < P.nrot; ++c) cand2pair.push_back(i);
        if (!contig) {
            hpos1.insert(hpos1.end(), pos1 + 3 * q.coord_off, pos1 + 3 * (q.coord_off + n));
            hpos2.insert(hpos2.end(), pos2 + 3 * q.coord_off, pos2 + 3 * (q.coord_off + n));
        }
        fgrid_n += (long long)M * M * M;
        grid_n += (long long)M * M * M;
        candatom += (long long)P.nrot * n;
        atom0 += n;
        cand0 += P.nrot;
        pl->maxL = std::max(pl->maxL, K);
        pl->maxG = std::max(pl->maxG, M);
        pl->maxn = std::max(pl->maxn, n);
    }
    pl->nslots = atom0;
    pl->ncand = cand0;
    pl->ngroups = (int)pl->hg.size();
    build_buckets(pl, rassign, cand_list);
    fo_status s = plan_common_alloc(ctx, pl, contig ? pos1 : hpos1.data(), contig ? pos2 : hpos2.data(),
                                    slot2orig, slot2pair, cand2pair, cand_list, 0, 0, 0, grid_n, fgrid_n,
                                    lap_total);
    if (s) { fo_plan_destroy(pl); return s; }
    *out = pl;
    return FO_OK;
}

// After the stream has drained: the tensor-core contraction's timeout flag.
static fo_status tc_status(fo_plan *pl) {
    if (!pl->tc) return FO_OK;
    int terr = 0;
    fo_status s = cuda_check(pl->ctx, cudaMemcpy(&terr, pl->tcb.err, sizeof(int), cudaMemcpyDeviceToHost), "status");
    if (s) return s;
    return terr ? set_err(pl->ctx, FO_ERR_CUDA, "tensor-core contraction (coefficients or Wigner-d): a pipeline wait timed out") : FO_OK;
}

// The coefficient contraction of a cluster plan and the inverse SO(3)
// transform of its coefficients onto its grids: on the tensor cores (the
// coefficient contraction, the Wigner-d contraction and its FFT stage) or the
// CUDA-core kernels.
static void launch_coef_isoft(fo_plan *pl, cudaStream_t st, bool events) {
    if (pl->tc) {
        cudaMemsetAsync(pl->tcb.err, 0, sizeof(int), st);
        fo::launch_coef_tc(pl->sb, pl->tcb.err, st);
        if (events) rec_event(pl, K_COEFF);
        fo::launch_wigner_tc(pl->tcb, st);
        if (events) rec_event(pl, K_WTC);
        fo::launch_isoft_tc(pl->tcb, st);
    } else {
        fo::launch_sph_coeff(pl->sb, pl->fp32, st);
        if (events) rec_event(pl, K_COEFF);
        fo::launch_isoft(pl->sb, pl->fp32, st);
    }
    if (events) rec_event(pl, K_ISOFT);
}

// The plan's launch sequence on the context's stream (the refinement buckets
// fork onto the auxiliary streams and join back).  events: per-stage profile
// events (not while a graph is captured).
static void plan_enqueue(fo_plan *pl, bool events) {
    fo_ctx *ctx = pl->ctx;
    cudaStream_t st = ctx->stream;
    auto rec_event = [&](fo_plan *p, int kid) {
        if (events) ::rec_event(p, kid);
    };
    rec_event(pl, -1);
    cudaMemsetAsync(pl->d_pstatus, 0, pl->npairs * sizeof(int), st);
    cudaMemsetAsync(pl->d_npeaks, 0, 2 * pl->npairs * sizeof(int), st);
    if (!pl->bulk) {
        cudaMemsetAsync(pl->d_coef, 0, pl->coef_bytes, st);
        rec_event(pl, K_MEMSET);
        fo::launch_sph_center(pl->sb, st);     rec_event(pl, K_CENTER);
        fo::launch_sph_ylm(pl->sb, pl->fp32, st); rec_event(pl, K_YLM);
        fo::launch_sph_radial(pl->sb, pl->fp32, ctx->opts.cutoff, st); rec_event(pl, K_RADIAL);
        launch_coef_isoft(pl, st, events);
    } else {
        cudaMemsetAsync(pl->d_fgrid, 0, pl->fgrid_bytes, st);
        rec_event(pl, K_MEMSET);
        fo::launch_bulk_prep(pl->bb, st);          rec_event(pl, K_BPREP);
        fo::launch_bulk_sf(pl->bb, pl->fp32, st);  rec_event(pl, K_BSF);
        fo::launch_bulk_fft(pl->bb, pl->fp32, st); rec_event(pl, K_BFFT);
    }
    fo::launch_findpeaks(pl->rb, pl->fp32, st); rec_event(pl, K_PEAKS);
    fo::launch_refine(pl->rb, st, ctx->aux, fo_ctx::kAux, ctx->fork, ctx->join);
    rec_event(pl, K_REFINE);
    fo::launch_select(pl->rb, st);              rec_event(pl, K_SELECT);
}

fo_status fo_plan_run(fo_plan *pl) {
    if (!pl) return FO_ERR_BAD_ARGS;
    fo_ctx *ctx = pl->ctx;
    cudaSetDevice(ctx->opts.device);
    cudaStream_t st = ctx->stream;
    if (pl->use_graph && pl->gexec) return cuda_check(ctx, cudaGraphLaunch(pl->gexec, st), "graph launch");
    for (auto e : pl->evs) cudaEventDestroy(e);
    pl->evs.clear();
    pl->ev_kid.clear();
    plan_enqueue(pl, !pl->use_graph);
    fo_status s = cuda_check(ctx, cudaGetLastError(), "kernel launch");
    if (s || !pl->use_graph) return s;
    // this run went eagerly (kernel attributes are set once, outside any
    // capture); the same sequence is captured for the runs that follow
    s = cuda_check(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
    if (s) return s;
    plan_enqueue(pl, false);
    cudaGraph_t g = nullptr;
    s = cuda_check(ctx, cudaStreamEndCapture(st, &g), "end capture");
    if (s) return s;
    pl->graph = g;
    return cuda_check(ctx, cudaGraphInstantiate(&pl->gexec, g, 0), "graph instantiate");
}

static void drop_graph(fo_plan *pl) {
    if (pl->gexec) cudaGraphExecDestroy(pl->gexec);
    if (pl->graph) cudaGraphDestroy(pl->graph);
    pl->gexec = nullptr;
    pl->graph = nullptr;
}

fo_status fo_plan_set_graph(fo_plan *pl, int on) {
    if (!pl) return FO_ERR_BAD_ARGS;
    cudaSetDevice(pl->ctx->opts.device);
    if (!on) drop_graph(pl);
    pl->use_graph = on != 0;
    return FO_OK;
}

fo_status fo_plan_wait(fo_plan *pl) {
    if (!pl) return FO_ERR_BAD_ARGS;
    fo_ctx *ctx = pl->ctx;
    fo_status s = cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "pipeline");
    if (s) return s;
    s = tc_status(pl);
    if (s) return s;
    if (ctx->opts.profile && pl->evs.size() > 1) {
        for (size_t i = 1; i < pl->evs.size(); ++i) {
            float ms = 0;
            cudaEventElapsedTime(&ms, pl->evs[i - 1], pl->evs[i]);
            int k = pl->ev_kid[i];
            if (k >= 0 && k < kNumKernels) {
                ctx->prof_ms[k] += ms;
                ctx->prof_n[k] += 1;
            }
        }
    }
    return FO_OK;
}

fo_status fo_plan_results(fo_plan *pl, double *aligned, int *permbest, fo_pair_result *results) {
    if (!pl) return FO_ERR_BAD_ARGS;
    fo_ctx *ctx = pl->ctx;
    const int np = pl->npairs, ns = pl->nslots;
    std::vector<fo_pair_result> res(np);
    cudaStream_t st = ctx->stream;
    // pairs packed in slot order: the per-atom outputs go straight to the caller
    bool direct = true;
    for (int i = 0; i < np && direct; ++i) direct = pl->caller_off[i] == pl->hp[i].atom0;
    if (direct) {
        cudaMemcpyAsync(res.data(), pl->rb.results, np * sizeof(fo_pair_result), cudaMemcpyDeviceToHost, st);
        if (aligned)
            cudaMemcpyAsync(aligned, pl->rb.aligned, 3 * (size_t)ns * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (permbest) cudaMemcpyAsync(permbest, pl->rb.permbest, (size_t)ns * sizeof(int), cudaMemcpyDeviceToHost, st);
        fo_status s = cuda_check(ctx, cudaStreamSynchronize(st), "result download");
        if (s) return s;
        if (permbest && pl->index_base)
            for (int j = 0; j < ns; ++j) permbest[j] += pl->index_base;
        if (results) memcpy(results, res.data(), np * sizeof(fo_pair_result));
        return FO_OK;
    }
    std::vector<double> al(aligned ? 3 * (size_t)ns : 0);
    std::vector<int> pb(permbest ? ns : 0);
    cudaMemcpyAsync(res.data(), pl->rb.results, np * sizeof(fo_pair_result), cudaMemcpyDeviceToHost, st);
    if (aligned) cudaMemcpyAsync(al.data(), pl->rb.aligned, al.size() * sizeof(double), cudaMemcpyDeviceToHost, st);
    if (permbest) cudaMemcpyAsync(pb.data(), pl->rb.permbest, pb.size() * sizeof(int), cudaMemcpyDeviceToHost, st);
    fo_status s = cuda_check(ctx, cudaStreamSynchronize(st), "result download");
    if (s) return s;
    int worst = FO_OK;
    for (int i = 0; i < np; ++i) {
        const fo::PairDev &P = pl->hp[i];
        if (results) results[i] = res[i];
        if (res[i].status > worst) worst = res[i].status;
        long long co = pl->caller_off[i];
        if (aligned) memcpy(aligned + 3 * co, al.data() + 3 * (size_t)P.atom0, 3 * (size_t)P.n * sizeof(double));
        if (permbest)
            for (int j = 0; j < P.n; ++j) permbest[co + j] = pb[P.atom0 + j] + pl->index_base;
    }
    (void)worst;
    return FO_OK;
}

size_t fo_plan_device_bytes(const fo_plan *pl) { return pl ? pl->dbytes : 0; }

int fo_plan_launches(const fo_plan *pl) {
    if (!pl) return 0;
    int nb = 0;
    for (const auto &b : pl->buckets) nb += b.count > 0;
    // cluster: centre, ylm, radial, coefficients, inverse transform (with the
    // tensor cores: the FFT stage, after the Wigner contraction's launches);
    // bulk: prep, sf, 3 fft passes; then findpeaks (5^3 window, wider
    // windows), the mixed form's fixed-structure copy, one refinement launch
    // per bucket, select
    const int tcl = pl->tc ? (int)pl->tcb.launches.size() : 0;
    return 5 + tcl + 2 + (pl->fp32 ? 1 : 0) + nb + 1;
}

void fo_plan_destroy(fo_plan *pl) {
    if (!pl) return;
    cudaSetDevice(pl->ctx->opts.device);
    cudaStreamSynchronize(pl->ctx->stream);
    drop_graph(pl);
    for (auto e : pl->evs) cudaEventDestroy(e);
    fo_ctx *ctx = pl->ctx;
    if (pl->dmem) {
        ctx->pool.push_back({pl->dmem, pl->block_bytes});
        if ((int)ctx->pool.size() > fo_ctx::kPoolMax) {   // drop the smallest block
            auto it = std::min_element(ctx->pool.begin(), ctx->pool.end(),
                                       [](const std::pair<unsigned char *, size_t> &a,
                                          const std::pair<unsigned char *, size_t> &b) { return a.second < b.second; });
            cudaFree(it->first);
            ctx->pool.erase(it);
        }
    }
    delete pl;
}

static fo_status run_batch(fo_ctx *ctx, fo_plan *pl, double *aligned, int *permbest,
                           fo_pair_result *results) {
    fo_status s = fo_plan_run(pl);
    if (!s) s = fo_plan_wait(pl);
    if (!s) s = fo_plan_results(pl, aligned, permbest, results);
    fo_plan_destroy(pl);
    (void)ctx;
    return s;
}

fo_status fo_cluster_align_batch(fo_ctx *ctx, int npairs, const fo_cluster_pair *pairs,
                                 const double *pos1, const double *pos2, const int *perm,
                                 const int *group_sizes, int index_base, double *aligned,
                                 int *permbest, fo_pair_result *results) {
    fo_plan *pl = nullptr;
    fo_status s = fo_cluster_plan_create(ctx, npairs, pairs, pos1, pos2, perm, group_sizes, index_base, &pl);
    if (s) return s;
    return run_batch(ctx, pl, aligned, permbest, results);
}

// Operation op (0..47) of the cubic point group O_h as a signed permutation
// of the axes, row-major: output axis r takes input axis P[op / 8][r] with
// the sign of bit r of op % 8.  Operation 0 is the identity.
static void oh_operation(int op, double M[9]) {
    static const int P[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    for (int k = 0; k < 9; ++k) M[k] = 0.0;
    for (int r = 0; r < 3; ++r) M[3 * r + P[op / 8][r]] = ((op % 8) >> r & 1) ? -1.0 : 1.0;
}

fo_status fo_bulk_align_batch(fo_ctx *ctx, int npairs, const fo_bulk_pair *pairs, const double *pos1,
                              const double *pos2, const int *perm, const int *group_sizes,
                              int index_base, double *aligned, int *permbest, fo_pair_result *results) {
    bool oh = false;
    for (int i = 0; pairs && i < npairs; ++i) oh = oh || pairs[i].ohcell;
    if (!oh) {
        fo_plan *pl = nullptr;
        fo_status s = fo_bulk_plan_create(ctx, npairs, pairs, pos1, pos2, perm, group_sizes, index_base, &pl);
        if (s) return s;
        return run_batch(ctx, pl, aligned, permbest, results);
    }
    // OHCELLT (ALIGN1, fastbulk.f90:458-481): every operation of an ohcell pair
    // is a pair of its own, pos2 transformed; the best of the 48 is kept
    if (!ctx || !pos1 || !pos2 || !results) return set_err(ctx, FO_ERR_BAD_ARGS, "null argument");
    std::vector<fo_bulk_pair> q;
    std::vector<int> first(npairs);
    size_t natoms = 0;
    for (int i = 0; i < npairs; ++i) {
        first[i] = (int)q.size();
        for (int op = 0; op < (pairs[i].ohcell ? 48 : 1); ++op) {
            fo_bulk_pair e = pairs[i];
            e.ohcell = 0;
            e.coord_off = (int64_t)natoms;
            natoms += (size_t)std::max(0, e.natoms);
            q.push_back(e);
        }
    }
    std::vector<double> p1(3 * natoms), p2(3 * natoms), al(aligned ? 3 * natoms : 0);
    std::vector<int> pb(permbest ? natoms : 0);
    std::vector<fo_pair_result> res(q.size());
    for (int i = 0; i < npairs; ++i) {
        const size_t n = (size_t)std::max(0, pairs[i].natoms);
        const double *a1 = pos1 + 3 * pairs[i].coord_off, *a2 = pos2 + 3 * pairs[i].coord_off;
        for (int k = first[i]; k < (i + 1 < npairs ? first[i + 1] : (int)q.size()); ++k) {
            double M[9];
            oh_operation(k - first[i], M);
            double *b1 = &p1[3 * q[k].coord_off], *b2 = &p2[3 * q[k].coord_off];
            memcpy(b1, a1, 3 * n * sizeof(double));
            for (size_t j = 0; j < n; ++j)
                for (int r = 0; r < 3; ++r)
                    b2[3 * j + r] = M[3 * r] * a2[3 * j] + M[3 * r + 1] * a2[3 * j + 1] + M[3 * r + 2] * a2[3 * j + 2];
        }
    }
    fo_status s = fo_bulk_align_batch(ctx, (int)q.size(), q.data(), p1.data(), p2.data(), perm, group_sizes,
                                      index_base, aligned ? al.data() : nullptr, permbest ? pb.data() : nullptr,
                                      res.data());
    if (s) return s;
    for (int i = 0; i < npairs; ++i) {
        const int k0 = first[i], k1 = (i + 1 < npairs) ? first[i + 1] : (int)q.size();
        int best = k0, ncand = 0;
        for (int k = k0; k < k1; ++k) {
            ncand += res[k].ncand;
            const bool ok = res[k].status == 0, bok = res[best].status == 0;
            if ((ok && !bok) || (ok && bok && res[k].dist < res[best].dist)) best = k;
        }
        results[i] = res[best];
        results[i].ncand = ncand;
        if (pairs[i].ohcell) oh_operation(best - k0, results[i].rmat);
        const size_t n = (size_t)std::max(0, pairs[i].natoms);
        if (aligned) memcpy(aligned + 3 * pairs[i].coord_off, &al[3 * q[best].coord_off], 3 * n * sizeof(double));
        if (permbest) memcpy(permbest + pairs[i].coord_off, &pb[q[best].coord_off], n * sizeof(int));
    }
    return FO_OK;
}

// ---------------------------------------------------------------------------
// stage outputs of one pair

fo_status fo_cluster_overlap(fo_ctx *ctx, const fo_cluster_pair *pair, const double *pos1,
                             const double *pos2, const int *perm, const int *group_sizes,
                             int index_base, double *coeffs, double *grid) {
    if (!ctx || !pair) return FO_ERR_BAD_ARGS;
    fo_cluster_pair q = *pair;
    q.coord_off = q.perm_off = q.group_off = 0;
    fo_plan *pl = nullptr;
    fo_status s = fo_cluster_plan_create(ctx, 1, &q, pos1, pos2, perm, group_sizes, index_base, &pl);
    if (s) return s;
    cudaStream_t st = ctx->stream;
    cudaMemsetAsync(pl->d_coef, 0, pl->coef_bytes, st);
    fo::launch_sph_center(pl->sb, st);
    fo::launch_sph_ylm(pl->sb, pl->fp32, st);
    fo::launch_sph_radial(pl->sb, pl->fp32, ctx->opts.cutoff, st);
    launch_coef_isoft(pl, st, false);
    s = cuda_check(ctx, cudaStreamSynchronize(st), "cluster overlap");
    if (!s) s = tc_status(pl);
    const int L = q.jmax, W = 2 * L + 1, G = 2 * (L + 1);
    const size_t ncoef = 2 * (size_t)(L + 1) * W * W, ngrid = (size_t)G * G * G;
    const size_t tsz = pl->fp32 ? 4 : 8;
    std::vector<unsigned char> buf(std::max(ncoef, ngrid) * tsz);
    if (!s && coeffs) {
        s = cuda_check(ctx, cudaMemcpy(buf.data(), pl->d_coef, ncoef * tsz, cudaMemcpyDeviceToHost), "copy");
        if (!s) widen(buf.data(), coeffs, ncoef, pl->fp32);
    }
    if (!s && grid) {
        s = cuda_check(ctx, cudaMemcpy(buf.data(), pl->sb.grid, ngrid * tsz, cudaMemcpyDeviceToHost), "copy");
        if (!s) widen(buf.data(), grid, ngrid, pl->fp32);
    }
    fo_plan_destroy(pl);
    return s;
}

fo_status fo_bulk_overlap(fo_ctx *ctx, const fo_bulk_pair *pair, const double *pos1,
                          const double *pos2, const int *perm, const int *group_sizes,
                          int index_base, double *grid) {
    if (!ctx || !pair) return FO_ERR_BAD_ARGS;
    fo_bulk_pair q = *pair;
    q.coord_off = q.perm_off = q.group_off = 0;
    fo_plan *pl = nullptr;
    fo_status s = fo_bulk_plan_create(ctx, 1, &q, pos1, pos2, perm, group_sizes, index_base, &pl);
    if (s) return s;
    cudaStream_t st = ctx->stream;
    cudaMemsetAsync(pl->d_fgrid, 0, pl->fgrid_bytes, st);
    fo::launch_bulk_prep(pl->bb, st);
    fo::launch_bulk_sf(pl->bb, pl->fp32, st);
    fo::launch_bulk_fft(pl->bb, pl->fp32, st);
    s = cuda_check(ctx, cudaStreamSynchronize(st), "bulk overlap");
    const int M = pl->hp[0].G;
    const size_t ngrid = (size_t)M * M * M, tsz = pl->fp32 ? 4 : 8;
    std::vector<unsigned char> buf(ngrid * tsz);
    if (!s && grid) {
        s = cuda_check(ctx, cudaMemcpy(buf.data(), pl->bb.grid, ngrid * tsz, cudaMemcpyDeviceToHost), "copy");
        if (!s) widen(buf.data(), grid, ngrid, pl->fp32);
    }
    fo_plan_destroy(pl);
    return s;
}

fo_status fo_findpeaks(fo_ctx *ctx, const double *grid, int n, int npeaks, int width, double *peaks,
                       double *amps, int *nfound) {
    if (!ctx) return FO_ERR_BAD_ARGS;
    if (!grid || !peaks || !nfound) return set_err(ctx, FO_ERR_BAD_ARGS, "null argument");
    *nfound = 0;
    if (n < 2 || n > kMaxM) return set_err(ctx, FO_ERR_BAD_ARGS, "grid side %d outside [2,%d]", n, kMaxM);
    if (npeaks < 1 || npeaks > kMaxNrot)
        return set_err(ctx, FO_ERR_BAD_ARGS, "npeaks %d outside [1,%d]", npeaks, kMaxNrot);
    if (width < 1 || width > 7) return set_err(ctx, FO_ERR_BAD_ARGS, "width %d outside [1,7]", width);
    cudaSetDevice(ctx->opts.device);
    const bool fp32 = ctx->opts.precision == FO_PREC_MIXED;
    const size_t N = (size_t)n * n * n, tsz = fp32 ? 4 : 8;
    fo::PairDev P{};
    P.n = 1;
    P.G = n;
    P.nrot = npeaks;
    P.norient = 1;
    // one allocation: descriptor, grid, overlap max, peaks, amplitudes, counts
    const size_t o_grid = 256, o_omax = o_grid + ((N * tsz + 255) & ~(size_t)255), o_pk = o_omax + 256,
                 o_amp = o_pk + ((24 * (size_t)npeaks + 255) & ~(size_t)255),
                 o_np = o_amp + ((8 * (size_t)npeaks + 255) & ~(size_t)255), total = o_np + 256;
    unsigned char *d = nullptr;
    fo_status s = cuda_check(ctx, cudaMalloc(&d, total), "findpeaks allocation");
    if (s) return s;
    cudaStream_t st = ctx->stream;
    std::vector<unsigned char> g(N * tsz);
    if (fp32)
        for (size_t i = 0; i < N; ++i) ((float *)g.data())[i] = (float)grid[i];
    else
        memcpy(g.data(), grid, N * tsz);
    cudaMemsetAsync(d, 0, total, st);
    cudaMemcpyAsync(d, &P, sizeof P, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d + o_grid, g.data(), N * tsz, cudaMemcpyHostToDevice, st);
    int *d_np = (int *)(d + o_np);
    fo::launch_findpeaks_from((const fo::PairDev *)d, 1, d + o_grid, (double *)(d + o_omax), (double *)(d + o_pk),
                              (double *)(d + o_amp), d_np, d_np + 2, fp32, width, st);
    int cnt[3] = {0, 0, 0};
    std::vector<double> pk(3 * (size_t)npeaks), am(npeaks);
    s = cuda_check(ctx, cudaGetLastError(), "findpeaks launch");
    if (!s) s = cuda_check(ctx, cudaMemcpyAsync(cnt, d_np, sizeof cnt, cudaMemcpyDeviceToHost, st), "copy");
    if (!s) s = cuda_check(ctx, cudaMemcpyAsync(pk.data(), d + o_pk, 24 * (size_t)npeaks, cudaMemcpyDeviceToHost, st), "copy");
    if (!s) s = cuda_check(ctx, cudaMemcpyAsync(am.data(), d + o_amp, 8 * (size_t)npeaks, cudaMemcpyDeviceToHost, st), "copy");
    if (!s) s = cuda_check(ctx, cudaStreamSynchronize(st), "findpeaks");
    cudaFree(d);
    if (s) return s;
    *nfound = cnt[0];
    memcpy(peaks, pk.data(), 24 * (size_t)cnt[0]);
    if (amps) memcpy(amps, am.data(), 8 * (size_t)cnt[0]);
    return cnt[0] > 0 ? FO_OK : set_err(ctx, FO_ERR_NO_PEAKS, "no peak found with half-width up to %d", std::min(n / 2, 7));
}

// ---------------------------------------------------------------------------
// Fortran-style entry points
fo_status fo_setperm(fo_ctx *ctx, int natoms, const int *permgroup, const int *npermsize, int npermgroup) {
    if (!ctx || natoms < 1 || !permgroup || !npermsize || npermgroup < 1) return FO_ERR_BAD_ARGS;
    long long tot = 0;
    for (int g = 0; g < npermgroup; ++g) tot += npermsize[g];
    ctx->permgroup.assign(permgroup, permgroup + tot);
    ctx->npermsize.assign(npermsize, npermsize + npermgroup);
    ctx->perm_natoms = natoms;
    return FO_OK;
}

fo_status fo_set_ohcell(fo_ctx *ctx, int ohcell) {
    if (!ctx) return FO_ERR_BAD_ARGS;
    ctx->ohcell = ohcell ? 1 : 0;
    return FO_OK;
}

fo_status fo_get_bestperm(const fo_ctx *ctx, int *bestperm) {
    if (!ctx || !bestperm || ctx->bestperm.empty()) return FO_ERR_BAD_ARGS;
    memcpy(bestperm, ctx->bestperm.data(), ctx->bestperm.size() * sizeof(int));
    return FO_OK;
}

static void current_groups(fo_ctx *ctx, int natoms, std::vector<int> &perm, std::vector<int> &sizes) {
    if (ctx->perm_natoms == natoms && !ctx->permgroup.empty()) {
        perm = ctx->permgroup;
        sizes = ctx->npermsize;
    } else {
        perm.resize(natoms);
        for (int i = 0; i < natoms; ++i) perm[i] = i + 1;
        sizes.assign(1, natoms);
    }
}

fo_status fo_cluster_align(fo_ctx *ctx, double *coordsb, double *coordsa, int natoms, int debug, int l,
                           double *kwidth, int nrotations, int perminvopt, double *distance,
                           double *dist2, double *rmatbest) {
    (void)debug;
    if (!ctx || !coordsb || !coordsa || natoms < 1 || !kwidth) return FO_ERR_BAD_ARGS;
    std::vector<int> perm, sizes;
    current_groups(ctx, natoms, perm, sizes);
    fo_cluster_pair q{};
    q.natoms = natoms;
    q.ngroups = (int)sizes.size();
    q.jmax = l;
    q.nrot = nrotations;
    q.invert = perminvopt ? 1 : 0;
    q.sigma = *kwidth;
    std::vector<double> al(3 * (size_t)natoms);
    std::vector<int> pb(natoms);
    fo_pair_result r{};
    fo_status s = fo_cluster_align_batch(ctx, 1, &q, coordsb, coordsa, perm.data(), sizes.data(), 1,
                                         al.data(), pb.data(), &r);
    if (s) return s;
    if (r.status) return (fo_status)r.status;
    double cb[3] = {0, 0, 0};
    for (int j = 0; j < natoms; ++j)
        for (int k = 0; k < 3; ++k) cb[k] += coordsb[3 * j + k];
    for (int j = 0; j < natoms; ++j)
        for (int k = 0; k < 3; ++k) coordsb[3 * j + k] -= cb[k] / natoms;
    memcpy(coordsa, al.data(), al.size() * sizeof(double));
    *kwidth = r.sigma;
    if (distance) *distance = r.dist;
    if (dist2) *dist2 = r.dist * r.dist;
    if (rmatbest)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) rmatbest[i + 3 * j] = r.rmat[3 * i + j];
    ctx->bestperm = pb;
    return FO_OK;
}

fo_status fo_bulk_align(fo_ctx *ctx, double *coordsb, double *coordsa, int natoms, int debug, double boxlx,
                        double boxly, double boxlz, double kwidth, int ndisplacements, int nwave,
                        int nfspace, double *distance, double *dist2) {
    (void)debug;
    if (!ctx || !coordsb || !coordsa || natoms < 1) return FO_ERR_BAD_ARGS;
    std::vector<int> perm, sizes;
    current_groups(ctx, natoms, perm, sizes);
    fo_bulk_pair q{};
    q.natoms = natoms;
    q.ngroups = (int)sizes.size();
    q.nwave = nwave;
    q.nfspace = nfspace;
    q.ndisps = ndisplacements;
    q.ohcell = ctx->ohcell;
    q.sigma = kwidth;
    q.box[0] = boxlx;
    q.box[1] = boxly;
    q.box[2] = boxlz;
    std::vector<double> al(3 * (size_t)natoms);
    std::vector<int> pb(natoms);
    fo_pair_result r{};
    fo_status s = fo_bulk_align_batch(ctx, 1, &q, coordsb, coordsa, perm.data(), sizes.data(), 1,
                                      al.data(), pb.data(), &r);
    if (s) return s;
    if (r.status) return (fo_status)r.status;
    memcpy(coordsa, al.data(), al.size() * sizeof(double));
    if (distance) *distance = r.dist;
    if (dist2) *dist2 = r.dist * r.dist;
    ctx->bestperm = pb;
    return FO_OK;
}

// ALIGNGROUP: pair (i, j) is ALIGN of structure j of list 2 onto structure i
// of list 1 with the same parameters, so the pairs run as bulk batches
// (chunks bound the host and device staging).  With sym only i >= j are
// aligned, as the reference's triangular loop does.
fo_status fo_bulk_align_group(fo_ctx *ctx, const double *coords1list, int n1list, const double *coords2list,
                              int n2list, int natoms, int debug, double boxlx, double boxly, double boxlz,
                              double kwidth, int ndisplacements, int nwave, int nfspace, double *distmat,
                              double *alignedcoords2, int sym) {
    (void)debug;
    if (!ctx) return FO_ERR_BAD_ARGS;
    if (!coords1list || !coords2list || !distmat || natoms < 1 || n1list < 1 || n2list < 1)
        return set_err(ctx, FO_ERR_BAD_ARGS, "null argument or empty list");
    if (sym && n2list > n1list) return set_err(ctx, FO_ERR_BAD_ARGS, "sym needs n2list <= n1list");
    std::vector<int> perm, sizes;
    current_groups(ctx, natoms, perm, sizes);
    const size_t per = 3 * (size_t)natoms;
    std::vector<std::pair<int, int>> todo;
    for (int j = 0; j < n2list; ++j)
        for (int i = sym ? j : 0; i < n1list; ++i) todo.emplace_back(i, j);
    for (size_t k = 0; k < (size_t)n1list * n2list; ++k) distmat[k] = 0.0;
    if (alignedcoords2) memset(alignedcoords2, 0, (size_t)n1list * n2list * per * sizeof(double));
    // about 64 MiB of coordinates per side and at most 4096 pairs per batch
    const size_t chunk = std::max<size_t>(1, std::min<size_t>(4096, ((size_t)8 << 20) / per));
    std::vector<double> p1, p2, al;
    std::vector<int> pb;
    std::vector<fo_bulk_pair> q;
    std::vector<fo_pair_result> res;
    for (size_t c0 = 0; c0 < todo.size(); c0 += chunk) {
        const size_t nb = std::min(chunk, todo.size() - c0);
        p1.resize(nb * per);
        p2.resize(nb * per);
        al.resize(nb * per);
        pb.resize(nb * natoms);
        q.assign(nb, fo_bulk_pair{});
        res.assign(nb, fo_pair_result{});
        for (size_t k = 0; k < nb; ++k) {
            const int i = todo[c0 + k].first, j = todo[c0 + k].second;
            memcpy(&p1[k * per], coords1list + (size_t)i * per, per * sizeof(double));
            memcpy(&p2[k * per], coords2list + (size_t)j * per, per * sizeof(double));
            fo_bulk_pair &b = q[k];
            b.natoms = natoms;
            b.ngroups = (int)sizes.size();
            b.nwave = nwave;
            b.nfspace = nfspace;
            b.ndisps = ndisplacements;
            b.sigma = kwidth;
            b.box[0] = boxlx;
            b.box[1] = boxly;
            b.box[2] = boxlz;
            b.coord_off = (int64_t)(k * natoms);
        }
        fo_status s = fo_bulk_align_batch(ctx, (int)nb, q.data(), p1.data(), p2.data(), perm.data(), sizes.data(),
                                          1, al.data(), pb.data(), res.data());
        if (s) return s;
        for (size_t k = 0; k < nb; ++k) {
            if (res[k].status) return set_err(ctx, (fo_status)res[k].status, "pair (%d, %d): %s",
                                              todo[c0 + k].first + 1, todo[c0 + k].second + 1,
                                              fo_status_string((fo_status)res[k].status));
            const size_t ij = (size_t)todo[c0 + k].first + (size_t)n1list * todo[c0 + k].second;
            distmat[ij] = res[k].dist;
            if (alignedcoords2) memcpy(alignedcoords2 + ij * per, &al[k * per], per * sizeof(double));
        }
    }
    return FO_OK;
}

fo_status fo_cluster_harm_align_batch(fo_ctx *ctx, int npairs, const fo_cluster_pair *pairs, const double *pos1,
                                      const double *pos2, const int *perm, const int *group_sizes, int index_base,
                                      int nmax, double hwidth, double *aligned, int *permbest,
                                      fo_pair_result *results) {
    fo_plan *pl = nullptr;
    fo_status s = fo_cluster_harm_plan_create(ctx, npairs, pairs, pos1, pos2, perm, group_sizes, index_base, nmax,
                                              hwidth, &pl);
    if (s) return s;
    return run_batch(ctx, pl, aligned, permbest, results);
}

// ALIGNHARM: the coordinates as given (COORDSB is not centred), the
// harmonic-basis coefficients, then ALIGNCOEFFS and the inversion as ALIGN.
fo_status fo_cluster_align_harm(fo_ctx *ctx, double *coordsb, double *coordsa, int natoms, int debug, int n, int l,
                                double hwidth, double kwidth, double *distance, double *dist2, double *rmatbest,
                                int nrotations, int perminvopt) {
    (void)debug;
    if (!ctx || !coordsb || !coordsa || natoms < 1) return FO_ERR_BAD_ARGS;
    std::vector<int> perm, sizes;
    current_groups(ctx, natoms, perm, sizes);
    fo_cluster_pair q{};
    q.natoms = natoms;
    q.ngroups = (int)sizes.size();
    q.jmax = l;
    q.nrot = nrotations;
    q.invert = perminvopt ? 1 : 0;
    q.sigma = kwidth;
    std::vector<double> al(3 * (size_t)natoms);
    std::vector<int> pb(natoms);
    fo_pair_result r{};
    fo_status s = fo_cluster_harm_align_batch(ctx, 1, &q, coordsb, coordsa, perm.data(), sizes.data(), 1, n,
                                              hwidth, al.data(), pb.data(), &r);
    if (s) return s;
    if (r.status) return (fo_status)r.status;
    memcpy(coordsa, al.data(), al.size() * sizeof(double));
    if (distance) *distance = r.dist;
    if (dist2) *dist2 = r.dist * r.dist;
    if (rmatbest)
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) rmatbest[i + 3 * j] = r.rmat[3 * i + j];
    ctx->bestperm = pb;
    return FO_OK;
}

// CALCOVERLAPMATRICES: CALCSIMILARITY of every pair i1 <= i2 (list member i1
// as the target), mirrored.  The pairs run as harmonic-basis plans through
// the coefficient and inverse-SOFT stages only.
fo_status fo_calc_overlap_matrices(fo_ctx *ctx, const double *coordslist, int natoms, int nlist, int n, int l,
                                   double hwidth, double kwidth, double *norms, double *maxovers) {
    if (!ctx) return FO_ERR_BAD_ARGS;
    if (!coordslist || !norms || !maxovers || natoms < 1 || nlist < 1)
        return set_err(ctx, FO_ERR_BAD_ARGS, "null argument or empty list");
    cudaSetDevice(ctx->opts.device);
    std::vector<int> perm, sizes;
    current_groups(ctx, natoms, perm, sizes);
    const size_t per = 3 * (size_t)natoms;
    std::vector<std::pair<int, int>> todo;
    for (int i1 = 0; i1 < nlist; ++i1)
        for (int i2 = i1; i2 < nlist; ++i2) todo.emplace_back(i1, i2);
    const size_t chunk = std::max<size_t>(1, std::min<size_t>(4096, ((size_t)8 << 20) / per));
    double *d_out = nullptr;
    fo_status s = cuda_check(ctx, cudaMalloc(&d_out, 2 * chunk * sizeof(double)), "cudaMalloc");
    if (s) return s;
    std::vector<double> p1, p2, h(2 * chunk);
    std::vector<fo_cluster_pair> q;
    cudaStream_t st = ctx->stream;
    for (size_t c0 = 0; c0 < todo.size() && !s; c0 += chunk) {
        const size_t nb = std::min(chunk, todo.size() - c0);
        p1.resize(nb * per);
        p2.resize(nb * per);
        q.assign(nb, fo_cluster_pair{});
        for (size_t k = 0; k < nb; ++k) {
            memcpy(&p1[k * per], coordslist + (size_t)todo[c0 + k].first * per, per * sizeof(double));
            memcpy(&p2[k * per], coordslist + (size_t)todo[c0 + k].second * per, per * sizeof(double));
            q[k].natoms = natoms;
            q[k].ngroups = (int)sizes.size();
            q[k].jmax = l;
            q[k].nrot = 1;
            q[k].invert = 0;
            q[k].sigma = kwidth;
            q[k].coord_off = (int64_t)(k * natoms);
        }
        fo_plan *pl = nullptr;
        s = fo_cluster_harm_plan_create(ctx, (int)nb, q.data(), p1.data(), p2.data(), perm.data(), sizes.data(), 1,
                                        n, hwidth, &pl);
        if (s) break;
        cudaMemsetAsync(pl->d_coef, 0, pl->coef_bytes, st);
        fo::launch_sph_center(pl->sb, st);
        fo::launch_sph_ylm(pl->sb, pl->fp32, st);
        fo::launch_sph_radial(pl->sb, pl->fp32, ctx->opts.cutoff, st);
        launch_coef_isoft(pl, st, false);
        fo::launch_pair_stats(pl->sb, pl->fp32, d_out, st);
        cudaMemcpyAsync(h.data(), d_out, 2 * nb * sizeof(double), cudaMemcpyDeviceToHost, st);
        s = cuda_check(ctx, cudaStreamSynchronize(st), "overlap matrices");
        if (!s) s = tc_status(pl);
        fo_plan_destroy(pl);
        for (size_t k = 0; k < nb && !s; ++k) {
            const int i1 = todo[c0 + k].first, i2 = todo[c0 + k].second;
            norms[i1 + (size_t)nlist * i2] = norms[i2 + (size_t)nlist * i1] = h[2 * k];
            maxovers[i1 + (size_t)nlist * i2] = maxovers[i2 + (size_t)nlist * i1] = h[2 * k + 1];
        }
    }
    cudaFree(d_out);
    return s;
}

fo_status fo_bulk_calcdefaults(int natoms, double boxlx, double boxly, double boxlz, double *kernelwidth,
                               int *nwave, int *nfspace) {
    if (natoms < 1 || !kernelwidth || !nwave || !nfspace) return FO_ERR_BAD_ARGS;
    double kw = std::cbrt(boxlx * boxly * boxlz / natoms) / 3.0;
    double maxk = 1.5 / kw;
    int nw = (int)std::ceil(2 * 3.14159265359 / std::min(boxlx, std::min(boxly, boxlz)) * maxk);
    *kernelwidth = kw;
    *nwave = nw;
    if (2 * nw + 1 <= 200) {
        *nfspace = fastlen(4 * nw + 3);
    } else {   // the next power of two
        int m = 1;
        while (m < 4 * nw + 3) m *= 2;
        *nfspace = m;
    }
    return FO_OK;
}

fo_status fo_ctx_record(fo_ctx *ctx, int slot) {
    if (!ctx || slot < 0 || slot >= 64) return FO_ERR_BAD_ARGS;
    cudaSetDevice(ctx->opts.device);
    if (!ctx->ev[slot]) {
        fo_status s = cuda_check(ctx, cudaEventCreate(&ctx->ev[slot]), "cudaEventCreate");
        if (s) return s;
    }
    return cuda_check(ctx, cudaEventRecord(ctx->ev[slot], ctx->stream), "cudaEventRecord");
}

fo_status fo_ctx_elapsed_ms(fo_ctx *ctx, int a, int b, float *ms) {
    if (!ctx || !ms || a < 0 || b < 0 || a >= 64 || b >= 64 || !ctx->ev[a] || !ctx->ev[b])
        return FO_ERR_BAD_ARGS;
    fo_status s = cuda_check(ctx, cudaEventSynchronize(ctx->ev[b]), "cudaEventSynchronize");
    if (s) return s;
    return cuda_check(ctx, cudaEventElapsedTime(ms, ctx->ev[a], ctx->ev[b]), "cudaEventElapsedTime");
}

fo_status fo_ctx_flush_l2(fo_ctx *ctx, size_t bytes) {
    if (!ctx) return FO_ERR_BAD_ARGS;
    cudaSetDevice(ctx->opts.device);
    if (bytes > ctx->flush_bytes) {
        cudaFree(ctx->flush_buf);
        ctx->flush_buf = nullptr;
        ctx->flush_bytes = 0;
        fo_status s = cuda_check(ctx, cudaMalloc(&ctx->flush_buf, bytes), "cudaMalloc(flush)");
        if (s) return s;
        ctx->flush_bytes = bytes;
    }
    static int salt = 0;
    return cuda_check(ctx, cudaMemsetAsync(ctx->flush_buf, (++salt) & 0xff, bytes, ctx->stream),
                      "flush");
}

fo_status fo_ctx_synchronize(fo_ctx *ctx) {
    if (!ctx) return FO_ERR_BAD_ARGS;
    return cuda_check(ctx, cudaStreamSynchronize(ctx->stream), "synchronize");
}

int fo_profile_kernels(const fo_ctx *ctx, const char **names, double *ms_total, int *launches, int cap) {
    if (!ctx) return 0;
    int k = 0;
    for (int i = 0; i < kNumKernels && k < cap; ++i) {
        if (ctx->prof_n[i] == 0) continue;
        if (names) names[k] = kKernelNames[i];
        if (ms_total) ms_total[k] = ctx->prof_ms[i];
        if (launches) launches[k] = ctx->prof_n[i];
        ++k;
    }
    return k;
}

void fo_profile_reset(fo_ctx *ctx) {
    if (!ctx) return;
    for (int i = 0; i < kNumKernels; ++i) { ctx->prof_ms[i] = 0; ctx->prof_n[i] = 0; }
}

}  // extern "C"

// library-internal (not in the public header): the server's worker contexts
namespace fo {
fo_opts ctx_opts(const fo_ctx *ctx) { return ctx->opts; }
void ctx_set_budget(fo_ctx *ctx, size_t bytes) { ctx->opts.hbm_budget_bytes = bytes; }
cudaStream_t ctx_stream(fo_ctx *ctx) { return ctx->stream; }
fo_status ctx_error(fo_ctx *ctx, fo_status s, const char *msg) { return set_err(ctx, s, "%s", msg); }
}  // namespace fo

