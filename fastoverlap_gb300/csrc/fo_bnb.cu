// fo_bnb.cu -- branch and bound over rotations for many cluster pairs.
//
// The search of the upstream Python BranchandBoundMaster with
// BranchNodeCluster (fastoverlap/bnbAlignment.py:23-104, 204-277): nodes are
// cubes of angle-axis vectors (start width 2 pi, 8 children of half width);
// a node's lower bound is the assignment over the smallest squared distances
// any rotation in its cube can reach (angular bound on each atom pair), its
// upper bound the assignment distance at the cube's centre; a cheap
// nearest-neighbour screen replaces both when it cannot beat the best; the
// search is best-first by lower bound until the lower bound is within
// rtol * best + atol of the best upper bound.
//
// GB300 form: every search keeps its heap on the host (Python heapq's order)
// and pops until it has a node to branch; one launch then evaluates the
// children of all searches, one warp per child -- the rotated structure, the
// nearest-neighbour bounds and the two dense assignments (Hungarian shortest
// augmenting paths, the column scans across the lanes).  The kernel returns
// all four bounds of a child and the host replays the sequential decisions
// with the live best bound, so the expansion order is the sequential one.
#include "../../include/fastoverlap_gb300.h"
#include "fo_common.cuh"
#include "fo_kernels.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <vector>

namespace fo {

constexpr int kMaxBnbAtoms = 256;

struct BnbChild {
    double rot[3];
    double width;
    int pair;
    int sign;   // +1: pos2, -1: the inverted pos2
};

// Scratch of one child (doubles): rotated structure 3n, lower-bound and
// squared-distance matrices n^2 each, potentials u, v and minv (n+1 each),
// per-column values 2n, then p, way (ints) and used (bytes).
__host__ __device__ inline long long bnb_stride(int n) {
    return 3LL * n + 2LL * n * n + 3LL * (n + 1) + 2LL * n + (n + 1) + (n + 1) / 8 + 2;
}

__device__ __forceinline__ void bnb_angle_axis(const double w[3], double M[9]) {
    const double th = sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
    if (th == 0.0) {
        for (int k = 0; k < 9; ++k) M[k] = (k % 4 == 0) ? 1.0 : 0.0;
        return;
    }
    const double x = w[0] / th, y = w[1] / th, z = w[2] / th, c = cos(th), s = sin(th), C = 1 - c;
    const double xs = x * s, ys = y * s, zs = z * s, xC = x * C, yC = y * C, zC = z * C;
    const double xyC = x * yC, yzC = y * zC, zxC = z * xC;
    M[0] = x * xC + c; M[1] = xyC - zs;    M[2] = zxC + ys;
    M[3] = xyC + zs;   M[4] = y * yC + c;  M[5] = yzC - xs;
    M[6] = zxC - ys;   M[7] = yzC + xs;    M[8] = z * zC + c;
}

// Dense assignment of the n x n costs c (row-major) by shortest augmenting
// paths with row and column potentials, 1-based with a virtual column 0, as
// the sequential form does it step for step: per step the lanes scan their
// columns and the warp takes the smallest reduced cost (lowest column on
// ties).  Fills col_of_row (0-based) through p; returns false when a row's
// search exceeds n + 1 steps (it never should).
__device__ bool bnb_warp_lap(const double *c, int n, double *u, double *v, double *minv, int *p, int *way,
                             unsigned char *used) {
    const int lane = threadIdx.x & 31;
    for (int j = lane; j <= n; j += 32) { u[j] = 0.0; v[j] = 0.0; p[j] = 0; way[j] = 0; }
    __syncwarp();
    for (int i = 1; i <= n; ++i) {
        if (lane == 0) p[0] = i;
        for (int j = lane; j <= n; j += 32) { minv[j] = INFINITY; used[j] = 0; }
        __syncwarp();
        int j0 = 0, steps = 0;
        do {
            if (++steps > n + 1) return false;
            if (lane == 0) used[j0] = 1;
            __syncwarp();
            const int i0 = p[j0];
            double delta = INFINITY;
            int j1 = n + 1;
            for (int j = lane + 1; j <= n; j += 32)
                if (!used[j]) {
                    const double cur = c[(size_t)(i0 - 1) * n + (j - 1)] - u[i0] - v[j];
                    if (cur < minv[j]) { minv[j] = cur; way[j] = j0; }
                    if (minv[j] < delta) { delta = minv[j]; j1 = j; }
                }
            for (int o = 16; o > 0; o >>= 1) {
                const double od = __shfl_xor_sync(0xffffffffu, delta, o);
                const int oj = __shfl_xor_sync(0xffffffffu, j1, o);
                if (od < delta || (od == delta && oj < j1)) { delta = od; j1 = oj; }
            }
            if (j1 > n) return false;   // no unused column left: cannot happen with finite costs
            __syncwarp();
            for (int j = lane; j <= n; j += 32) {
                if (used[j]) {
                    u[p[j]] += delta;
                    v[j] -= delta;
                } else {
                    minv[j] -= delta;
                }
            }
            __syncwarp();
            j0 = j1;
        } while (p[j0] != 0);
        if (lane == 0) {
            int guard = 0;
            do {
                const int j1 = way[j0];
                p[j0] = p[j1];
                j0 = j1;
            } while (j0 && ++guard <= n + 1);
        }
        __syncwarp();
    }
    return true;
}

// One warp per child.  out[4c..4c+3] = nearest-neighbour upper bound, its
// lower bound, assignment lower bound, assignment upper bound; st[c] = 1 if
// an assignment hit its step guard.
__global__ void __launch_bounds__(128) k_bnb_children(const BnbChild *ch, int nch, const double *X1,
                                                      const double *X2, const double *r1, const double *r2,
                                                      const int *atom0, const int *natoms, double *scratch,
                                                      long long sstride, double *out, int *st) {
    const int w = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (w >= nch) return;   // whole warps only (blockDim is a multiple of 32)
    const BnbChild c = ch[w];
    const int n = natoms[c.pair], a0 = atom0[c.pair];
    const double *x1 = X1 + 3LL * a0, *x2 = X2 + 3LL * a0, *R1 = r1 + a0, *R2 = r2 + a0;
    double *rp = scratch + (long long)w * sstride;
    double *lb = rp + 3LL * n, *d2 = lb + (long long)n * n, *u = d2 + (long long)n * n, *v = u + (n + 1);
    double *minv = v + (n + 1), *nnd = minv + (n + 1), *nnl = nnd + n;
    int *p = (int *)(nnl + n), *way = p + (n + 1);
    unsigned char *used = (unsigned char *)(way + (n + 1));
    double M[9];
    bnb_angle_axis(c.rot, M);
    for (int j = lane; j < n; j += 32)
        for (int k = 0; k < 3; ++k)
            rp[3 * j + k] = c.sign * (x2[3 * j] * M[k] + x2[3 * j + 1] * M[3 + k] + x2[3 * j + 2] * M[6 + k]);
    __syncwarp();
    const double theta = fmin(sqrt(3.0) * c.width / 2, FO_PI), cosd = cos(theta), sind = fabs(sin(theta));
    // nearest atom of the fixed structure to each rotated atom
    for (int j = lane; j < n; j += 32) {
        double best = INFINITY;
        int bi = 0;
        for (int i = 0; i < n; ++i) {
            double t = 0;
            for (int k = 0; k < 3; ++k) {
                const double e = x1[3 * i + k] - rp[3 * j + k];
                t += e * e;
            }
            if (t < best) { best = t; bi = i; }
        }
        const double a = R1[bi], b = R2[j];
        const double cosa = 0.5 * (a * a + b * b - best) / a / b;
        const double sina = sqrt(fmin(fmax(1.0 - cosa * cosa, 0.0), 1.0));
        const double cdm = (cosa > cosd) ? 1.0 : cosa * cosd + sina * sind;
        nnd[j] = best;
        nnl[j] = fmax(a * a + b * b - 2 * a * b * cdm, 0.0);
    }
    // the two cost matrices
    for (long long e = lane; e < (long long)n * n; e += 32) {
        const int i = (int)(e / n), j = (int)(e % n);
        double t = 0;
        for (int k = 0; k < 3; ++k) {
            const double q = x1[3 * i + k] - rp[3 * j + k];
            t += q * q;
        }
        const double rr = R1[i] * R2[j], rs = R1[i] * R1[i] + R2[j] * R2[j];
        const double cosa = 0.5 * (rs - t) / rr, sina = sqrt(fmin(fmax(1.0 - cosa * cosa, 0.0), 1.0));
        const double cdm = (cosa > cosd) ? 1.0 : cosa * cosd + sina * sind;
        d2[e] = t;
        lb[e] = fmax(rs - 2 * rr * cdm, 0.0);
    }
    __syncwarp();
    double res[4] = {0, 0, 0, 0};
    if (lane == 0) {   // sums in the sequential order
        double s = 0, q = 0;
        for (int j = 0; j < n; ++j) { s += nnd[j]; q += nnl[j]; }
        res[0] = sqrt(s);
        res[1] = sqrt(q);
    }
    bool ok = bnb_warp_lap(lb, n, u, v, minv, p, way, used);
    if (lane == 0 && ok) {
        double tot = 0;
        for (int j = 1; j <= n; ++j) tot += lb[(size_t)(p[j] - 1) * n + (j - 1)];
        res[2] = sqrt(tot);
    }
    __syncwarp();
    ok = ok && bnb_warp_lap(d2, n, u, v, minv, p, way, used);
    if (lane == 0) {
        if (ok) {
            // row p[j] - 1 takes column j - 1: the distance at the cube's centre
            for (int j = 1; j <= n; ++j) way[p[j] - 1] = j - 1;
            double s = 0;
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) {
                    const double e = x1[3 * i + k] - rp[3 * way[i] + k];
                    s += e * e;
                }
            res[3] = sqrt(s);
        }
        for (int k = 0; k < 4; ++k) out[4LL * w + k] = res[k];
        st[w] = ok ? 0 : 1;
    }
}

void launch_bnb_children(const BnbChild *ch, int nch, const double *X1, const double *X2, const double *r1,
                         const double *r2, const int *atom0, const int *natoms, double *scratch, long long sstride,
                         double *out, int *st, cudaStream_t s) {
    const int threads = 128, warps = threads / 32;
    k_bnb_children<<<(nch + warps - 1) / warps, threads, 0, s>>>(ch, nch, X1, X2, r1, r2, atom0, natoms, scratch,
                                                                 sstride, out, st);
}

}  // namespace fo

namespace {

fo_status bnb_err(fo_ctx *ctx, fo_status s, const char *fmt, ...) {
    char buf[256];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return fo::ctx_error(ctx, s, buf);
}

fo_status bnb_cuda(fo_ctx *ctx, cudaError_t e, const char *what) {
    if (e == cudaSuccess) return FO_OK;
    return bnb_err(ctx, FO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

struct BnbNode {
    double rot[3];
    double width, lower, upper;
    int sign;
};

// binary min-heap on lower with the sift rules of Python's heapq (a push
// sifts up past strictly larger parents; a pop moves the last item to the
// root, walks it to a leaf along the smaller child -- the right one only
// when strictly smaller -- and sifts it up)
struct BnbHeap {
    std::vector<BnbNode> a;
    void up(size_t pos) {
        BnbNode it = a[pos];
        while (pos > 0) {
            const size_t par = (pos - 1) >> 1;
            if (it.lower < a[par].lower) { a[pos] = a[par]; pos = par; }
            else break;
        }
        a[pos] = it;
    }
    void push(const BnbNode &x) {
        a.push_back(x);
        up(a.size() - 1);
    }
    BnbNode pop() {
        BnbNode last = a.back();
        a.pop_back();
        if (a.empty()) return last;
        BnbNode top = a[0];
        a[0] = last;
        size_t pos = 0, child = 1;
        const size_t end = a.size();
        BnbNode it = a[0];
        while (child < end) {
            const size_t right = child + 1;
            if (right < end && !(a[child].lower < a[right].lower)) child = right;
            a[pos] = a[child];
            pos = child;
            child = 2 * pos + 1;
        }
        a[pos] = it;
        up(pos);
        return top;
    }
};

struct BnbSearch {
    BnbHeap heap;
    BnbNode best{};
    long long nodes = 0;
    bool active = true;
    bool failed = false;   // an assignment of one of its children hit the step guard
};

}  // namespace

extern "C" {

fo_status fo_bnb_cluster_batch(fo_ctx *ctx, int npairs, const int *natoms, const double *pos1, const double *pos2,
                               int invert, long long niter, double rtol, double atol, double *dist,
                               double *aligned, long long *nodes) {
    using namespace fo;
    if (!ctx) return FO_ERR_BAD_ARGS;
    if (npairs < 1 || !natoms || !pos1 || !pos2 || !dist) return bnb_err(ctx, FO_ERR_BAD_ARGS, "null argument or npairs < 1");
    cudaSetDevice(fo::ctx_opts(ctx).device);
    std::vector<int> a0(npairs);
    int tot = 0, maxn = 0;
    for (int p = 0; p < npairs; ++p) {
        if (natoms[p] < 1 || natoms[p] > kMaxBnbAtoms)
            return bnb_err(ctx, FO_ERR_BAD_ARGS, "pair %d: natoms %d outside [1,%d]", p, natoms[p], kMaxBnbAtoms);
        a0[p] = tot;
        tot += natoms[p];
        maxn = std::max(maxn, natoms[p]);
    }
    // both structures centred, with their radii (as the search takes them)
    std::vector<double> X1(3 * (size_t)tot), X2(3 * (size_t)tot), r1(tot), r2(tot), c1(3 * (size_t)npairs);
    for (int p = 0; p < npairs; ++p) {
        const int n = natoms[p];
        double s1[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < 3; ++k) {
                const double a = pos1[3 * (size_t)(a0[p] + j) + k], b = pos2[3 * (size_t)(a0[p] + j) + k];
                if (!std::isfinite(a) || !std::isfinite(b)) return bnb_err(ctx, FO_ERR_BAD_ARGS, "pair %d: non-finite coordinate", p);
                s1[k] += a;
                s2[k] += b;
            }
        for (int k = 0; k < 3; ++k) { s1[k] /= n; s2[k] /= n; c1[3 * p + k] = s1[k]; }
        for (int j = 0; j < n; ++j) {
            const size_t q = 3 * (size_t)(a0[p] + j);
            for (int k = 0; k < 3; ++k) { X1[q + k] = pos1[q + k] - s1[k]; X2[q + k] = pos2[q + k] - s2[k]; }
            r1[a0[p] + j] = std::sqrt(X1[q] * X1[q] + X1[q + 1] * X1[q + 1] + X1[q + 2] * X1[q + 2]);
            r2[a0[p] + j] = std::sqrt(X2[q] * X2[q] + X2[q + 1] * X2[q + 1] + X2[q + 2] * X2[q + 2]);
        }
    }
    // device inputs and per-launch buffers for up to maxch children: all the
    // searches' 8 children at once, or fewer launches' worth when the
    // context's HBM budget (caller's, else 80% of the free memory) is smaller
    const long long sstride = bnb_stride(maxn);
    const size_t fixed = (2 * 3 * (size_t)tot + 2 * (size_t)tot) * sizeof(double) + 2 * (size_t)npairs * sizeof(int) +
                         16 * 256;
    const size_t per_child = sizeof(BnbChild) + 4 * sizeof(double) + sizeof(int) + sstride * sizeof(double) + 64;
    size_t budget = fo::ctx_opts(ctx).hbm_budget_bytes;
    if (!budget) {
        size_t fr = 0, tt = 0;
        cudaMemGetInfo(&fr, &tt);
        budget = (size_t)(0.8 * fr);
    }
    if (budget < fixed + 8 * per_child)
        return bnb_err(ctx, FO_ERR_OOM_BUDGET, "branch and bound needs %zu bytes, budget %zu", fixed + 8 * per_child,
                       budget);
    const size_t maxch = std::min(8 * (size_t)npairs, std::max((size_t)8, (budget - fixed) / per_child));
    const size_t bytes = fixed + maxch * per_child;
    unsigned char *dm = nullptr;
    fo_status s = bnb_cuda(ctx, cudaMalloc(&dm, bytes), "cudaMalloc");
    if (s) return s;
    size_t off = 0;
    auto take = [&](size_t b) { void *q = dm + off; off += (b + 255) & ~(size_t)255; return q; };
    double *dX1 = (double *)take(3 * (size_t)tot * sizeof(double)), *dX2 = (double *)take(3 * (size_t)tot * sizeof(double));
    double *dr1 = (double *)take(tot * sizeof(double)), *dr2 = (double *)take(tot * sizeof(double));
    int *da0 = (int *)take(npairs * sizeof(int)), *dn = (int *)take(npairs * sizeof(int));
    BnbChild *dch = (BnbChild *)take(maxch * sizeof(BnbChild));
    double *dout = (double *)take(maxch * 4 * sizeof(double));
    int *dst = (int *)take(maxch * sizeof(int));
    double *dscr = (double *)take(maxch * sstride * sizeof(double));
    (void)bytes;
    cudaStream_t st = fo::ctx_stream(ctx);
    cudaMemcpyAsync(dX1, X1.data(), X1.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dX2, X2.data(), X2.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dr1, r1.data(), r1.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dr2, r2.data(), r2.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(da0, a0.data(), npairs * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dn, natoms, npairs * sizeof(int), cudaMemcpyHostToDevice, st);
    std::vector<BnbChild> ch;
    std::vector<double> vals;
    std::vector<int> stat;
    // every child of ch, in launches of at most maxch; stat[k] != 0 marks a
    // child whose assignment hit its step guard
    auto evaluate = [&]() -> fo_status {
        if (ch.empty()) return FO_OK;
        vals.resize(4 * ch.size());
        stat.resize(ch.size());
        for (size_t c0 = 0; c0 < ch.size(); c0 += maxch) {
            const size_t nc = std::min(maxch, ch.size() - c0);
            cudaMemcpyAsync(dch, ch.data() + c0, nc * sizeof(BnbChild), cudaMemcpyHostToDevice, st);
            launch_bnb_children(dch, (int)nc, dX1, dX2, dr1, dr2, da0, dn, dscr, sstride, dout, dst, st);
            cudaMemcpyAsync(vals.data() + 4 * c0, dout, 4 * nc * sizeof(double), cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(stat.data() + c0, dst, nc * sizeof(int), cudaMemcpyDeviceToHost, st);
            fo_status e = bnb_cuda(ctx, cudaStreamSynchronize(st), "branch and bound");
            if (e) return e;
        }
        return FO_OK;
    };
    std::vector<BnbSearch> S(npairs);
    // start nodes, bounds forced: the assignment bounds with no best yet
    const int nstart = invert ? 2 : 1;
    for (int p = 0; p < npairs; ++p)
        for (int k = 0; k < nstart; ++k) ch.push_back(BnbChild{{0, 0, 0}, 2 * FO_PI, p, k ? -1 : 1});
    s = evaluate();
    for (int p = 0; !s && p < npairs; ++p) {
        for (int k = 0; k < nstart; ++k)
            if (stat[p * nstart + k]) S[p].failed = true;
        if (S[p].failed) {
            S[p].active = false;
            continue;
        }
        BnbNode st0[2];
        for (int k = 0; k < nstart; ++k) {
            const double *v = &vals[4 * (size_t)(p * nstart + k)];
            st0[k] = BnbNode{{0, 0, 0}, 2 * FO_PI, v[2], v[3], k ? -1 : 1};
        }
        S[p].best = st0[0];
        S[p].heap.push(st0[0]);
        for (int k = 1; k < nstart; ++k) {
            if (st0[k].upper < S[p].best.upper) S[p].best = st0[k];
            if (st0[k].lower < S[p].best.upper) S[p].heap.push(st0[k]);
        }
    }
    std::vector<int> owner;
    while (!s) {
        ch.clear();
        owner.clear();
        for (int p = 0; p < npairs; ++p) {
            BnbSearch &q = S[p];
            while (q.active && !q.heap.a.empty()) {
                const BnbNode nd = q.heap.pop();
                ++q.nodes;
                if (nd.lower < q.best.upper - rtol * q.best.upper - atol) {
                    for (int a = 0; a < 2; ++a)   // children in numpy.indices order
                        for (int b = 0; b < 2; ++b)
                            for (int c = 0; c < 2; ++c) {
                                const double h = 0.25 * nd.width;
                                ch.push_back(BnbChild{{(2 * a - 1) * h + nd.rot[0], (2 * b - 1) * h + nd.rot[1],
                                                       (2 * c - 1) * h + nd.rot[2]},
                                                      0.5 * nd.width, p, nd.sign});
                            }
                    owner.push_back(p);
                    break;
                }
            }
            if (q.heap.a.empty() && (owner.empty() || owner.back() != p)) q.active = false;
        }
        if (ch.empty()) break;
        s = evaluate();
        // the sequential decisions, with the best bound as it moves
        for (size_t o = 0; !s && o < owner.size(); ++o) {
            BnbSearch &q = S[owner[o]];
            for (int k = 0; k < 8; ++k)
                if (stat[8 * o + k]) q.failed = true;
            if (q.failed) {   // this search stops; the others go on
                q.active = false;
                continue;
            }
            for (int k = 0; k < 8; ++k) {
                const BnbChild &c = ch[8 * o + k];
                const double *v = &vals[4 * (8 * o + k)];
                BnbNode nd{{c.rot[0], c.rot[1], c.rot[2]}, c.width, 0, 0, c.sign};
                if (v[0] < q.best.upper) {   // full bounds
                    nd.lower = v[2];
                    nd.upper = (v[2] < q.best.upper) ? v[3] : INFINITY;
                } else {                     // nearest-neighbour bounds
                    nd.lower = v[1];
                    nd.upper = v[0];
                }
                if (nd.lower < q.best.upper) {
                    if (nd.upper < q.best.upper) q.best = nd;
                    q.heap.push(nd);
                }
            }
            if (q.nodes > niter) q.active = false;
        }
    }
    cudaFree(dm);
    if (s) return s;
    // outputs: the best node's rotated pos2 on pos1's centroid, in pos2's order
    int nfailed = 0;
    for (int p = 0; p < npairs; ++p) {
        if (nodes) nodes[p] = S[p].nodes;
        if (S[p].failed) {
            ++nfailed;
            dist[p] = NAN;
            if (aligned)
                for (int j = 0; j < 3 * natoms[p]; ++j) aligned[3 * (size_t)a0[p] + j] = NAN;
            continue;
        }
        dist[p] = S[p].best.upper;
        if (aligned) {
            const BnbNode &b = S[p].best;
            const double th = std::sqrt(b.rot[0] * b.rot[0] + b.rot[1] * b.rot[1] + b.rot[2] * b.rot[2]);
            double M[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
            if (th != 0.0) {
                const double x = b.rot[0] / th, y = b.rot[1] / th, z = b.rot[2] / th, cc = std::cos(th),
                             ss = std::sin(th), C = 1 - cc;
                const double xs = x * ss, ys = y * ss, zs = z * ss, xC = x * C, yC = y * C, zC = z * C;
                const double xyC = x * yC, yzC = y * zC, zxC = z * xC;
                const double R[9] = {x * xC + cc, xyC - zs, zxC + ys, xyC + zs, y * yC + cc, yzC - xs,
                                     zxC - ys, yzC + xs, z * zC + cc};
                memcpy(M, R, sizeof M);
            }
            for (int j = 0; j < natoms[p]; ++j) {
                const size_t q = 3 * (size_t)(a0[p] + j);
                for (int k = 0; k < 3; ++k)
                    aligned[q + k] = b.sign * (X2[q] * M[k] + X2[q + 1] * M[3 + k] + X2[q + 2] * M[6 + k]) + c1[3 * p + k];
            }
        }
    }
    if (nfailed)
        return bnb_err(ctx, FO_ERR_LAP_FAILED, "branch and bound: assignment step guard in %d of %d searches",
                       nfailed, npairs);
    return FO_OK;
}

fo_status fo_bnb_cluster(fo_ctx *ctx, const double *pos1, const double *pos2, int natoms, int invert,
                         long long niter, double rtol, double atol, double *dist, double *aligned,
                         long long *nodes) {
    return fo_bnb_cluster_batch(ctx, 1, &natoms, pos1, pos2, invert, niter, rtol, atol, dist, aligned, nodes);
}

}  // extern "C"
