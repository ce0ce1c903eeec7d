// fo_refine.cu -- candidate refinement and selection.
//
// One warp per candidate (pair, orientation, peak): rotate (cluster) or shift
// (bulk) the moved structure by the candidate, then alternate
//   per-group squared distances (60 nearest per row when a group has more
//   than 60 atoms) -> integer costs INT(d^2 * 1e6) -> sparse Jonker-Volgenant
//   assignment -> best rotation (cluster) or mean minimum-image
//   displacement (bulk)
// until no atom changes partner, the distance grows, or 21 tries.  The FP64
// form takes the rotation from the Kearsley matrix as FINDROTATION does; the
// mixed form from Horn's matrix of the 3x3 correlation (the same minimiser),
// with its FP64 work spread one matrix entry per lane.
// Candidates are launched in buckets of equal shared-memory footprint so
// small problems pack many warps per SM; the assignment arrays live in
// shared memory when they fit and in per-candidate global scratch otherwise.
// In the mixed-precision form the costs are not stored: the assignment
// recomputes each one from the FP32 coordinates (float4 per atom) where it
// reads it, which keeps the per-warp footprint small enough for many warps
// per SM.
//
// Reference behaviour (matthewghgriffiths/fastoverlap):
//   ITERATIVEALIGN   fastoverlap/f90/alignutils.f90:111-286
//   FINDBESTPERM     fastoverlap/f90/alignutils.f90:482-580
//   PAIRDISTS        fastoverlap/f90/alignutils.f90:582-730
//   JOVOSAP          fastoverlap/f90/alignutils.f90:989-1259
//   FINDROTATION     fastoverlap/f90/alignutils.f90:304-379
//   FINDDISPLACEMENT fastoverlap/f90/alignutils.f90:381-419
//   ALIGNCOEFFS      fastoverlap/f90/fastclusters.f90:393-470 (candidate loop,
//                    best by distance) and ALIGN :214-254 (inversion choice);
//                    bulk ALIGNCOEFFS fastoverlap/f90/fastbulk.f90:501-565
#include "../../include/fastoverlap_gb300.h"
#include "fo_common.cuh"
#include "fo_kernels.h"
#include "fo_refine.cuh"

#include <cstdint>

// 1: the mixed form runs the augmenting row reduction too (as the FP64 form)
#ifndef FO_MIXED_ARR
#define FO_MIXED_ARR 0
#endif
// 1: dense groups of the mixed form use the register-resident assignment
// (jv_dense_reg) instead of the sequential method's warp form
#ifndef FO_DENSE_REG
#define FO_DENSE_REG 1
#endif

namespace fo {

constexpr unsigned kFull = 0xffffffffu;
constexpr long long kLLMax = 0x7fffffffffffffffLL;
constexpr unsigned long long kNoKey = ~0ull;
// Row scans order entries by the key ((h + kKeyBias) << 6) | t: reduced cost
// h first, scan position t (< 64) second.  Reduced costs are >= 0 (column
// prices only decrease from the column minima) and below BIGINT = 1e12 <
// 2^40 where they enter a key, so the key is exact and below 2^63.
constexpr long long kKeyBias = 1LL << 56;

// Warp minimum of a 64-bit unsigned key: redux on the high words, then on
// the low words of the lanes holding the minimal high word.
__device__ __forceinline__ unsigned long long wmin_u64(unsigned long long k) {
    const unsigned hi = (unsigned)(k >> 32), lo = (unsigned)k;
    const unsigned mh = __reduce_min_sync(kFull, hi);
    const unsigned ml = __reduce_min_sync(kFull, hi == mh ? lo : 0xffffffffu);
    return ((unsigned long long)mh << 32) | ml;
}

// Warp minimum of a signed 64-bit value (sign bit flipped: unsigned order).
__device__ __forceinline__ long long wmin_ll(long long v) {
    const unsigned long long s = 0x8000000000000000ull;
    return (long long)(wmin_u64((unsigned long long)v ^ s) ^ s);
}

// ---------------------------------------------------------------------------
// Squared distances and integer costs in FP32 (mixed form).  Every rounding
// is explicit so that a distance recomputed anywhere equals the one the
// neighbour heap ordered.
__device__ __forceinline__ float d2_f4(const float4 p, const float4 q) {
    const float dx = __fsub_rn(p.x, q.x), dy = __fsub_rn(p.y, q.y), dz = __fsub_rn(p.z, q.z);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// minimum image along one axis of length bk (no wrap when bk == 0)
__device__ __forceinline__ float min_image_f(float t, float bk) {
    return bk != 0.f ? __fsub_rn(t, __fmul_rn(bk, roundf(__fdiv_rn(t, bk)))) : t;
}

// minimum image with the reciprocal box length (mixed form: the costs and the
// neighbour lists of a pair use this same function throughout)
__device__ __forceinline__ float min_image_rcp(float t, float bk, float rk) {
    return bk != 0.f ? __fsub_rn(t, __fmul_rn(bk, rintf(__fmul_rn(t, rk)))) : t;
}

__device__ __forceinline__ float d2_f4_box_rcp(const float4 p, const float4 q, const float *bx,
                                               const float *rx) {
    const float dx = min_image_rcp(__fsub_rn(p.x, q.x), bx[0], rx[0]);
    const float dy = min_image_rcp(__fsub_rn(p.y, q.y), bx[1], rx[1]);
    const float dz = min_image_rcp(__fsub_rn(p.z, q.z), bx[2], rx[2]);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

__device__ __forceinline__ float d2_f4_box(const float4 p, const float4 q, const float *bx) {
    const float dx = min_image_f(__fsub_rn(p.x, q.x), bx[0]);
    const float dy = min_image_f(__fsub_rn(p.y, q.y), bx[1]);
    const float dz = min_image_f(__fsub_rn(p.z, q.z), bx[2]);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// INT(d2 * 1e6) of an FP32 squared distance d2 >= 0, equal to truncating the
// FP64 product (double)d2 * 1e6, without FP64 instructions.  1e6 is exact in
// FP32 and the product splits exactly into hi + lo (hi the rounded FP32
// product, lo its FMA residual).  When hi is an integer the floor of hi + lo
// is hi + floor(lo); otherwise |lo| <= ulp(hi)/2 keeps hi + lo strictly
// between the two integers around hi, so it is floor(hi).  CT = int needs
// d2 * 1e6 < 2^31.
template <typename CT>
__device__ __forceinline__ CT cost_of_f32(float d2) {
    const float hi = __fmul_rn(d2, 1.0e6f);
    const float lo = __fmaf_rn(d2, 1.0e6f, -hi);
    const float fh = floorf(hi);
    if (fh == hi) return (CT)hi + (CT)floorf(lo);
    return (CT)fh;
}

// Cost of row i, scan position t, column j.
// kByColumn: the cost depends on the column only, not on its scan position.
template <typename CT>
struct CostStored {      // costs kept in a row-major table of width m
    static constexpr bool kByColumn = false;
    const CT *cc;
    int m;
    __device__ __forceinline__ long long operator()(int i, int t, int) const { return (long long)cc[i * m + t]; }
};

template <typename CT, bool BOX>
struct CostF32 {         // costs recomputed from FP32 coordinates (minimum image when BOX)
    static constexpr bool kByColumn = true;
    const float4 *b, *a;
    float bx[3], rx[3];  // box lengths and their reciprocals (0 for no wrap)
    __device__ __forceinline__ float d2(int i, int j) const {
        if constexpr (BOX) return d2_f4_box_rcp(b[i], a[j], bx, rx);
        else return d2_f4(b[i], a[j]);
    }
    __device__ __forceinline__ long long operator()(int i, int, int j) const {
        return (long long)cost_of_f32<CT>(d2(i, j));
    }
};

// ---------------------------------------------------------------------------
// Sparse Jonker-Volgenant (Computing 38, 1987) executed by one warp.  The
// sequence of steps -- column reduction, reduction transfer in row order,
// two augmenting-row-reduction passes over the free list, shortest
// augmenting paths -- and every tie rule are those of the sequential method
// (first row wins a column minimum; the lowest scan position wins a row
// minimum; the label list is searched last-in first-out; the first free
// column in scan / index order ends a path).  Only the scans inside a step
// (a row's <= 60 entries, or all columns) are spread over the 32 lanes, so
// the assignment is the one the sequential method produces.  Rows have a
// fixed width m <= 60; dense rows (m == n) have implicit column index t,
// sparse rows the column indices kk.  All lanes must call; returns 0 on
// success, > 0 when the matching fails.
// kARR = false skips the augmenting row reduction: the shortest augmenting
// paths then start from the prices of the reduction transfer.  The result is
// still an optimal assignment (the same one when the optimum is unique); only
// the choice among tied optima may differ from the sequential method.
template <bool kARR, typename KT, typename CF>
__device__ int jv_warp(const int n, const int m, const bool dense, const CF &cost, const KT *__restrict__ kk,
                       long long *v, long long *dd, int *x, int *y, int *lab, int *fr, int *todo,
                       unsigned char *ok) {
    const int lane = threadIdx.x & 31;
    const unsigned ltmask = (1u << lane) - 1u;
    auto COL = [&](int i, int t) -> int { return dense ? t : (int)kk[i * m + t]; };

    // 1. column reduction: v_j = min_i c_ij, the first row attaining it owns j.
    if (dense) {
        // one lane per column, rows in order
        for (int j = lane; j < n; j += 32) {
            long long best = kBigInt;
            int bi = -1;
            for (int i = 0; i < n; ++i) {
                const long long c = cost(i, j, j);
                if (c < best) { best = c; bi = i; }
            }
            v[j] = best;
            y[j] = bi;
        }
    } else {
        // rows in order; a row's columns are distinct, so lanes never collide.
        // The next row's neighbour-list entries are loaded one row ahead.
        for (int j = lane; j < n; j += 32) { v[j] = kBigInt; y[j] = -1; }
        __syncwarp();
        int nx[2];
        for (int q = 0; q < 2; ++q) nx[q] = (lane + 32 * q < m) ? COL(0, lane + 32 * q) : -1;
        for (int i = 0; i < n; ++i) {
            const int cur[2] = {nx[0], nx[1]};
            if (i + 1 < n)
                for (int q = 0; q < 2; ++q) nx[q] = (lane + 32 * q < m) ? COL(i + 1, lane + 32 * q) : -1;
            for (int q = 0; q < 2; ++q) {
                const int t = lane + 32 * q;
                if (t < m) {
                    const int j = cur[q];
                    const long long c = cost(i, t, j);
                    if (c < v[j]) { v[j] = c; y[j] = i; }
                }
            }
            __syncwarp();
        }
    }
    __syncwarp();
    int bad = 0;
    for (int j = lane; j < n; j += 32)
        if (y[j] < 0) bad = 1;
    if (__any_sync(kFull, bad)) return 1;
    for (int i = lane; i < n; i += 32) { x[i] = -1; lab[i] = 0; }
    __syncwarp();
    // columns are visited from the last: a row keeps the highest of its columns
    for (int j = lane; j < n; j += 32) {
        int i = y[j];
        atomicMax(&x[i], j);
        atomicAdd(&lab[i], 1);
    }
    __syncwarp();
    for (int j = lane; j < n; j += 32) {
        int i = y[j];
        if (x[i] != j) y[j] = -1;
    }
    for (int i = lane; i < n; i += 32) ok[i] = (lab[i] > 1);  // row owns several minima
    __syncwarp();

    // 2. reduction transfer, rows in order
    int nfree = 0;
    int nx2[2];
    for (int q = 0; q < 2; ++q) nx2[q] = (lane + 32 * q < m) ? COL(0, lane + 32 * q) : -1;
    for (int i = 0; i < n; ++i) {
        const int cur[2] = {nx2[0], nx2[1]};   // this row's entries; the next row's are loaded ahead
        if (i + 1 < n)
            for (int q = 0; q < 2; ++q) nx2[q] = (lane + 32 * q < m) ? COL(i + 1, lane + 32 * q) : -1;
        const int xi = x[i];
        if (xi < 0) {
            if (lane == 0) fr[nfree] = i;
            ++nfree;
            continue;
        }
        if (ok[i]) continue;
        long long mn = kBigInt;
        for (int q = 0; q < 2; ++q) {
            const int t = lane + 32 * q;
            if (t >= m) continue;
            const int j = cur[q];
            if (j == xi) continue;
            const long long h = cost(i, t, j) - v[j];
            mn = h < mn ? h : mn;
        }
        mn = wmin_ll(mn);
        if (lane == 0) v[xi] -= mn;
        __syncwarp();
    }
    __syncwarp();
    if (nfree == 0) return 0;

    // 3. augmenting row reduction, two passes
    long long guard = 0;
    const long long gmax = 64LL * n * (long long)n * m + 100000;
    int j0 = -1, j1 = -1;
    for (int pass = 0; kARR && pass < 2 && nfree > 0; ++pass) {
        const int l0 = nfree;
        int k = 0;
        nfree = 0;
        while (k < l0) {
            if (++guard > gmax) return 9;
            const int i = fr[k++];
            // the two smallest (h, t) of the row with h < BIGINT, and their count
            unsigned long long k1 = kNoKey, k2 = kNoKey;
            bool val[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int t = lane + 32 * q;
                val[q] = false;
                if (t < m) {
                    const int j = COL(i, t);
                    const long long h = cost(i, t, j) - v[j];
                    if (h < kBigInt) {   // never enters the two smallest
                        val[q] = true;
                        const unsigned long long key = ((unsigned long long)(h + kKeyBias) << 6) | (unsigned)t;
                        if (key < k1) { k2 = k1; k1 = key; }
                        else if (key < k2) k2 = key;
                    }
                }
            }
            const int cnt = __popc(__ballot_sync(kFull, val[0])) + __popc(__ballot_sync(kFull, val[1]));
            const unsigned long long m1 = wmin_u64(k1);
            const unsigned long long m2 = wmin_u64(k1 == m1 ? k2 : k1);   // keys are distinct
            const int t1 = (int)(m1 & 63u), t2 = (int)(m2 & 63u);
            const long long h1 = (long long)(m1 >> 6) - kKeyBias, h2 = (long long)(m2 >> 6) - kKeyBias;
            long long u1, u2;
            if (cnt >= 2) { u1 = h1; u2 = h2; j0 = COL(i, t1); j1 = COL(i, t2); }
            else if (cnt == 1) { u1 = h1; u2 = kBigInt; j1 = j0; j0 = COL(i, t1); }
            else { u1 = kBigInt; u2 = kBigInt; }
            if (j0 < 0) return 2;
            int i0 = y[j0];
            bool reins = false;
            __syncwarp();
            if (u1 < u2) {
                if (lane == 0) v[j0] = v[j0] - u2 + u1;
                reins = (i0 >= 0);
            } else if (i0 >= 0) {
                if (j1 < 0) return 3;
                j0 = j1;
                i0 = y[j1];
                reins = (i0 >= 0);
            }
            if (reins) {
                if (u1 < u2) {
                    --k;
                    if (lane == 0) fr[k] = i0;
                } else {
                    if (lane == 0) fr[nfree] = i0;
                    ++nfree;
                }
            }
            if (lane == 0) { x[i] = j0; y[j0] = i; }
            __syncwarp();
        }
    }

    // 4. shortest augmenting paths for the remaining free rows
    const int l0 = nfree;
    for (int f = 0; f < l0; ++f) {
        for (int j = lane; j < n; j += 32) { ok[j] = 0; dd[j] = kBigInt; }
        __syncwarp();
        const int i0 = fr[f];
        int td = n - 1, k = 0, jend = -1;
        bool price = false;
        long long hl[2];
        int jl[2];
        for (int q = 0; q < 2; ++q) {
            int t = lane + 32 * q;
            hl[q] = kLLMax;
            jl[q] = -1;
            if (t < m) {
                int j = COL(i0, t);
                long long h = cost(i0, t, j) - v[j];
                dd[j] = h;
                lab[j] = i0;
                hl[q] = h;
                jl[q] = j;
            }
        }
        long long mn = wmin_ll(hl[0] < hl[1] ? hl[0] : hl[1]);
        if (mn > kBigInt) mn = kBigInt;
        __syncwarp();
        for (int q = 0; q < 2; ++q) {
            bool sel = (hl[q] == mn);
            unsigned msk = __ballot_sync(kFull, sel);
            if (sel) todo[k + __popc(msk & ltmask)] = jl[q];
            k += __popc(msk);
        }
        __syncwarp();
        for (int b = 0; b < k && jend < 0; b += 32) {   // first free column ends the search
            int h = b + lane, j = (h < k) ? todo[h] : -1;
            bool fre = (h < k) && y[j] < 0;
            unsigned fm = __ballot_sync(kFull, fre);
            if (fm) {
                int first = b + __ffs(fm) - 1;
                if (h < first) ok[j] = 1;
                jend = todo[first];
            } else if (h < k) {
                ok[j] = 1;
            }
        }
        __syncwarp();
        // Neighbour-list entries of the row to be scanned next, loaded one
        // scan ahead: the row of the last column on the label list, which is
        // the next one taken unless the current scan adds columns to it.
        int pf_row = -1, pf_col[2] = {-1, -1};
        while (jend < 0) {
            if (++guard > gmax) return 9;
            if (k == 0) return 4;
            --k;
            const int jc = todo[k];
            const int i = y[jc];
            __syncwarp();
            if (lane == 0) todo[td] = jc;
            --td;
            int rcol[2] = {pf_col[0], pf_col[1]};
            if (!dense && pf_row != i)
                for (int q = 0; q < 2; ++q) rcol[q] = (lane + 32 * q < m) ? COL(i, lane + 32 * q) : -1;
            pf_row = -1;
            if (!dense && k > 0) {
                pf_row = y[todo[k - 1]];
                for (int q = 0; q < 2; ++q) pf_col[q] = (lane + 32 * q < m) ? COL(pf_row, lane + 32 * q) : -1;
            }
            // scan position of jc in row i: jc is the column row i holds, and
            // rows only ever hold columns of their own list
            int tpos = jc;
            if (!CF::kByColumn && !dense) {
                tpos = -1;
                for (int q = 0; q < 2; ++q) {
                    int t = lane + 32 * q;
                    bool hit = (t < m) && COL(i, t) == jc;
                    unsigned hm = __ballot_sync(kFull, hit);
                    if (hm && tpos < 0) tpos = 32 * q + __ffs(hm) - 1;
                }
                if (tpos < 0) return 5;
            }
            const long long hh = cost(i, tpos, jc) - v[jc] - mn;
            bool eq[2];
            int jq[2];
            // every load of the row's entries is issued at once (nothing of
            // these columns is written before the compares below), so the
            // scan waits for one round of shared-memory latency
            bool okq[2];
            long long cq[2], vq[2], dq[2];
            int yq[2];
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int t = lane + 32 * q;
                const bool in = t < m;
                const int j = in ? (dense ? t : rcol[q]) : 0;
                jq[q] = in ? j : -1;
                okq[q] = in ? ok[j] != 0 : true;
                cq[q] = in ? cost(i, t, j) : 0;
                vq[q] = in ? v[j] : 0;
                dq[q] = in ? dd[j] : 0;
                yq[q] = in ? y[j] : 0;
            }
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                eq[q] = false;
                if (!okq[q]) {
                    const long long vj = cq[q] - hh - vq[q];
                    if (vj < dq[q]) {
                        dd[jq[q]] = vj;
                        lab[jq[q]] = i;
                        eq[q] = (vj == mn);
                    }
                }
            }
            __syncwarp();
            for (int q = 0; q < 2 && jend < 0; ++q) {
                bool isf = eq[q] && yq[q] < 0;
                unsigned em = __ballot_sync(kFull, eq[q]), fm = __ballot_sync(kFull, isf);
                unsigned upto = em;
                if (fm) {
                    int fl = __ffs(fm) - 1;
                    upto = em & ((1u << fl) - 1u);
                    jend = __shfl_sync(kFull, jq[q], fl);
                    price = true;
                }
                if (eq[q] && ((upto >> lane) & 1u)) {
                    todo[k + __popc(upto & ltmask)] = jq[q];
                    ok[jq[q]] = 1;
                }
                k += __popc(upto);
            }
            __syncwarp();
            if (jend >= 0) break;
            if (k != 0) continue;
            // next level: the smallest label among the unscanned columns.  One
            // pass keeps each lane's minimum, its first column and its count;
            // a single column at the minimum (the usual case) is taken
            // directly, ties are collected in index order by a second pass.
            long long lm = kLLMax;
            int lj = -1, lc = 0;
#pragma unroll 4
            for (int j = lane; j < n; j += 32) {
                const long long dj = dd[j];
                if (!ok[j] && dj <= kBigInt - 1) {
                    if (dj < lm) { lm = dj; lj = j; lc = 1; }
                    else if (dj == lm) ++lc;
                }
            }
            const long long wm = wmin_ll(lm);
            if (wm == kLLMax) { mn = kBigInt - 1; k = 0; continue; }
            mn = wm;
            const int nat = __reduce_add_sync(kFull, lm == wm ? lc : 0);
            if (nat == 1) {
                const unsigned who = __ballot_sync(kFull, lm == wm);
                const int j1 = __shfl_sync(kFull, lj, __ffs(who) - 1);
                if (lane == 0) todo[0] = j1;
                k = 1;
            } else {
                for (int b = 0; b < n; b += 32) {
                    int j = b + lane;
                    bool sel = (j < n) && !ok[j] && dd[j] == mn;
                    unsigned sm = __ballot_sync(kFull, sel);
                    if (sel) todo[k + __popc(sm & ltmask)] = j;
                    k += __popc(sm);
                }
            }
            __syncwarp();
            for (int b = 0; b < k && jend < 0; b += 32) {
                int h = b + lane, j = (h < k) ? todo[h] : -1;
                bool fre = (h < k) && y[j] < 0;
                unsigned fm = __ballot_sync(kFull, fre);
                if (fm) {
                    int first = b + __ffs(fm) - 1;
                    if (h < first) ok[j] = 1;
                    jend = todo[first];
                    price = true;
                } else if (h < k) {
                    ok[j] = 1;
                }
            }
            __syncwarp();
        }
        if (price && mn != 0)
            for (int q = td + 1 + lane; q < n; q += 32) {
                int jj = todo[q];
                v[jj] += dd[jj] - mn;
            }
        __syncwarp();
        int fail = 0;
        if (lane == 0) {
            int je = jend;
            for (int steps = 0;; ++steps) {
                if (steps > n + 1) { fail = 1; break; }
                int i = lab[je];
                y[je] = i;
                int ks = je;
                je = x[i];
                x[i] = ks;
                if (i == i0) break;
            }
        }
        if (__shfl_sync(kFull, fail, 0)) return 6;
        __syncwarp();
    }
    return 0;
}

// Dense assignment of the mixed form (groups of at most 64 atoms, every
// column in every row), one warp, the columns in registers: lane l owns
// columns l and l + 32 (price, distance label, scanned flag, owning row).
// Column reduction (each column to its cheapest row, a row keeping the
// highest of its columns), then for every free row a Dijkstra search for the
// shortest augmenting path (Jonker & Volgenant, Computing 38, 1987, the
// shortest-path phase): each step is one warp minimum over the unscanned
// columns (lowest column on ties) and one relaxation of the owning row's
// costs by every lane; prices of the scanned columns move by d_j - d_end and
// the path is flipped.  The result is an optimal assignment -- the same one
// as the sequential method's whenever the optimum is unique; only the choice
// among tied optima may differ.  x (shared, n ints) receives row -> column.
// Returns 0, or 4 if a search ends without a free column (cannot happen for a
// complete cost matrix).
template <typename CF>
__device__ int jv_dense_reg(const int n, const CF &cost, int *x) {
    const int lane = threadIdx.x & 31, j0 = lane, j1 = lane + 32;
    const bool has0 = j0 < n, has1 = j1 < n;
    long long v0 = kBigInt, v1 = kBigInt;
    int y0 = -1, y1 = -1;
    for (int i = 0; i < n; ++i) {
        if (has0) { const long long c = cost(i, j0, j0); if (c < v0) { v0 = c; y0 = i; } }
        if (has1) { const long long c = cost(i, j1, j1); if (c < v1) { v1 = c; y1 = i; } }
    }
    for (int i = lane; i < n; i += 32) x[i] = -1;
    __syncwarp();
    if (has0) atomicMax(&x[y0], j0);
    if (has1) atomicMax(&x[y1], j1);
    __syncwarp();
    if (has0 && x[y0] != j0) y0 = -1;
    if (has1 && x[y1] != j1) y1 = -1;
    __syncwarp();
    for (int i0 = 0; i0 < n; ++i0) {
        if (x[i0] >= 0) continue;
        long long d0 = has0 ? cost(i0, j0, j0) - v0 : kLLMax, d1 = has1 ? cost(i0, j1, j1) - v1 : kLLMax;
        int lab0 = i0, lab1 = i0;
        bool sc0 = !has0, sc1 = !has1;
        long long mn = 0;
        int jend = -1;
        for (int step = 0; step <= n; ++step) {
            const unsigned long long k0 = sc0 ? kNoKey : ((unsigned long long)(d0 + kKeyBias) << 6) | (unsigned)j0;
            const unsigned long long k1 = sc1 ? kNoKey : ((unsigned long long)(d1 + kKeyBias) << 6) | (unsigned)j1;
            const unsigned long long km = wmin_u64(k0 < k1 ? k0 : k1);
            if (km == kNoKey) break;
            const int jm = (int)(km & 63u), own = jm & 31;
            const bool hi = jm >= 32;
            mn = (long long)(km >> 6) - kKeyBias;
            const int yj = __shfl_sync(kFull, hi ? y1 : y0, own);
            const long long vj = __shfl_sync(kFull, hi ? v1 : v0, own);
            if (lane == own) {
                if (hi) sc1 = true;
                else sc0 = true;
            }
            if (yj < 0) { jend = jm; break; }
            const long long h = cost(yj, jm, jm) - vj - mn;   // the same on every lane
            if (!sc0) { const long long nd = cost(yj, j0, j0) - v0 - h; if (nd < d0) { d0 = nd; lab0 = yj; } }
            if (!sc1) { const long long nd = cost(yj, j1, j1) - v1 - h; if (nd < d1) { d1 = nd; lab1 = yj; } }
        }
        if (jend < 0) return 4;
        if (has0 && sc0) v0 += d0 - mn;
        if (has1 && sc1) v1 += d1 - mn;
        int j = jend;
        for (int guard = 0; guard <= n; ++guard) {
            const int own = j & 31;
            const bool hi = j >= 32;
            const int i = __shfl_sync(kFull, hi ? lab1 : lab0, own);
            if (lane == own) {
                if (hi) y1 = i;
                else y0 = i;
            }
            const int next = x[i];
            __syncwarp();
            if (lane == 0) x[i] = j;
            __syncwarp();
            if (i == i0) break;
            j = next;
        }
    }
    return 0;
}

__device__ __forceinline__ double wsum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

template <typename DT>
__device__ __forceinline__ DT pdist2(const DT *c1, const DT *c2, int bulk, const double *box) {
    DT d = 0;
    for (int k = 0; k < 3; ++k) {
        DT t = c1[k] - c2[k];
        if (bulk) {
            if (box[k] == 0.0) continue;
            DT bk = (DT)box[k];
            t -= bk * round(t / bk);
        }
        d += t * t;
    }
    return d;
}

// ---------------------------------------------------------------------------
// FP64 building blocks of the mixed form.  GB300 issues FP64 at a small
// fraction of its FP32 rate, and one warp-wide FP64 instruction costs the
// same with one lane active as with 32, so the mixed form counts FP64
// instructions rather than lanes: small matrix work runs one entry per lane,
// sums over the warp are halved level by level, and the eigen-solve iterates
// in FP32 with one FP64 correction.

template <int N>
__host__ __device__ constexpr unsigned long long pack_nibbles(const int (&a)[N]) {
    unsigned long long r = 0;
    for (int i = 0; i < N; ++i) r |= (unsigned long long)(a[i] & 15) << (4 * i);
    return r;
}
template <int N>
__host__ __device__ constexpr unsigned pack_flags(const int (&a)[N]) {
    unsigned r = 0;
    for (int i = 0; i < N; ++i) r |= (a[i] ? 1u : 0u) << i;
    return r;
}
__device__ __forceinline__ int nibble(unsigned long long t, int i) { return (int)((t >> (4 * i)) & 15); }
__device__ __forceinline__ bool flag(unsigned t, int i) { return (t >> i) & 1u; }

// x or -x, by the sign bit (an integer instruction).
__device__ __forceinline__ double flip_sign(double x, bool s) {
    return __hiloint2double(__double2hiint(x) ^ (s ? (int)0x80000000 : 0), __double2loint(x));
}

// Warp sum of M doubles per lane by recursive halving: at each butterfly
// level a lane keeps half of its values and adds its partner's copy of that
// half, ceil(M/2) + ceil(M/4) + ... additions in all instead of 5M.  Value k's
// total ends in v[0] of lane halve_lane(k, M) (and of the lanes that differ
// from it only in levels where one value was left).
__host__ __device__ constexpr int halve_lane(int k, int m) {
    int lane = 0;
    for (int o = 16; o > 0; o >>= 1) {
        if (m == 1) continue;
        const int h = (m + 1) / 2;
        if (k >= h) { lane |= o; k -= h; }
        m = h;
    }
    return lane;
}
template <int M, int O = 16>
__device__ __forceinline__ void warp_halve(double *v, int lane) {
    if constexpr (O > 0) {
        if constexpr (M == 1) {
            v[0] += __shfl_xor_sync(kFull, v[0], O);
            warp_halve<1, O / 2>(v, lane);
        } else {
            constexpr int H = (M + 1) / 2;
            const bool up = (lane & O) != 0;
#pragma unroll
            for (int i = 0; i < H; ++i) {
                const double lo = v[i], hi = (H + i < M) ? v[H + i] : 0.0;
                v[i] = (up ? hi : lo) + __shfl_xor_sync(kFull, up ? lo : hi, O);
            }
            warp_halve<H, O / 2>(v, lane);
        }
    }
}

// Cyclic Jacobi rotations (Golub & Van Loan 8.5) on a symmetric 4x4 FP32
// matrix scaled to unit largest element; a sweep in which every off-diagonal
// element is at most 2^-22 ends it.  Columns of V are the eigenvectors.  The
// rotation angles use the hardware reciprocal and reciprocal square root: the
// result only starts the FP64 correction, and every rotation is orthogonal
// to FP32 rounding whatever its angle.
__device__ __forceinline__ void jacobi4f(float (&a)[4][4], float (&V)[4][4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) V[i][j] = (i == j) ? 1.f : 0.f;
    for (int sweep = 0; sweep < 16; ++sweep) {
        bool rotated = false;
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
            for (int r = p + 1; r < 4; ++r) {
                const float apr = a[p][r];
                if (fabsf(apr) <= 2.384185791015625e-7f) continue;
                rotated = true;
                // |apr| > 2^-22 and |a| <= ~2 keep |theta| below 2^23
                const float theta = __fdividef(a[r][r] - a[p][p], 2.f * apr);
                const float th2 = fmaf(theta, theta, 1.f);
                const float t = __fdividef(copysignf(1.f, theta), fabsf(theta) + th2 * rsqrtf(th2));
                const float c = rsqrtf(fmaf(t, t, 1.f)), s = t * c;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float akp = a[k][p], akr = a[k][r];
                    a[k][p] = c * akp - s * akr;
                    a[k][r] = s * akp + c * akr;
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float apk = a[p][k], ark = a[r][k];
                    a[p][k] = c * apk - s * ark;
                    a[r][k] = s * apk + c * ark;
                }
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float vkp = V[k][p], vkr = V[k][r];
                    V[k][p] = c * vkp - s * vkr;
                    V[k][r] = s * vkp + c * vkr;
                }
            }
        if (!rotated) break;
    }
}

// Horn's matrix (J. Opt. Soc. Am. A 4, 629 (1987)) of H = sum_j a_j b_j^T,
// H[3p+q] = sum a_p b_q: the best rotation (b ~ R a) is the unit quaternion
// of N's largest eigenvalue mu, and min_R sum |b - R a|^2 = S - 2 mu with
// S = sum |a|^2 + |b|^2 -- the minimiser of the Kearsley matrix of
// FINDROTATION (alignutils.f90:304-379), which is S I - 2 N up to the order
// and signs of the quaternion components.  Upper-triangle entry e (row-major)
// is +-H[i0] +- H[i1] (+- H[i2]).
constexpr int kHornI0[10] = {0, 5, 6, 1, 0, 1, 6, 0, 5, 0};
constexpr int kHornI1[10] = {4, 7, 2, 3, 4, 3, 2, 4, 7, 4};
constexpr int kHornI2[10] = {8, 0, 0, 0, 8, 0, 0, 8, 0, 8};
constexpr int kHornNeg0[10] = {0, 0, 0, 0, 0, 0, 0, 1, 0, 1};
constexpr int kHornNeg1[10] = {0, 1, 1, 1, 1, 0, 0, 0, 0, 1};
constexpr int kHornNeg2[10] = {0, 0, 0, 0, 1, 0, 0, 1, 0, 0};
constexpr int kHornHas2[10] = {1, 0, 0, 0, 1, 0, 0, 1, 0, 1};
// upper-triangle index of element (i, j) of a symmetric 4x4, row-major over (i, j)
constexpr int kSym4[16] = {0, 1, 2, 3, 1, 4, 5, 6, 2, 5, 7, 8, 3, 6, 8, 9};
// rotation matrix of quaternion q (row-major entry k, |q| = 1):
// 2 (q[qa] q[qb] +- q[qc] q[qd]) - (1 on the diagonal)
constexpr int kQuatA[9] = {0, 1, 1, 1, 0, 2, 1, 2, 0};
constexpr int kQuatB[9] = {0, 2, 3, 2, 0, 3, 3, 3, 0};
constexpr int kQuatC[9] = {1, 0, 0, 0, 2, 0, 0, 0, 3};
constexpr int kQuatD[9] = {1, 3, 2, 3, 2, 1, 2, 1, 3};
constexpr int kQuatNeg[9] = {0, 1, 0, 0, 0, 1, 1, 0, 0};
constexpr int kQuatDiag[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
// the tables packed into integer constants for device code
constexpr unsigned long long kHornI0p = pack_nibbles(kHornI0), kHornI1p = pack_nibbles(kHornI1),
                             kHornI2p = pack_nibbles(kHornI2), kSym4p = pack_nibbles(kSym4),
                             kQuatAp = pack_nibbles(kQuatA), kQuatBp = pack_nibbles(kQuatB),
                             kQuatCp = pack_nibbles(kQuatC), kQuatDp = pack_nibbles(kQuatD);
constexpr unsigned kHornNeg0p = pack_flags(kHornNeg0), kHornNeg1p = pack_flags(kHornNeg1),
                   kHornNeg2p = pack_flags(kHornNeg2), kHornHas2p = pack_flags(kHornHas2),
                   kQuatNegp = pack_flags(kQuatNeg), kQuatDiagp = pack_flags(kQuatDiag);

// Euler rotation matrix (entry k, row-major) from sF = {cos a, sin a, cos b,
// sin b, cos g, sin g, 1, 0}: +-sF[x] sF[y] sF[z] +- sF[u] sF[w], the matrix of
// euler_matrix.
constexpr int kEulerX[9] = {4, 5, 3, 4, 5, 3, 4, 5, 2};
constexpr int kEulerY[9] = {2, 2, 0, 2, 2, 1, 3, 3, 6};
constexpr int kEulerZ[9] = {0, 0, 6, 1, 1, 6, 6, 6, 6};
constexpr int kEulerU[9] = {5, 4, 7, 5, 4, 7, 7, 7, 7};
constexpr int kEulerW[9] = {1, 1, 7, 0, 0, 7, 7, 7, 7};
constexpr int kEulerNeg1[9] = {0, 0, 0, 1, 1, 1, 1, 1, 0};
constexpr int kEulerNeg2[9] = {1, 0, 0, 1, 0, 0, 0, 0, 0};
constexpr unsigned long long kEulerXp = pack_nibbles(kEulerX), kEulerYp = pack_nibbles(kEulerY),
                             kEulerZp = pack_nibbles(kEulerZ), kEulerUp = pack_nibbles(kEulerU),
                             kEulerWp = pack_nibbles(kEulerW);
constexpr unsigned kEulerNeg1p = pack_flags(kEulerNeg1), kEulerNeg2p = pack_flags(kEulerNeg2);

__device__ __forceinline__ double sel3(double a0, double a1, double a2, int i) {
    return (i == 0) ? a0 : (i == 1) ? a1 : a2;
}

// Best rotation of the moved atoms onto the fixed ones from this lane's
// partial sums h of H (destroyed) and S.  FP32 Jacobi gives N's top
// eigenpair (v0, mu0); one correction in the FP32 eigenbasis from the FP64
// residual r = (N - mu0) v0, v1 = v0 + sum_k V_k (V_k . r) / (mu0 - mu_k),
// brings v1 to FP64 accuracy, and the FP64 Rayleigh quotient of v1 gives
// mu.  Writes R (row-major) to sR[0..8] and returns sqrt(S - 2 mu) (the
// clamp of a negative value as in the Kearsley solution) to every lane.
__device__ double horn_rotation(double (&h)[9], const double S, const int lane, double *sR) {
    constexpr unsigned long long kHL9 = (unsigned long long)halve_lane(0, 9) | ((unsigned long long)halve_lane(1, 9) << 5) |
                                        ((unsigned long long)halve_lane(2, 9) << 10) | ((unsigned long long)halve_lane(3, 9) << 15) |
                                        ((unsigned long long)halve_lane(4, 9) << 20) | ((unsigned long long)halve_lane(5, 9) << 25) |
                                        ((unsigned long long)halve_lane(6, 9) << 30) | ((unsigned long long)halve_lane(7, 9) << 35) |
                                        ((unsigned long long)halve_lane(8, 9) << 40);
    warp_halve<9>(h, lane);
    auto hsrc = [](int k) { return (int)((kHL9 >> (5 * k)) & 31); };
    // entry e = lane of N (lanes 10-31 repeat entry 0)
    const int e = lane < 10 ? lane : 0;
    const double h0 = __shfl_sync(kFull, h[0], hsrc(nibble(kHornI0p, e)));
    const double h1 = __shfl_sync(kFull, h[0], hsrc(nibble(kHornI1p, e)));
    const double h2 = __shfl_sync(kFull, h[0], hsrc(nibble(kHornI2p, e)));
    const double t2 = flag(kHornHas2p, e) ? flip_sign(h2, flag(kHornNeg2p, e)) : 0.0;
    const double ne = (flip_sign(h0, flag(kHornNeg0p, e)) + flip_sign(h1, flag(kHornNeg1p, e))) + t2;
    // FP32 eigen-decomposition, every lane the same
    const float nf = (float)ne;
    float a[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = i; j < 4; ++j) a[i][j] = a[j][i] = __shfl_sync(kFull, nf, nibble(kSym4p, 4 * i + j));
    float mx = 0.f;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = i; j < 4; ++j) mx = fmaxf(mx, fabsf(a[i][j]));
    if (!(mx > 0.f)) {   // H = 0: every rotation is optimal
        if (lane < 9) sR[lane] = (lane % 4 == 0) ? 1.0 : 0.0;
        __syncwarp();
        return sqrt(fmax(S, 0.0));
    }
    const float sc = 1.f / mx;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) a[i][j] *= sc;
    float V[4][4];
    jacobi4f(a, V);
    float mu[4], v0[4];
    int jm = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        mu[k] = a[k][k] * mx;
        if (k > 0 && mu[k] > mu[jm]) jm = k;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        v0[i] = V[i][0];
#pragma unroll
        for (int k = 1; k < 4; ++k)
            if (k == jm) v0[i] = V[i][k];
    }
    const float mu0f = (jm == 0) ? mu[0] : (jm == 1) ? mu[1] : (jm == 2) ? mu[2] : mu[3];
    // FP64 residual, lane i (mod 4) computes component i
    const int i = lane & 3;
    const double vd = (double)((i == 0) ? v0[0] : (i == 1) ? v0[1] : (i == 2) ? v0[2] : v0[3]);
    double vj[4], nr[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        vj[j] = __shfl_sync(kFull, vd, j);
        nr[j] = __shfl_sync(kFull, ne, nibble(kSym4p, 4 * i + j));
    }
    double r = nr[0] * vj[0];
    r = fma(nr[1], vj[1], r);
    r = fma(nr[2], vj[2], r);
    r = fma(nr[3], vj[3], r);
    r = fma(flip_sign((double)mu0f, true), vd, r);
    const float rf = (float)r;
    float rr[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) rr[j] = __shfl_sync(kFull, rf, j);
    // correction in the FP32 eigenbasis (components with no gap are left out)
    float d[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float gap = mu0f - mu[k];
        if (k == jm || !(gap > 1e-6f * mx)) continue;
        const float cf = (V[0][k] * rr[0] + V[1][k] * rr[1] + V[2][k] * rr[2] + V[3][k] * rr[3]) / gap;
#pragma unroll
        for (int j = 0; j < 4; ++j) d[j] = fmaf(cf, V[j][k], d[j]);
    }
    if (!(d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3] < 1e-6f))   // no contraction
        d[0] = d[1] = d[2] = d[3] = 0.f;
    const double v1 = vd + (double)((i == 0) ? d[0] : (i == 1) ? d[1] : (i == 2) ? d[2] : d[3]);
#pragma unroll
    for (int j = 0; j < 4; ++j) vj[j] = __shfl_sync(kFull, v1, j);
    double nv = nr[0] * vj[0];
    nv = fma(nr[1], vj[1], nv);
    nv = fma(nr[2], vj[2], nv);
    nv = fma(nr[3], vj[3], nv);
    // v1.N v1 on even lanes, |v1|^2 on odd lanes of each group of 4
    const bool odd = lane & 1;
    const double t = v1 * nv, w = v1 * v1;
    double x = (odd ? w : t) + __shfl_xor_sync(kFull, odd ? t : w, 1);
    x += __shfl_xor_sync(kFull, x, 2);
    const double num = __shfl_sync(kFull, x, 0), den = __shfl_sync(kFull, x, 1);
    const double inv = 1.0 / den;
    double lam = fma(-2.0, num * inv, S);
    if (lam < 0.0) lam = (fabs(lam) < 1e-6) ? 0.0 : -lam;
    // rotation matrix, entry k on lane k
    const int k = lane < 9 ? lane : 0;
    auto q = [&](int c) { return (c == 0) ? vj[0] : (c == 1) ? vj[1] : (c == 2) ? vj[2] : vj[3]; };
    double p = q(nibble(kQuatAp, k)) * q(nibble(kQuatBp, k));
    p = fma(flip_sign(q(nibble(kQuatCp, k)), flag(kQuatNegp, k)),
            q(nibble(kQuatDp, k)), p);
    const double Rk = fma(inv + inv, p, flag(kQuatDiagp, k) ? -1.0 : 0.0);
    if (lane < 9) sR[lane] = Rk;
    __syncwarp();
    return sqrt(lam);
}

// sRb <- sRn sRb (lanes 0-8); then the affine map of the input coordinates
// that gives the moved structure, x -> T x + t with T = sRb sRs and
// t = add - sRb ca, into sT[0..8] (T, row-major) and sT[9..11] (t).
__device__ __forceinline__ void compose_affine(const double *sRn, double *sRb, const double *sRs, const double (&nca)[3],
                                               const double (&add)[3], double *sT, const int lane) {
    const int k = lane < 9 ? lane : 0, r = k / 3, c = k % 3;
    double v = sRn[3 * r] * sRb[c];
    v = fma(sRn[3 * r + 1], sRb[3 + c], v);
    v = fma(sRn[3 * r + 2], sRb[6 + c], v);
    __syncwarp();
    if (lane < 9) sRb[lane] = v;
    __syncwarp();
    const bool tl = lane >= 9;   // lanes 9-11: translation
    const int rr = tl ? ((lane < 12) ? lane - 9 : 0) : r;
    const double x0 = tl ? nca[0] : sRs[c], x1 = tl ? nca[1] : sRs[3 + c], x2 = tl ? nca[2] : sRs[6 + c];
    double w = fma(sRb[3 * rr], x0, tl ? sel3(add[0], add[1], add[2], rr) : 0.0);
    w = fma(sRb[3 * rr + 1], x1, w);
    w = fma(sRb[3 * rr + 2], x2, w);
    if (lane < 12) sT[lane] = w;
    __syncwarp();
}

// The m nearest columns of one row as the binary max-heap of PAIRDISTS
// (alignutils.f90:641-701): the first m columns are sifted up in order, each
// later closer column replaces the root and is sifted down.  The heap's array
// order is the stored order of the row.  dist(j) is the squared distance to
// column j.
template <typename DT, typename KT, typename DF>
__device__ __forceinline__ void nearest_heap(DT *hd, KT *hk, int ns, int m, const DF &dist) {
    // sift-up and sift-down move a hole instead of swapping: the same
    // comparisons and the same final array as element swaps, one store each
    for (int j = 0; j < m; ++j) {
        const DT d = dist(j);
        int l = j + 1;
        while (l > 1) {
            const int l2 = l / 2;
            const DT p = hd[l2 - 1];
            if (!(p < d)) break;
            hd[l - 1] = p;
            hk[l - 1] = hk[l2 - 1];
            l = l2;
        }
        hd[l - 1] = d;
        hk[l - 1] = (KT)j;
    }
    DT root = hd[0];
    for (int j = m; j < ns; ++j) {
        const DT d = dist(j);
        if (!(d < root)) continue;
        DT nroot = d;
        int l = 1;
        for (int guard = 0; guard < 64; ++guard) {
            const int l2 = 2 * l;
            if (l2 + 1 > m) {
                if (l2 <= m) {
                    const DT c = hd[l2 - 1];
                    if (c > d) {
                        hd[l - 1] = c;
                        hk[l - 1] = hk[l2 - 1];
                        if (l == 1) nroot = c;
                        l = l2;
                    }
                }
                break;
            }
            const DT c0 = hd[l2 - 1], c1 = hd[l2];
            const bool right = c1 > c0;
            const int a = right ? l2 + 1 : l2;
            const DT ca = right ? c1 : c0;
            if (!(ca > d)) break;
            hd[l - 1] = ca;
            hk[l - 1] = hk[a - 1];
            if (l == 1) nroot = ca;
            l = a;
        }
        hd[l - 1] = d;
        hk[l - 1] = (KT)j;
        root = nroot;
    }
}

// The m nearest columns of each lane's own row (mixed form, rows of at most
// kHeapMaxRow columns, 32 rows at once): the m smallest squared distances
// dist(j), j < ns (m < ns), as column indices in increasing order, ties at
// the m-th value to the lowest indices; the same set as the PAIRDISTS heap
// whenever the m-th and (m+1)-th distances differ.  Each lane bisects on the
// bit patterns of its row's distances (recomputed per pass; all lanes read
// the same column at a time) until a threshold has exactly m distances below
// it, starting from the bracket [0.99 thr, 1.01 thr] of its previous m-th
// distance when warm, and stores the new one.  Replaces a heap per lane,
// whose sift steps cost several times more.
template <typename KT, typename DF>
__device__ void nearest_lane(KT *krow, const int ns, const int m, const DF &dist, float *thr, bool warm) {
    auto count_below = [&](unsigned t) -> int {
        int c = 0;
#pragma unroll 4
        for (int j = 0; j < ns; ++j) c += __float_as_uint(dist(j)) < t;
        return c;
    };
    unsigned lo = 0, hi = 0x7f800000u, v = 0;
    bool exact = false;
    const float g = warm ? *thr : 0.f;
    if (g <= 0.f) {   // cold: bisect between the row's smallest and largest distance
        unsigned mn = 0x7f800000u, mx = 0;
#pragma unroll 4
        for (int j = 0; j < ns; ++j) {
            const unsigned u = __float_as_uint(dist(j));
            mn = min(mn, u);
            mx = max(mx, u);
        }
        lo = mn;                            // count(< mn) = 0 <= m
        hi = mx < 0x7f800000u ? mx + 1 : mx;   // count(< mx + 1) = ns > m
    } else {
        const unsigned a = __float_as_uint(g * 0.99f), b = __float_as_uint(g * 1.01f);
        const int ca = count_below(a);
        if (ca == m) { exact = true; v = a; }
        else if (ca > m) hi = a;
        else {
            lo = a;
            const int cb = count_below(b);
            if (cb == m) { exact = true; v = b; }
            else if (cb > m) hi = b;
            else lo = b;
        }
    }
    while (!exact && hi - lo > 1u) {
        const unsigned mid = lo + (hi - lo) / 2u;
        const int c = count_below(mid);
        if (c == m) { exact = true; v = mid; }
        else if (c < m) lo = mid;
        else hi = mid;
    }
    int need_eq = 0;
    if (!exact) {   // lo is the m-th smallest: ties at lo, lowest index first
        v = lo;
        need_eq = m - count_below(v);
    }
    *thr = __uint_as_float(v);
    int out = 0;
    for (int j = 0; j < ns && out < m; ++j) {
        const unsigned u = __float_as_uint(dist(j));
        if (u < v || (u == v && need_eq > 0)) {
            if (u == v) --need_eq;
            krow[out++] = (KT)j;
        }
    }
}

// The m nearest columns of one row (mixed form): the m smallest squared
// distances dist(j), j < ns (m < ns), as column indices in increasing order;
// ties at the m-th value go to the lowest indices.  The whole warp works on
// the row: the distances go to the scratch d (ns floats) unless they fit in
// registers, and the m-th smallest is found by bisection on their bit
// patterns (non-negative floats order like their bits) with warp-wide counts,
// keeping count(< lo) <= m < count(< hi); it stops as soon as a threshold has
// exactly m distances below it.  The chosen columns are compacted in column
// order.  It picks the same set as the PAIRDISTS heap whenever the m-th and
// (m+1)-th distances differ; the order within the row only decides between
// tied optimal assignments.
// thr (optional): this row's m-th distance from the previous call; with warm
// set, the bisection starts from the bracket [0.99 thr, 1.01 thr], which
// usually holds the new m-th distance (the structures move little between
// iterations) and gives the same result in a few counts instead of ~20.  The
// new m-th distance (or exact threshold) is stored back.
// Rows of up to 32*kNearReg columns keep their distances in registers.
constexpr int kNearReg = 16;

template <typename KT, int NR, typename DF>
__device__ void nearest_warp(KT *krow, float *d, const int ns, const int m, const DF &dist, float *thr = nullptr,
                             bool warm = false) {
    const int lane = threadIdx.x & 31;
    const unsigned ltmask = (1u << lane) - 1u;
    const bool inreg = ns <= 32 * NR;
    unsigned r[NR];   // bit patterns of columns lane + 32k (all ones beyond ns)
#pragma unroll
    for (int k = 0; k < NR; ++k) {
        const int j = lane + 32 * k;
        r[k] = (inreg && j < ns) ? __float_as_uint(dist(j)) : 0xffffffffu;
    }
    if (!inreg)
        for (int j = lane; j < ns; j += 32) d[j] = dist(j);
    __syncwarp();
    auto count_below = [&](unsigned t) -> int {
        int c = 0;
        if (inreg) {
#pragma unroll
            for (int k = 0; k < NR; ++k) c += r[k] < t;
        } else {
            for (int j = lane; j < ns; j += 32) c += __float_as_uint(d[j]) < t;
        }
        return (int)__reduce_add_sync(kFull, (unsigned)c);
    };
    unsigned lo = 0, hi = 0x7f800000u, v = 0;   // count(< 0) = 0 <= m < ns = count(< +inf)
    bool exact = false;
    const float g = (thr && warm) ? *thr : 0.f;
    if (g > 0.f) {
        const unsigned a = __float_as_uint(g * 0.99f), b = __float_as_uint(g * 1.01f);
        const int ca = count_below(a);
        if (ca == m) { exact = true; v = a; }
        else if (ca > m) hi = a;
        else {
            lo = a;
            const int cb = count_below(b);
            if (cb == m) { exact = true; v = b; }
            else if (cb > m) hi = b;
            else lo = b;
        }
    }
    while (!exact && hi - lo > 1u) {
        const unsigned mid = lo + (hi - lo) / 2u;
        const int c = count_below(mid);
        if (c == m) { exact = true; v = mid; }
        else if (c < m) lo = mid;
        else hi = mid;
    }
    int need_eq = 0, out = 0;
    if (!exact) {   // lo is the m-th smallest: ties at lo, lowest index first
        v = lo;
        need_eq = m - count_below(v);
    }
    if (thr && lane == 0) *thr = __uint_as_float(v);
    for (int b0 = 0; b0 < ns; b0 += 32) {
        const int j = b0 + lane;
        unsigned u = 0xffffffffu;
        if (inreg) {
#pragma unroll
            for (int k = 0; k < NR; ++k)
                if (b0 == 32 * k) u = r[k];
        } else if (j < ns) {
            u = __float_as_uint(d[j]);
        }
        const unsigned em = __ballot_sync(kFull, u == v);
        const bool sel = u < v || (u == v && __popc(em & ltmask) < need_eq);
        const unsigned sm = __ballot_sync(kFull, sel);
        if (sel) krow[out + __popc(sm & ltmask)] = (KT)j;
        out += __popc(sm);
        need_eq -= min(need_eq, __popc(em));
    }
    __syncwarp();
}

// Neighbour-list work of one group handed from the first warp of a
// multi-warp block to the others (shared memory; mixed form).
struct NbrCmd {
    int op;                  // 1: rows of this group; 0: the candidate is done
    int ns, m, warm;
    const float4 *b4, *a4;   // the group's FP32 coordinates
    void *kk;                // its neighbour lists (ns rows of m)
    float *thr;              // its rows' last m-th distances
    float bx[3], rx[3];      // box lengths and reciprocals (0: no wrap)
};

__device__ __forceinline__ void named_bar(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Rows w, w + nw, ... of the group in cmd, one row per warp at a time.
template <typename KT, bool BOX>
__device__ void nbr_rows(const NbrCmd &cmd, int w, int nw) {
    const CostF32<int, BOX> cf{cmd.b4, cmd.a4, {cmd.bx[0], cmd.bx[1], cmd.bx[2]}, {cmd.rx[0], cmd.rx[1], cmd.rx[2]}};
    KT *kk = (KT *)cmd.kk;
    for (int i = w; i < cmd.ns; i += nw)
        nearest_warp<KT, kNearRegMW>(kk + (size_t)i * cmd.m, nullptr, cmd.ns, cmd.m, [&](int j) { return cf.d2(i, j); },
                                     cmd.thr + i, cmd.warm != 0);
}

// The warps after the first of a multi-warp block: wait for neighbour-list
// work (barrier 1), do their rows, report them done (barrier 2), until the
// first warp posts op 0.  The first warp passes barrier 1 exactly once per
// command it posts and once more with op 0 before it finishes the candidate.
template <bool BOX>
__device__ void nbr_helper(volatile NbrCmd *cmdv, int kkbytes) {
    const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (;;) {
        named_bar(1, blockDim.x);
        if (cmdv->op == 0) return;
        const NbrCmd &cmd = *(const NbrCmd *)cmdv;
        if (kkbytes == 1) nbr_rows<uint8_t, BOX>(cmd, w, nw);
        else nbr_rows<uint16_t, BOX>(cmd, w, nw);
        named_bar(2, blockDim.x);
    }
}

// Coordinates of one permutation group as the assignment sees them: rows are
// atoms of the fixed structure, columns atoms of the moved one.
struct GroupCoords {
    const double *xb;        // fixed structure as input (3 per atom)
    double cmb[3];           // its centroid (cluster) or 0 (bulk)
    const double *A;         // moved structure, FP64 (3 per atom)
    const float4 *B4, *A4;   // FP32 copies (mixed form)
    int bulk;
    double box[3];
    float bxf[3], rxf[3];    // FP32 box lengths and reciprocals (0: no wrap)
    // fixed-structure atom i as ITERATIVEALIGN holds it (centred for clusters)
    __device__ __forceinline__ void b(int i, double *o) const {
        for (int k = 0; k < 3; ++k) o[k] = xb[3 * i + k] - cmb[k];
    }
};

// Neighbour lists / costs of one group, then its assignment (PAIRDISTS +
// JOVOSAP for one group).  Returns the assignment's status.
template <typename KT, typename DT, typename CT, bool RECOMP, bool BOX>
__device__ int assign_group(const int ns, const int m, const GroupCoords &G, unsigned char *lb, unsigned char *lbk,
                            const RefLayout &L, float *thr = nullptr, bool warm = false, NbrCmd *cmd = nullptr,
                            int *frg = nullptr) {
    const int lane = threadIdx.x & 31;
    const bool dense = (m == ns);
    constexpr bool kF32 = sizeof(DT) == 4;   // mixed form: no augmenting row reduction
    KT *kk = (KT *)(lbk + L.lap_kk);
    long long *v = (long long *)(lb + L.lap_v), *dd = (long long *)(lb + L.lap_d);
    int *x = (int *)(lb + L.lap_x), *y = (int *)(lb + L.lap_y), *lab = (int *)(lb + L.lap_lab);
    int *fr = frg ? frg : (int *)(lb + L.lap_fr), *todo = (int *)(lb + L.lap_todo);   // frg: free list in global scratch
    unsigned char *ok = lb + L.lap_ok;
    if constexpr (RECOMP) {
        auto run = [&](const auto &cf) {
            if (!dense) {
                if (cmd && thr && ns <= 32 * kNearRegMW) {
                    // every warp of the block on its own rows (the first warp is
                    // the caller); in multi-warp blocks this serves the smaller
                    // sparse groups of the pair as well
                    if (lane == 0) {
                        cmd->op = 1;
                        cmd->ns = ns;
                        cmd->m = m;
                        cmd->warm = warm ? 1 : 0;
                        cmd->b4 = cf.b;
                        cmd->a4 = cf.a;
                        cmd->kk = kk;
                        cmd->thr = thr;
                        for (int k = 0; k < 3; ++k) { cmd->bx[k] = cf.bx[k]; cmd->rx[k] = cf.rx[k]; }
                    }
                    __syncwarp();
                    named_bar(1, blockDim.x);
                    nbr_rows<KT, BOX>(*cmd, 0, blockDim.x >> 5);
                    named_bar(2, blockDim.x);
                } else if (ns <= kHeapMaxRow) {   // one row per lane (32 rows at once)
                    for (int i = lane; i < ns; i += 32)
                        nearest_lane<KT>(kk + i * m, ns, m, [&](int j) { return cf.d2(i, j); }, thr + i, warm);
                } else {   // the warp on one row at a time, from the row's last m-th distance when warm
                    float *dr = (float *)(lb + L.lap_heap);
                    for (int i = 0; i < ns; ++i)
                        nearest_warp<KT, kNearReg>(kk + i * m, dr, ns, m, [&](int j) { return cf.d2(i, j); },
                                                   thr ? thr + i : nullptr, warm);
                }
            }
            __syncwarp();
#if FO_DENSE_REG
            if (dense && ns <= 64) return jv_dense_reg(ns, cf, x);
#endif
            return jv_warp<!kF32 || FO_MIXED_ARR, KT>(ns, m, dense, cf, kk, v, dd, x, y, lab, fr, todo, ok);
        };
        return run(CostF32<CT, BOX>{G.B4, G.A4, {G.bxf[0], G.bxf[1], G.bxf[2]}, {G.rxf[0], G.rxf[1], G.rxf[2]}});
    } else {
        CT *cc = (CT *)(lbk + L.lap_cc);
        // squared distance of row i (bi: its FP64 coordinates) and column j
        auto dist = [&](int i, const double *bi, int j) -> DT {
            if constexpr (kF32)
                return G.bulk ? d2_f4_box(G.B4[i], G.A4[j], G.bxf) : d2_f4(G.B4[i], G.A4[j]);
            else
                return pdist2<double>(bi, G.A + 3 * j, G.bulk, G.box);
        };
        auto cost = [&](DT d) -> CT {
            if constexpr (kF32) return cost_of_f32<CT>(d);
            else return (CT)(d * kPScale);
        };
        if (dense) {
            // lanes over columns: conflict-free row stores
            for (int i = 0; i < ns; ++i) {
                double bi[3] = {0, 0, 0};
                if constexpr (!kF32) G.b(i, bi);
                for (int j = lane; j < ns; j += 32) cc[i * m + j] = cost(dist(i, bi, j));
            }
        } else if constexpr (sizeof(DT) <= sizeof(CT)) {
            // heap kept in place: distances in the row's cost slots, then
            // converted from the last slot down (a slot is never overwritten
            // before it is read)
            for (int i = lane; i < ns; i += 32) {
                double bi[3] = {0, 0, 0};
                if constexpr (!kF32) G.b(i, bi);
                CT *crow = cc + i * m;
                DT *hd = reinterpret_cast<DT *>(crow);
                nearest_heap<DT, KT>(hd, kk + i * m, ns, m, [&](int j) { return dist(i, bi, j); });
                for (int j = m - 1; j >= 0; --j) crow[j] = cost(hd[j]);
            }
        } else {
            for (int i = lane; i < ns; i += 32) {
                double bi[3] = {0, 0, 0};
                if constexpr (!kF32) G.b(i, bi);
                DT hd[kMaxNei];
                nearest_heap<DT, KT>(hd, kk + i * m, ns, m, [&](int j) { return dist(i, bi, j); });
                CT *crow = cc + i * m;
                for (int j = 0; j < m; ++j) crow[j] = cost(hd[j]);
            }
        }
        __syncwarp();
        return jv_warp<!kF32, KT>(ns, m, dense, CostStored<CT>{cc, m}, kk, v, dd, x, y, lab, fr, todo, ok);
    }
}

// Centroids of a pair's two inputs (XA's in mx[0..2], XB's in mx[3..5]),
// every lane getting all six.  The refinement and k_ref_b4 both use it, so
// the fixed structure's centred FP32 copy has the same bits in both.
__device__ __forceinline__ void pair_centroids(const double *XA, const double *XB, int n, int lane,
                                               double (&mx)[6]) {
    double v6[6] = {0, 0, 0, 0, 0, 0};
    for (int j = lane; j < n; j += 32)
        for (int r = 0; r < 3; ++r) {
            v6[r] += XA[3 * j + r];
            v6[3 + r] += XB[3 * j + r];
        }
    warp_halve<6>(v6, lane);
    const double mean = v6[0] / n;
    for (int r = 0; r < 6; ++r) mx[r] = __shfl_sync(kFull, mean, halve_lane(r, 6));
}

// Mixed form: the FP32 copy of every pair's fixed structure as the
// refinement reads it (centred on its centroid for clusters, as given for
// periodic pairs), one warp per pair, written once to global memory and
// read by all candidates of the pair (it used to be rebuilt in every
// candidate's shared memory).
template <bool BOX>
__global__ void __launch_bounds__(32) k_ref_b4(const PairDev *pairs, const double *xa, const double *xb,
                                               float4 *b4) {
    const int lane = threadIdx.x;
    const PairDev &P = pairs[blockIdx.x];
    const int n = P.n, a0 = P.atom0;
    const double *XA = xa + 3LL * a0, *XB = xb + 3LL * a0;
    double cm[3] = {0, 0, 0};
    if constexpr (!BOX) {
        double mx[6];
        pair_centroids(XA, XB, n, lane, mx);
        for (int r = 0; r < 3; ++r) cm[r] = mx[3 + r];
    }
    for (int j = lane; j < n; j += 32)
        b4[a0 + j] = make_float4((float)(XB[3 * j] - cm[0]), (float)(XB[3 * j + 1] - cm[1]),
                                 (float)(XB[3 * j + 2] - cm[2]), 0.f);
}

// Resident one-warp blocks per SM the register allocation is sized for
// (65536 / (32 * FO_REFINE_MINB) registers per thread at most).
#ifndef FO_REFINE_MINB
#define FO_REFINE_MINB 16
#endif

// ---------------------------------------------------------------------------
// ITERATIVEALIGN from one candidate, executed by one warp (block of 32).
// Shared memory holds the FP32 coordinate copies, the permutations and the
// assignment arrays.  The moved structure's FP64 working coordinates live in
// the candidate's output slot (cxyz); the fixed structure and the rotated
// starting structure are recomputed from the inputs where they are read, with
// the same expressions as when they are first formed.
// MW: blocks of up to kRefMaxWarps warps (mixed form, groups of more than
// kHeapMaxRow atoms): the first warp runs the candidate, the others help with
// its neighbour lists.  The register budget per thread equals the one-warp
// kernel's (FO_REFINE_MINB one-warp blocks per SM).
template <typename DT, typename CT, bool RECOMP, bool BOX, bool MW = false>
__global__ void __launch_bounds__(MW ? 32 * kRefMaxWarps : 32, MW ? FO_REFINE_MINB / kRefMaxWarps : FO_REFINE_MINB)
    k_refine_warp(const PairDev *pairs, const GroupDev *groups, const int *cand_list, const int *cand2pair,
                  const double *xa, const double *xb, const double *peaks, const int *npeaks, unsigned char *lapg,
                  double *cdist, double *cR, double *cdisp, double *cxyz, int *cperm, int *cniter, int *cstat,
                  float *cthr, const float4 *b4g, int *cscr) {
    constexpr bool kF32 = sizeof(DT) == 4;
    static_assert(kF32 || !RECOMP, "costs are recomputed only from FP32 coordinates");
    static_assert(!MW || (kF32 && RECOMP), "helper warps serve the mixed form's neighbour lists only");
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ NbrCmd scmd;
    const int lane = threadIdx.x & 31;
    const int c = cand_list[blockIdx.x];
    const int p = cand2pair[c];
    const PairDev &P = pairs[p];
    const int local = c - P.cand0, o = local / P.nrot, ci = local % P.nrot;
    if (ci >= npeaks[2 * p + o]) {
        if (lane == 0) { cdist[c] = INFINITY; cstat[c] = -1; }
        return;
    }
    const int n = P.n, bulk = P.bulk, a0 = P.atom0;
    int maxg = 0;
    for (int gi = 0; gi < P.ngroups; ++gi) maxg = max(maxg, groups[P.group0 + gi].n);
    RefLayout L;
    ref_layout(n, maxg, kF32, (int)sizeof(CT), RECOMP, L);
    // FP32 coordinate copies: the moved structure per candidate in shared
    // memory; the fixed structure per pair in global memory (mixed form) or
    // in shared memory (B4w, the FP32 form with stored costs)
    float4 *A4 = (float4 *)(smem + L.DAf), *B4w = (float4 *)(smem + L.DBf);
    const float4 *B4 = RECOMP ? b4g + P.atom0 : B4w;
    // permutations: the best one in the candidate's output slot and two
    // working arrays in its global scratch (mixed form), or in shared memory
    const long long ob = P.candatom0 + (long long)local * n;
    int *permbest = RECOMP ? cperm + ob : (int *)(smem + L.perm);
    int *newperm = RECOMP ? cscr + 3 * ob : (int *)(smem + L.nperm);
    int *ptmp = RECOMP ? cscr + 3 * ob + n : (int *)(smem + L.ptmp);
    int *frlist = RECOMP ? cscr + 3 * ob + 2 * n : nullptr;   // the assignment's free list (mixed form)
    // assignment block: on chip; or split (working arrays on chip, costs and
    // neighbour lists in the candidate's global scratch); or all in global
    unsigned char *lbk = P.lapstride ? lapg + P.lap0 + (long long)local * P.lapstride : smem + L.coord_end;
    unsigned char *lb = (P.lapstride && !P.lapsplit) ? lbk : smem + L.coord_end;
    int *lx = (int *)(lb + L.lap_x);
    const double box[3] = {P.box[0], P.box[1], P.box[2]};
    const double *pk = peaks + 3LL * (P.cand0 + o * P.nrot + ci);
    double *DA = cxyz + 3 * ob;                            // moved structure, FP64
    const double *XA = xa + 3LL * a0, *XB = xb + 3LL * a0;   // inputs of the pair
    if constexpr (kF32 && RECOMP) {
        // Mixed form: FP32 coordinates for the costs, FP64 superposition built
        // from few FP64 instructions (Horn rotation, one affine map per step).
        __shared__ double sRb[9], sRn[9], sRc[9], sRs[9], sT[12], sF[8];
        float *thrc = cthr + ob;   // per row: its m-th neighbour distance in the last iteration
        if constexpr (MW) {
            if (threadIdx.x >= 32) {   // helper warps: neighbour-list rows until the first warp is done
                nbr_helper<BOX>(&scmd, L.kkbytes);
                return;
            }
        }
        NbrCmd *cmd = MW ? &scmd : nullptr;
        GroupCoords GC;
        GC.bulk = bulk;
        GC.xb = XB;
        double S = 0, d0[3] = {0, 0, 0}, rb[3] = {0, 0, 0}, nbox[3], off[3] = {0, 0, 0}, nca[3] = {0, 0, 0};
        const double zero3[3] = {0, 0, 0};
        for (int k = 0; k < 3; ++k) nbox[k] = flip_sign(box[k], true);
        if constexpr (BOX) {
            // lanes 0-2: shift of the candidate (peak_k - 1) box_k / G; lanes 3-5: 1 / box_k
            const int k = lane % 3;
            const double bk = sel3(box[0], box[1], box[2], k);
            const double num = (lane < 3) ? (pk[k] - 1.0) * bk : 1.0;
            const double den = (lane < 3) ? (double)P.G : bk;
            const double qv = (den != 0.0) ? num / den : 0.0;
            for (int j = 0; j < 3; ++j) {
                d0[j] = __shfl_sync(kFull, qv, j);
                rb[j] = __shfl_sync(kFull, qv, 3 + j);
                off[j] = flip_sign(d0[j], true);
                GC.cmb[j] = 0.0;
                GC.box[j] = box[j];
                GC.bxf[j] = (float)box[j];
                GC.rxf[j] = (float)rb[j];
            }
            for (int j = lane; j < n; j += 32) {
                double a[3];
                for (int r = 0; r < 3; ++r) {
                    a[r] = XA[3 * j + r] + off[r];
                    DA[3 * j + r] = a[r];
                }
                A4[j] = make_float4((float)a[0], (float)a[1], (float)a[2], 0.f);
                permbest[j] = j;
            }
        } else {
            // Euler angles of the candidate over pi: lanes 0-2 take sin and cos of one each
            const double num = (lane == 1) ? pk[1] - 0.5 : (pk[(lane < 3) ? lane : 0] - 1.0) * 2.0;
            double sn, cs;
            sincospi(num / (double)P.G, &sn, &cs);
            if (lane < 3) { sF[2 * lane] = cs; sF[2 * lane + 1] = sn; }
            if (lane == 3) { sF[6] = 1.0; sF[7] = 0.0; }
            __syncwarp();
            const int k = lane < 9 ? lane : 0;
            double rc = sF[nibble(kEulerXp, k)] * sF[nibble(kEulerYp, k)];
            rc = rc * sF[nibble(kEulerZp, k)];
            rc = fma(flip_sign(sF[nibble(kEulerUp, k)], flag(kEulerNeg2p, k)), sF[nibble(kEulerWp, k)],
                     flip_sign(rc, flag(kEulerNeg1p, k)));
            if (lane < 9) {
                sRc[lane] = rc;
                sRs[lane] = flip_sign(rc, o == 1);   // with the inversion
                sRb[lane] = (lane % 4 == 0) ? 1.0 : 0.0;
            }
            // centroids of both inputs
            double mx[6];
            pair_centroids(XA, XB, n, lane, mx);
            __syncwarp();
            // centroid of the rotated moved structure, lanes 0-2
            const int r3 = lane % 3;
            double cv = sRs[3 * r3] * mx[0];
            cv = fma(sRs[3 * r3 + 1], mx[1], cv);
            cv = fma(sRs[3 * r3 + 2], mx[2], cv);
            for (int r = 0; r < 3; ++r) {
                nca[r] = flip_sign(__shfl_sync(kFull, cv, r), true);
                GC.cmb[r] = mx[3 + r];
                GC.box[r] = box[r];
                GC.bxf[r] = 0.f;
                GC.rxf[r] = 0.f;
            }
            double Rs[9];
            for (int r = 0; r < 9; ++r) Rs[r] = sRs[r];
            double s = 0;
            for (int j = lane; j < n; j += 32) {
                const double x0 = XA[3 * j], x1 = XA[3 * j + 1], x2 = XA[3 * j + 2];
                double a[3], b[3];
                GC.b(j, b);
                for (int r = 0; r < 3; ++r) {
                    a[r] = fma(Rs[3 * r], x0, fma(Rs[3 * r + 1], x1, fma(Rs[3 * r + 2], x2, nca[r])));
                    DA[3 * j + r] = a[r];
                    s = fma(a[r], a[r], s);
                    s = fma(b[r], b[r], s);
                }
                A4[j] = make_float4((float)a[0], (float)a[1], (float)a[2], 0.f);
                permbest[j] = j;
            }
            S = wsum_d(s);
        }
        __syncwarp();
        const GroupCoords GB = GC;   // whole-structure view of the fixed structure
        const double thr = sqrt((double)n) / kPScale;
        double db[3] = {0, 0, 0}, newdist = 0;
        int ntries = 0, nperm = n, fail = 0;
        // mean minimum-image displacement of the moved atoms (a(j)) onto the
        // fixed ones, and the distance after that shift
        auto displacement = [&](const auto &a_of, double *dn) {
            double v3[3] = {0, 0, 0};
            for (int j = lane; j < n; j += 32) {
                const double *a = a_of(j);
                for (int r = 0; r < 3; ++r) {
                    const double t = XB[3 * j + r] - a[r];
                    v3[r] += fma(nbox[r], rint(t * rb[r]), t);
                }
            }
            warp_halve<3>(v3, lane);
            const double mv = v3[0] / n;
            for (int r = 0; r < 3; ++r) dn[r] = __shfl_sync(kFull, mv, halve_lane(r, 3));
            double s1 = 0;
            for (int j = lane; j < n; j += 32) {
                const double *a = a_of(j);
                for (int r = 0; r < 3; ++r) {
                    double t = (XB[3 * j + r] - a[r]) - dn[r];
                    t = fma(nbox[r], rint(t * rb[r]), t);
                    s1 = fma(t, t, s1);
                }
            }
            return sqrt(wsum_d(s1));
        };
        for (int iter = 0; iter < 64 && nperm > 0; ++iter) {
            for (int j = lane; j < n; j += 32) newperm[j] = j;
            double pdsum = 0;
            __syncwarp();
            for (int gi = 0; gi < P.ngroups; ++gi) {
                const GroupDev g = groups[P.group0 + gi];
                const int ns = g.n, m = g.m, s0 = g.slot0 - a0;
                GC.xb = XB + 3 * s0;
                GC.A = DA + 3 * s0;
                GC.B4 = B4 + s0;
                GC.A4 = A4 + s0;
                const int rc = (L.kkbytes == 1) ? assign_group<uint8_t, DT, CT, RECOMP, BOX>(ns, m, GC, lb, lbk, L, thrc + s0, iter > 0, cmd, frlist)
                                                : assign_group<uint16_t, DT, CT, RECOMP, BOX>(ns, m, GC, lb, lbk, L, thrc + s0, iter > 0, cmd, frlist);
                if (rc) fail += 1;
                __syncwarp();
                for (int i = lane; i < ns; i += 32) {
                    int col = lx[i];
                    if (col >= ns) { col = ns - 1; fail += 1; }
                    if (col < 0) { col = 0; fail += 1; }
                    newperm[s0 + i] = s0 + col;
                    const double *a = DA + 3 * (s0 + col);
                    if constexpr (BOX) {
                        for (int r = 0; r < 3; ++r) {
                            double t = GC.xb[3 * i + r] - a[r];
                            t = fma(nbox[r], rint(t * rb[r]), t);
                            pdsum = fma(t, t, pdsum);
                        }
                    } else {
                        double b[3];
                        GC.b(i, b);
                        pdsum += pdist2<double>(b, a, 0, box);
                    }
                }
                __syncwarp();
            }
            pdsum = wsum_d(pdsum);
            int cnt = 0;
            for (int j = lane; j < n; j += 32) {
                int q = newperm[j];
                ptmp[j] = permbest[q];
                if (q != j) ++cnt;
            }
            for (int o2 = 16; o2 > 0; o2 >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o2);
            if constexpr (BOX) {
                double dn[3];
                newdist = displacement([&](int j) { return DA + 3 * newperm[j]; }, dn);
                for (int r = 0; r < 3; ++r) {
                    db[r] += dn[r];
                    off[r] += dn[r];
                }
                __syncwarp();
                for (int j = lane; j < n; j += 32) {
                    const int pj = ptmp[j];
                    permbest[j] = pj;
                    double a[3];
                    for (int r = 0; r < 3; ++r) {
                        a[r] = XA[3 * pj + r] + off[r];
                        DA[3 * j + r] = a[r];
                    }
                    A4[j] = make_float4((float)a[0], (float)a[1], (float)a[2], 0.f);
                }
            } else {
                double h[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
                for (int j = lane; j < n; j += 32) {
                    const double *a = DA + 3 * newperm[j];
                    const double a3[3] = {a[0], a[1], a[2]};
                    double b[3];
                    GB.b(j, b);
                    for (int p2 = 0; p2 < 3; ++p2)
                        for (int q2 = 0; q2 < 3; ++q2) h[3 * p2 + q2] = fma(a3[p2], b[q2], h[3 * p2 + q2]);
                }
                newdist = horn_rotation(h, S, lane, sRn);
                compose_affine(sRn, sRb, sRs, nca, zero3, sT, lane);
                double T[12];
                for (int r = 0; r < 12; ++r) T[r] = sT[r];
                for (int j = lane; j < n; j += 32) {
                    const int pj = ptmp[j];
                    permbest[j] = pj;
                    const double x0 = XA[3 * pj], x1 = XA[3 * pj + 1], x2 = XA[3 * pj + 2];
                    double a[3];
                    for (int r = 0; r < 3; ++r) {
                        a[r] = fma(T[3 * r], x0, fma(T[3 * r + 1], x1, fma(T[3 * r + 2], x2, T[9 + r])));
                        DA[3 * j + r] = a[r];
                    }
                    A4[j] = make_float4((float)a[0], (float)a[1], (float)a[2], 0.f);
                }
            }
            __syncwarp();
            nperm = cnt;
            ntries += 1;
            // (newdist - pd) / newdist > sqrt(n) / PSCALE, without the division
            const double pd = sqrt(pdsum);
            if (newdist - pd > thr * newdist) nperm = 0;
            if (ntries > kMaxTries) nperm = 0;
        }
        // final superposition without a new permutation
        if constexpr (BOX) {
            double dn[3];
            newdist = displacement([&](int j) { return DA + 3 * j; }, dn);
            for (int r = 0; r < 3; ++r) db[r] += dn[r];
            __syncwarp();
            for (int j = lane; j < n; j += 32)
                for (int r = 0; r < 3; ++r) DA[3 * j + r] += dn[r];
        } else {
            double h[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int j = lane; j < n; j += 32) {
                const double a3[3] = {DA[3 * j], DA[3 * j + 1], DA[3 * j + 2]};
                double b[3];
                GB.b(j, b);
                for (int p2 = 0; p2 < 3; ++p2)
                    for (int q2 = 0; q2 < 3; ++q2) h[3 * p2 + q2] = fma(a3[p2], b[q2], h[3 * p2 + q2]);
            }
            newdist = horn_rotation(h, S, lane, sRn);
            compose_affine(sRn, sRb, sRs, nca, GB.cmb, sT, lane);   // back to the fixed centroid
            double T[12];
            for (int r = 0; r < 12; ++r) T[r] = sT[r];
            for (int j = lane; j < n; j += 32) {
                const int pj = permbest[j];
                const double x0 = XA[3 * pj], x1 = XA[3 * pj + 1], x2 = XA[3 * pj + 2];
                for (int r = 0; r < 3; ++r)
                    DA[3 * j + r] = fma(T[3 * r], x0, fma(T[3 * r + 1], x1, fma(T[3 * r + 2], x2, T[9 + r])));
            }
        }
        __syncwarp();   // permbest is the candidate's output slot
        for (int o2 = 16; o2 > 0; o2 >>= 1) fail += __shfl_xor_sync(kFull, fail, o2);
        if constexpr (BOX) {
            if (lane < 9) cR[9LL * c + lane] = (lane % 4 == 0) ? 1.0 : 0.0;
        } else {   // rotation of the input: sRb sRc, entry k on lane k
            const int k = lane < 9 ? lane : 0, r = k / 3, cc = k % 3;
            double v = sRb[3 * r] * sRc[cc];
            v = fma(sRb[3 * r + 1], sRc[3 + cc], v);
            v = fma(sRb[3 * r + 2], sRc[6 + cc], v);
            if (lane < 9) cR[9LL * c + lane] = v;
        }
        if (lane == 0) {
            cdist[c] = newdist;
            for (int k = 0; k < 3; ++k) cdisp[3LL * c + k] = db[k] - d0[k];
            cniter[c] = ntries;
            cstat[c] = fail ? (int)ST_LAP_FAILED : 0;
        }
        if constexpr (MW) {   // release the helper warps
            __syncwarp();
            if (lane == 0) scmd.op = 0;
            __syncwarp();
            named_bar(1, blockDim.x);
        }
    } else {
        __shared__ double sRb[9], sRn[9], sRc[9];
        double d0[3] = {0, 0, 0};
        if (lane == 0) {
            for (int k = 0; k < 9; ++k) { sRb[k] = (k % 4 == 0) ? 1.0 : 0.0; sRc[k] = sRb[k]; }
            if (!bulk) {
                const double conv = FO_PI / P.G;
                euler_matrix((pk[0] - 1.0) * 2 * conv, (pk[1] - 0.5) * conv, (pk[2] - 1.0) * 2 * conv, sRc);
            }
        }
        if (bulk)
            for (int k = 0; k < 3; ++k) d0[k] = (pk[k] - 1.0) * box[k] / P.G;
        __syncwarp();
        const double sgn = (o == 1) ? -1.0 : 1.0;
        // moved atom j rotated by the candidate (cluster) or shifted (bulk)
        auto a_raw = [&](int j, double *out) {
            const double *a = XA + 3 * j;
            if (bulk) {
                for (int k = 0; k < 3; ++k) out[k] = a[k] - d0[k];
            } else {
                for (int k = 0; k < 3; ++k)
                    out[k] = sgn * (sRc[3 * k] * a[0] + sRc[3 * k + 1] * a[1] + sRc[3 * k + 2] * a[2]);
            }
        };
        double cs[6] = {0, 0, 0, 0, 0, 0};
        for (int j = lane; j < n; j += 32) {
            double t[3];
            a_raw(j, t);
            for (int k = 0; k < 3; ++k) { cs[k] += t[k]; cs[3 + k] += XB[3 * j + k]; }
        }
        for (int k = 0; k < 6; ++k) cs[k] = wsum_d(cs[k]);
        // ITERATIVEALIGN works on structures centred at their centroids
        double ca[3] = {0, 0, 0};
        GroupCoords GC;
        GC.bulk = bulk;
        for (int k = 0; k < 3; ++k) {
            GC.cmb[k] = bulk ? 0.0 : cs[3 + k] / n;
            ca[k] = cs[k] / n;
            GC.box[k] = box[k];
            GC.bxf[k] = (float)box[k];
            GC.rxf[k] = box[k] != 0.0 ? (float)(1.0 / box[k]) : 0.f;
        }
        // starting moved structure A0 (centred for clusters)
        auto a_start = [&](int j, double *out) {
            a_raw(j, out);
            if (!bulk)
                for (int k = 0; k < 3; ++k) out[k] -= ca[k];
        };
        GC.xb = XB;
        for (int j = lane; j < n; j += 32) {
            double a[3];
            a_start(j, a);
            for (int k = 0; k < 3; ++k) DA[3 * j + k] = a[k];
            if constexpr (kF32) {
                double b[3];
                GC.b(j, b);
                A4[j] = make_float4((float)a[0], (float)a[1], (float)a[2], 0.f);
                B4w[j] = make_float4((float)b[0], (float)b[1], (float)b[2], 0.f);
            }
            permbest[j] = j;
        }
        __syncwarp();
        const GroupCoords GB = GC;   // whole-structure view of the fixed structure
        double db[3] = {0, 0, 0}, newdist = 0;
        int ntries = 0, nperm = n, fail = 0;
        for (int iter = 0; iter < 64 && nperm > 0; ++iter) {
            for (int j = lane; j < n; j += 32) newperm[j] = j;
            double pdsum = 0;
            __syncwarp();
            for (int gi = 0; gi < P.ngroups; ++gi) {
                const GroupDev g = groups[P.group0 + gi];
                const int ns = g.n, m = g.m, s0 = g.slot0 - a0;
                GC.xb = XB + 3 * s0;
                GC.A = DA + 3 * s0;
                GC.B4 = B4 + s0;
                GC.A4 = A4 + s0;
                const int rc = (L.kkbytes == 1) ? assign_group<uint8_t, DT, CT, RECOMP, BOX>(ns, m, GC, lb, lbk, L)
                                                : assign_group<uint16_t, DT, CT, RECOMP, BOX>(ns, m, GC, lb, lbk, L);
                if (rc) fail += 1;
                __syncwarp();
                for (int i = lane; i < ns; i += 32) {
                    int col = lx[i];
                    if (col >= ns) { col = ns - 1; fail += 1; }
                    if (col < 0) { col = 0; fail += 1; }
                    newperm[s0 + i] = s0 + col;
                    double b[3];
                    GC.b(i, b);
                    pdsum += pdist2<double>(b, DA + 3 * (s0 + col), bulk, box);
                }
                __syncwarp();
            }
            pdsum = wsum_d(pdsum);
            int cnt = 0;
            for (int j = lane; j < n; j += 32) {
                int q = newperm[j];
                ptmp[j] = permbest[q];
                if (q != j) ++cnt;
            }
            for (int o2 = 16; o2 > 0; o2 >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o2);
            if (bulk) {
                double s3[3] = {0, 0, 0};
                for (int j = lane; j < n; j += 32) {
                    const double *a = DA + 3 * newperm[j];
                    double b[3];
                    GB.b(j, b);
                    for (int k = 0; k < 3; ++k) {
                        double t = b[k] - a[k];
                        s3[k] += t - box[k] * round(t / box[k]);
                    }
                }
                double dn[3];
                for (int k = 0; k < 3; ++k) dn[k] = wsum_d(s3[k]) / n;
                double s1 = 0;
                for (int j = lane; j < n; j += 32) {
                    const double *a = DA + 3 * newperm[j];
                    double ad[3] = {a[0] + dn[0], a[1] + dn[1], a[2] + dn[2]}, b[3];
                    GB.b(j, b);
                    s1 += pdist2<double>(b, ad, 1, box);
                }
                newdist = sqrt(wsum_d(s1));
                for (int k = 0; k < 3; ++k) db[k] += dn[k];
                __syncwarp();
                for (int j = lane; j < n; j += 32) {
                    permbest[j] = ptmp[j];
                    double a[3];
                    a_start(ptmp[j], a);
                    for (int k = 0; k < 3; ++k) DA[3 * j + k] = a[k] + db[k];
                    if constexpr (kF32)
                        A4[j] = make_float4((float)DA[3 * j], (float)DA[3 * j + 1], (float)DA[3 * j + 2], 0.f);
                }
            } else {
                double q[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
                for (int j = lane; j < n; j += 32) {
                    const double *a = DA + 3 * newperm[j];
                    double b[3];
                    GB.b(j, b);
                    double xm = b[0] - a[0], ym = b[1] - a[1], zm = b[2] - a[2];
                    double xp = b[0] + a[0], yp = b[1] + a[1], zp = b[2] + a[2];
                    q[0] += xm * xm + ym * ym + zm * zm;
                    q[1] += yp * zm - ym * zp;
                    q[2] += xm * zp - xp * zm;
                    q[3] += xp * ym - xm * yp;
                    q[4] += yp * yp + zp * zp + xm * xm;
                    q[5] += xm * ym - xp * yp;
                    q[6] += xm * zm - xp * zp;
                    q[7] += xp * xp + zp * zp + ym * ym;
                    q[8] += ym * zm - yp * zp;
                    q[9] += xp * xp + yp * yp + zm * zm;
                }
                for (int k = 0; k < 10; ++k) q[k] = wsum_d(q[k]);
                if (lane == 0) {
                    newdist = kearsley_rotation_fast(q, sRn);
                    matmul3(sRn, sRb, sRb);
                }
                newdist = __shfl_sync(kFull, newdist, 0);
                __syncwarp();
                for (int j = lane; j < n; j += 32) {
                    permbest[j] = ptmp[j];
                    double a[3];
                    a_start(ptmp[j], a);
                    for (int k = 0; k < 3; ++k)
                        DA[3 * j + k] = sRb[3 * k] * a[0] + sRb[3 * k + 1] * a[1] + sRb[3 * k + 2] * a[2];
                    if constexpr (kF32)
                        A4[j] = make_float4((float)DA[3 * j], (float)DA[3 * j + 1], (float)DA[3 * j + 2], 0.f);
                }
            }
            __syncwarp();
            nperm = cnt;
            ntries += 1;
            double pd = sqrt(pdsum);
            if ((newdist - pd) / newdist > sqrt((double)n) / kPScale) nperm = 0;
            if (ntries > kMaxTries) nperm = 0;
        }
        // final minimisation without a new permutation
        if (bulk) {
            double s3[3] = {0, 0, 0};
            for (int j = lane; j < n; j += 32) {
                double b[3];
                GB.b(j, b);
                for (int k = 0; k < 3; ++k) {
                    double t = b[k] - DA[3 * j + k];
                    s3[k] += t - box[k] * round(t / box[k]);
                }
            }
            double dn[3];
            for (int k = 0; k < 3; ++k) dn[k] = wsum_d(s3[k]) / n;
            double s1 = 0;
            for (int j = lane; j < n; j += 32) {
                double ad[3] = {DA[3 * j] + dn[0], DA[3 * j + 1] + dn[1], DA[3 * j + 2] + dn[2]}, b[3];
                GB.b(j, b);
                s1 += pdist2<double>(b, ad, 1, box);
            }
            newdist = sqrt(wsum_d(s1));
            for (int k = 0; k < 3; ++k) db[k] += dn[k];
            __syncwarp();
            for (int j = lane; j < n; j += 32)
                for (int k = 0; k < 3; ++k) DA[3 * j + k] += dn[k];
        } else {
            double q[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int j = lane; j < n; j += 32) {
                const double *a = DA + 3 * j;
                double b[3];
                GB.b(j, b);
                double xm = b[0] - a[0], ym = b[1] - a[1], zm = b[2] - a[2];
                double xp = b[0] + a[0], yp = b[1] + a[1], zp = b[2] + a[2];
                q[0] += xm * xm + ym * ym + zm * zm;
                q[1] += yp * zm - ym * zp;
                q[2] += xm * zp - xp * zm;
                q[3] += xp * ym - xm * yp;
                q[4] += yp * yp + zp * zp + xm * xm;
                q[5] += xm * ym - xp * yp;
                q[6] += xm * zm - xp * zp;
                q[7] += xp * xp + zp * zp + ym * ym;
                q[8] += ym * zm - yp * zp;
                q[9] += xp * xp + yp * yp + zm * zm;
            }
            for (int k = 0; k < 10; ++k) q[k] = wsum_d(q[k]);
            if (lane == 0) {
                newdist = kearsley_rotation_fast(q, sRn);
                matmul3(sRn, sRb, sRb);
            }
            newdist = __shfl_sync(kFull, newdist, 0);
            __syncwarp();
            for (int j = lane; j < n; j += 32) {
                double a[3] = {DA[3 * j], DA[3 * j + 1], DA[3 * j + 2]};
                for (int k = 0; k < 3; ++k)
                    DA[3 * j + k] = sRn[3 * k] * a[0] + sRn[3 * k + 1] * a[1] + sRn[3 * k + 2] * a[2] + GB.cmb[k];
            }
        }
        __syncwarp();
        for (int j = lane; j < n; j += 32) cperm[ob + j] = permbest[j];
        for (int o2 = 16; o2 > 0; o2 >>= 1) fail += __shfl_xor_sync(kFull, fail, o2);
        if (lane == 0) {
            cdist[c] = newdist;
            double R[9];
            matmul3(sRb, sRc, R);
            for (int k = 0; k < 9; ++k) cR[9LL * c + k] = bulk ? ((k % 4 == 0) ? 1.0 : 0.0) : R[k];
            for (int k = 0; k < 3; ++k) cdisp[3LL * c + k] = db[k] - d0[k];
            cniter[c] = ntries;
            cstat[c] = fail ? (int)ST_LAP_FAILED : 0;
        }
    }
}

// Winner per pair: smallest distance among the non-inverted candidates (the
// first wins ties), replaced by the inverted winner only when strictly
// smaller.  Per-atom outputs are scattered back to original atom order.
__global__ void k_select(const PairDev *pairs, const int *slot2orig, const int *npeaks,
                         const int *pstatus, const double *omax, const double *cdist,
                         const double *cR, const double *cdisp, const double *cxyz,
                         const int *cperm, const int *cniter, const int *cstat,
                         fo_pair_result *res, double *aligned, int *permbest) {
    __shared__ int s_win;
    const int p = blockIdx.x;
    const PairDev &P = pairs[p];
    if (threadIdx.x == 0) {
        int win = -1, inv = 0;
        double best = INFINITY;
        for (int ci = 0; ci < npeaks[2 * p]; ++ci) {
            double d = cdist[P.cand0 + ci];
            if (d < best) { best = d; win = ci; }
        }
        if (P.norient == 2) {
            double bi = INFINITY;
            int wi = -1;
            for (int ci = 0; ci < npeaks[2 * p + 1]; ++ci) {
                double d = cdist[P.cand0 + P.nrot + ci];
                if (d < bi) { bi = d; wi = ci; }
            }
            if (wi >= 0 && (win < 0 || bi < best)) { best = bi; win = P.nrot + wi; inv = 1; }
        }
        fo_pair_result r;
        r.sigma = P.sigma;
        r.inverted = inv;
        r.ncand = npeaks[2 * p] + (P.norient == 2 ? npeaks[2 * p + 1] : 0);
        if (win < 0) {
            r.dist = NAN;
            for (int k = 0; k < 9; ++k) r.rmat[k] = NAN;
            for (int k = 0; k < 3; ++k) r.disp[k] = NAN;
            r.overlap_max = omax[2 * p];
            r.status = pstatus[p] ? pstatus[p] : (int)ST_NO_PEAKS;
            r.niter = 0;
        } else {
            const int c = P.cand0 + win;
            r.dist = cdist[c];
            for (int k = 0; k < 9; ++k) r.rmat[k] = cR[9LL * c + k];
            for (int k = 0; k < 3; ++k) r.disp[k] = cdisp[3LL * c + k];
            r.overlap_max = omax[2 * p + inv];
            r.status = cstat[c] > 0 ? cstat[c] : 0;
            r.niter = cniter[c];
        }
        res[p] = r;
        s_win = win;
    }
    __syncthreads();
    const int win = s_win, n = P.n, a0 = P.atom0;
    if (win < 0) return;
    const long long ob = P.candatom0 + (long long)win * n;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        int oj = slot2orig[a0 + j];
        if (aligned)
            for (int k = 0; k < 3; ++k) aligned[3LL * (a0 + oj) + k] = cxyz[3 * (ob + j) + k];
        if (permbest) permbest[a0 + oj] = slot2orig[a0 + cperm[ob + j]];
    }
}


// Warps per block for a bucket of the mixed form whose groups take the
// multi-warp neighbour lists: as many as the register file holds next to the
// blocks that the shared-memory footprint already lets share an SM (at most
// kRefMaxWarps; 1 when the footprint allows many blocks anyway).
int refine_block_warps(bool bulk, bool ct64, size_t smem) {
    const void *fn = bulk ? (ct64 ? (const void *)k_refine_warp<float, long long, true, true, true>
                                  : (const void *)k_refine_warp<float, int, true, true, true>)
                          : (ct64 ? (const void *)k_refine_warp<float, long long, true, false, true>
                                  : (const void *)k_refine_warp<float, int, true, false, true>);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) { cudaGetLastError(); return 1; }
    int dev = 0, smsm = 0, regsm = 0, thrsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smsm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&regsm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&thrsm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    const size_t per_block = smem + fa.sharedSizeBytes + 1024;
    const int blocks = per_block ? (int)((size_t)smsm / per_block) : 0;
    if (blocks < 1 || blocks >= FO_REFINE_MINB / 2) return 1;
    const int regs = fa.numRegs > 0 ? fa.numRegs : 128;
    int nw = regsm / (blocks * 32 * regs);
    nw = min(nw, thrsm / (blocks * 32));
    return max(1, min(nw, kRefMaxWarps));
}

// Buckets run concurrently on the auxiliary streams (fork/join through
// events on the main stream) so that small and large problems share the SMs.
void launch_refine(const RefineBuffers &b, cudaStream_t main, cudaStream_t *aux, int naux,
                   cudaEvent_t fork, cudaEvent_t *join) {
    if (b.fp32 && b.recomp) {
        if (b.bulk) k_ref_b4<true><<<b.npairs, 32, 0, main>>>(b.pairs, b.xa, b.xb, b.b4);
        else k_ref_b4<false><<<b.npairs, 32, 0, main>>>(b.pairs, b.xa, b.xb, b.b4);
    }
    cudaEventRecord(fork, main);
    for (int a = 0; a < naux; ++a) cudaStreamWaitEvent(aux[a], fork, 0);
    for (int k = 0; k < b.nbuckets; ++k) {
        const RefineBucket &bk = b.buckets[k];
        if (bk.count == 0) continue;
        const int *list = b.cand_list + bk.offset;
        cudaStream_t s = naux ? aux[k % naux] : main;
#define FO_LAUNCH_REFINE(DT, CT, RC, BX)                                                              \
    do {                                                                                              \
        allow_max_smem<k_refine_warp<DT, CT, RC, BX>>();                                             \
        k_refine_warp<DT, CT, RC, BX><<<bk.count, 32, bk.smem, s>>>(                                  \
            b.pairs, b.groups, list, b.cand2pair, b.xa, b.xb, b.peaks, b.npeaks, b.lap, b.cdist,      \
            b.cR, b.cdisp, b.cxyz, b.cperm, b.cniter, b.cstat, b.cthr, b.b4, b.cscr);                 \
    } while (0)
#define FO_LAUNCH_REFINE_MW(CT, BX)                                                                   \
    do {                                                                                              \
        allow_max_smem<k_refine_warp<float, CT, true, BX, true>>();                                  \
        k_refine_warp<float, CT, true, BX, true><<<bk.count, 32 * bk.nw, bk.smem, s>>>(               \
            b.pairs, b.groups, list, b.cand2pair, b.xa, b.xb, b.peaks, b.npeaks, b.lap, b.cdist,      \
            b.cR, b.cdisp, b.cxyz, b.cperm, b.cniter, b.cstat, b.cthr, b.b4, b.cscr);                 \
    } while (0)
        if (b.fp32 && b.recomp && bk.nw > 1) {
            if (b.bulk) {
                if (bk.ct64) FO_LAUNCH_REFINE_MW(long long, true);
                else FO_LAUNCH_REFINE_MW(int, true);
            } else {
                if (bk.ct64) FO_LAUNCH_REFINE_MW(long long, false);
                else FO_LAUNCH_REFINE_MW(int, false);
            }
        } else if (b.fp32 && b.recomp) {
            if (b.bulk) {
                if (bk.ct64) FO_LAUNCH_REFINE(float, long long, true, true);
                else FO_LAUNCH_REFINE(float, int, true, true);
            } else {
                if (bk.ct64) FO_LAUNCH_REFINE(float, long long, true, false);
                else FO_LAUNCH_REFINE(float, int, true, false);
            }
        } else if (b.fp32) {
            if (bk.ct64) FO_LAUNCH_REFINE(float, long long, false, false);
            else FO_LAUNCH_REFINE(float, int, false, false);
        } else {
            if (bk.ct64) FO_LAUNCH_REFINE(double, long long, false, false);
            else FO_LAUNCH_REFINE(double, int, false, false);
        }
#undef FO_LAUNCH_REFINE
#undef FO_LAUNCH_REFINE_MW
    }
    for (int a = 0; a < naux; ++a) {
        cudaEventRecord(join[a], aux[a]);
        cudaStreamWaitEvent(main, join[a], 0);
    }
}

void launch_select(const RefineBuffers &b, cudaStream_t s) {
    k_select<<<b.npairs, 256, 0, s>>>(b.pairs, b.slot2orig, b.npeaks, b.pstatus, b.overlap_max,
                                      b.cdist, b.cR, b.cdisp, b.cxyz, b.cperm, b.cniter, b.cstat,
                                      (fo_pair_result *)b.results, b.aligned, b.permbest);
}

}  // namespace fo
