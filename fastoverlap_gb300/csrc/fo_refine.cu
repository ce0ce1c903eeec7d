// fo_refine.cu -- candidate refinement and selection.
//
// One warp per candidate (pair, orientation, peak): rotate (cluster) or shift
// (bulk) the moved structure by the candidate, then alternate
//   per-group squared distances (60 nearest per row when a group has more
//   than 60 atoms) -> integer costs INT(d^2 * 1e6) -> sparse Jonker-Volgenant
//   assignment -> Kearsley rotation (cluster) or mean minimum-image
//   displacement (bulk)
// until no atom changes partner, the distance grows, or 21 tries.
// Candidates are launched in buckets of equal shared-memory footprint so
// small problems pack many warps per SM; the assignment arrays live in
// shared memory when they fit and in per-candidate global scratch otherwise.
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

namespace fo {

constexpr unsigned kFull = 0xffffffffu;
constexpr long long kLLMax = 0x7fffffffffffffffLL;

__device__ __forceinline__ long long wmin_ll(long long v) {
    for (int o = 16; o > 0; o >>= 1) {
        long long w = __shfl_xor_sync(kFull, v, o);
        v = w < v ? w : v;
    }
    return v;
}

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
// fixed width m; dense rows (m == n) have implicit column index t.  All
// lanes must call; returns 0 on success, > 0 when the matching fails.
template <typename CT>
__device__ int jv_warp(const int n, const int m, const bool dense, const CT *__restrict__ cc,
                       const unsigned short *__restrict__ kk, long long *v, long long *dd, int *x,
                       int *y, int *lab, int *fr, int *todo, unsigned char *ok) {
    const int lane = threadIdx.x & 31;
    const unsigned ltmask = (1u << lane) - 1u;
    auto COL = [&](int i, int t) -> int { return dense ? t : (int)kk[(long long)i * m + t]; };
    auto CST = [&](int i, int t) -> long long { return (long long)cc[(long long)i * m + t]; };

    // 1. column reduction: v_j = min_i c_ij, the first row attaining it owns j.
    // Rows in order; a row's columns are distinct, so lanes never collide.
    for (int j = lane; j < n; j += 32) { v[j] = kBigInt; y[j] = -1; }
    __syncwarp();
    for (int i = 0; i < n; ++i) {
        for (int t = lane; t < m; t += 32) {
            const int j = COL(i, t);
            const long long c = CST(i, t);
            if (c < v[j]) { v[j] = c; y[j] = i; }
        }
        __syncwarp();
    }
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
    for (int i = 0; i < n; ++i) {
        const int xi = x[i];
        if (xi < 0) {
            if (lane == 0) fr[nfree] = i;
            ++nfree;
            continue;
        }
        if (ok[i]) continue;
        long long mn = kBigInt;
        for (int t = lane; t < m; t += 32) {
            int j = COL(i, t);
            if (j == xi) continue;
            long long h = CST(i, t) - v[j];
            mn = h < mn ? h : mn;
        }
        mn = wmin_ll(mn);
        __syncwarp();
        if (lane == 0) v[xi] -= mn;
        __syncwarp();
    }
    __syncwarp();
    if (nfree == 0) return 0;

    // 3. augmenting row reduction, two passes
    long long guard = 0;
    const long long gmax = 64LL * n * (long long)n * m + 100000;
    int j0 = -1, j1 = -1;
    for (int pass = 0; pass < 2 && nfree > 0; ++pass) {
        const int l0 = nfree;
        int k = 0;
        nfree = 0;
        while (k < l0) {
            if (++guard > gmax) return 9;
            const int i = fr[k++];
            long long h1 = kLLMax, h2 = kLLMax;
            int t1 = 0x7fffffff, t2 = 0x7fffffff, cnt = 0;
            for (int t = lane; t < m; t += 32) {
                long long h = CST(i, t) - v[COL(i, t)];
                if (!(h < kBigInt)) continue;   // never enters the two smallest
                ++cnt;
                if (h < h1 || (h == h1 && t < t1)) { h2 = h1; t2 = t1; h1 = h; t1 = t; }
                else if (h < h2 || (h == h2 && t < t2)) { h2 = h; t2 = t; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                long long oh1 = __shfl_xor_sync(kFull, h1, o), oh2 = __shfl_xor_sync(kFull, h2, o);
                int ot1 = __shfl_xor_sync(kFull, t1, o), ot2 = __shfl_xor_sync(kFull, t2, o);
                cnt += __shfl_xor_sync(kFull, cnt, o);
                bool afirst = (h1 < oh1) || (h1 == oh1 && t1 < ot1);
                long long fh, sh;
                int ft, st;
                if (afirst) {
                    fh = h1; ft = t1;
                    bool a2 = (h2 < oh1) || (h2 == oh1 && t2 < ot1);
                    sh = a2 ? h2 : oh1; st = a2 ? t2 : ot1;
                } else {
                    fh = oh1; ft = ot1;
                    bool b2 = (oh2 < h1) || (oh2 == h1 && ot2 < t1);
                    sh = b2 ? oh2 : h1; st = b2 ? ot2 : t1;
                }
                h1 = fh; t1 = ft; h2 = sh; t2 = st;
            }
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
                long long h = CST(i0, t) - v[j];
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
        while (jend < 0) {
            if (++guard > gmax) return 9;
            if (k == 0) return 4;
            --k;
            const int jc = todo[k];
            const int i = y[jc];
            __syncwarp();
            if (lane == 0) todo[td] = jc;
            --td;
            int tpos = -1;
            for (int q = 0; q < 2; ++q) {
                int t = lane + 32 * q;
                bool hit = (t < m) && COL(i, t) == jc;
                unsigned hm = __ballot_sync(kFull, hit);
                if (hm && tpos < 0) tpos = 32 * q + __ffs(hm) - 1;
            }
            if (tpos < 0) return 5;
            const long long hh = CST(i, tpos) - v[jc] - mn;
            bool eq[2];
            int jq[2];
            for (int q = 0; q < 2; ++q) {
                int t = lane + 32 * q;
                eq[q] = false;
                jq[q] = -1;
                if (t < m) {
                    int j = COL(i, t);
                    jq[q] = j;
                    if (!ok[j]) {
                        long long vj = CST(i, t) - hh - v[j];
                        if (vj < dd[j]) {
                            dd[j] = vj;
                            lab[j] = i;
                            eq[q] = (vj == mn);
                        }
                    }
                }
            }
            __syncwarp();
            for (int q = 0; q < 2 && jend < 0; ++q) {
                bool isf = eq[q] && y[jq[q]] < 0;
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
            long long lm = kLLMax;
            for (int j = lane; j < n; j += 32)
                if (!ok[j] && dd[j] <= kBigInt - 1 && dd[j] < lm) lm = dd[j];
            lm = wmin_ll(lm);
            if (lm == kLLMax) { mn = kBigInt - 1; k = 0; continue; }
            mn = lm;
            for (int b = 0; b < n; b += 32) {
                int j = b + lane;
                bool sel = (j < n) && !ok[j] && dd[j] == mn;
                unsigned sm = __ballot_sync(kFull, sel);
                if (sel) todo[k + __popc(sm & ltmask)] = j;
                k += __popc(sm);
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

// The m nearest columns of one row as the binary max-heap of PAIRDISTS
// (alignutils.f90:641-701): the first m columns are sifted up in order, each
// later closer column replaces the root and is sifted down.  The heap's array
// order is the stored order of the row.
template <typename DT, typename KT>
__device__ __forceinline__ void nearest_heap(DT *hd, KT *hk, const DT *bi, const DT *acol, int ns, int m,
                                             int bulk, const double *box) {
    for (int j = 0; j < m; ++j) {
        hd[j] = pdist2<DT>(bi, acol + 3 * j, bulk, box);
        hk[j] = (KT)j;
        int l = j + 1;
        while (l > 1) {
            int l2 = l / 2;
            if (hd[l2 - 1] < hd[l - 1]) {
                DT h = hd[l2 - 1]; hd[l2 - 1] = hd[l - 1]; hd[l - 1] = h;
                KT t = hk[l2 - 1]; hk[l2 - 1] = hk[l - 1]; hk[l - 1] = t;
                l = l2;
            } else break;
        }
    }
    for (int j = m; j < ns; ++j) {
        DT d = pdist2<DT>(bi, acol + 3 * j, bulk, box);
        if (!(d < hd[0])) continue;
        hd[0] = d;
        hk[0] = (KT)j;
        int l = 1;
        for (int guard = 0; guard < 64; ++guard) {
            int l2 = 2 * l;
            if (l2 + 1 > m) {
                if (l2 <= m && hd[l2 - 1] > hd[l - 1]) {
                    DT h = hd[l2 - 1]; hd[l2 - 1] = hd[l - 1]; hd[l - 1] = h;
                    KT t = hk[l2 - 1]; hk[l2 - 1] = hk[l - 1]; hk[l - 1] = t;
                }
                break;
            }
            int a = (hd[l2] > hd[l2 - 1]) ? l2 + 1 : l2;
            if (hd[a - 1] > hd[l - 1]) {
                DT h = hd[a - 1]; hd[a - 1] = hd[l - 1]; hd[l - 1] = h;
                KT t = hk[a - 1]; hk[a - 1] = hk[l - 1]; hk[l - 1] = t;
                l = a;
            } else break;
        }
    }
}

// ---------------------------------------------------------------------------
// ITERATIVEALIGN from one candidate, executed by one warp (block of 32).
template <typename DT, typename CT>
__global__ void __launch_bounds__(32) k_refine_warp(
    const PairDev *pairs, const GroupDev *groups, const int *cand_list, const int *cand2pair,
    const double *xa, const double *xb, const double *peaks, const int *npeaks, unsigned char *lapg,
    double *cdist, double *cR, double *cdisp, double *cxyz, int *cperm, int *cniter, int *cstat) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double sRb[9], sRn[9], sRc[9];
    const int lane = threadIdx.x;
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
    ref_layout(n, maxg, sizeof(DT) == 4, (int)sizeof(CT), L);
    double *DB = (double *)(smem + L.DB), *A0 = (double *)(smem + L.A0), *DA = (double *)(smem + L.DA);
    DT *DBf = (DT *)(smem + L.DBf), *DAf = (DT *)(smem + L.DAf);
    int *permbest = (int *)(smem + L.perm), *newperm = (int *)(smem + L.nperm), *ptmp = (int *)(smem + L.ptmp);
    unsigned char *lb = P.lapstride ? lapg + P.lap0 + (long long)local * P.lapstride : smem + L.coord_end;
    CT *lcc = (CT *)(lb + L.lap_cc);
    unsigned short *lkk = (unsigned short *)(lb + L.lap_kk);
    long long *lv = (long long *)(lb + L.lap_v), *ld = (long long *)(lb + L.lap_d);
    int *lx = (int *)(lb + L.lap_x), *ly = (int *)(lb + L.lap_y), *llab = (int *)(lb + L.lap_lab);
    int *lfr = (int *)(lb + L.lap_fr), *ltodo = (int *)(lb + L.lap_todo);
    unsigned char *lok = lb + L.lap_ok;
    const double box[3] = {P.box[0], P.box[1], P.box[2]};
    const double *pk = peaks + 3LL * (P.cand0 + o * P.nrot + ci);
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
    double cs[6] = {0, 0, 0, 0, 0, 0};
    for (int j = lane; j < n; j += 32) {
        const double *a = xa + 3LL * (a0 + j), *b = xb + 3LL * (a0 + j);
        for (int k = 0; k < 3; ++k) DB[3 * j + k] = b[k];
        if (bulk) {
            for (int k = 0; k < 3; ++k) A0[3 * j + k] = a[k] - d0[k];
        } else {
            for (int k = 0; k < 3; ++k)
                A0[3 * j + k] = sgn * (sRc[3 * k] * a[0] + sRc[3 * k + 1] * a[1] + sRc[3 * k + 2] * a[2]);
        }
        for (int k = 0; k < 3; ++k) { cs[k] += A0[3 * j + k]; cs[3 + k] += DB[3 * j + k]; }
    }
    for (int k = 0; k < 6; ++k) cs[k] = wsum_d(cs[k]);
    double cmb[3] = {0, 0, 0};
    __syncwarp();
    if (!bulk) {  // ITERATIVEALIGN works on structures centred at their centroids
        for (int k = 0; k < 3; ++k) cmb[k] = cs[3 + k] / n;
        for (int j = lane; j < n; j += 32)
            for (int k = 0; k < 3; ++k) {
                A0[3 * j + k] -= cs[k] / n;
                DB[3 * j + k] -= cmb[k];
            }
    }
    __syncwarp();
    for (int j = lane; j < n; j += 32) {
        for (int k = 0; k < 3; ++k) {
            DA[3 * j + k] = A0[3 * j + k];
            if (sizeof(DT) == 4) { DAf[3 * j + k] = (DT)A0[3 * j + k]; DBf[3 * j + k] = (DT)DB[3 * j + k]; }
        }
        permbest[j] = j;
    }
    __syncwarp();
    double db[3] = {0, 0, 0}, newdist = 0;
    int ntries = 0, nperm = n, fail = 0;
    for (int iter = 0; iter < 64 && nperm > 0; ++iter) {
        for (int j = lane; j < n; j += 32) newperm[j] = j;
        double pdsum = 0;
        __syncwarp();
        for (int gi = 0; gi < P.ngroups; ++gi) {
            const GroupDev g = groups[P.group0 + gi];
            const int ns = g.n, m = g.m, s0 = g.slot0 - a0;
            const bool dense = (m == ns);
            for (int i = lane; i < ns; i += 32) {
                const DT *bi = DBf + 3 * (s0 + i);
                CT *crow = lcc + (long long)i * m;
                if (dense) {
                    for (int j = 0; j < ns; ++j)
                        crow[j] = (CT)((double)pdist2<DT>(bi, DAf + 3 * (s0 + j), bulk, box) * kPScale);
                } else if (sizeof(DT) == 4 && sizeof(CT) == 4) {
                    // heap kept in place: float distances in the 32-bit cost slots
                    float *hd = reinterpret_cast<float *>(crow);
                    unsigned short *hk = lkk + (long long)i * m;
                    nearest_heap<float, unsigned short>(hd, hk, (const float *)bi, (const float *)DAf + 3 * s0,
                                                        ns, m, bulk, box);
                    for (int j = 0; j < m; ++j) crow[j] = (CT)((double)hd[j] * kPScale);
                } else {
                    DT hd[kMaxNei];
                    int hk[kMaxNei];
                    nearest_heap<DT, int>(hd, hk, bi, DAf + 3 * s0, ns, m, bulk, box);
                    unsigned short *krow = lkk + (long long)i * m;
                    for (int j = 0; j < m; ++j) {
                        crow[j] = (CT)((double)hd[j] * kPScale);
                        krow[j] = (unsigned short)hk[j];
                    }
                }
            }
            __syncwarp();
            int rc = jv_warp<CT>(ns, m, dense, lcc, lkk, lv, ld, lx, ly, llab, lfr, ltodo, lok);
            if (rc) fail += 1;
            __syncwarp();
            for (int i = lane; i < ns; i += 32) {
                int col = lx[i];
                if (col >= ns) { col = ns - 1; fail += 1; }
                if (col < 0) { col = 0; fail += 1; }
                newperm[s0 + i] = s0 + col;
                pdsum += pdist2<double>(DB + 3 * (s0 + i), DA + 3 * (s0 + col), bulk, box);
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
                for (int k = 0; k < 3; ++k) {
                    double t = DB[3 * j + k] - a[k];
                    s3[k] += t - box[k] * round(t / box[k]);
                }
            }
            double dn[3];
            for (int k = 0; k < 3; ++k) dn[k] = wsum_d(s3[k]) / n;
            double s1 = 0;
            for (int j = lane; j < n; j += 32) {
                const double *a = DA + 3 * newperm[j];
                double ad[3] = {a[0] + dn[0], a[1] + dn[1], a[2] + dn[2]};
                s1 += pdist2<double>(DB + 3 * j, ad, 1, box);
            }
            newdist = sqrt(wsum_d(s1));
            for (int k = 0; k < 3; ++k) db[k] += dn[k];
            __syncwarp();
            for (int j = lane; j < n; j += 32) {
                permbest[j] = ptmp[j];
                for (int k = 0; k < 3; ++k) {
                    DA[3 * j + k] = A0[3 * ptmp[j] + k] + db[k];
                    if (sizeof(DT) == 4) DAf[3 * j + k] = (DT)DA[3 * j + k];
                }
            }
        } else {
            double q[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int j = lane; j < n; j += 32) {
                const double *b = DB + 3 * j, *a = DA + 3 * newperm[j];
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
                const double *a = A0 + 3 * ptmp[j];
                for (int k = 0; k < 3; ++k) {
                    DA[3 * j + k] = sRb[3 * k] * a[0] + sRb[3 * k + 1] * a[1] + sRb[3 * k + 2] * a[2];
                    if (sizeof(DT) == 4) DAf[3 * j + k] = (DT)DA[3 * j + k];
                }
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
        for (int j = lane; j < n; j += 32)
            for (int k = 0; k < 3; ++k) {
                double t = DB[3 * j + k] - DA[3 * j + k];
                s3[k] += t - box[k] * round(t / box[k]);
            }
        double dn[3];
        for (int k = 0; k < 3; ++k) dn[k] = wsum_d(s3[k]) / n;
        double s1 = 0;
        for (int j = lane; j < n; j += 32) {
            double ad[3] = {DA[3 * j] + dn[0], DA[3 * j + 1] + dn[1], DA[3 * j + 2] + dn[2]};
            s1 += pdist2<double>(DB + 3 * j, ad, 1, box);
        }
        newdist = sqrt(wsum_d(s1));
        for (int k = 0; k < 3; ++k) db[k] += dn[k];
        __syncwarp();
        for (int j = lane; j < n; j += 32)
            for (int k = 0; k < 3; ++k) DA[3 * j + k] += dn[k];
    } else {
        double q[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int j = lane; j < n; j += 32) {
            const double *b = DB + 3 * j, *a = DA + 3 * j;
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
                DA[3 * j + k] = sRn[3 * k] * a[0] + sRn[3 * k + 1] * a[1] + sRn[3 * k + 2] * a[2] + cmb[k];
        }
    }
    __syncwarp();
    const long long ob = P.candatom0 + (long long)local * n;
    for (int j = lane; j < n; j += 32) {
        cperm[ob + j] = permbest[j];
        for (int k = 0; k < 3; ++k) cxyz[3 * (ob + j) + k] = DA[3 * j + k];
    }
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


// Buckets run concurrently on the auxiliary streams (fork/join through
// events on the main stream) so that small and large problems share the SMs.
void launch_refine(const RefineBuffers &b, cudaStream_t main, cudaStream_t *aux, int naux,
                   cudaEvent_t fork, cudaEvent_t *join) {
    cudaEventRecord(fork, main);
    for (int a = 0; a < naux; ++a) cudaStreamWaitEvent(aux[a], fork, 0);
    for (int k = 0; k < b.nbuckets; ++k) {
        const RefineBucket &bk = b.buckets[k];
        if (bk.count == 0) continue;
        const int *list = b.cand_list + bk.offset;
        cudaStream_t s = naux ? aux[k % naux] : main;
#define FO_LAUNCH_REFINE(DT, CT)                                                                   \
    do {                                                                                          \
        cudaFuncSetAttribute(k_refine_warp<DT, CT>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                             (int)bk.smem);                                                       \
        k_refine_warp<DT, CT><<<bk.count, 32, bk.smem, s>>>(                                      \
            b.pairs, b.groups, list, b.cand2pair, b.xa, b.xb, b.peaks, b.npeaks, b.lap, b.cdist,  \
            b.cR, b.cdisp, b.cxyz, b.cperm, b.cniter, b.cstat);                                   \
    } while (0)
        if (b.fp32) {
            if (bk.ct64) FO_LAUNCH_REFINE(float, long long); else FO_LAUNCH_REFINE(float, int);
        } else {
            if (bk.ct64) FO_LAUNCH_REFINE(double, long long); else FO_LAUNCH_REFINE(double, int);
        }
#undef FO_LAUNCH_REFINE
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
