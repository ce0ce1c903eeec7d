// fo_refine.cu -- candidate refinement and selection.
//
// One block per candidate (pair, orientation, peak): rotate (cluster) or shift
// (bulk) the moved structure by the candidate, then alternate
//   per-group squared distances (60 nearest per row when a group has more
//   than 60 atoms) -> integer costs INT(d^2 * 1e6) -> sparse Jonker-Volgenant
//   assignment -> Kearsley rotation (cluster) or mean minimum-image
//   displacement (bulk)
// until no atom changes partner, the distance grows, or 21 tries.
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

namespace fo {

struct LapView {
    long long *cc;
    int *kk;
    long long *v, *d;
    int *x, *y, *lab, *fr, *todo;
    unsigned char *ok;
};

__host__ __device__ inline long long lap_align8(long long b) { return (b + 7) & ~7LL; }

__host__ __device__ inline long long lap_bytes(int maxg) {
    int m = maxg < kMaxNei ? maxg : kMaxNei;
    long long b = 0;
    b += lap_align8(8LL * maxg * m);
    b += lap_align8(4LL * maxg * m);
    b += 2 * lap_align8(8LL * maxg);
    b += 5 * lap_align8(4LL * maxg);
    b += lap_align8(maxg);
    return b;
}

__device__ inline LapView lap_view(unsigned char *base, int maxg) {
    int m = maxg < kMaxNei ? maxg : kMaxNei;
    LapView L;
    long long o = 0;
    L.cc = (long long *)(base + o); o += lap_align8(8LL * maxg * m);
    L.kk = (int *)(base + o); o += lap_align8(4LL * maxg * m);
    L.v = (long long *)(base + o); o += lap_align8(8LL * maxg);
    L.d = (long long *)(base + o); o += lap_align8(8LL * maxg);
    L.x = (int *)(base + o); o += lap_align8(4LL * maxg);
    L.y = (int *)(base + o); o += lap_align8(4LL * maxg);
    L.lab = (int *)(base + o); o += lap_align8(4LL * maxg);
    L.fr = (int *)(base + o); o += lap_align8(4LL * maxg);
    L.todo = (int *)(base + o); o += lap_align8(4LL * maxg);
    L.ok = base + o;
    return L;
}

// Sparse Jonker-Volgenant (Computing 38, 1987) on CSR rows of fixed width m:
// column reduction, reduction transfer, two augmenting-row-reduction passes,
// shortest augmenting paths.  Sequential (one thread).  Returns 0 on success;
// a failed matching leaves x[i] = -1 for unmatched rows.  Every loop is
// bounded; a guard trip reports failure instead of spinning.
__device__ int jv_sparse(int n, int m, const long long *cc, const int *kk, LapView &L) {
    long long *v = L.v, *dd = L.d;
    int *x = L.x, *y = L.y, *lab = L.lab, *fr = L.fr, *todo = L.todo;
    unsigned char *ok = L.ok;  // also used as the "several minima" flag in phase 1
    for (int j = 0; j < n; ++j) { v[j] = kBigInt; y[j] = -1; ok[j] = 0; }
    for (int i = 0; i < n; ++i) {
        x[i] = -1;
        for (int t = i * m; t < i * m + m; ++t) {
            int j = kk[t];
            if (cc[t] < v[j]) { v[j] = cc[t]; y[j] = i; }
        }
    }
    for (int j = n - 1; j >= 0; --j) {
        int i = y[j];
        if (i < 0) return 1;
        if (x[i] >= 0) { ok[i] = 1; y[j] = -1; }
        else x[i] = j;
    }
    int nfree = 0;
    for (int i = 0; i < n; ++i) {
        if (x[i] < 0) fr[nfree++] = i;
        else if (ok[i]) ok[i] = 0;
        else {
            int j1 = x[i];
            long long mn = kBigInt;
            for (int t = i * m; t < i * m + m; ++t) {
                int j = kk[t];
                if (j == j1) continue;
                if (cc[t] - v[j] < mn) mn = cc[t] - v[j];
            }
            v[j1] -= mn;
        }
    }
    if (nfree == 0) return 0;
    long long guard = 0;
    const long long gmax = 64LL * n * (long long)n * m + 100000;
    int j0 = -1, j1 = -1;
    for (int pass = 0; pass < 2 && nfree > 0; ++pass) {
        int l0 = nfree, k = 0;
        nfree = 0;
        while (k < l0) {
            if (++guard > gmax) return 9;
            int i = fr[k++];
            long long u1 = kBigInt, u2 = kBigInt;
            for (int t = i * m; t < i * m + m; ++t) {
                int j = kk[t];
                long long h = cc[t] - v[j];
                if (h < u2) {
                    if (h >= u1) { u2 = h; j1 = j; }
                    else { u2 = u1; u1 = h; j1 = j0; j0 = j; }
                }
            }
            if (j0 < 0) return 2;
            int i0 = y[j0];
            bool reinsert = false;
            if (u1 < u2) {
                v[j0] = v[j0] - u2 + u1;
                reinsert = (i0 >= 0);
            } else if (i0 >= 0) {
                if (j1 < 0) return 3;
                j0 = j1;
                i0 = y[j1];
                reinsert = (i0 >= 0);
            }
            if (reinsert) {
                if (u1 < u2) fr[--k] = i0;
                else fr[nfree++] = i0;
            }
            x[i] = j0;
            y[j0] = i;
        }
    }
    const int l0 = nfree;
    for (int f = 0; f < l0; ++f) {
        for (int j = 0; j < n; ++j) { ok[j] = 0; dd[j] = kBigInt; }
        long long mn = kBigInt;
        const int i0 = fr[f];
        int td = n - 1, k = 0, jend = -1;
        bool price = false;
        for (int t = i0 * m; t < i0 * m + m; ++t) {
            int j = kk[t];
            long long dj = cc[t] - v[j];
            dd[j] = dj;
            lab[j] = i0;
            if (dj <= mn) {
                if (dj < mn) { mn = dj; k = 0; }
                todo[k++] = j;
            }
        }
        for (int h = 0; h < k; ++h) {
            int j = todo[h];
            if (y[j] < 0) { jend = j; break; }
            ok[j] = 1;
        }
        while (jend < 0) {
            if (++guard > gmax) return 9;
            if (k == 0) return 4;
            int jc = todo[--k];
            int i = y[jc];
            todo[td--] = jc;
            int t = i * m;
            while (t < i * m + m && kk[t] != jc) ++t;
            if (t == i * m + m) return 5;
            long long h = cc[t] - v[jc] - mn;
            for (t = i * m; t < i * m + m; ++t) {
                int j = kk[t];
                if (ok[j]) continue;
                long long vj = cc[t] - h - v[j];
                if (vj < dd[j]) {
                    dd[j] = vj;
                    lab[j] = i;
                    if (vj == mn) {
                        if (y[j] < 0) { jend = j; price = true; break; }
                        todo[k++] = j;
                        ok[j] = 1;
                    }
                }
            }
            if (jend >= 0) break;
            if (k != 0) continue;
            mn = kBigInt - 1;
            for (int j = 0; j < n; ++j) {
                if (dd[j] <= mn && !ok[j]) {
                    if (dd[j] < mn) { mn = dd[j]; k = 0; }
                    todo[k++] = j;
                }
            }
            for (int h2 = 0; h2 < k; ++h2) {
                int j = todo[h2];
                if (y[j] < 0) { jend = j; price = true; break; }
                ok[j] = 1;
            }
        }
        if (price && mn != 0)
            for (int q = td + 1; q < n; ++q) {
                int jj = todo[q];
                v[jj] += dd[jj] - mn;
            }
        for (int steps = 0;; ++steps) {
            if (steps > n + 1) return 6;
            int i = lab[jend];
            y[jend] = i;
            int ks = jend;
            jend = x[i];
            x[i] = ks;
            if (i == i0) break;
        }
    }
    return 0;
}

__device__ inline double pairdist2(const double *c1, const double *c2, int bulk, const double *box) {
    double d = 0;
    for (int k = 0; k < 3; ++k) {
        double t = c1[k] - c2[k];
        if (bulk) {
            if (box[k] == 0.0) continue;
            t -= box[k] * round(t / box[k]);
        }
        d += t * t;
    }
    return d;
}

struct RefineCtl {
    double Rb[9], Rc[9], Rn[9], cmb[3], db[3], dn[3], d0[3];
    double newdist, pdsum;
    int nperm, ntries, fail, done;
};

__global__ void __launch_bounds__(256) k_refine(const PairDev *pairs, const GroupDev *groups,
                                                const int *cand2pair, const double *xa,
                                                const double *xb, const double *peaks,
                                                const int *npeaks, unsigned char *lap,
                                                double *cdist, double *cR, double *cdisp,
                                                double *cxyz, int *cperm, int *cniter, int *cstat) {
    extern __shared__ double sm[];
    __shared__ RefineCtl C;
    __shared__ double red[32 * 10];
    const int c = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const int p = cand2pair[c];
    const PairDev &P = pairs[p];
    const int local = c - P.cand0, o = local / P.nrot, ci = local % P.nrot;
    if (ci >= npeaks[2 * p + o]) {
        if (tid == 0) { cdist[c] = INFINITY; cstat[c] = -1; }
        return;
    }
    const int n = P.n, bulk = P.bulk, a0 = P.atom0;
    double *DB = sm, *A0 = DB + 3 * n, *DA = A0 + 3 * n, *DUM = DA + 3 * n;
    int *permbest = (int *)(DUM + 3 * n), *saveperm = permbest + n, *newperm = saveperm + n;
    const double box[3] = {P.box[0], P.box[1], P.box[2]};
    const double *pk = peaks + 3LL * (P.cand0 + o * P.nrot + ci);
    if (tid == 0) {
        for (int k = 0; k < 9; ++k) C.Rb[k] = (k % 4 == 0) ? 1.0 : 0.0;
        for (int k = 0; k < 3; ++k) { C.db[k] = 0; C.cmb[k] = 0; C.d0[k] = 0; }
        if (bulk) {
            for (int k = 0; k < 9; ++k) C.Rc[k] = (k % 4 == 0) ? 1.0 : 0.0;
            for (int k = 0; k < 3; ++k) C.d0[k] = (pk[k] - 1.0) * box[k] / P.G;
        } else {
            const double conv = FO_PI / P.G;
            euler_matrix((pk[0] - 1.0) * 2 * conv, (pk[1] - 0.5) * conv, (pk[2] - 1.0) * 2 * conv, C.Rc);
        }
        C.fail = 0;
    }
    __syncthreads();
    const double sgn = (o == 1) ? -1.0 : 1.0;
    double cs[6] = {0, 0, 0, 0, 0, 0};
    for (int j = tid; j < n; j += nt) {
        const double *a = xa + 3LL * (a0 + j), *b = xb + 3LL * (a0 + j);
        for (int k = 0; k < 3; ++k) DB[3 * j + k] = b[k];
        if (bulk) {
            for (int k = 0; k < 3; ++k) A0[3 * j + k] = a[k] - C.d0[k];
        } else {
            for (int k = 0; k < 3; ++k)
                A0[3 * j + k] = sgn * (C.Rc[3 * k] * a[0] + C.Rc[3 * k + 1] * a[1] + C.Rc[3 * k + 2] * a[2]);
        }
        for (int k = 0; k < 3; ++k) { cs[k] += A0[3 * j + k]; cs[3 + k] += DB[3 * j + k]; }
    }
    block_sum<double, 6>(cs, red);
    if (!bulk) {  // ITERATIVEALIGN works on structures centred at their centroids
        for (int j = tid; j < n; j += nt)
            for (int k = 0; k < 3; ++k) {
                A0[3 * j + k] -= cs[k] / n;
                DB[3 * j + k] -= cs[3 + k] / n;
            }
        if (tid == 0)
            for (int k = 0; k < 3; ++k) C.cmb[k] = cs[3 + k] / n;
    }
    for (int j = tid; j < n; j += nt) {
        for (int k = 0; k < 3; ++k) DA[3 * j + k] = A0[3 * j + k];
        permbest[j] = j;
    }
    if (tid == 0) { C.ntries = 0; C.nperm = n; C.done = 0; }
    __syncthreads();
    const int maxg_m = 0;
    (void)maxg_m;
    unsigned char *lapbase = lap + P.lap0 + (long long)local * P.lapstride;
    int maxg = 0;
    for (int gi = 0; gi < P.ngroups; ++gi) maxg = max(maxg, groups[P.group0 + gi].n);
    LapView LV = lap_view(lapbase, maxg);

    for (int iter = 0; iter < 64 && C.nperm > 0; ++iter) {
        for (int j = tid; j < n; j += nt) {
            for (int k = 0; k < 3; ++k) DUM[3 * j + k] = DA[3 * j + k];
            saveperm[j] = permbest[j];
            newperm[j] = j;
        }
        if (tid == 0) C.pdsum = 0;
        __syncthreads();
        for (int gi = 0; gi < P.ngroups; ++gi) {
            const GroupDev g = groups[P.group0 + gi];
            const int ns = g.n, m = g.m, s0 = g.slot0 - a0;
            for (int i = tid; i < ns; i += nt) {
                const double *bi = DB + 3 * (s0 + i);
                long long *crow = LV.cc + (long long)i * m;
                int *krow = LV.kk + (long long)i * m;
                if (m == ns) {
                    for (int j = 0; j < ns; ++j) {
                        crow[j] = (long long)(pairdist2(bi, DA + 3 * (s0 + j), bulk, box) * kPScale);
                        krow[j] = j;
                    }
                } else {
                    double hd[kMaxNei];
                    int hk[kMaxNei];
                    for (int j = 0; j < m; ++j) {
                        hd[j] = pairdist2(bi, DA + 3 * (s0 + j), bulk, box);
                        hk[j] = j;
                        int l = j + 1;
                        while (l > 1) {
                            int l2 = l / 2;
                            if (hd[l2 - 1] < hd[l - 1]) {
                                double h = hd[l2 - 1]; hd[l2 - 1] = hd[l - 1]; hd[l - 1] = h;
                                int t = hk[l2 - 1]; hk[l2 - 1] = hk[l - 1]; hk[l - 1] = t;
                                l = l2;
                            } else break;
                        }
                    }
                    for (int j = m; j < ns; ++j) {
                        double d = pairdist2(bi, DA + 3 * (s0 + j), bulk, box);
                        if (!(d < hd[0])) continue;
                        hd[0] = d;
                        hk[0] = j;
                        int l = 1;
                        for (int guard = 0; guard < 64; ++guard) {
                            int l2 = 2 * l;
                            if (l2 + 1 > m) {
                                if (l2 <= m && hd[l2 - 1] > hd[l - 1]) {
                                    double h = hd[l2 - 1]; hd[l2 - 1] = hd[l - 1]; hd[l - 1] = h;
                                    int t = hk[l2 - 1]; hk[l2 - 1] = hk[l - 1]; hk[l - 1] = t;
                                }
                                break;
                            }
                            int a = (hd[l2] > hd[l2 - 1]) ? l2 + 1 : l2;
                            if (hd[a - 1] > hd[l - 1]) {
                                double h = hd[a - 1]; hd[a - 1] = hd[l - 1]; hd[l - 1] = h;
                                int t = hk[a - 1]; hk[a - 1] = hk[l - 1]; hk[l - 1] = t;
                                l = a;
                            } else break;
                        }
                    }
                    for (int j = 0; j < m; ++j) {
                        crow[j] = (long long)(hd[j] * kPScale);
                        krow[j] = hk[j];
                    }
                }
            }
            __syncthreads();
            if (tid == 0) {
                int rc = jv_sparse(ns, m, LV.cc, LV.kk, LV);
                if (rc) C.fail += 1;
                double pd = 0;
                for (int i = 0; i < ns; ++i) {
                    int col = LV.x[i];
                    if (col >= ns) { col = ns - 1; C.fail += 1; }
                    if (col < 0) { col = 0; C.fail += 1; }
                    newperm[s0 + i] = s0 + col;
                    pd += pairdist2(DB + 3 * (s0 + i), DA + 3 * (s0 + col), bulk, box);
                }
                C.pdsum += pd;
            }
            __syncthreads();
        }
        int cnt[1] = {0};
        for (int j = tid; j < n; j += nt) {
            int q = newperm[j];
            for (int k = 0; k < 3; ++k) DA[3 * j + k] = DUM[3 * q + k];
            permbest[j] = saveperm[q];
            if (q != j) ++cnt[0];
        }
        block_sum<int, 1>(cnt, (int *)red);
        if (bulk) {
            double s3[3] = {0, 0, 0};
            for (int j = tid; j < n; j += nt)
                for (int k = 0; k < 3; ++k) {
                    double t = DB[3 * j + k] - DA[3 * j + k];
                    s3[k] += t - box[k] * round(t / box[k]);
                }
            block_sum<double, 3>(s3, red);
            double dn[3] = {s3[0] / n, s3[1] / n, s3[2] / n};
            double s1[1] = {0};
            for (int j = tid; j < n; j += nt) {
                double a[3] = {DA[3 * j] + dn[0], DA[3 * j + 1] + dn[1], DA[3 * j + 2] + dn[2]};
                s1[0] += pairdist2(DB + 3 * j, a, 1, box);
            }
            block_sum<double, 1>(s1, red);
            if (tid == 0) {
                C.newdist = sqrt(s1[0]);
                for (int k = 0; k < 3; ++k) C.db[k] += dn[k];
            }
            __syncthreads();
            for (int j = tid; j < n; j += nt)
                for (int k = 0; k < 3; ++k) DA[3 * j + k] = A0[3 * permbest[j] + k] + C.db[k];
        } else {
            double q[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
            for (int j = tid; j < n; j += nt) {
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
            block_sum<double, 10>(q, red);
            if (tid == 0) {
                C.newdist = kearsley_rotation(q, C.Rn);
                matmul3(C.Rn, C.Rb, C.Rb);
            }
            __syncthreads();
            for (int j = tid; j < n; j += nt) {
                const double *a = A0 + 3 * permbest[j];
                for (int k = 0; k < 3; ++k)
                    DA[3 * j + k] = C.Rb[3 * k] * a[0] + C.Rb[3 * k + 1] * a[1] + C.Rb[3 * k + 2] * a[2];
            }
        }
        if (tid == 0) {
            C.nperm = cnt[0];
            C.ntries += 1;
            double pd = sqrt(C.pdsum);
            if ((C.newdist - pd) / C.newdist > sqrt((double)n) / kPScale) C.done = 1;
            if (C.ntries > kMaxTries) C.done = 1;
            if (C.done) C.nperm = 0;
        }
        __syncthreads();
    }
    // final minimisation
    if (bulk) {
        double s3[3] = {0, 0, 0};
        for (int j = tid; j < n; j += nt)
            for (int k = 0; k < 3; ++k) {
                double t = DB[3 * j + k] - DA[3 * j + k];
                s3[k] += t - box[k] * round(t / box[k]);
            }
        block_sum<double, 3>(s3, red);
        double dn[3] = {s3[0] / n, s3[1] / n, s3[2] / n};
        double s1[1] = {0};
        for (int j = tid; j < n; j += nt) {
            double a[3] = {DA[3 * j] + dn[0], DA[3 * j + 1] + dn[1], DA[3 * j + 2] + dn[2]};
            s1[0] += pairdist2(DB + 3 * j, a, 1, box);
        }
        block_sum<double, 1>(s1, red);
        for (int j = tid; j < n; j += nt)
            for (int k = 0; k < 3; ++k) DA[3 * j + k] += dn[k];
        if (tid == 0) {
            C.newdist = sqrt(s1[0]);
            for (int k = 0; k < 3; ++k) C.db[k] += dn[k];
        }
    } else {
        double q[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        for (int j = tid; j < n; j += nt) {
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
        block_sum<double, 10>(q, red);
        if (tid == 0) {
            C.newdist = kearsley_rotation(q, C.Rn);
            matmul3(C.Rn, C.Rb, C.Rb);
        }
        __syncthreads();
        for (int j = tid; j < n; j += nt) {
            double a[3] = {DA[3 * j], DA[3 * j + 1], DA[3 * j + 2]};
            for (int k = 0; k < 3; ++k)
                DA[3 * j + k] = C.Rn[3 * k] * a[0] + C.Rn[3 * k + 1] * a[1] + C.Rn[3 * k + 2] * a[2] + C.cmb[k];
        }
    }
    __syncthreads();
    const long long ob = P.candatom0 + (long long)local * n;
    for (int j = tid; j < n; j += nt) {
        cperm[ob + j] = permbest[j];
        for (int k = 0; k < 3; ++k) cxyz[3 * (ob + j) + k] = DA[3 * j + k];
    }
    if (tid == 0) {
        cdist[c] = C.newdist;
        double R[9];
        matmul3(C.Rb, C.Rc, R);
        for (int k = 0; k < 9; ++k) cR[9LL * c + k] = bulk ? ((k % 4 == 0) ? 1.0 : 0.0) : R[k];
        for (int k = 0; k < 3; ++k) cdisp[3LL * c + k] = C.db[k] - C.d0[k];
        cniter[c] = C.ntries;
        cstat[c] = C.fail ? (int)ST_LAP_FAILED : 0;
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

long long lap_bytes_host(int maxg) { return lap_bytes(maxg); }

size_t refine_smem_bytes(int maxn) { return (size_t)maxn * (12 * sizeof(double) + 3 * sizeof(int)); }

void launch_refine(const RefineBuffers &b, cudaStream_t s) {
    size_t sm = refine_smem_bytes(b.maxn);
    cudaFuncSetAttribute(k_refine, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_refine<<<b.ncand, 256, sm, s>>>(b.pairs, b.groups, b.cand2pair, b.xa, b.xb, b.peaks, b.npeaks,
                                      b.lap, b.cdist, b.cR, b.cdisp, b.cxyz, b.cperm, b.cniter, b.cstat);
}

void launch_select(const RefineBuffers &b, cudaStream_t s) {
    k_select<<<b.npairs, 256, 0, s>>>(b.pairs, b.slot2orig, b.npeaks, b.pstatus, b.overlap_max,
                                      b.cdist, b.cR, b.cdisp, b.cxyz, b.cperm, b.cniter, b.cstat,
                                      (fo_pair_result *)b.results, b.aligned, b.permbest);
}

}  // namespace fo
