// fo_peaks.cu -- peak extraction on the overlap grids (rotations or
// translations): repeated first-maximum search, periodic window, 11-parameter
// Gaussian fit by Levenberg-Marquardt, subtraction of the fitted peak from
// the whole grid.
//
// One warp per (orientation, pair).  The fit of the 5^3 window (half-width 2,
// the case nearly every search ends in) keeps the window, the parameters and
// the factorisation of the damped normal equations in registers: every lane
// solves the same 11x11 system, so no lane waits on another and nothing goes
// through shared memory but the 77 reduced sums.  A search that finds no peak
// with half-width 2 is continued with wider windows (3 .. kMaxWin) by a second
// kernel that holds the window in shared memory.
//
// Reference behaviour: FINDPEAKS / FINDPEAK / FIT / FCN / GAUSSIAN,
// fastoverlap/f90/fastutils.f90:231-548 (fit tolerance 1e-6, :69; window
// half-width 2, :68; 100*(11+1) model evaluations, lmder1 at :395).
#include "fo_common.cuh"
#include "fo_kernels.h"

namespace fo {

constexpr int kMaxWin = 7;   // largest window half-width handled on chip
constexpr unsigned kAll = 0xffffffffu;

template <typename T, typename P>
__device__ inline T peak_model(const P *p, T u1, T u2, T u3, T *e_out) {
    T Y = T(p[2]) * u1 * u1 + T(p[3]) * u2 * u2 + T(p[4]) * u3 * u3 + T(p[5]) * u1 * u2 +
          T(p[6]) * u2 * u3 + T(p[7]) * u1 * u3;
    T e = exp(-Y);
    if (e_out) *e_out = e;
    return T(p[0]) * e + T(p[1]);
}

// Residual and Jacobian row of one window point (value w at 1-based window
// coordinates X1..X3), added into the packed normal equations h[0..65]
// (lower triangle of J^T J) and h[66..76] (J^T r).
template <typename T>
__device__ __forceinline__ void lm_point(const T (&q)[11], T w, T X1, T X2, T X3, T (&h)[77]) {
    const T u1 = X1 - q[8], u2 = X2 - q[9], u3 = X3 - q[10];
    T e;
    const T f = peak_model<T, T>(q, u1, u2, u3, &e);
    const T r = f - w;
    const T ae = q[0] * e;
    T J[11];
    J[0] = e; J[1] = 1;
    J[2] = -ae * u1 * u1; J[3] = -ae * u2 * u2; J[4] = -ae * u3 * u3;
    J[5] = -ae * u1 * u2; J[6] = -ae * u2 * u3; J[7] = -ae * u1 * u3;
    J[8] = ae * (T(2) * q[2] * u1 + q[5] * u2 + q[7] * u3);
    J[9] = ae * (T(2) * q[3] * u2 + q[5] * u1 + q[6] * u3);
    J[10] = ae * (T(2) * q[4] * u3 + q[6] * u2 + q[7] * u1);
    int k = 0;
#pragma unroll
    for (int a = 0; a < 11; ++a)
#pragma unroll
        for (int b = 0; b <= a; ++b) h[k++] += J[a] * J[b];
#pragma unroll
    for (int a = 0; a < 11; ++a) h[66 + a] += J[a] * r;
}

template <typename T>
__device__ __forceinline__ T lm_resid2(const T (&q)[11], T w, T X1, T X2, T X3) {
    const T r = peak_model<T, T>(q, X1 - q[8], X2 - q[9], X3 - q[10], (T *)nullptr) - w;
    return r * r;
}

// Half-width-2 window: point t = lane + 32k (k < 4, t < 125) of the 5^3 block,
// value and coordinates in registers.
template <typename T>
struct WinRegs {
    T v[4], x1[4], x2[4], x3[4];
    unsigned valid;   // bit k: point lane + 32k exists
    __device__ T cost(const T (&q)[11]) const {
        T s = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if ((valid >> k) & 1u) s += lm_resid2<T>(q, v[k], x1[k], x2[k], x3[k]);
        return warp_sum(s);
    }
    __device__ void accumulate(const T (&q)[11], T (&h)[77]) const {
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if ((valid >> k) & 1u) lm_point<T>(q, v[k], x1[k], x2[k], x3[k], h);
    }
};

// Wider windows: (2w+1)^3 values in shared memory, i1 fastest.
template <typename T>
struct WinSmem {
    const T *win;
    int n, npts;
    __device__ T cost(const T (&q)[11]) const {
        T s = 0;
        for (int t = threadIdx.x & 31; t < npts; t += 32)
            s += lm_resid2<T>(q, win[t], T(t % n + 1), T((t / n) % n + 1), T(t / (n * n) + 1));
        return warp_sum(s);
    }
    __device__ void accumulate(const T (&q)[11], T (&h)[77]) const {
        for (int t = threadIdx.x & 31; t < npts; t += 32)
            lm_point<T>(q, win[t], T(t % n + 1), T((t / n) % n + 1), T(t / (n * n) + 1), h);
    }
};

// Warp sums of the 77 per-lane accumulators, written to out[0..76], by
// recursive halving: at each level a lane keeps one half of its values and
// adds the partner's copy of that half (77 shuffles in all instead of 5 per
// value).  Lane L ends with the totals of up to 3 indices.
template <typename T>
__device__ __forceinline__ void warp_reduce77(const T (&h)[77], T *out) {
    const int lane = threadIdx.x & 31;
    const bool b16 = lane & 16, b8 = lane & 8, b4 = lane & 4, b2 = lane & 2, b1 = lane & 1;
    T a[39], b[20], c[10], d[5], e[3];
#pragma unroll
    for (int i = 0; i < 39; ++i) {   // 77 (+1 zero) -> 39
        const T lo = h[i], hi = (i + 39 < 77) ? h[i + 39] : T(0);
        a[i] = (b16 ? hi : lo) + __shfl_xor_sync(kAll, b16 ? lo : hi, 16);
    }
#pragma unroll
    for (int i = 0; i < 20; ++i) {   // 39 (+1 zero) -> 20
        const T lo = a[i], hi = (i + 20 < 39) ? a[i + 20] : T(0);
        b[i] = (b8 ? hi : lo) + __shfl_xor_sync(kAll, b8 ? lo : hi, 8);
    }
#pragma unroll
    for (int i = 0; i < 10; ++i) {   // 20 -> 10
        const T lo = b[i], hi = b[i + 10];
        c[i] = (b4 ? hi : lo) + __shfl_xor_sync(kAll, b4 ? lo : hi, 4);
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {    // 10 -> 5
        const T lo = c[i], hi = c[i + 5];
        d[i] = (b2 ? hi : lo) + __shfl_xor_sync(kAll, b2 ? lo : hi, 2);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {    // 5 (+1 zero) -> 3
        const T lo = d[i], hi = (i + 3 < 5) ? d[i + 3] : T(0);
        e[i] = (b1 ? hi : lo) + __shfl_xor_sync(kAll, b1 ? lo : hi, 1);
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int i4 = i + (b1 ? 3 : 0);
        const int i1 = i4 + (b2 ? 5 : 0) + (b4 ? 10 : 0) + (b8 ? 20 : 0);
        const int i0 = i1 + (b16 ? 39 : 0);
        if (i4 < 5 && i1 < 39 && i0 < 77) out[i0] = e[i];
    }
}

// Damped normal equations (H + lambda diag(H)) dl = -g, H packed in Hg[0..65]
// and g in Hg[66..76], solved by Cholesky in registers; in FP32 after scaling
// the system to unit diagonal, which leaves the step unchanged.  The FP32
// scale factors and pivot reciprocals come from the hardware reciprocal
// square root (a step's direction, not its acceptance, depends on them).
// Returns false when the matrix is not positive definite (dl is then
// meaningless).
template <typename T>
__device__ __forceinline__ bool lm_solve(const T *Hg, T lambda, T (&dl)[11]) {
    constexpr bool kScale = sizeof(T) == 4;
    T A[66], sc[11], inv[11], y[11];
#pragma unroll
    for (int a = 0; a < 11; ++a) {
        const T dgl = Hg[a * (a + 1) / 2 + a];
        if constexpr (kScale) sc[a] = rsqrtf(dgl > T(1e-30) ? dgl : T(1e-30));
        else sc[a] = T(1);
    }
#pragma unroll
    for (int a = 0; a < 11; ++a)
#pragma unroll
        for (int b = 0; b <= a; ++b) {
            const int q = a * (a + 1) / 2 + b;
            T v = Hg[q];
            if (a == b) v += lambda * (v > T(1e-30) ? v : T(1e-30));
            A[q] = v * sc[a] * sc[b];
        }
    bool ok = true;
#pragma unroll
    for (int j = 0; j < 11; ++j) {
        const int jj = j * (j + 1) / 2;
        T s = A[jj + j];
#pragma unroll
        for (int k = 0; k < j; ++k) s -= A[jj + k] * A[jj + k];
        ok = ok && (s > T(0));
        if constexpr (kScale) {
            inv[j] = rsqrtf(s > T(0) ? s : T(1));
        } else {
            const T djj = sqrt(s > T(0) ? s : T(1));
            inv[j] = T(1) / djj;
        }
#pragma unroll
        for (int i = j + 1; i < 11; ++i) {
            const int ii = i * (i + 1) / 2;
            T t = A[ii + j];
#pragma unroll
            for (int k = 0; k < j; ++k) t -= A[ii + k] * A[jj + k];
            A[ii + j] = t * inv[j];
        }
    }
#pragma unroll
    for (int i = 0; i < 11; ++i) {
        const int ii = i * (i + 1) / 2;
        T t = -Hg[66 + i] * sc[i];
#pragma unroll
        for (int k = 0; k < i; ++k) t -= A[ii + k] * y[k];
        y[i] = t * inv[i];
    }
#pragma unroll
    for (int i = 10; i >= 0; --i) {
        T t = y[i];
#pragma unroll
        for (int k = i + 1; k < 11; ++k) t -= A[k * (k + 1) / 2 + i] * dl[k];
        dl[i] = t * inv[i];
    }
#pragma unroll
    for (int a = 0; a < 11; ++a) dl[a] *= sc[a];
    return ok;
}

// Levenberg-Marquardt (Marquardt 1963): diagonal damping lambda*diag(J^T J),
// lambda /10 after an accepted step, *10 after a rejected one; stop when the
// relative decrease or the relative step is <= tol (info 1/2/3), when lambda
// exceeds 1e16 (info 4) or after maxfev model evaluations (info 5); info 0:
// the starting cost is not finite.  Executed by one full warp in the
// precision T of the grid; every lane holds the same parameters q (in: the
// start, out: the fit).  Hg: 77 elements of shared memory.
template <typename T, typename W>
__device__ int lm_fit(T (&q)[11], const W &win, T *Hg, T tol) {
    const int maxfev = 1200;
    T lambda = T(1e-3);
    T cost = win.cost(q);
    int nfev = 1;
    if (!isfinite(cost)) return 0;
    for (int outer = 0; outer < 100000; ++outer) {
        T h[77];
#pragma unroll
        for (int k = 0; k < 77; ++k) h[k] = 0;
        win.accumulate(q, h);
        __syncwarp();   // the previous system is no longer read
        warp_reduce77<T>(h, Hg);
        __syncwarp();
        for (int inner = 0; inner < 64; ++inner) {
            T dl[11], pn[11];
            const bool ok = lm_solve<T>(Hg, lambda, dl);
#pragma unroll
            for (int a = 0; a < 11; ++a) pn[a] = q[a] + dl[a];
            T cn = T(INFINITY);
            if (ok) {
                cn = win.cost(pn);
                ++nfev;
            }
            if (ok && cn < cost) {
                T rel = (cost - cn) / cost, step = 0, pnorm = 0;
#pragma unroll
                for (int a = 0; a < 11; ++a) {
                    step += dl[a] * dl[a];
                    pnorm += pn[a] * pn[a];
                }
                step = sqrt(step);
                pnorm = sqrt(pnorm);
#pragma unroll
                for (int a = 0; a < 11; ++a) q[a] = pn[a];
                cost = cn;
                lambda = lambda * T(0.1) > T(1e-15) ? lambda * T(0.1) : T(1e-15);
                const bool c1 = rel <= tol, c2 = step <= tol * (pnorm + tol);
                if (c1 && c2) return 3;
                if (c1) return 1;
                if (c2) return 2;
                if (nfev >= maxfev) return 5;
                break;
            }
            lambda *= T(10);
            if (lambda > T(1e16)) return 4;
            if (nfev >= maxfev) return 5;
        }
    }
    return 5;
}

// Per-lane running sum of a grid: FP64 for FP64 grids; for FP32 grids a
// compensated (Kahan) FP32 sum, which keeps about FP64 accuracy over the few
// hundred terms a lane adds without issuing FP64 instructions in the grid
// loop.  Lane sums are combined in FP64.
template <typename T>
struct GridSum {
    double s = 0;
    __device__ void add(T v) { s += (double)v; }
    __device__ double get() const { return s; }
};
template <>
struct GridSum<float> {
    float s = 0, c = 0;
    __device__ void add(float v) {
        const float y = v - c, t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ double get() const { return (double)s - (double)c; }
};

// warp-wide (max value, first index) and sum; every lane gets the result
template <typename T>
__device__ __forceinline__ void warp_argmax_finish(T best, int bi, double s, T &mx, int &amax, double &sum) {
    for (int o = 16; o > 0; o >>= 1) {
        const T ov = __shfl_xor_sync(kAll, best, o);
        const int oi = __shfl_xor_sync(kAll, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        s += __shfl_xor_sync(kAll, s, o);
    }
    mx = best;
    amax = bi;
    sum = s;
}

// Loads in flight per lane in the full-grid passes.  One warp per grid runs
// them, so the depth of its load pipeline sets their speed on large grids
// (edge >= kDeepGrid: 16 loads per lane, measured 20.8 -> 12.8 ms for 64^3
// grids); grids of edge <= 32 measured faster with 4.
#ifndef FO_DEEP_GRID
#define FO_DEEP_GRID 48
#endif
#ifndef FO_DEEP_UNROLL
#define FO_DEEP_UNROLL 16
#endif
constexpr int kDeepGrid = FO_DEEP_GRID;

// (max value, first index) and sum over a grid of N points by one warp;
// U loads in flight per lane.
template <typename T, int kGridUnroll = 4>
__device__ void warp_argmax_sum(const T *f, int N, T &mx, int &amax, double &sum) {
    const int lane = threadIdx.x & 31;
    T best = -INFINITY;
    int bi = N, i = lane;
    GridSum<T> acc;
    for (; i + 32 * (kGridUnroll - 1) < N; i += 32 * kGridUnroll) {
        T v[kGridUnroll];
#pragma unroll
        for (int u = 0; u < kGridUnroll; ++u) v[u] = f[i + 32 * u];
#pragma unroll
        for (int u = 0; u < kGridUnroll; ++u) {
            acc.add(v[u]);
            if (v[u] > best) { best = v[u]; bi = i + 32 * u; }
        }
    }
    for (; i < N; i += 32) {
        const T v = f[i];
        acc.add(v);
        if (v > best) { best = v; bi = i; }
    }
    warp_argmax_finish<T>(best, bi, acc.get(), mx, amax, sum);
}

// f -= model(p, q - c) over the whole G^3 grid (p: the fit, c: the peak
// centre in 1-based grid coordinates, the model evaluated in the grid's
// precision), then (max value, first index) and sum of the result, in one
// pass by one warp with kGridUnroll loads in flight per lane.
template <typename T, int kGridUnroll = 4>
__device__ void warp_subtract_argmax_sum(T *f, int G, const T (&q)[11], double c1, double c2, double c3,
                                         T &mx, int &amax, double &sum) {
    const int lane = threadIdx.x & 31, N = G * G * G;
    const T t1 = T(c1), t2 = T(c2), t3 = T(c3);
    int i = lane, i1 = i % G, i2 = (i / G) % G, i3 = i / (G * G);
    const int d1 = 32 % G, d2 = (32 / G) % G, d3 = 32 / (G * G);
    T best = -INFINITY;
    int bi = N;
    GridSum<T> acc;
    auto point = [&](T fv, int idx) {
        const T v = fv - peak_model<T, T>(q, T(i1 + 1) - t1, T(i2 + 1) - t2, T(i3 + 1) - t3, (T *)nullptr);
        f[idx] = v;
        acc.add(v);
        if (v > best) { best = v; bi = idx; }
        i1 += d1; i2 += d2; i3 += d3;
        if (i1 >= G) { i1 -= G; ++i2; }
        if (i2 >= G) { i2 -= G; ++i3; }
    };
    for (; i + 32 * (kGridUnroll - 1) < N; i += 32 * kGridUnroll) {
        T v[kGridUnroll];
#pragma unroll
        for (int u = 0; u < kGridUnroll; ++u) v[u] = f[i + 32 * u];
#pragma unroll
        for (int u = 0; u < kGridUnroll; ++u) point(v[u], i + 32 * u);
    }
    for (; i < N; i += 32) point(f[i], i);
    warp_argmax_finish<T>(best, bi, acc.get(), mx, amax, sum);
}

// Start of a fit: amplitude above the grid mean, the mean, unit widths, no
// cross terms, centre at the window's middle (1-based).
template <typename T>
__device__ __forceinline__ void lm_start(T (&q)[11], T mx, double mean, int width) {
    const double init[11] = {(double)mx - mean, mean, 1, 1, 1, 0, 0, 0, width + 1.0, width + 1.0, width + 1.0};
#pragma unroll
    for (int a = 0; a < 11; ++a) q[a] = T(init[a]);
}

// Resident one-warp blocks per SM the register allocation of k_findpeaks is
// sized for (1: as many registers as the fit can use).
#ifndef FO_PEAKS_MINB
#define FO_PEAKS_MINB 1
#endif

// Peaks of one (orientation, pair) grid with the 5^3 window.  Peaks are
// written as 1-based fractional grid coordinates (as FINDPEAKS returns
// them).  A search that finds none leaves npeaks 0 for k_findpeaks_wide.
template <typename T>
__global__ void __launch_bounds__(32, FO_PEAKS_MINB) k_findpeaks(const PairDev *pairs, T *grids, double *omax,
                                                                  double *peaks, double *amps, int *npeaks,
                                                                  double tol) {
    __shared__ T Hg[77];
    constexpr int width = 2, wn = 5;
    const int lane = threadIdx.x, o = blockIdx.x, p = blockIdx.y;
    const PairDev &P = pairs[p];
    if (o >= P.norient) return;
    const int G = P.G, N = G * G * G, nrot = P.nrot;
    T *f = grids + P.grid0 + (long long)o * N;
    T mx;
    int amax;
    double sum;
    const bool deep = G >= kDeepGrid;
    if (deep) warp_argmax_sum<T, FO_DEEP_UNROLL>(f, N, mx, amax, sum);
    else warp_argmax_sum<T>(f, N, mx, amax, sum);
    if (lane == 0) omax[2 * p + o] = (double)mx;
    int nfound = 0;
    double *pk = peaks + 3LL * (P.cand0 + o * nrot);
    for (int np = 0; np < nrot; ++np) {
        const double mean = sum / (double)N;
        const int a1 = amax % G, a2 = (amax / G) % G, a3 = amax / (G * G);
        WinRegs<T> W;
        W.valid = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int t = lane + 32 * k;
            const int i1 = t % wn, i2 = (t / wn) % wn, i3 = t / (wn * wn);
            W.x1[k] = T(i1 + 1);
            W.x2[k] = T(i2 + 1);
            W.x3[k] = T(i3 + 1);
            W.v[k] = 0;
            if (t < wn * wn * wn) {
                const int j1 = ((a1 + i1 - width) % G + G) % G, j2 = ((a2 + i2 - width) % G + G) % G,
                          j3 = ((a3 + i3 - width) % G + G) % G;
                W.v[k] = f[j1 + G * (j2 + G * j3)];
                W.valid |= 1u << k;
            }
        }
        T q[11];
        lm_start<T>(q, mx, mean, width);
        const int info = lm_fit<T>(q, W, Hg, T(tol));
        if (info == 0 || info == 5) break;
        const double c1 = (double)q[8] - width - 1 + (a1 + 1), c2 = (double)q[9] - width - 1 + (a2 + 1),
                     c3 = (double)q[10] - width - 1 + (a3 + 1);
        if (lane == 0) {
            pk[3 * nfound] = c1;
            pk[3 * nfound + 1] = c2;
            pk[3 * nfound + 2] = c3;
            if (amps) amps[P.cand0 + o * nrot + nfound] = (double)q[0];
        }
        ++nfound;
        // subtract the fitted peak (not wrapped) and its mean level; the same
        // pass finds the next first maximum and the new grid sum
        if (deep) warp_subtract_argmax_sum<T, FO_DEEP_UNROLL>(f, G, q, c1, c2, c3, mx, amax, sum);
        else warp_subtract_argmax_sum<T>(f, G, q, c1, c2, c3, mx, amax, sum);
    }
    if (lane == 0) npeaks[2 * p + o] = nfound;
}

// Searches that found no peak yet (npeaks 0) on the untouched grid, with
// half-widths width0, width0 + 1, ... while the half-width stays within G/2
// (the first one unchecked when !check_first, as FINDPEAKS tries its current
// width before widening) and within kMaxWin.
template <typename T>
__global__ void __launch_bounds__(32) k_findpeaks_wide(const PairDev *pairs, T *grids, double *omax,
                                                       double *peaks, double *amps, int *npeaks, int *pstatus,
                                                       int width0, int check_first, double tol) {
    __shared__ T Hg[77];
    __shared__ T win[(2 * kMaxWin + 1) * (2 * kMaxWin + 1) * (2 * kMaxWin + 1)];
    const int lane = threadIdx.x, o = blockIdx.x, p = blockIdx.y;
    const PairDev &P = pairs[p];
    if (o >= P.norient || npeaks[2 * p + o] != 0) return;
    const int G = P.G, N = G * G * G, nrot = P.nrot;
    T *f = grids + P.grid0 + (long long)o * N;
    T mx;
    int amax;
    double sum;
    warp_argmax_sum<T>(f, N, mx, amax, sum);
    if (omax && lane == 0) omax[2 * p + o] = (double)mx;
    int nfound = 0;
    double *pk = peaks + 3LL * (P.cand0 + o * nrot);
    for (int width = width0; nfound == 0 && width >= 1 && width <= kMaxWin; ++width) {
        if ((check_first || width > width0) && width > G / 2) break;
        const int wn = 2 * width + 1;
        for (int np = 0; np < nrot; ++np) {
            const double mean = sum / (double)N;
            const int a1 = amax % G, a2 = (amax / G) % G, a3 = amax / (G * G);
            __syncwarp();   // the previous window is no longer read
            for (int t = lane; t < wn * wn * wn; t += 32) {
                const int i1 = t % wn, i2 = (t / wn) % wn, i3 = t / (wn * wn);
                const int j1 = ((a1 + i1 - width) % G + G) % G, j2 = ((a2 + i2 - width) % G + G) % G,
                          j3 = ((a3 + i3 - width) % G + G) % G;
                win[t] = f[j1 + G * (j2 + G * j3)];
            }
            __syncwarp();
            WinSmem<T> W{win, wn, wn * wn * wn};
            T q[11];
            lm_start<T>(q, mx, mean, width);
            const int info = lm_fit<T>(q, W, Hg, T(tol));
            if (info == 0 || info == 5) break;
            const double c1 = (double)q[8] - width - 1 + (a1 + 1), c2 = (double)q[9] - width - 1 + (a2 + 1),
                         c3 = (double)q[10] - width - 1 + (a3 + 1);
            if (lane == 0) {
                pk[3 * nfound] = c1;
                pk[3 * nfound + 1] = c2;
                pk[3 * nfound + 2] = c3;
                if (amps) amps[P.cand0 + o * nrot + nfound] = (double)q[0];
            }
            ++nfound;
            warp_subtract_argmax_sum<T>(f, G, q, c1, c2, c3, mx, amax, sum);
        }
    }
    if (lane == 0) {
        npeaks[2 * p + o] = nfound;
        if (nfound == 0) atomicMax(&pstatus[p], (int)ST_NO_PEAKS);
    }
}

// width0 == 2: the 5^3 kernel, then wider windows from 3 for the grids left
// without a peak; other starting half-widths go to the wide kernel directly.
// amps may be null.  npeaks must be zero on entry.
void launch_findpeaks_from(const PairDev *pairs, int npairs, void *grid, double *omax, double *peaks,
                           double *amps, int *npeaks, int *pstatus, bool fp32, int width0, cudaStream_t s) {
    dim3 g(2, npairs);
    const double tol = fp32 ? 1e-5 : 1e-6;
    if (fp32) {
        if (width0 == 2)
            k_findpeaks<float><<<g, 32, 0, s>>>(pairs, (float *)grid, omax, peaks, amps, npeaks, tol);
        k_findpeaks_wide<float><<<g, 32, 0, s>>>(pairs, (float *)grid, width0 == 2 ? nullptr : omax, peaks,
                                                 amps, npeaks, pstatus, width0 == 2 ? 3 : width0,
                                                 width0 == 2 ? 1 : 0, tol);
    } else {
        if (width0 == 2)
            k_findpeaks<double><<<g, 32, 0, s>>>(pairs, (double *)grid, omax, peaks, amps, npeaks, tol);
        k_findpeaks_wide<double><<<g, 32, 0, s>>>(pairs, (double *)grid, width0 == 2 ? nullptr : omax, peaks,
                                                  amps, npeaks, pstatus, width0 == 2 ? 3 : width0,
                                                  width0 == 2 ? 1 : 0, tol);
    }
}

void launch_findpeaks(const RefineBuffers &b, bool fp32, cudaStream_t s) {
    launch_findpeaks_from(b.pairs, b.npairs, b.grid, b.overlap_max, b.peaks, nullptr, b.npeaks, b.pstatus, fp32,
                          2, s);
}

}  // namespace fo
