// fo_peaks.cu -- peak extraction on the overlap grids (rotations or
// translations): repeated first-maximum search, periodic window, 11-parameter
// Gaussian fit by Levenberg-Marquardt on one warp, subtraction of the fitted
// peak from the whole grid.
//
// Reference behaviour: FINDPEAKS / FINDPEAK / FIT / FCN / GAUSSIAN,
// fastoverlap/f90/fastutils.f90:231-548 (fit tolerance 1e-6, :69; window
// half-width 2, :68; 100*(11+1) model evaluations, lmder1 at :395).
#include "fo_common.cuh"
#include "fo_kernels.h"

namespace fo {

constexpr int kMaxWin = 7;  // largest window half-width handled on chip
constexpr int kPeakThreads = 64;

template <typename T>
struct LMShared {
    T H[66];   // packed lower triangle of J^T J
    T g[11];   // J^T r
    T A[66];   // Cholesky factor
    T dl[11];  // step
    T p[11];
    T pn[11];
    int info;
    int ok;
};

template <typename T, typename P>
__device__ inline T peak_model(const P *p, T u1, T u2, T u3, T *e_out) {
    T Y = T(p[2]) * u1 * u1 + T(p[3]) * u2 * u2 + T(p[4]) * u3 * u3 + T(p[5]) * u1 * u2 +
          T(p[6]) * u2 * u3 + T(p[7]) * u1 * u3;
    T e = exp(-Y);
    if (e_out) *e_out = e;
    return T(p[0]) * e + T(p[1]);
}

// sum of squared residuals over the window (every lane gets the total)
template <typename T>
__device__ T lm_cost(const T *p, const T *win, int w) {
    const int n = 2 * w + 1, npts = n * n * n, lane = threadIdx.x & 31;
    T S = 0;
    for (int i = lane; i < npts; i += 32) {
        int i1 = i % n, i2 = (i / n) % n, i3 = i / (n * n);
        T r = peak_model<T, T>(p, T(i1 + 1) - p[8], T(i2 + 1) - p[9], T(i3 + 1) - p[10], (T *)nullptr) - win[i];
        S += r * r;
    }
    return warp_sum(S);
}

// Levenberg-Marquardt (Marquardt 1963): diagonal damping lambda*diag(J^T J),
// lambda /10 after an accepted step, *10 after a rejected one; stop when the
// relative decrease or the relative step is <= tol (info 1/2/3), when lambda
// exceeds 1e16 (info 4) or after maxfev model evaluations (info 5).
// Executed by one full warp in the precision T of the grid; the damped
// normal equations are solved by lane 0 (Cholesky; in FP32 after scaling the
// system to unit diagonal, which leaves the step unchanged).
template <typename T>
__device__ int lm_fit_warp(LMShared<T> &S, const T *win, int w, T tol) {
    const int lane = threadIdx.x & 31, n = 2 * w + 1, npts = n * n * n, maxfev = 1200;
    constexpr bool kScale = sizeof(T) == 4;
    T lambda = T(1e-3);
    T cost = lm_cost<T>(S.p, win, w);
    int nfev = 1;
    if (!isfinite(cost)) return 0;
    for (int outer = 0; outer < 100000; ++outer) {
        T h[77];
#pragma unroll
        for (int q = 0; q < 77; ++q) h[q] = 0;
        for (int i = lane; i < npts; i += 32) {
            int i1 = i % n, i2 = (i / n) % n, i3 = i / (n * n);
            T u1 = T(i1 + 1) - S.p[8], u2 = T(i2 + 1) - S.p[9], u3 = T(i3 + 1) - S.p[10], e;
            T f = peak_model<T, T>(S.p, u1, u2, u3, &e);
            T r = f - win[i];
            T ae = S.p[0] * e, J[11];
            J[0] = e; J[1] = 1;
            J[2] = -ae * u1 * u1; J[3] = -ae * u2 * u2; J[4] = -ae * u3 * u3;
            J[5] = -ae * u1 * u2; J[6] = -ae * u2 * u3; J[7] = -ae * u1 * u3;
            J[8] = ae * (T(2) * S.p[2] * u1 + S.p[5] * u2 + S.p[7] * u3);
            J[9] = ae * (T(2) * S.p[3] * u2 + S.p[5] * u1 + S.p[6] * u3);
            J[10] = ae * (T(2) * S.p[4] * u3 + S.p[6] * u2 + S.p[7] * u1);
            int q = 0;
#pragma unroll
            for (int a = 0; a < 11; ++a)
#pragma unroll
                for (int b = 0; b <= a; ++b) h[q++] += J[a] * J[b];
#pragma unroll
            for (int a = 0; a < 11; ++a) h[66 + a] += J[a] * r;
        }
#pragma unroll
        for (int q = 0; q < 77; ++q) h[q] = warp_sum(h[q]);
        if (lane == 0) {
            for (int q = 0; q < 66; ++q) S.H[q] = h[q];
            for (int a = 0; a < 11; ++a) S.g[a] = h[66 + a];
        }
        __syncwarp();
        for (int inner = 0; inner < 64; ++inner) {
            if (lane == 0) {
                int ok = 1;
                T sc[11];
                for (int a = 0; a < 11; ++a) {
                    T dgl = S.H[a * (a + 1) / 2 + a];
                    sc[a] = kScale ? T(1) / sqrt(dgl > T(1e-30) ? dgl : T(1e-30)) : T(1);
                }
                // A = S (H + lambda diag(H)) S with S = diag(sc); packed Cholesky
                for (int a = 0, q = 0; a < 11; ++a)
                    for (int b = 0; b <= a; ++b, ++q) {
                        T v = S.H[q];
                        if (a == b) v += lambda * (S.H[q] > T(1e-30) ? S.H[q] : T(1e-30));
                        S.A[q] = v * sc[a] * sc[b];
                    }
                T inv[11];
                for (int j = 0; j < 11 && ok; ++j) {
                    int jj = j * (j + 1) / 2;
                    T s = S.A[jj + j];
                    for (int k = 0; k < j; ++k) s -= S.A[jj + k] * S.A[jj + k];
                    if (!(s > T(0))) { ok = 0; break; }
                    T djj = sqrt(s);
                    inv[j] = T(1) / djj;
                    S.A[jj + j] = djj;
                    for (int i = j + 1; i < 11; ++i) {
                        int ii = i * (i + 1) / 2;
                        T t = S.A[ii + j];
                        for (int k = 0; k < j; ++k) t -= S.A[ii + k] * S.A[jj + k];
                        S.A[ii + j] = t * inv[j];
                    }
                }
                if (ok) {
                    T y[11];
                    for (int i = 0; i < 11; ++i) {
                        int ii = i * (i + 1) / 2;
                        T t = -S.g[i] * sc[i];
                        for (int k = 0; k < i; ++k) t -= S.A[ii + k] * y[k];
                        y[i] = t * inv[i];
                    }
                    for (int i = 10; i >= 0; --i) {
                        T t = y[i];
                        for (int k = i + 1; k < 11; ++k) t -= S.A[k * (k + 1) / 2 + i] * S.dl[k];
                        S.dl[i] = t * inv[i];
                    }
                    for (int a = 0; a < 11; ++a) {
                        S.dl[a] *= sc[a];
                        S.pn[a] = S.p[a] + S.dl[a];
                    }
                }
                S.ok = ok;
            }
            __syncwarp();
            T cn = T(INFINITY);
            const int okk = S.ok;
            if (okk) {
                cn = lm_cost<T>(S.pn, win, w);
                ++nfev;
            }
            if (okk && cn < cost) {
                T rel = (cost - cn) / cost, step = 0, pnorm = 0;
                for (int a = 0; a < 11; ++a) {
                    step += S.dl[a] * S.dl[a];
                    pnorm += S.pn[a] * S.pn[a];
                }
                step = sqrt(step);
                pnorm = sqrt(pnorm);
                __syncwarp();
                if (lane == 0)
                    for (int a = 0; a < 11; ++a) S.p[a] = S.pn[a];
                __syncwarp();
                cost = cn;
                lambda = lambda * T(0.1) > T(1e-15) ? lambda * T(0.1) : T(1e-15);
                bool c1 = rel <= tol, c2 = step <= tol * (pnorm + tol);
                if (c1 && c2) return 3;
                if (c1) return 1;
                if (c2) return 2;
                if (nfev >= maxfev) return 5;
                break;
            }
            lambda *= T(10);
            if (lambda > T(1e16)) return 4;
            if (nfev >= maxfev) return 5;
            __syncwarp();
        }
    }
    return 5;
}

// Per-thread running sum of a grid: FP64 for FP64 grids; for FP32 grids a
// compensated (Kahan) FP32 sum, which keeps about FP64 accuracy over the few
// thousand terms a thread adds without issuing FP64 instructions in the grid
// loop.  Partial sums are combined across threads in FP64.
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

// block-wide (max value, first index) and sum over a grid; all threads get it
template <typename T>
__device__ void block_argmax_sum(const T *f, int N, T &mx, long long &amax, double &sum,
                                 double *sred, T *vred, long long *ired) {
    T best = -INFINITY;
    int bl = N;
    GridSum<T> acc;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        T v = f[i];
        acc.add(v);
        if (v > best) { best = v; bl = i; }
    }
    long long bi = bl;
    double s = acc.get();
    // warp level
    for (int o = 16; o > 0; o >>= 1) {
        T ov = __shfl_xor_sync(0xffffffffu, best, o);
        long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
        s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) { vred[wid] = best; ired[wid] = bi; sred[wid] = s; }
    __syncthreads();
    best = vred[0]; bi = ired[0]; s = sred[0];
    for (int w = 1; w < nw; ++w) {
        if (vred[w] > best || (vred[w] == best && ired[w] < bi)) { best = vred[w]; bi = ired[w]; }
        s += sred[w];
    }
    mx = best; amax = bi; sum = s;
    __syncthreads();
}

// f -= model(p, q - c) over the whole G^3 grid, then block-wide (max, first
// index) and sum of the result; 32-bit index counters, one pass.
template <typename T>
__device__ void subtract_argmax_sum(T *f, int G, const double *pp, double c1, double c2, double c3,
                                    T &mx, long long &amax, double &sum, double *sred, T *vred,
                                    long long *ired) {
    const int N = G * G * G, step = blockDim.x;
    int i = threadIdx.x, i1 = i % G, i2 = (i / G) % G, i3 = i / (G * G);
    const int d1 = step % G, d2 = (step / G) % G, d3 = step / (G * G);
    // the model is evaluated in the grid's precision T
    T pt[11];
#pragma unroll
    for (int a = 0; a < 11; ++a) pt[a] = T(pp[a]);
    const T t1 = T(c1), t2 = T(c2), t3 = T(c3);
    T best = -INFINITY;
    int bi = N;
    GridSum<T> acc;
    for (; i < N; i += step) {
        T v = f[i] - peak_model<T, T>(pt, T(i1 + 1) - t1, T(i2 + 1) - t2, T(i3 + 1) - t3, (T *)nullptr);
        f[i] = v;
        acc.add(v);
        if (v > best) { best = v; bi = i; }
        i1 += d1; i2 += d2; i3 += d3;
        if (i1 >= G) { i1 -= G; ++i2; }
        if (i2 >= G) { i2 -= G; ++i3; }
    }
    long long bl = bi;
    double s = acc.get();
    for (int o = 16; o > 0; o >>= 1) {
        T ov = __shfl_xor_sync(0xffffffffu, best, o);
        long long oi = __shfl_xor_sync(0xffffffffu, bl, o);
        if (ov > best || (ov == best && oi < bl)) { best = ov; bl = oi; }
        s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    __syncthreads();
    if (lane == 0) { vred[wid] = best; ired[wid] = bl; sred[wid] = s; }
    __syncthreads();
    best = vred[0]; bl = ired[0]; s = sred[0];
    for (int w = 1; w < nw; ++w) {
        if (vred[w] > best || (vred[w] == best && ired[w] < bl)) { best = vred[w]; bl = ired[w]; }
        s += sred[w];
    }
    mx = best; amax = bl; sum = s;
    __syncthreads();
}

// One block per (orientation, pair).  Peaks are written as 1-based
// fractional grid coordinates (as FINDPEAKS returns them).
template <typename T>
__global__ void __launch_bounds__(kPeakThreads) k_findpeaks(const PairDev *pairs, T *grids, double *omax,
                                                   double *peaks, int *npeaks, int *pstatus,
                                                   double tol) {
    __shared__ LMShared<T> S;
    __shared__ T win[(2 * kMaxWin + 1) * (2 * kMaxWin + 1) * (2 * kMaxWin + 1)];
    __shared__ double sred[32];
    __shared__ T vred[32];
    __shared__ long long ired[32];
    __shared__ int s_info;
    const int o = blockIdx.x, p = blockIdx.y;
    const PairDev P = pairs[p];
    if (o >= P.norient) return;
    const int G = P.G;
    const long long N = (long long)G * G * G;
    T *f = grids + P.grid0 + (long long)o * N;
    T mx;
    long long amax;
    double sum;
    block_argmax_sum<T>(f, (int)N, mx, amax, sum, sred, vred, ired);
    if (threadIdx.x == 0) omax[2 * p + o] = (double)mx;
    int width = 2, nfound = 0;
    double *pk = peaks + 3LL * (P.cand0 + o * P.nrot);
    while (nfound == 0) {
        for (int np = 0; np < P.nrot; ++np) {
            const double mean = sum / (double)N;
            const int a1 = (int)(amax % G), a2 = (int)((amax / G) % G), a3 = (int)(amax / ((long long)G * G));
            const int wn = 2 * width + 1;
            for (int t = threadIdx.x; t < wn * wn * wn; t += blockDim.x) {
                int i1 = t % wn, i2 = (t / wn) % wn, i3 = t / (wn * wn);
                int j1 = ((a1 + i1 - width) % G + G) % G, j2 = ((a2 + i2 - width) % G + G) % G,
                    j3 = ((a3 + i3 - width) % G + G) % G;
                win[t] = f[j1 + (long long)G * (j2 + (long long)G * j3)];
            }
            if (threadIdx.x == 0) {
                double init[11] = {(double)mx - mean, mean, 1, 1, 1, 0, 0, 0, width + 1.0, width + 1.0, width + 1.0};
                for (int a = 0; a < 11; ++a) S.p[a] = T(init[a]);
            }
            __syncthreads();
            if (threadIdx.x < 32) {
                int info = lm_fit_warp<T>(S, win, width, T(tol));
                if (threadIdx.x == 0) s_info = info;
            }
            __syncthreads();
            const int info = s_info;
            if (info == 0 || info == 5) break;
            const double c1 = (double)S.p[8] - width - 1 + (a1 + 1), c2 = (double)S.p[9] - width - 1 + (a2 + 1),
                         c3 = (double)S.p[10] - width - 1 + (a3 + 1);
            if (threadIdx.x == 0) {
                pk[3 * nfound] = c1;
                pk[3 * nfound + 1] = c2;
                pk[3 * nfound + 2] = c3;
            }
            ++nfound;
            // subtract the fitted peak (not wrapped) and its mean level; the same
            // pass finds the next first maximum and the new grid sum
            double pp[11];
            for (int a = 0; a < 11; ++a) pp[a] = (double)S.p[a];
            __syncthreads();
            subtract_argmax_sum<T>(f, G, pp, c1, c2, c3, mx, amax, sum, sred, vred, ired);
        }
        if (nfound == 0) {
            ++width;
            if (width > G / 2 || width > kMaxWin) break;
        }
    }
    if (threadIdx.x == 0) {
        npeaks[2 * p + o] = nfound;
        if (nfound == 0) atomicMax(&pstatus[p], (int)ST_NO_PEAKS);
    }
}

void launch_findpeaks(const RefineBuffers &b, bool fp32, cudaStream_t s) {
    dim3 grid(2, b.npairs);
    if (fp32)
        k_findpeaks<float><<<grid, kPeakThreads, 0, s>>>(b.pairs, (float *)b.grid, b.overlap_max, b.peaks,
                                               b.npeaks, b.pstatus, 1e-5);
    else
        k_findpeaks<double><<<grid, kPeakThreads, 0, s>>>(b.pairs, (double *)b.grid, b.overlap_max, b.peaks,
                                                b.npeaks, b.pstatus, 1e-6);
}

}  // namespace fo
