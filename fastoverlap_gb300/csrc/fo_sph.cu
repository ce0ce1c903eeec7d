// fo_sph.cu -- spherical (cluster) front end: centring, spherical harmonics,
// radial pair weights, the SO(3) coefficient contraction, the Wigner-d table
// and the inverse SO(3) transform onto the rotation grid.
//
// Reference behaviour (paths inside matthewghgriffiths/fastoverlap):
//   centring                fastoverlap/f90/fastclusters.f90:173-185
//   CHOOSE_KWIDTH           fastoverlap/f90/fastclusters.f90:1046-1101
//   RYML (Y_lm)             fastoverlap/f90/fastclusters.f90:602-652
//   SPHI (i_l)              fastoverlap/f90/fastutils.f90:1000-1096
//   FOURIERCOEFFS           fastoverlap/f90/fastclusters.f90:868-916
//   CALCWIGNERD             fastoverlap/f90/DSOFT.f90:121-195
//   ISOFT + CALCOVERLAP     fastoverlap/f90/DSOFT.f90:265-329, fastclusters.f90:918-960
#include "fo_common.cuh"
#include "fo_kernels.h"

namespace fo {

// ---------------------------------------------------------------------------
// Centre both structures (not for the harmonic basis) and gather them into
// slot (group) order; choose the Gaussian width when the caller passed
// sigma <= 0.  One block per pair.
__global__ void k_sph_center(PairDev *pairs, const int *slot2orig, const double *pos1,
                             const double *pos2, double *xa, double *xb) {
    __shared__ double red[32 * 6];
    const int p = blockIdx.x;
    PairDev P = pairs[p];
    const int n = P.n, base = P.atom0;
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        for (int k = 0; k < 3; ++k) {
            s[k] += pos2[3 * (base + i) + k];
            s[3 + k] += pos1[3 * (base + i) + k];
        }
    block_sum<double, 6>(s, red);
    if (P.sigma <= 0.0) {  // CHOOSE_KWIDTH: mean nearest-neighbour distance / 3
        double acc[1] = {0.0};
        for (int t = threadIdx.x; t < 2 * n; t += blockDim.x) {
            const double *X = (t < n) ? pos2 : pos1;
            int i = (t < n) ? t : t - n;
            double best = 1.0e10;
            for (int j = 0; j < n; ++j) {
                if (j == i) continue;
                double dx = X[3 * (base + i)] - X[3 * (base + j)];
                double dy = X[3 * (base + i) + 1] - X[3 * (base + j) + 1];
                double dz = X[3 * (base + i) + 2] - X[3 * (base + j) + 2];
                double d = sqrt(dx * dx + dy * dy + dz * dz);
                if (d < best) best = d;
            }
            acc[0] += best;
        }
        block_sum<double, 1>(acc, red);
        if (threadIdx.x == 0) pairs[p].sigma = acc[0] / (6.0 * n);
    }
    // the harmonic basis (ALIGNHARM) takes the coordinates as given
    double c[6];
    for (int k = 0; k < 6; ++k) c[k] = P.harm ? 0.0 : s[k] / n;
    for (int sl = threadIdx.x; sl < n; sl += blockDim.x) {
        int o = slot2orig[base + sl];
        for (int k = 0; k < 3; ++k) {
            xa[3 * (base + sl) + k] = pos2[3 * (base + o) + k] - c[k];
            xb[3 * (base + sl) + k] = pos1[3 * (base + o) + k] - c[3 + k];
        }
    }
}

// ---------------------------------------------------------------------------
// Recurrence factors of the orthonormal associated Legendre functions, for
// l, m < kYlmMax (Jmax <= 31), in FP64 and FP32:
//   a[l][m] = sqrt((4l^2 - 1) / (l^2 - m^2))            (l >= m + 2)
//   b[l][m] = sqrt(((l-1)^2 - m^2) / (4(l-1)^2 - 1))     (l >= m + 2)
//   c[m] = sqrt(2m + 3)  (l = m + 1),   d[m] = sqrt((2m + 1) / 2m)  (m >= 1)
// Numerators and denominators are exact integers and the quotient and root
// are correctly rounded on host and device alike, so the table holds the
// values a direct FP64 evaluation gives.
constexpr int kYlmMax = 32;
constexpr int kYlmTab = 2 * kYlmMax * kYlmMax + 2 * kYlmMax;
__constant__ double c_ylm64[kYlmTab];
__constant__ float c_ylm32[kYlmTab];

void init_sph_tables() {
    double t64[kYlmTab] = {0};
    float t32[kYlmTab];
    for (int l = 0; l < kYlmMax; ++l)
        for (int m = 0; m + 2 <= l; ++m) {
            t64[l * kYlmMax + m] = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            t64[kYlmMax * kYlmMax + l * kYlmMax + m] =
                sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
        }
    for (int m = 0; m < kYlmMax; ++m) {
        t64[2 * kYlmMax * kYlmMax + m] = sqrt(2.0 * m + 3.0);
        t64[2 * kYlmMax * kYlmMax + kYlmMax + m] = m > 0 ? sqrt((2.0 * m + 1.0) / (2.0 * m)) : 0.0;
    }
    for (int q = 0; q < kYlmTab; ++q) t32[q] = (float)t64[q];
    cudaMemcpyToSymbol(c_ylm64, t64, sizeof t64);
    cudaMemcpyToSymbol(c_ylm32, t32, sizeof t32);
}

template <typename T> __device__ __forceinline__ const T *ylm_tab();
template <> __device__ __forceinline__ const double *ylm_tab<double>() { return c_ylm64; }
template <> __device__ __forceinline__ const float *ylm_tab<float>() { return c_ylm32; }

// Orthonormal Y_lm (Condon-Shortley phase) for l <= L of every slot of both
// structures; one thread per (slot, side), computed in the precision T of the
// output.  Output per slot: (L+1)^2 complex values at index l*l + l + m
// (TL: per pair [lm][atom], atom fastest, the layout of the tensor-core
// coefficient contraction).  An atom at the origin gets theta = 0.  FP64:
// e^{i m phi} from sincos(m phi); FP32: by repeated multiplication with e^{i phi}.
template <typename T, typename T2, bool TL>
__global__ void k_sph_ylm(const PairDev *pairs, const int *slot2pair, const double *xa,
                          const double *xb, double *ra, double *rb, T2 *ylmA, T2 *ylmB,
                          int nslots) {
    constexpr bool kF32 = sizeof(T) == 4;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * nslots) return;
    const int side = t / nslots, slot = t % nslots;
    const PairDev &P = pairs[slot2pair[slot]];
    const int L = P.L;
    const double *X = side ? xb : xa;
    const double x = X[3 * slot], y = X[3 * slot + 1], z = X[3 * slot + 2];
    const double r = sqrt(x * x + y * y + z * z);
    (side ? rb : ra)[slot] = r;
    const T *A = ylm_tab<T>(), *B = A + kYlmMax * kYlmMax, *C = B + kYlmMax * kYlmMax, *D = C + kYlmMax;
    T ct = 1, cph = 1, sph = 0;
    double phi = 0.0;
    if (r > 0.0) {
        if constexpr (kF32) {
            const float xf = (float)x, yf = (float)y, rho = sqrtf(xf * xf + yf * yf);
            ct = fminf(1.f, fmaxf(-1.f, (float)z / (float)r));
            if (rho > 0.f) { cph = xf / rho; sph = yf / rho; }
        } else {
            ct = fmin(1.0, fmax(-1.0, z / r));
            phi = atan2(y, x);
        }
    }
    const T st = sqrt(ct * ct < T(1) ? T(1) - ct * ct : T(0));
    const long long ostride = TL ? P.n : 1;   // between consecutive lm
    T2 *out = (side ? ylmB : ylmA) + P.ylm0 + (long long)(slot - P.atom0) * (TL ? 1 : (L + 1) * (L + 1));
    T pmm = T(0.28209479177387814347);  // 1/sqrt(4 pi)
    T cm = 1, sm = 0;
    for (int m = 0; m <= L; ++m) {
        if (m > 0) {
            pmm = -D[m] * st * pmm;
            if constexpr (kF32) {
                const T c2 = cm * cph - sm * sph;
                sm = sm * cph + cm * sph;
                cm = c2;
            }
        }
        if constexpr (!kF32) sincos(m * phi, &sm, &cm);
        const T sgn = (m & 1) ? T(-1) : T(1);
        T p2 = 0, p1 = pmm;
        for (int l = m; l <= L; ++l) {
            T pl;
            if (l == m) pl = pmm;
            else if (l == m + 1) pl = C[m] * ct * pmm;
            else pl = A[l * kYlmMax + m] * (ct * p1 - B[l * kYlmMax + m] * p2);
            if (l > m) { p2 = p1; p1 = pl; }
            out[(l * l + l + m) * ostride] = pack2<T2, T>(pl * cm, pl * sm);
            if (m > 0) out[(l * l + l - m) * ostride] = pack2<T2, T>(sgn * pl * cm, -sgn * pl * sm);
        }
    }
}

// ---------------------------------------------------------------------------
// Radial pair weights of FOURIERCOEFFS:
//   w_l(a,b) = 4 pi^{5/2} s^3 i_l(x) e^{-(r_a^2 + r_b^2)/4s^2},  x = r_a r_b / 2s^2
// evaluated as 4 pi^{5/2} s^3 [e^{-x} i_l(x)] e^{-(r_a - r_b)^2/4s^2} so
// nothing overflows.  e^{-x} i_l(x) comes from Miller's backward recurrence
// i_{l-1} = i_{l+1} + (2l+1)/x i_l started at l = L + 10 + 0.8x (full FP64
// accuracy for L <= 63) and normalised by e^{-x} i_0 = (1 - e^{-2x})/2x; for
// x < 1e-6 the leading series terms are used.  Evaluated in the precision T of
// the weights (the recurrence is rescaled before it can overflow T: by 1e-250
// above 1e250 in FP64, by 1e-28 above 1e28 in FP32, which leaves room for a
// step's growth (2k+1)/x < 1e8 at x >= 1e-6).  The cutoff test is made in
// FP64 in both precisions.  Layout per group: W[w0 + (l*n + b)*n + a]
// (TL: W[w0 + (l*n + a)*n + b], the layout of the tensor-core contraction).
template <typename T, bool TL>
__global__ void k_sph_radial(const PairDev *pairs, const GroupDev *groups, const double *ra,
                             const double *rb, T *W, int cutoff) {
    constexpr T kBig = sizeof(T) == 4 ? T(1.0e28) : T(1.0e250);
    constexpr T kShrink = sizeof(T) == 4 ? T(1.0e-28) : T(1.0e-250);
    const GroupDev g = groups[blockIdx.y];
    const int n = g.n;
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n * n) return;
    const int b = TL ? (int)(idx % n) : (int)(idx / n), a = TL ? (int)(idx / n) : (int)(idx % n);
    const PairDev &P = pairs[g.pair];
    const int L = P.L;
    const double r1d = ra[g.slot0 + a], r2d = rb[g.slot0 + b];
    T *out = W + g.w0 + idx;
    const long long lstride = (long long)n * n;
    if (cutoff && !(fabs(r1d - r2d) < 4.0 * P.sigma)) {
        for (int l = 0; l <= L; ++l) out[l * lstride] = T(0);
        return;
    }
    const T s = T(P.sigma), r1 = T(r1d), r2 = T(r2d);
    const T pre = T(4.0 * 17.493418327624862) /* 4 pi^2.5 */ * s * s * s *
                  exp(-(r1 - r2) * (r1 - r2) / (T(4) * s * s));
    const T x = r1 * r2 / (T(2) * s * s);
    if (x < T(1.0e-6)) {
        T t = exp(-x);
        for (int l = 0; l <= L; ++l) {
            if (l > 0) t *= x / (T(2) * l + T(1));
            out[l * lstride] = pre * t * (T(1) + x * x / (T(2) * (T(2) * l + T(3))));
        }
        return;
    }
    if (x >= T(1000) && x >= T(L) * T(L)) {
        // e^{-x} i_l(x) = (1/2x) sum_{k<=l} (l+k)!/(k!(l-k)!) (-1/2x)^k  (+ O(e^{-2x}));
        // terms shrink at least by half when x >= l^2, so the sum is stable.
        for (int l = 0; l <= L; ++l) {
            T term = 1, sum = 1;
            for (int k = 0; k < l; ++k) {
                term *= -T(l + k + 1) * T(l - k) / ((T(k) + T(1)) * T(2) * x);
                sum += term;
            }
            out[l * lstride] = pre * sum / (T(2) * x);
        }
        return;
    }
    T vals[64];
    const int n0 = L + 10 + (int)(T(0.8) * x);
    const T invx = T(1) / x;
    T fp1 = 0, f = 1;
    for (int k = n0; k >= 1; --k) {
        if (k <= L) vals[k] = f;
        T fm1 = (T(2) * k + T(1)) * invx * f + fp1;
        if (fabs(fm1) > kBig) {
            fm1 *= kShrink;
            f *= kShrink;
            for (int q = k; q <= L; ++q) vals[q] *= kShrink;
        }
        fp1 = f;
        f = fm1;
    }
    vals[0] = f;
    const T s0 = -expm1(T(-2) * x) / (T(2) * x);
    const T scale = pre * s0 / f;
    for (int l = 0; l <= L; ++l) out[l * lstride] = vals[l] * scale;
}

// ---------------------------------------------------------------------------
// Harmonic-oscillator basis (SphericalHarmonicAlign): the radial weights of the
// coefficient contraction are W_l(a, b) = sum_{n <= nmax} d_nl(r_a) d_nl(r_b),
// d_nl(r) being the overlap of the Gaussian kernel at distance r with the basis
// function of order (n, l) (HARMONICNL fastoverlap/f90/fastclusters.f90:492-540;
// IMML = sum_n conj(c_B) c_A of DOTHARMONICCOEFFS :740-759 expanded over atom
// pairs).  k_harm_dnl: d_nl of every slot of both structures in FP64 by the
// recurrence in n from the closed form at n = 0, which runs to l = L + 2 nmax.
// Output hd[((side * nslots + slot) * (nmax + 1) + n) * (maxL + 1) + l].
constexpr int kHarmRow = kYlmMax + 2 * kMaxHarmN + 1;

__global__ void k_harm_dnl(const PairDev *pairs, const int *slot2pair, const double *ra, const double *rb,
                           double *hd, int nslots, int nmax, int maxL) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * nslots) return;
    const int side = t / nslots, slot = t % nslots;
    const PairDev &P = pairs[slot2pair[slot]];
    const int L = P.L, lmax = L + 2 * nmax, w = maxL + 1;
    const double rj = side ? rb[slot] : ra[slot], sigma = P.sigma, r0 = P.harm_r0;
    double *out = hd + (size_t)t * (nmax + 1) * w;
    double rows[3][kHarmRow];
    double *pm2 = rows[0], *pm1 = rows[1], *cur = rows[2];
    const double rs = 1.0 / (r0 * r0 + sigma * sigma), x = r0 * rs;
    pm1[0] = sqrt(2.0 * sqrt(FO_PI) * (x * x * x)) * sigma * sigma * sigma * exp(-0.5 * rj * rj * rs) * 4 * FO_PI;
    const double f = sqrt(2.0) * r0 * rj * rs;
    for (int j = 1; j <= lmax; ++j) pm1[j] = f / sqrt(1.0 + 2.0 * j) * pm1[j - 1];
    for (int l = 0; l <= L; ++l) out[l] = pm1[l];
    const double q = sigma * sigma / rj / r0;
    for (int i = 1; i <= nmax; ++i) {
        const double si = sqrt((double)i), sm = sqrt(i - 1.0);
        for (int j = 0; j <= lmax - 2 * i; ++j) {
            double v = sqrt(i + j + 0.5) * pm1[j] - (2.0 * j + 3.0) * q * pm1[j + 1] - sqrt(i + j + 1.5) * pm1[j + 2];
            cur[j] = (i == 1) ? v : (v + sm * pm2[j + 2]) / si;
        }
        for (int l = 0; l <= L; ++l) out[i * w + l] = cur[l];
        double *tmp = pm2;
        pm2 = pm1;
        pm1 = cur;
        cur = tmp;
    }
}

// W_l(b, a) of every atom pair of every group, in the precision T of the
// contraction (same layouts as k_sph_radial).
template <typename T, bool TL>
__global__ void k_harm_radial(const PairDev *pairs, const GroupDev *groups, const double *hd, T *W, int nslots,
                              int nmax, int maxL) {
    const GroupDev g = groups[blockIdx.y];
    const int n = g.n;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)n * n) return;
    const int b = TL ? (int)(idx % n) : (int)(idx / n), a = TL ? (int)(idx / n) : (int)(idx % n);
    const int L = pairs[g.pair].L, w = maxL + 1;
    const double *da = hd + (size_t)(g.slot0 + a) * (nmax + 1) * w;
    const double *db = hd + (size_t)(nslots + g.slot0 + b) * (nmax + 1) * w;
    T *out = W + g.w0 + idx;
    const long long lstride = (long long)n * n;
    for (int l = 0; l <= L; ++l) {
        double acc = 0;
        for (int i = 0; i <= nmax; ++i) acc += da[i * w + l] * db[i * w + l];
        out[l * lstride] = T(acc);
    }
}

// ---------------------------------------------------------------------------
// Coefficient contraction, one block per (l, pair):
//   I^l[m1][m2] = sum_groups sum_a ( sum_b YB_l[m1](b) W_l(b,a) ) conj(YA_l[m2](a))
// as two tiled GEMMs through shared memory (a tiles of 32, b tiles of 32).
// Written to the ilmm layout coef[coef0 + (l*W + m1 mod W)*W + m2 mod W].
constexpr int kTA = 32, kTB = 32, kMaxWM = 63;

template <typename T, typename T2>
__global__ void __launch_bounds__(256) k_sph_coeff(const PairDev *pairs, const GroupDev *groups,
                                                   const T2 *ylmA, const T2 *ylmB, const T *W,
                                                   T2 *coef) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int l = blockIdx.x, p = blockIdx.y;
    const PairDev P = pairs[p];
    if (l > P.L) return;
    const int WM = 2 * l + 1, L = P.L, LL = (L + 1) * (L + 1), Wc = 2 * L + 1;
    T2 *sYB = (T2 *)smem_raw;              // [WM][kTB]
    T2 *sP = sYB + kMaxWM * kTB;           // [WM][kTA]
    T2 *sYA = sP + kMaxWM * kTA;           // [kTA][WM]
    T *sW = (T *)(sYA + kTA * kMaxWM);     // [kTB][kTA]
    const int tid = threadIdx.x, nt = blockDim.x;
    T2 acc[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) acc[k] = mk2<T2>(0, 0);
    for (int gi = 0; gi < P.ngroups; ++gi) {
        const GroupDev g = groups[P.group0 + gi];
        const int n = g.n;
        const T *Wl = W + g.w0 + (long long)l * n * n;
        const long long yb = P.ylm0 + (long long)(g.slot0 - P.atom0) * LL + l * l;
        for (int a0 = 0; a0 < n; a0 += kTA) {
            T2 pacc[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) pacc[k] = mk2<T2>(0, 0);
            for (int b0 = 0; b0 < n; b0 += kTB) {
                for (int t = tid; t < WM * kTB; t += nt) {
                    int m1 = t / kTB, bb = t % kTB;
                    sYB[m1 * kTB + bb] = (b0 + bb < n) ? ylmB[yb + (long long)(b0 + bb) * LL + m1] : mk2<T2>(0, 0);
                }
                for (int t = tid; t < kTB * kTA; t += nt) {
                    int bb = t / kTA, aa = t % kTA;
                    sW[t] = (b0 + bb < n && a0 + aa < n) ? Wl[(long long)(b0 + bb) * n + a0 + aa] : T(0);
                }
                __syncthreads();
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    int o = tid + k * nt;
                    if (o < WM * kTA) {
                        int m1 = o / kTA, aa = o % kTA;
                        T2 s = pacc[k];
                        for (int bb = 0; bb < kTB; ++bb) {
                            T2 y = sYB[m1 * kTB + bb];
                            T w = sW[bb * kTA + aa];
                            s.x += y.x * w;
                            s.y += y.y * w;
                        }
                        pacc[k] = s;
                    }
                }
                __syncthreads();
            }
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                int o = tid + k * nt;
                if (o < WM * kTA) sP[o] = pacc[k];
            }
            for (int t = tid; t < kTA * WM; t += nt) {
                int aa = t / WM, m2 = t % WM;
                sYA[t] = (a0 + aa < n) ? ylmA[yb + (long long)(a0 + aa) * LL + m2] : mk2<T2>(0, 0);
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                int o = tid + k * nt;
                if (o < WM * WM) {
                    int m1 = o / WM, m2 = o % WM;
                    T2 s = acc[k];
                    for (int aa = 0; aa < kTA; ++aa) {
                        T2 pv = sP[m1 * kTA + aa], ya = sYA[aa * WM + m2];
                        // pv * conj(ya)
                        s.x += pv.x * ya.x + pv.y * ya.y;
                        s.y += pv.y * ya.x - pv.x * ya.y;
                    }
                    acc[k] = s;
                }
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        int o = tid + k * nt;
        if (o < WM * WM) {
            int m1 = o / WM - l, m2 = o % WM - l;
            int i1 = (m1 + Wc) % Wc, i2 = (m2 + Wc) % Wc;
            coef[P.coef0 + ((long long)l * Wc + i1) * Wc + i2] = acc[k];
        }
    }
}

// ---------------------------------------------------------------------------
// Normalised Wigner little-d table sqrt((2l+1)/2) d^l_{m1 m2}(beta_k),
// beta_k = pi(2k+1)/(4 bw), by the Kostelec-Rockmore three-term recurrence
// in l from the closed-form seed at l = max(|m1|,|m2|).  FP64 always.
// Layout d[((k*W + m1i)*W + m2i)*bw + l], W = 2bw-1, entries below the seed 0.
__global__ void k_wigner_table(int bw, double *d64, float *d32) {
    const int W = 2 * bw - 1, G = 2 * bw;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= G * W * W) return;
    const int k = t / (W * W), i1 = (t / W) % W, i2 = t % W;
    const int m1 = (i1 < bw) ? i1 : i1 - W, m2 = (i2 < bw) ? i2 : i2 - W;
    const int l0 = max(abs(m1), abs(m2));
    // layout [k][l][m1][m2]: element l of this (k, m1, m2) at base + l W^2
    const long long W2 = (long long)W * W, base = (long long)k * bw * W2 + (long long)i1 * W + i2;
    auto put = [&](int l, double v) {
        d64[base + l * W2] = v;
        if (d32) d32[base + l * W2] = (float)v;
    };
    for (int l = 0; l < l0; ++l) put(l, 0.0);
    const double beta = FO_PI * (2.0 * k + 1.0) / (4.0 * bw);
    double c = cos(beta / 2), s = sin(beta / 2), cb = cos(beta);
    int M, pc, ps;
    double sgn_s;
    if (l0 == m1) { M = m2; pc = l0 + m2; ps = l0 - m2; sgn_s = -1; }
    else if (l0 == -m1) { M = m2; pc = l0 - m2; ps = l0 + m2; sgn_s = 1; }
    else if (l0 == m2) { M = m1; pc = l0 + m1; ps = l0 - m1; sgn_s = 1; }
    else { M = m1; pc = l0 - m1; ps = l0 + m1; sgn_s = -1; }
    double lf = lgamma(2.0 * l0 + 1.0) - lgamma((double)l0 + M + 1.0) - lgamma((double)l0 - M + 1.0);
    double seed = sqrt((2.0 * l0 + 1.0) / 2.0 * exp(lf));
    double sv = sgn_s * s;
    for (int q = 0; q < pc; ++q) seed *= c;
    for (int q = 0; q < ps; ++q) seed *= sv;
    double prev = 0.0, cur = seed;
    put(l0, cur);
    for (int l = l0; l <= bw - 2; ++l) {
        double dl = l, a = 0.0, cc = 0.0;
        double t5 = 1.0 / sqrt(((dl + 1) * (dl + 1) - (double)m1 * m1) * ((dl + 1) * (dl + 1) - (double)m2 * m2));
        double bb = sqrt((2 * dl + 3) / (2 * dl + 1)) * (dl + 1) * (2 * dl + 1) * t5;
        if (l > 0) {
            a = sqrt((2 * dl + 3) / (2 * dl - 1)) * (dl + 1) / dl *
                sqrt((dl * dl - (double)m1 * m1) * (dl * dl - (double)m2 * m2)) * t5;
            cc = (double)m1 * m2 / (dl * (dl + 1));
        }
        double nxt = bb * (cb - cc) * cur - a * prev;
        prev = cur;
        cur = nxt;
        put(l + 1, cur);
    }
}

// ---------------------------------------------------------------------------
// Inverse SO(3) transform, one block per (beta index k, pair) for both
// orientations:
//   S[m1][m2] = sum_{l >= max(|m1|,|m2|)} d^l_{m1m2}(beta_k) (+-1)^l I^l_{m1m2}
// (the inverted copy of A has I^l -> (-1)^l I^l since Y_lm(-r) = (-1)^l Y_lm(r),
// so the even-l and odd-l partial sums give both), then unnormalised backward
// DFTs m2 -> gamma and m1 -> alpha in shared memory and the real part written
// to grid[grid0 + o*G^3 + a + G*(k + G*g)].  The Wigner table and the
// coefficients are both [l][m1][m2], so a warp reads them contiguously.
template <typename T, typename T2>
__global__ void __launch_bounds__(256) k_isoft(const PairDev *pairs, const T2 *coef,
                                               const T *const *dtab, T *grid) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int k = blockIdx.x, p = blockIdx.y;
    const PairDev P = pairs[p];
    const int G = P.G, L = P.L, bw = L + 1, Wc = 2 * L + 1, W2 = Wc * Wc;
    if (k >= G) return;
    const bool inv = P.norient == 2;
    const int PL = isoft_plane(G), ld = isoft_ld(G);
    T2 *bufA = (T2 *)smem_raw, *bufB = bufA + PL, *bufC = bufB + PL, *tw = bufC + PL;
    for (int t = threadIdx.x; t < G; t += blockDim.x) {
        T sn, cs;
        if constexpr (sizeof(T) == 4) sincospif(2.0f * t / G, &sn, &cs);
        else sincospi(2.0 * t / G, &sn, &cs);
        tw[t] = pack2<T2, T>(cs, sn);
    }
    for (int t = threadIdx.x; t < PL; t += blockDim.x) {
        bufA[t] = pack2<T2, T>(0, 0);
        bufC[t] = pack2<T2, T>(0, 0);
    }
    __syncthreads();
    const T *d = dtab[bw] + (long long)k * bw * W2;
    const T2 *I = coef + P.coef0;
    for (int t = threadIdx.x; t < W2; t += blockDim.x) {
        const int i1 = t / Wc, i2 = t % Wc;
        const int m1 = (i1 <= L) ? i1 : i1 - Wc, m2 = (i2 <= L) ? i2 : i2 - Wc;
        const int l0 = max(abs(m1), abs(m2));
        T er = 0, ei = 0, orr = 0, oi = 0;   // even-l and odd-l partial sums
        for (int l = l0 + (l0 & 1); l <= L; l += 2) {
            const T2 c = I[(long long)l * W2 + t];
            const T dv = d[(long long)l * W2 + t];
            er += dv * c.x;
            ei += dv * c.y;
        }
        for (int l = l0 + 1 - (l0 & 1); l <= L; l += 2) {
            const T2 c = I[(long long)l * W2 + t];
            const T dv = d[(long long)l * W2 + t];
            orr += dv * c.x;
            oi += dv * c.y;
        }
        const int dst = ((m1 + G) % G) * ld + (m2 + G) % G;
        bufA[dst] = pack2<T2, T>(er + orr, ei + oi);
        bufC[dst] = pack2<T2, T>(er - orr, ei - oi);
    }
    __syncthreads();
    isoft_tail<T, T2>(bufA, bufB, bufC, tw, G, k, inv, grid + P.grid0);
}

// ---------------------------------------------------------------------------
// host launchers
void launch_sph_center(const SphBuffers &b, cudaStream_t s) {
    k_sph_center<<<b.npairs, 256, 0, s>>>(const_cast<PairDev *>(b.pairs), b.slot2orig, b.pos1,
                                          b.pos2, b.xa, b.xb);
}

void launch_sph_ylm(const SphBuffers &b, bool fp32, cudaStream_t s) {
    int nth = 2 * b.nslots, bs = 128;
    const unsigned nb = (nth + bs - 1) / bs;
    if (fp32 && b.tc_layout)
        k_sph_ylm<float, float2, true><<<nb, bs, 0, s>>>(b.pairs, b.slot2pair, b.xa, b.xb, b.ra, b.rb,
                                                        (float2 *)b.ylmA, (float2 *)b.ylmB, b.nslots);
    else if (fp32)
        k_sph_ylm<float, float2, false><<<nb, bs, 0, s>>>(b.pairs, b.slot2pair, b.xa, b.xb, b.ra, b.rb,
                                                         (float2 *)b.ylmA, (float2 *)b.ylmB, b.nslots);
    else
        k_sph_ylm<double, double2, false><<<nb, bs, 0, s>>>(b.pairs, b.slot2pair, b.xa, b.xb, b.ra, b.rb,
                                                           (double2 *)b.ylmA, (double2 *)b.ylmB, b.nslots);
}

void launch_sph_radial(const SphBuffers &b, bool fp32, int cutoff, cudaStream_t s) {
    long long nn = (long long)b.maxgroup * b.maxgroup;
    dim3 grid((unsigned)((nn + 255) / 256), (unsigned)b.ngroups);
    if (b.harm_n >= 0) {
        const int nth = 2 * b.nslots;
        k_harm_dnl<<<(nth + 127) / 128, 128, 0, s>>>(b.pairs, b.slot2pair, b.ra, b.rb, b.hd, b.nslots, b.harm_n,
                                                    b.maxL);
        if (fp32 && b.tc_layout)
            k_harm_radial<float, true><<<grid, 256, 0, s>>>(b.pairs, b.groups, b.hd, (float *)b.W, b.nslots,
                                                            b.harm_n, b.maxL);
        else if (fp32)
            k_harm_radial<float, false><<<grid, 256, 0, s>>>(b.pairs, b.groups, b.hd, (float *)b.W, b.nslots,
                                                             b.harm_n, b.maxL);
        else
            k_harm_radial<double, false><<<grid, 256, 0, s>>>(b.pairs, b.groups, b.hd, (double *)b.W, b.nslots,
                                                              b.harm_n, b.maxL);
        return;
    }
    if (fp32 && b.tc_layout)
        k_sph_radial<float, true><<<grid, 256, 0, s>>>(b.pairs, b.groups, b.ra, b.rb, (float *)b.W, cutoff);
    else if (fp32)
        k_sph_radial<float, false><<<grid, 256, 0, s>>>(b.pairs, b.groups, b.ra, b.rb, (float *)b.W, cutoff);
    else
        k_sph_radial<double, false><<<grid, 256, 0, s>>>(b.pairs, b.groups, b.ra, b.rb, (double *)b.W, cutoff);
}

void launch_sph_coeff(const SphBuffers &b, bool fp32, cudaStream_t s) {
    dim3 grid(b.maxL + 1, b.npairs);
    if (fp32) {
        size_t sm = sizeof(float2) * (kMaxWM * kTB + kMaxWM * kTA + kTA * kMaxWM) + sizeof(float) * kTB * kTA;
        allow_max_smem<k_sph_coeff<float, float2>>();
        k_sph_coeff<float, float2><<<grid, 256, sm, s>>>(b.pairs, b.groups, (const float2 *)b.ylmA,
                                                        (const float2 *)b.ylmB, (const float *)b.W,
                                                        (float2 *)b.coef);
    } else {
        size_t sm = sizeof(double2) * (kMaxWM * kTB + kMaxWM * kTA + kTA * kMaxWM) + sizeof(double) * kTB * kTA;
        allow_max_smem<k_sph_coeff<double, double2>>();
        k_sph_coeff<double, double2><<<grid, 256, sm, s>>>(b.pairs, b.groups, (const double2 *)b.ylmA,
                                                          (const double2 *)b.ylmB, (const double *)b.W,
                                                          (double2 *)b.coef);
    }
}

// CALCSIMILARITY's two numbers (fastoverlap/f90/fastclusters.f90:790-815) for
// every pair of a plan: the squared norm of its SO(3) coefficients and the
// maximum of its overlap grid (first orientation).  One block per pair;
// out[2p] = norm, out[2p+1] = maximum.
template <typename T, typename T2>
__global__ void __launch_bounds__(256) k_pair_stats(const PairDev *pairs, const T2 *coef, const T *grid,
                                                    double *out) {
    __shared__ double red[32 * 2];
    const PairDev &P = pairs[blockIdx.x];
    const int W = 2 * P.L + 1;
    const long long nc = (long long)(P.L + 1) * W * W, ng = (long long)P.G * P.G * P.G;
    double v[1] = {0.0}, mx = -INFINITY;
    for (long long i = threadIdx.x; i < nc; i += blockDim.x) {
        const T2 c = coef[P.coef0 + i];
        v[0] += (double)c.x * c.x + (double)c.y * c.y;
    }
    for (long long i = threadIdx.x; i < ng; i += blockDim.x) mx = fmax(mx, (double)grid[P.grid0 + i]);
    block_sum<double, 1>(v, red);
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[32 + (threadIdx.x >> 5)] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x + 31) / 32; ++w) mx = fmax(mx, red[32 + w]);
        out[2 * blockIdx.x] = v[0];
        out[2 * blockIdx.x + 1] = mx;
    }
}

void launch_pair_stats(const SphBuffers &b, bool fp32, double *out, cudaStream_t s) {
    if (fp32)
        k_pair_stats<float, float2><<<b.npairs, 256, 0, s>>>(b.pairs, (const float2 *)b.coef,
                                                            (const float *)b.grid, out);
    else
        k_pair_stats<double, double2><<<b.npairs, 256, 0, s>>>(b.pairs, (const double2 *)b.coef,
                                                              (const double *)b.grid, out);
}

void launch_isoft(const SphBuffers &b, bool fp32, cudaStream_t s) {
    dim3 grid(b.maxG, b.npairs);
    if (fp32) {
        size_t sm = sizeof(float2) * (3 * isoft_plane(b.maxG) + b.maxG);
        allow_max_smem<k_isoft<float, float2>>();
        k_isoft<float, float2><<<grid, 256, sm, s>>>(b.pairs, (const float2 *)b.coef,
                                                    (const float *const *)b.dtab, (float *)b.grid);
    } else {
        size_t sm = sizeof(double2) * (3 * isoft_plane(b.maxG) + b.maxG);
        allow_max_smem<k_isoft<double, double2>>();
        k_isoft<double, double2><<<grid, 256, sm, s>>>(b.pairs, (const double2 *)b.coef,
                                                      (const double *const *)b.dtab, (double *)b.grid);
    }
}

void launch_wigner_table(int bw, double *d64, float *d32, cudaStream_t s) {
    int W = 2 * bw - 1, n = 2 * bw * W * W;
    k_wigner_table<<<(n + 127) / 128, 128, 0, s>>>(bw, d64, d32);
}

}  // namespace fo
