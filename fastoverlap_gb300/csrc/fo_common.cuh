// fo_common.cuh -- shared device/host definitions of the GB300 FASTOVERLAP
// library: plan descriptors, complex helpers, reductions, the shared-memory
// Stockham FFT and small dense linear algebra used by several kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#ifndef FO_PI
#define FO_PI 3.141592653589793238462643383279502884
#endif

namespace fo {

// ---------------------------------------------------------------------------
// Plan descriptors (device-resident, built on the host).
// A "slot" is an atom position after the atoms of a pair are reordered so that
// each permutation group is contiguous; slot s of pair p holds original atom
// perm[s] (the concatenated group list is exactly the slot -> atom map).
struct PairDev {
    int n;          // atoms
    int ngroups;    // permutation groups
    int group0;     // first GroupDev of this pair
    int L;          // cluster: Jmax; bulk: nwave K
    int G;          // cluster: 2(L+1); bulk: nfspace M
    int nrot;       // candidate slots per orientation
    int norient;    // 2 when the inverted copy is aligned too, else 1
    int atom0;      // first slot (global)
    int cand0;      // first candidate (global), norient*nrot candidates
    int bulk;       // 1 periodic, 0 cluster
    long long ylm0;      // complex offset into the Y_lm arrays
    long long coef0;     // complex offset: cluster coefficients / bulk F grid
    long long grid0;     // offset into the real overlap grids (norient * G^3)
    long long candatom0; // offset of per-atom candidate outputs
    long long lap0;      // offset (bytes) of this pair's LAP scratch
    long long lapstride; // LAP scratch bytes per candidate
    double sigma;
    double box[3];
    int harm;         // cluster: 1 for the harmonic-oscillator basis (coordinates as given)
    int harm_n;       // its largest order nmax
    double harm_r0;   // its length scale (HWIDTH)
    int lapsplit;     // 1: assignment working arrays on chip, costs / neighbour lists in the LAP scratch
    int pad_;
};

struct GroupDev {
    int pair;
    int slot0;      // first slot (global)
    int n;          // atoms in the group
    int m;          // neighbours kept per row: min(n, 60)
    long long w0;   // offset of the radial weight block [(L+1)][n][n]
};

// status codes shared with the C ABI (fastoverlap_gb300.h)
enum : int {
    ST_OK = 0, ST_BAD_ARGS = 1, ST_NO_PEAKS = 2, ST_LAP_FAILED = 3, ST_TIMEOUT = 4
};

constexpr int kMaxNei = 60;          // PMAXNEI, alignutils.f90:79
constexpr double kPScale = 1.0e6;    // PSCALE, alignutils.f90:80
constexpr int kMaxTries = 20;        // MAXIMUMTRIES, alignutils.f90:81
constexpr long long kBigInt = 1000000000000LL;  // BIGINT, alignutils.f90:1007

// ---------------------------------------------------------------------------
// complex helpers over double2 / float2
template <typename T> struct cplx;
template <> struct cplx<double> { using type = double2; };
template <> struct cplx<float> { using type = float2; };

// a complex value from two parts of the element type itself (no FP64 detour)
template <typename T2, typename S> __host__ __device__ inline T2 pack2(S a, S b) {
    T2 r;
    r.x = a;
    r.y = b;
    return r;
}
template <typename T2> __host__ __device__ inline T2 mk2(double a, double b) {
    T2 r; r.x = a; r.y = b; return r;
}
template <typename T2> __device__ inline T2 cmul(T2 a, T2 b) {
    T2 r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename T2> __device__ inline T2 cadd(T2 a, T2 b) {
    T2 r; r.x = a.x + b.x; r.y = a.y + b.y; return r;
}

// ---------------------------------------------------------------------------
// reductions
template <typename T> __device__ inline T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of K values per thread; result broadcast to every thread.
// scratch: >= 32*K elements of T in shared memory.  All threads must call.
template <typename T, int K>
__device__ inline void block_sum(T (&v)[K], T *scratch) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) scratch[wid * K + k] = v[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) {
        T s = 0;
        for (int w = 0; w < nw; ++w) s += scratch[w * K + k];
        v[k] = s;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Stockham autosort FFT over a batch of lines held in shared memory.
// Element e of line l lives at buf[l*lstride + e*estride].  Radix 2,3,4,5
// passes; lengths with another prime factor use a direct DFT.  sign = -1 is
// the forward transform, +1 the unnormalised backward one.  tw[t] holds
// exp(+2 pi i t/n).  Returns the buffer (x or y) that holds the result.
// All threads of the block must call it.
__host__ __device__ inline int fft_factor(int n, int *rad) {
    int k = 0;
    while (n % 4 == 0) { rad[k++] = 4; n /= 4; }
    while (n % 2 == 0) { rad[k++] = 2; n /= 2; }
    while (n % 3 == 0) { rad[k++] = 3; n /= 3; }
    while (n % 5 == 0) { rad[k++] = 5; n /= 5; }
    if (n != 1) return -1;
    return k;
}

// twiddle exp(sign 2 pi i e/n) for 0 <= e < n
template <typename T2>
__device__ __forceinline__ T2 tw_at(const T2 *tw, int e, int sign) {
    T2 w = tw[e];
    if (sign < 0) w.y = -w.y;
    return w;
}

// One radix-P Stockham pass over all lines (Ns: product of the earlier
// radices).  The twiddle index k r n/(Ns P) of the inputs stays below n, and
// the butterfly's own twiddles W_P^{rq} are tw[((r q) mod P) n/P] with the
// exponent reduced at compile time.
template <int P, typename T2>
__device__ __forceinline__ void fft_pass(const T2 *x, T2 *y, int n, int nlines, int lstride, int estride,
                                         int sign, const T2 *tw, int Ns) {
    const int nb = n / P, tstep = n / (Ns * P);
    for (int t = threadIdx.x; t < nlines * nb; t += blockDim.x) {
        const int l = t / nb, j = t % nb, k = j % Ns;
        const T2 *xl = x + (long long)l * lstride;
        T2 *yl = y + (long long)l * lstride;
        T2 v[P];
#pragma unroll
        for (int r = 0; r < P; ++r) {
            const T2 a = xl[(long long)(j + r * nb) * estride];
            v[r] = (r == 0 || k == 0) ? a : cmul(a, tw_at(tw, k * r * tstep, sign));
        }
        const int idxD = (j / Ns) * Ns * P + k;
#pragma unroll
        for (int q = 0; q < P; ++q) {
            T2 acc = v[0];
#pragma unroll
            for (int r = 1; r < P; ++r) {
                const int m = (r * q) % P;
                acc = cadd(acc, m == 0 ? v[r] : cmul(v[r], tw_at(tw, m * nb, sign)));
            }
            yl[(long long)(idxD + q * Ns) * estride] = acc;
        }
    }
}

template <typename T2>
__device__ T2 *fft_lines(T2 *x, T2 *y, int n, int nlines, int lstride, int estride, int sign,
                         const T2 *tw) {
    int rad[24];
    int nr = fft_factor(n, rad);
    if (nr < 0) {  // direct DFT (n <= 256, so j q < 2^31)
        for (int t = threadIdx.x; t < nlines * n; t += blockDim.x) {
            int l = t / n, q = t % n;
            const T2 *xl = x + (long long)l * lstride;
            T2 acc = mk2<T2>(0, 0);
            for (int j = 0; j < n; ++j)
                acc = cadd(acc, cmul(xl[(long long)j * estride], tw_at(tw, (j * q) % n, sign)));
            y[(long long)l * lstride + (long long)q * estride] = acc;
        }
        __syncthreads();
        return y;
    }
    int Ns = 1;
    for (int s = 0; s < nr; ++s) {
        const int p = rad[s];
        switch (p) {
            case 4: fft_pass<4, T2>(x, y, n, nlines, lstride, estride, sign, tw, Ns); break;
            case 2: fft_pass<2, T2>(x, y, n, nlines, lstride, estride, sign, tw, Ns); break;
            case 3: fft_pass<3, T2>(x, y, n, nlines, lstride, estride, sign, tw, Ns); break;
            default: fft_pass<5, T2>(x, y, n, nlines, lstride, estride, sign, tw, Ns); break;
        }
        __syncthreads();
        T2 *tmp = x; x = y; y = tmp;
        Ns *= p;
    }
    return x;
}

// Shared-memory (m1, m2) planes of the inverse SO(3) transform: G rows of
// G + 1 elements (the pad keeps column walks free of bank conflicts).
__host__ __device__ inline int isoft_ld(int G) { return G + 1; }
__host__ __device__ inline int isoft_plane(int G) { return G * (G + 1); }

// The transform tail of one beta index k of the inverse SO(3) transform (both
// orientations): bufA / bufC hold the (m1, m2) sums of the direct and the
// inverted orientation at ((m1 mod G) * ld + (m2 mod G)), ld = G + 1; the
// unnormalised backward 2-D DFT (m2 -> gamma, m1 -> alpha) in shared memory,
// then the real part to grid_pair[o * G^3 + a + G * (k + G * g)] (alpha
// fastest).  Only real parts are kept, and Re F(X) = F(H(X)) with H(X)[m] =
// (X[m] + conj X[-m]) / 2 (H(X) transforms to a real grid), so both
// orientations go through ONE complex transform of Z = H(A) + i H(C): its
// real part is the direct grid, its imaginary part the inverted one.  bufB
// is scratch; tw[t] = exp(+2 pi i t / G).  All threads of the block call it.
template <typename T, typename T2>
__device__ void isoft_tail(T2 *bufA, T2 *bufB, T2 *bufC, const T2 *tw, int G, int k, bool inv,
                           T *grid_pair) {
    const int ld = isoft_ld(G);
    T2 *src = bufA, *scr = bufB;
    if (inv) {
        for (int t = threadIdx.x; t < G * G; t += blockDim.x) {
            const int i1 = t / G, i2 = t % G;
            const int e = i1 * ld + i2, em = ((G - i1) % G) * ld + (G - i2) % G;
            const T2 a = bufA[e], am = bufA[em], c = bufC[e], cm = bufC[em];
            T2 z;
            z.x = T(0.5) * ((a.x + am.x) - (c.y - cm.y));
            z.y = T(0.5) * ((a.y - am.y) + (c.x + cm.x));
            bufB[e] = z;
        }
        __syncthreads();
        src = bufB;
        scr = bufA;
    }
    T2 *r1 = fft_lines(src, scr, G, G, ld, 1, +1, tw);      // m2 -> gamma
    T2 *o1 = (r1 == src) ? scr : src;
    T2 *r2 = fft_lines(r1, o1, G, G, 1, ld, +1, tw);        // m1 -> alpha
    T *out0 = grid_pair + (long long)G * k, *out1 = out0 + (long long)G * G * G;
    for (int t = threadIdx.x; t < G * G; t += blockDim.x) {
        const int a = t % G, g = t / G;
        const T2 v = r2[a * ld + g];
        out0[a + (long long)G * G * g] = v.x;
        if (inv) out1[a + (long long)G * G * g] = v.y;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Euler matrix of EULERM (fastclusters.f90:990-1016), row-major.
__host__ __device__ inline void euler_matrix(double a, double b, double g, double *R) {
    double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cg = cos(g), sg = sin(g);
    R[0] = cg * cb * ca - sg * sa;  R[1] = sg * cb * ca + cg * sa;  R[2] = sb * ca;
    R[3] = -cg * cb * sa - sg * ca; R[4] = -sg * cb * sa + cg * ca; R[5] = -sb * sa;
    R[6] = -cg * sb;                R[7] = -sg * sb;                R[8] = cb;
}

__host__ __device__ inline void matmul3(const double *X, const double *Y, double *Z) {
    double T[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            T[3 * i + j] = X[3 * i] * Y[j] + X[3 * i + 1] * Y[3 + j] + X[3 * i + 2] * Y[6 + j];
    for (int i = 0; i < 9; ++i) Z[i] = T[i];
}

// Symmetric 4x4 eigenproblem by cyclic Jacobi rotations (Golub & Van Loan
// 8.5); replaces LAPACK DSYEV in FINDROTATION (alignutils.f90:346).
__host__ __device__ inline void jacobi4(double a[4][4], double w[4], double V[4][4]) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
    // An off-diagonal element below 1e-17 sqrt(|a_pp a_qq|) is already zero
    // at double precision: it is set to zero instead of rotated, and a sweep
    // without rotations ends the iteration (typically after 4-6 sweeps).
    for (int sweep = 0; sweep < 64; ++sweep) {
        int rotated = 0;
        for (int p = 0; p < 4; ++p)
            for (int q = p + 1; q < 4; ++q) {
                if (fabs(a[p][q]) <= 1e-17 * sqrt(fabs(a[p][p] * a[q][q]))) {
                    a[p][q] = a[q][p] = 0.0;
                    continue;
                }
                rotated = 1;
                double theta = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 4; ++k) {
                    double akp = a[k][p], akq = a[k][q];
                    a[k][p] = c * akp - s * akq;
                    a[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 4; ++k) {
                    double apk = a[p][k], aqk = a[q][k];
                    a[p][k] = c * apk - s * aqk;
                    a[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 4; ++k) {
                    double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
        if (!rotated) break;
    }
    for (int i = 0; i < 4; ++i) w[i] = a[i][i];
}

// Quaternion rotation from the 10 unique Kearsley sums (FINDROTATION,
// alignutils.f90:323-377).  q = {Q11,Q12,Q13,Q14,Q22,Q23,Q24,Q33,Q34,Q44}.
__host__ __device__ inline double kearsley_rotation(const double *q, double *R) {
    double Q[4][4] = {{q[0], q[1], q[2], q[3]},
                      {q[1], q[4], q[5], q[6]},
                      {q[2], q[5], q[7], q[8]},
                      {q[3], q[6], q[8], q[9]}};
    double w[4], V[4][4];
    jacobi4(Q, w, V);
    int jmin = 0;
    double minv = 1.0e100;
    for (int j = 0; j < 4; ++j)
        if (w[j] < minv) { minv = w[j]; jmin = j; }
    if (minv < 0.0) minv = (fabs(minv) < 1e-6) ? 0.0 : -minv;
    double q1 = V[0][jmin], q2 = V[1][jmin], q3 = V[2][jmin], q4 = V[3][jmin];
    R[0] = q1 * q1 + q2 * q2 - q3 * q3 - q4 * q4;
    R[1] = 2 * (q2 * q3 + q1 * q4);
    R[2] = 2 * (q2 * q4 - q1 * q3);
    R[3] = 2 * (q2 * q3 - q1 * q4);
    R[4] = q1 * q1 + q3 * q3 - q2 * q2 - q4 * q4;
    R[5] = 2 * (q3 * q4 + q1 * q2);
    R[6] = 2 * (q2 * q4 + q1 * q3);
    R[7] = 2 * (q3 * q4 - q1 * q2);
    R[8] = q1 * q1 + q4 * q4 - q2 * q2 - q3 * q3;
    return sqrt(minv);
}

// Smallest eigenpair of the Kearsley matrix with few FP64 operations:
// cyclic Jacobi on the matrix scaled to unit norm in FP32 gives an
// approximate eigenvector v0; in FP64 the Rayleigh quotient lambda of v0 and
// one inverse-iteration step (Q - lambda I) x = v0 (Gaussian elimination with
// partial pivoting) bring it to double precision -- the error contracts by
// |lambda - lambda_min| / gap, and lambda is already accurate to O(|v0
// error|^2).  Returns the distance sqrt(lambda_min) and R as
// kearsley_rotation does.
__host__ __device__ inline double kearsley_rotation_fast(const double *q, double *R) {
    const double Q[4][4] = {{q[0], q[1], q[2], q[3]},
                            {q[1], q[4], q[5], q[6]},
                            {q[2], q[5], q[7], q[8]},
                            {q[3], q[6], q[8], q[9]}};
    double nrm = 0;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) nrm = fmax(nrm, fabs(Q[i][j]));
    if (!(nrm > 0.0)) {
        for (int k = 0; k < 9; ++k) R[k] = (k % 4 == 0) ? 1.0 : 0.0;
        return 0.0;
    }
    float a[4][4], V[4][4];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
            a[i][j] = (float)(Q[i][j] / nrm);
            V[i][j] = (i == j) ? 1.f : 0.f;
        }
    for (int sweep = 0; sweep < 32; ++sweep) {
        int rotated = 0;
        for (int p = 0; p < 4; ++p)
            for (int r = p + 1; r < 4; ++r) {
                if (fabsf(a[p][r]) <= 1e-8f * sqrtf(fabsf(a[p][p] * a[r][r])) || fabsf(a[p][r]) < 1e-30f) {
                    a[p][r] = a[r][p] = 0.f;
                    continue;
                }
                rotated = 1;
                float theta = (a[r][r] - a[p][p]) / (2.f * a[p][r]);
                float t = (theta >= 0 ? 1.f : -1.f) / (fabsf(theta) + sqrtf(theta * theta + 1.f));
                float c = 1.f / sqrtf(t * t + 1.f), s = t * c;
                for (int k = 0; k < 4; ++k) {
                    float akp = a[k][p], akr = a[k][r];
                    a[k][p] = c * akp - s * akr;
                    a[k][r] = s * akp + c * akr;
                }
                for (int k = 0; k < 4; ++k) {
                    float apk = a[p][k], ark = a[r][k];
                    a[p][k] = c * apk - s * ark;
                    a[r][k] = s * apk + c * ark;
                }
                for (int k = 0; k < 4; ++k) {
                    float vkp = V[k][p], vkr = V[k][r];
                    V[k][p] = c * vkp - s * vkr;
                    V[k][r] = s * vkp + c * vkr;
                }
            }
        if (!rotated) break;
    }
    int jmin = 0;
    for (int j = 1; j < 4; ++j)
        if (a[j][j] < a[jmin][jmin]) jmin = j;
    double v[4] = {V[0][jmin], V[1][jmin], V[2][jmin], V[3][jmin]};
    auto rayleigh = [&](const double *x) {
        double num = 0, den = 0;
        for (int i = 0; i < 4; ++i) {
            double qi = 0;
            for (int j = 0; j < 4; ++j) qi += Q[i][j] * x[j];
            num += x[i] * qi;
            den += x[i] * x[i];
        }
        return num / den;
    };
    double lam = rayleigh(v);
    // one step of inverse iteration on (Q - lam I)
    double M[4][5];
    for (int i = 0; i < 4; ++i) {
        for (int j = 0; j < 4; ++j) M[i][j] = Q[i][j] - (i == j ? lam : 0.0);
        M[i][4] = v[i];
    }
    const double tiny = 1e-300 + 1e-18 * nrm;
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int i = c + 1; i < 4; ++i)
            if (fabs(M[i][c]) > fabs(M[piv][c])) piv = i;
        if (piv != c)
            for (int j = 0; j < 5; ++j) { double t = M[c][j]; M[c][j] = M[piv][j]; M[piv][j] = t; }
        if (fabs(M[c][c]) < tiny) M[c][c] = (M[c][c] < 0 ? -tiny : tiny);
        double inv = 1.0 / M[c][c];
        for (int i = c + 1; i < 4; ++i) {
            double f = M[i][c] * inv;
            for (int j = c; j < 5; ++j) M[i][j] -= f * M[c][j];
        }
    }
    double x[4];
    for (int i = 3; i >= 0; --i) {
        double t = M[i][4];
        for (int j = i + 1; j < 4; ++j) t -= M[i][j] * x[j];
        x[i] = t / M[i][i];
    }
    double xn = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2] + x[3] * x[3]);
    if (xn > 0.0 && isfinite(xn)) {
        for (int i = 0; i < 4; ++i) v[i] = x[i] / xn;
        lam = rayleigh(v);
    }
    double minv = lam;
    if (minv < 0.0) minv = (fabs(minv) < 1e-6) ? 0.0 : -minv;
    double q1 = v[0], q2 = v[1], q3 = v[2], q4 = v[3];
    R[0] = q1 * q1 + q2 * q2 - q3 * q3 - q4 * q4;
    R[1] = 2 * (q2 * q3 + q1 * q4);
    R[2] = 2 * (q2 * q4 - q1 * q3);
    R[3] = 2 * (q2 * q3 - q1 * q4);
    R[4] = q1 * q1 + q3 * q3 - q2 * q2 - q4 * q4;
    R[5] = 2 * (q3 * q4 + q1 * q2);
    R[6] = 2 * (q2 * q4 + q1 * q3);
    R[7] = 2 * (q3 * q4 - q1 * q2);
    R[8] = q1 * q1 + q4 * q4 - q2 * q2 - q3 * q3;
    return sqrt(minv);
}

}  // namespace fo
