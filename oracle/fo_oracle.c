/*
 * fo_oracle.c -- CPU FP64 restatement of the FASTOVERLAP alignment path.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and CPU baseline); the product is
 * the CUDA library under fastoverlap_gb300/csrc.  Written from the upstream
 * algorithm descriptions, not translated line by line; every routine names the
 * upstream file:line whose behaviour it restates.  Plain sequential C99, no
 * globals, so the batch helper can run pairs on several threads.
 */
#include "fo_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.141592653589793238462643383279502884
#define ORC_BIG ((int64_t)1000000000000LL) /* alignutils.f90:1007-1008 */
#define ORC_PSCALE 1.0e6                   /* alignutils.f90:80 */
#define ORC_MAXNEI 60                      /* alignutils.f90:79 */
#define ORC_MAXTRIES 20                    /* alignutils.f90:81 */
#define ORC_LM_TOL 1.0e-6                  /* fastutils.f90:69 */

/* ------------------------------------------------------------------------ */
/* FASTLEN table (fastutils.f90:78-90): smallest 5-smooth integer >= n.      */
int orc_fastlen(int n) {
    if (n <= 1) return 1;
    for (int m = n;; ++m) {
        int k = m;
        while (k % 2 == 0) k /= 2;
        while (k % 3 == 0) k /= 3;
        while (k % 5 == 0) k /= 5;
        if (k == 1) return m;
    }
}

/* ------------------------------------------------------------------------ */
/* Orthonormal spherical harmonics with the Condon-Shortley phase, the
 * convention of RYML (fastclusters.f90:602-652) and scipy sph_harm used by
 * sphericalAlignment.py:57-65.  Output index l*(2L+1) + (m+L); entries with
 * |m| > l are zero.  An atom exactly at the origin gets theta = 0 (the
 * upstream code divides by r there and produces NaN).                       */
void orc_ylm(const double xyz[3], int L, double *re, double *im) {
    const int W = 2 * L + 1;
    double r = sqrt(xyz[0] * xyz[0] + xyz[1] * xyz[1] + xyz[2] * xyz[2]);
    double ct = 1.0, phi = 0.0;
    if (r > 0.0) {
        ct = xyz[2] / r;
        if (ct > 1.0) ct = 1.0;
        if (ct < -1.0) ct = -1.0;
        phi = atan2(xyz[1], xyz[0]);
    }
    double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    memset(re, 0, sizeof(double) * (size_t)(L + 1) * W);
    memset(im, 0, sizeof(double) * (size_t)(L + 1) * W);
    double *P = (double *)malloc(sizeof(double) * (size_t)(L + 1) * (L + 1));
    /* P[l*(L+1)+m] = N_lm P_l^m(cos theta), m >= 0, CS phase included */
    P[0] = 1.0 / sqrt(4.0 * ORC_PI);
    for (int m = 1; m <= L; ++m)
        P[m * (L + 1) + m] = -sqrt((2.0 * m + 1.0) / (2.0 * m)) * st * P[(m - 1) * (L + 1) + (m - 1)];
    for (int m = 0; m < L; ++m)
        P[(m + 1) * (L + 1) + m] = sqrt(2.0 * m + 3.0) * ct * P[m * (L + 1) + m];
    for (int m = 0; m <= L; ++m) {
        for (int l = m + 2; l <= L; ++l) {
            double a = sqrt((4.0 * l * l - 1.0) / ((double)l * l - (double)m * m));
            double b = sqrt(((l - 1.0) * (l - 1.0) - (double)m * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
            P[l * (L + 1) + m] = a * (ct * P[(l - 1) * (L + 1) + m] - b * P[(l - 2) * (L + 1) + m]);
        }
    }
    for (int m = 0; m <= L; ++m) {
        double c = cos(m * phi), s = sin(m * phi);
        double sgn = (m & 1) ? -1.0 : 1.0;
        for (int l = m; l <= L; ++l) {
            double p = P[l * (L + 1) + m];
            re[l * W + L + m] = p * c;
            im[l * W + L + m] = p * s;
            if (m > 0) { /* Y_l^{-m} = (-1)^m conj(Y_l^m) */
                re[l * W + L - m] = sgn * p * c;
                im[l * W + L - m] = -sgn * p * s;
            }
        }
    }
    free(P);
}

/* ------------------------------------------------------------------------ */
/* Modified spherical Bessel functions of the first kind i_l(x), l = 0..L,
 * the quantity SPHI (fastutils.f90:1000-1096) returns and that the Python
 * path forms as iv(l+1/2, x) sqrt(pi/2x) (sphericalAlignment.py:270-271).
 * Miller-type backward recurrence on the ratios r_l = i_l / i_{l-1}
 * (r_l = 1 / ((2l+1)/x + r_{l+1})), normalised by i_0 = sinh(x)/x.          */
static int orc_sphi_start(int L, double x) {
    return L + 24 + (int)(x + 8.0 * sqrt(x + 1.0));
}

void orc_sphi(int L, double x, double *out) {
    if (x == 0.0) {
        out[0] = 1.0;
        for (int l = 1; l <= L; ++l) out[l] = 0.0;
        return;
    }
    out[0] = (x < 1e-4) ? 1.0 + x * x / 6.0 : sinh(x) / x;
    if (L == 0) return;
    int n0 = orc_sphi_start(L, x);
    double r = 0.0;
    double *ratio = (double *)malloc(sizeof(double) * (size_t)(L + 1));
    for (int l = n0; l >= 1; --l) {
        r = 1.0 / ((2.0 * l + 1.0) / x + r);
        if (l <= L) ratio[l] = r;
    }
    for (int l = 1; l <= L; ++l) out[l] = out[l - 1] * ratio[l];
    free(ratio);
}

/* ------------------------------------------------------------------------ */
/* CHOOSE_KWIDTH (fastclusters.f90:1046-1101): 1/3 of the mean nearest-
 * neighbour separation over both structures.                               */
double orc_choose_kwidth(const double *A, const double *B, int n) {
    double sum = 0.0;
    const double *S[2] = {A, B};
    for (int s = 0; s < 2; ++s) {
        const double *X = S[s];
        for (int i = 0; i < n; ++i) {
            double best = 1.0e10;
            for (int j = 0; j < n; ++j) {
                if (i == j) continue;
                double dx = X[3 * i] - X[3 * j], dy = X[3 * i + 1] - X[3 * j + 1], dz = X[3 * i + 2] - X[3 * j + 2];
                double d = sqrt(dx * dx + dy * dy + dz * dz);
                if (d < best) best = d;
            }
            sum += best;
        }
    }
    return sum / (3.0 * 2.0 * n);
}

/* ------------------------------------------------------------------------ */
/* FOURIERCOEFFS (fastclusters.f90:868-916): direct pair sum
 *   I^l_{m1 m2} += 4 pi^{5/2} s^3 i_l(r_a r_b / 2s^2) e^{-(r_a^2+r_b^2)/4s^2}
 *                  Y_{l m1}(b) conj(Y_{l m2}(a))
 * with the optional |r_a - r_b| < 4 s cutoff of :901 (the Python path,
 * sphericalAlignment.py:260-273, has no cutoff).  Output is ADDED to ilmm.  */
void orc_cluster_coeffs(const double *B, const double *A, int n, int L,
                        double sigma, int cutoff, double *ilmm) {
    const int W = 2 * L + 1;
    const size_t ny = (size_t)(L + 1) * W;
    double *YAr = malloc(sizeof(double) * ny * n), *YAi = malloc(sizeof(double) * ny * n);
    double *YBr = malloc(sizeof(double) * ny * n), *YBi = malloc(sizeof(double) * ny * n);
    double *RA = malloc(sizeof(double) * n), *RB = malloc(sizeof(double) * n);
    double *EA = malloc(sizeof(double) * n), *EB = malloc(sizeof(double) * n);
    double *il = malloc(sizeof(double) * (L + 1));
    for (int i = 0; i < n; ++i) {
        orc_ylm(A + 3 * i, L, YAr + ny * i, YAi + ny * i);
        orc_ylm(B + 3 * i, L, YBr + ny * i, YBi + ny * i);
        RA[i] = sqrt(A[3 * i] * A[3 * i] + A[3 * i + 1] * A[3 * i + 1] + A[3 * i + 2] * A[3 * i + 2]);
        RB[i] = sqrt(B[3 * i] * B[3 * i] + B[3 * i + 1] * B[3 * i + 1] + B[3 * i + 2] * B[3 * i + 2]);
        EA[i] = exp(-0.25 * RA[i] * RA[i] / (sigma * sigma));
        EB[i] = exp(-0.25 * RB[i] * RB[i] / (sigma * sigma));
    }
    const double fact = 4.0 * pow(ORC_PI, 2.5) * sigma * sigma * sigma;
    for (int ia = 0; ia < n; ++ia) {
        for (int ib = 0; ib < n; ++ib) {
            if (cutoff && !(fabs(RA[ia] - RB[ib]) < 4.0 * sigma)) continue;
            double x = 0.5 * RA[ia] * RB[ib] / (sigma * sigma);
            orc_sphi(L, x, il);
            double tmp = fact * EA[ia] * EB[ib];
            for (int l = 0; l <= L; ++l) {
                double w = il[l] * tmp;
                const double *ybr = YBr + ny * ib + (size_t)l * W, *ybi = YBi + ny * ib + (size_t)l * W;
                const double *yar = YAr + ny * ia + (size_t)l * W, *yai = YAi + ny * ia + (size_t)l * W;
                for (int m1 = -l; m1 <= l; ++m1) {
                    double br = ybr[L + m1] * w, bi = ybi[L + m1] * w;
                    int i1 = (m1 + W) % W;
                    double *row = ilmm + 2 * (((size_t)l * W + i1) * W);
                    for (int m2 = -l; m2 <= l; ++m2) {
                        double ar = yar[L + m2], ai = yai[L + m2];
                        int i2 = (m2 + W) % W;
                        /* (br + i bi) * (ar - i ai) */
                        row[2 * i2] += br * ar + bi * ai;
                        row[2 * i2 + 1] += bi * ar - br * ai;
                    }
                }
            }
        }
    }
    free(YAr); free(YAi); free(YBr); free(YBi); free(RA); free(RB); free(EA); free(EB); free(il);
}

/* ------------------------------------------------------------------------ */
/* Normalised Wigner little-d table (CALCWIGNERD, DSOFT.f90:121-195):
 * sqrt((2l+1)/2) d^l_{m1 m2}(beta_k), beta_k = pi(2k+1)/(4 bw), by the
 * Kostelec-Rockmore three-term recurrence in l seeded at l = max(|m1|,|m2|).
 * Layout d[((l*W + m1i)*W + m2i)*G + k], W = 2bw-1, G = 2bw (the Python
 * SOFT.Ds layout, soft.py:81).                                             */
static double orc_seed_factor(int J, int M) {
    /* sqrt((2J+1)/2 * (2J)! / ((J+M)! (J-M)!)) via log-gamma for range */
    double lf = lgamma(2.0 * J + 1.0) - lgamma((double)J + M + 1.0) - lgamma((double)J - M + 1.0);
    return sqrt((2.0 * J + 1.0) / 2.0 * exp(lf));
}

static double orc_ipow(double b, int e) {
    double r = 1.0;
    for (int i = 0; i < e; ++i) r *= b;
    return r;
}

void orc_wigner_d(int bw, double *d) {
    const int W = 2 * bw - 1, G = 2 * bw;
    memset(d, 0, sizeof(double) * (size_t)bw * W * W * G);
    for (int m1 = -(bw - 1); m1 <= bw - 1; ++m1) {
        for (int m2 = -(bw - 1); m2 <= bw - 1; ++m2) {
            int i1 = (m1 + W) % W, i2 = (m2 + W) % W;
            int l0 = abs(m1) > abs(m2) ? abs(m1) : abs(m2);
            for (int k = 0; k < G; ++k) {
                double beta = ORC_PI * (2.0 * k + 1.0) / (4.0 * bw);
                double c = cos(beta / 2), s = sin(beta / 2), cb = cos(beta);
                double seed;
                if (l0 == m1)
                    seed = orc_seed_factor(l0, m2) * orc_ipow(c, l0 + m2) * orc_ipow(-s, l0 - m2);
                else if (l0 == -m1)
                    seed = orc_seed_factor(l0, m2) * orc_ipow(c, l0 - m2) * orc_ipow(s, l0 + m2);
                else if (l0 == m2)
                    seed = orc_seed_factor(l0, m1) * orc_ipow(c, l0 + m1) * orc_ipow(s, l0 - m1);
                else
                    seed = orc_seed_factor(l0, m1) * orc_ipow(c, l0 - m1) * orc_ipow(-s, l0 + m1);
                double prev = 0.0, cur = seed;
                d[(((size_t)l0 * W + i1) * W + i2) * G + k] = cur;
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
                    d[(((size_t)(l + 1) * W + i1) * W + i2) * G + k] = cur;
                }
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* In-place complex DFT of length n (mixed radix 2/3/5 recursion, direct sum
 * for other prime factors).  sign = -1: forward (FFTW_FORWARD), +1: backward
 * (FFTW_BACKWARD, unnormalised), as FFTW is used at DSOFT.f90:282 and
 * fastutils.f90:554-569.                                                   */
static void orc_dft_rec(int n, int stride, const double *in, double *out, int sign, double *tmp) {
    if (n == 1) {
        out[0] = in[0];
        out[1] = in[1];
        return;
    }
    int p = 0;
    for (int f = 2; f * f <= n; ++f)
        if (n % f == 0) { p = f; break; }
    if (p == 0) p = n; /* prime: direct DFT */
    int m = n / p;
    if (p == n) {
        for (int k = 0; k < n; ++k) {
            double sr = 0, si = 0;
            for (int j = 0; j < n; ++j) {
                double ang = sign * 2.0 * ORC_PI * (double)((long)j * k % n) / n;
                double c = cos(ang), s = sin(ang);
                double xr = in[2 * j * stride], xi = in[2 * j * stride + 1];
                sr += xr * c - xi * s;
                si += xr * s + xi * c;
            }
            out[2 * k] = sr;
            out[2 * k + 1] = si;
        }
        return;
    }
    /* decimation in time: sub-transforms of the p interleaved subsequences */
    for (int q = 0; q < p; ++q)
        orc_dft_rec(m, stride * p, in + 2 * q * stride, tmp + 2 * q * m, sign, out);
    for (int k = 0; k < m; ++k) {
        for (int r = 0; r < p; ++r) {
            int kk = k + r * m;
            double sr = 0, si = 0;
            for (int q = 0; q < p; ++q) {
                double ang = sign * 2.0 * ORC_PI * (double)((long)q * kk % n) / n;
                double c = cos(ang), s = sin(ang);
                double xr = tmp[2 * (q * m + k)], xi = tmp[2 * (q * m + k) + 1];
                sr += xr * c - xi * s;
                si += xr * s + xi * c;
            }
            out[2 * kk] = sr;
            out[2 * kk + 1] = si;
        }
    }
}

static void orc_fft1d(int n, double *data /* interleaved, stride 1 */, int sign) {
    double *in = malloc(sizeof(double) * 2 * n), *tmp = malloc(sizeof(double) * 2 * n);
    double *scratch = malloc(sizeof(double) * 2 * n);
    memcpy(in, data, sizeof(double) * 2 * n);
    (void)scratch;
    orc_dft_rec(n, 1, in, data, sign, tmp);
    free(in); free(tmp); free(scratch);
}

/* ------------------------------------------------------------------------ */
/* ISOFT (DSOFT.f90:265-329) followed by the real part (CALCOVERLAP,
 * fastclusters.f90:918-960): Wigner contraction over l, then unnormalised
 * backward DFTs over m2 -> gamma and m1 -> alpha.                           */
void orc_isoft(int bw, const double *ilmm, double *grid_re) {
    const int W = 2 * bw - 1, G = 2 * bw;
    double *d = malloc(sizeof(double) * (size_t)bw * W * W * G);
    orc_wigner_d(bw, d);
    /* S[m1g][beta][m2g] complex, m index mod G */
    double *S = calloc((size_t)2 * G * G * G, sizeof(double));
    for (int m1 = -(bw - 1); m1 <= bw - 1; ++m1) {
        for (int m2 = -(bw - 1); m2 <= bw - 1; ++m2) {
            int i1 = (m1 + W) % W, i2 = (m2 + W) % W;
            int g1 = (m1 + G) % G, g2 = (m2 + G) % G;
            int l0 = abs(m1) > abs(m2) ? abs(m1) : abs(m2);
            for (int k = 0; k < G; ++k) {
                double sr = 0, si = 0;
                for (int l = l0; l < bw; ++l) {
                    double dv = d[(((size_t)l * W + i1) * W + i2) * G + k];
                    const double *c = ilmm + 2 * (((size_t)l * W + i1) * W + i2);
                    sr += dv * c[0];
                    si += dv * c[1];
                }
                double *o = S + 2 * (((size_t)g1 * G + k) * G + g2);
                o[0] = sr;
                o[1] = si;
            }
        }
    }
    double *line = malloc(sizeof(double) * 2 * G);
    /* gamma axis (contiguous) */
    for (int a = 0; a < G; ++a)
        for (int k = 0; k < G; ++k) orc_fft1d(G, S + 2 * (((size_t)a * G + k) * G), +1);
    /* alpha axis */
    for (int k = 0; k < G; ++k) {
        for (int g = 0; g < G; ++g) {
            for (int a = 0; a < G; ++a) {
                line[2 * a] = S[2 * (((size_t)a * G + k) * G + g)];
                line[2 * a + 1] = S[2 * (((size_t)a * G + k) * G + g) + 1];
            }
            orc_fft1d(G, line, +1);
            for (int a = 0; a < G; ++a) grid_re[a + (size_t)G * (k + (size_t)G * g)] = line[2 * a];
        }
    }
    free(line); free(S); free(d);
}

/* ------------------------------------------------------------------------ */
/* Peak model of GAUSSIAN / FCN (fastutils.f90:231-349):
 *   f(q) = p0 exp(-Y) + p1,  u = q - c,
 *   Y = p2 u1^2 + p3 u2^2 + p4 u3^2 + p5 u1 u2 + p6 u2 u3 + p7 u1 u3,
 *   c = (p8, p9, p10), q = 1-based integer grid coordinates.
 * Fitted by Levenberg-Marquardt (Marquardt 1963) on the residuals f - data
 * with the analytic Jacobian, diagonal scaling, lambda /= 10 on success and
 * *= 10 on failure, stopping on relative reduction or relative step <= tol
 * (info 1/2/3), no further progress (info 4) or after 100*(11+1) model
 * evaluations (info 5), the limits lmder1 is called with at :395.           */
static double orc_peak_model(const double *p, double u1, double u2, double u3, double *e_out) {
    double Y = p[2] * u1 * u1 + p[3] * u2 * u2 + p[4] * u3 * u3 + p[5] * u1 * u2 + p[6] * u2 * u3 + p[7] * u1 * u3;
    double e = exp(-Y);
    if (e_out) *e_out = e;
    return p[0] * e + p[1];
}

static double orc_lm_cost(const double *p, const double *data, int w) {
    int n = 2 * w + 1;
    double S = 0;
    for (int i3 = 0; i3 < n; ++i3)
        for (int i2 = 0; i2 < n; ++i2)
            for (int i1 = 0; i1 < n; ++i1) {
                double r = orc_peak_model(p, i1 + 1 - p[8], i2 + 1 - p[9], i3 + 1 - p[10], NULL) -
                           data[i1 + n * (i2 + n * i3)];
                S += r * r;
            }
    return S;
}

static int orc_chol_solve(double A[11][11], const double *b, double *x) {
    double Lm[11][11];
    memset(Lm, 0, sizeof Lm);
    for (int j = 0; j < 11; ++j) {
        double s = A[j][j];
        for (int k = 0; k < j; ++k) s -= Lm[j][k] * Lm[j][k];
        if (!(s > 0.0)) return -1;
        Lm[j][j] = sqrt(s);
        for (int i = j + 1; i < 11; ++i) {
            double t = A[i][j];
            for (int k = 0; k < j; ++k) t -= Lm[i][k] * Lm[j][k];
            Lm[i][j] = t / Lm[j][j];
        }
    }
    double y[11];
    for (int i = 0; i < 11; ++i) {
        double t = b[i];
        for (int k = 0; k < i; ++k) t -= Lm[i][k] * y[k];
        y[i] = t / Lm[i][i];
    }
    for (int i = 10; i >= 0; --i) {
        double t = y[i];
        for (int k = i + 1; k < 11; ++k) t -= Lm[k][i] * x[k];
        x[i] = t / Lm[i][i];
    }
    return 0;
}

static int orc_lm_fit(double *p, const double *data, int w, double tol) {
    const int n = 2 * w + 1, maxfev = 100 * (11 + 1);
    double lambda = 1e-3;
    double S = orc_lm_cost(p, data, w);
    int nfev = 1;
    if (!isfinite(S)) return 0;
    for (;;) {
        double H[11][11], g[11];
        memset(H, 0, sizeof H);
        memset(g, 0, sizeof g);
        for (int i3 = 0; i3 < n; ++i3)
            for (int i2 = 0; i2 < n; ++i2)
                for (int i1 = 0; i1 < n; ++i1) {
                    double u1 = i1 + 1 - p[8], u2 = i2 + 1 - p[9], u3 = i3 + 1 - p[10], e;
                    double f = orc_peak_model(p, u1, u2, u3, &e);
                    double r = f - data[i1 + n * (i2 + n * i3)];
                    double ae = p[0] * e, J[11];
                    J[0] = e;
                    J[1] = 1.0;
                    J[2] = -ae * u1 * u1;
                    J[3] = -ae * u2 * u2;
                    J[4] = -ae * u3 * u3;
                    J[5] = -ae * u1 * u2;
                    J[6] = -ae * u2 * u3;
                    J[7] = -ae * u1 * u3;
                    J[8] = ae * (2 * p[2] * u1 + p[5] * u2 + p[7] * u3);
                    J[9] = ae * (2 * p[3] * u2 + p[5] * u1 + p[6] * u3);
                    J[10] = ae * (2 * p[4] * u3 + p[6] * u2 + p[7] * u1);
                    for (int a = 0; a < 11; ++a) {
                        g[a] += J[a] * r;
                        for (int b = 0; b <= a; ++b) H[a][b] += J[a] * J[b];
                    }
                }
        for (int a = 0; a < 11; ++a)
            for (int b = 0; b < a; ++b) H[b][a] = H[a][b];
        for (;;) {
            double A[11][11], mg[11], dlt[11], pn[11];
            memcpy(A, H, sizeof A);
            for (int a = 0; a < 11; ++a) {
                A[a][a] += lambda * fmax(H[a][a], 1e-30);
                mg[a] = -g[a];
            }
            int ok = orc_chol_solve(A, mg, dlt);
            double Sn = INFINITY;
            if (ok == 0) {
                for (int a = 0; a < 11; ++a) pn[a] = p[a] + dlt[a];
                Sn = orc_lm_cost(pn, data, w);
                ++nfev;
            }
            if (ok == 0 && Sn < S) {
                double rel = (S - Sn) / S, step = 0, pnorm = 0;
                for (int a = 0; a < 11; ++a) {
                    step += dlt[a] * dlt[a];
                    pnorm += pn[a] * pn[a];
                }
                step = sqrt(step);
                pnorm = sqrt(pnorm);
                memcpy(p, pn, sizeof(double) * 11);
                S = Sn;
                lambda = fmax(lambda * 0.1, 1e-15);
                int c1 = rel <= tol, c2 = step <= tol * (pnorm + tol);
                if (c1 && c2) return 3;
                if (c1) return 1;
                if (c2) return 2;
                if (nfev >= maxfev) return 5;
                break;
            }
            lambda *= 10.0;
            if (lambda > 1e16) return 4;
            if (nfev >= maxfev) return 5;
        }
    }
}

/* FINDPEAKS / FINDPEAK (fastutils.f90:401-548): repeat up to npeaks times:
 * first maximum in Fortran (column-major) order, periodic (2w+1)^3 window,
 * Gaussian fit, record the centre, subtract the fitted Gaussian (not
 * wrapped) plus its mean from the whole grid.  A failed fit (info 0 or 5)
 * ends the search; if nothing was found the window grows by one.          */
int orc_findpeaks(const double *grid, int n1, int n2, int n3, int npeaks,
                  double *peaks, double *amps) {
    return orc_findpeaks_w(grid, n1, n2, n3, npeaks, 2, peaks, amps);
}

/* The same search starting from half-width width0 (FINDPEAKS reads its
 * width from the module variable WIDTH, :68; the first width is tried
 * without the MINVAL(FSHAPE)/2 check, later ones with it, :538-544). */
int orc_findpeaks_w(const double *grid, int n1, int n2, int n3, int npeaks, int width0,
                    double *peaks, double *amps) {
    const size_t N = (size_t)n1 * n2 * n3;
    double *f = malloc(sizeof(double) * N);
    int width = width0, nfound = 0;
    int minshape = n1 < n2 ? n1 : n2;
    if (n3 < minshape) minshape = n3;
    while (nfound == 0) {
        memcpy(f, grid, sizeof(double) * N);
        for (int np = 0; np < npeaks; ++np) {
            size_t amax = 0;
            double sum = 0, mx = f[0];
            for (size_t i = 0; i < N; ++i) {
                sum += f[i];
                if (f[i] > mx) {
                    mx = f[i];
                    amax = i;
                }
            }
            double mean = sum / (double)N;
            int a1 = (int)(amax % n1), a2 = (int)((amax / n1) % n2), a3 = (int)(amax / ((size_t)n1 * n2));
            int wn = 2 * width + 1;
            double *win = malloc(sizeof(double) * (size_t)wn * wn * wn);
            for (int i3 = 0; i3 < wn; ++i3)
                for (int i2 = 0; i2 < wn; ++i2)
                    for (int i1 = 0; i1 < wn; ++i1) {
                        int j1 = ((a1 + i1 - width) % n1 + n1) % n1;
                        int j2 = ((a2 + i2 - width) % n2 + n2) % n2;
                        int j3 = ((a3 + i3 - width) % n3 + n3) % n3;
                        win[i1 + wn * (i2 + wn * i3)] = f[j1 + (size_t)n1 * (j2 + (size_t)n2 * j3)];
                    }
            double p[11] = {mx - mean, mean, 1, 1, 1, 0, 0, 0, width + 1.0, width + 1.0, width + 1.0};
            int info = orc_lm_fit(p, win, width, ORC_LM_TOL);
            free(win);
            if (info == 0 || info == 5) break;
            double c[3] = {p[8] - width - 1 + (a1 + 1), p[9] - width - 1 + (a2 + 1), p[10] - width - 1 + (a3 + 1)};
            peaks[3 * nfound] = c[0];
            peaks[3 * nfound + 1] = c[1];
            peaks[3 * nfound + 2] = c[2];
            amps[nfound] = p[0];
            ++nfound;
            for (int i3 = 0; i3 < n3; ++i3)
                for (int i2 = 0; i2 < n2; ++i2)
                    for (int i1 = 0; i1 < n1; ++i1)
                        f[i1 + (size_t)n1 * (i2 + (size_t)n2 * i3)] -=
                            orc_peak_model(p, i1 + 1 - c[0], i2 + 1 - c[1], i3 + 1 - c[2], NULL);
        }
        if (nfound == 0) {
            ++width;
            if (width > minshape / 2) {
                free(f);
                return -1;
            }
        }
    }
    free(f);
    return nfound;
}

/* EULERM (fastclusters.f90:990-1016) as a row-major matrix. */
void orc_eulerm(double a, double b, double g, double R[9]) {
    double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cg = cos(g), sg = sin(g);
    R[0] = cg * cb * ca - sg * sa;
    R[1] = sg * cb * ca + cg * sa;
    R[2] = sb * ca;
    R[3] = -cg * cb * sa - sg * ca;
    R[4] = -sg * cb * sa + cg * ca;
    R[5] = -sb * sa;
    R[6] = -cg * sb;
    R[7] = -sg * sb;
    R[8] = cb;
}

/* ------------------------------------------------------------------------ */
/* PAIRDIST / PAIRDISTS (alignutils.f90:582-730): squared (minimum-image when
 * bulk) distances from each p_i to the q_j; for n > maxnei only the maxnei
 * nearest per row, kept in a binary max-heap whose array order is the
 * stored order.  kk is 0-based.                                            */
static double orc_pairdist(const double *c1, const double *c2, int bulk, const double box[3]) {
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

void orc_pairdists(int n, const double *p, const double *q, int bulk,
                   const double box[3], int maxnei, double *cc, int *kk) {
    int m = n <= maxnei ? n : maxnei;
    for (int i = 0; i < n; ++i) {
        double *c = cc + (size_t)i * m;
        int *k = kk + (size_t)i * m;
        if (m == n) {
            for (int j = 0; j < n; ++j) {
                c[j] = orc_pairdist(p + 3 * i, q + 3 * j, bulk, box);
                k[j] = j;
            }
            continue;
        }
        /* heap positions are 1-based in the arithmetic below */
        for (int j = 0; j < m; ++j) {
            c[j] = orc_pairdist(p + 3 * i, q + 3 * j, bulk, box);
            k[j] = j;
            int l = j + 1;
            while (l > 1) {
                int l2 = l / 2;
                if (c[l2 - 1] < c[l - 1]) {
                    double h = c[l2 - 1]; c[l2 - 1] = c[l - 1]; c[l - 1] = h;
                    int t = k[l2 - 1]; k[l2 - 1] = k[l - 1]; k[l - 1] = t;
                    l = l2;
                } else break;
            }
        }
        for (int j = m; j < n; ++j) {
            double d = orc_pairdist(p + 3 * i, q + 3 * j, bulk, box);
            if (!(d < c[0])) continue;
            c[0] = d;
            k[0] = j;
            int l = 1;
            for (;;) {
                int l2 = 2 * l;
                if (l2 + 1 > m) {
                    if (l2 <= m && c[l2 - 1] > c[l - 1]) {
                        double h = c[l2 - 1]; c[l2 - 1] = c[l - 1]; c[l - 1] = h;
                        int t = k[l2 - 1]; k[l2 - 1] = k[l - 1]; k[l - 1] = t;
                    }
                    break;
                }
                int a = (c[l2] > c[l2 - 1]) ? l2 + 1 : l2;
                if (c[a - 1] > c[l - 1]) {
                    double h = c[a - 1]; c[a - 1] = c[l - 1]; c[l - 1] = h;
                    int t = k[a - 1]; k[a - 1] = k[l - 1]; k[l - 1] = t;
                    l = a;
                } else break;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Sparse linear assignment, Jonker & Volgenant (Computing 38, 1987), the
 * method of JOVOSAP (alignutils.f90:989-1259): column reduction, reduction
 * transfer, two passes of augmenting row reduction, then shortest augmenting
 * paths for the remaining free rows.  Rows are CSR (first[], kk[] 0-based
 * columns, cc[] int64 costs).  Returns 0 on success, >0 when the matching
 * fails (the upstream routine then returns silently with a partial
 * assignment; unassigned entries stay -1 here).                            */
int orc_jv(int n, const int64_t *cc, const int *kk, const int *first, int *x, int *y) {
    int64_t *v = malloc(sizeof(int64_t) * n), *dd = malloc(sizeof(int64_t) * n);
    int *lab = malloc(sizeof(int) * n), *fr = malloc(sizeof(int) * n), *todo = malloc(sizeof(int) * n);
    char *ok = malloc((size_t)n), *multi = calloc((size_t)n, 1);
    int rc = 0;
    /* column reduction */
    for (int j = 0; j < n; ++j) {
        v[j] = ORC_BIG;
        y[j] = -1;
    }
    for (int i = 0; i < n; ++i) {
        x[i] = -1;
        for (int t = first[i]; t < first[i + 1]; ++t) {
            int j = kk[t];
            if (cc[t] < v[j]) {
                v[j] = cc[t];
                y[j] = i;
            }
        }
    }
    for (int j = n - 1; j >= 0; --j) {
        int i = y[j];
        if (i < 0) { rc = 1; goto done; }
        if (x[i] >= 0) {
            multi[i] = 1;
            y[j] = -1;
        } else {
            x[i] = j;
        }
    }
    /* reduction transfer */
    int nfree = 0;
    for (int i = 0; i < n; ++i) {
        if (x[i] < 0) {
            fr[nfree++] = i;
        } else if (multi[i]) {
            multi[i] = 0;
        } else {
            int j1 = x[i];
            int64_t mn = ORC_BIG;
            for (int t = first[i]; t < first[i + 1]; ++t) {
                int j = kk[t];
                if (j == j1) continue;
                if (cc[t] - v[j] < mn) mn = cc[t] - v[j];
            }
            v[j1] -= mn;
        }
    }
    if (nfree == 0) goto done;
    /* augmenting row reduction, two passes */
    int j0 = -1, j1 = -1;
    for (int pass = 0; pass < 2 && nfree > 0; ++pass) {
        int l0 = nfree, k = 0;
        nfree = 0;
        while (k < l0) {
            int i = fr[k++];
            int64_t u1 = ORC_BIG, u2 = ORC_BIG;
            for (int t = first[i]; t < first[i + 1]; ++t) {
                int j = kk[t];
                int64_t h = cc[t] - v[j];
                if (h < u2) {
                    if (h >= u1) {
                        u2 = h;
                        j1 = j;
                    } else {
                        u2 = u1;
                        u1 = h;
                        j1 = j0;
                        j0 = j;
                    }
                }
            }
            if (j0 < 0) { rc = 2; goto done; }
            int i0 = y[j0];
            int reinsert = 0;
            if (u1 < u2) {
                v[j0] = v[j0] - u2 + u1;
                reinsert = (i0 >= 0);
            } else if (i0 >= 0) {
                if (j1 < 0) { rc = 3; goto done; }
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
    /* augmentation */
    {
        int l0 = nfree;
        for (int f = 0; f < l0; ++f) {
            for (int j = 0; j < n; ++j) {
                ok[j] = 0;
                dd[j] = ORC_BIG;
            }
            int64_t mn = ORC_BIG;
            int i0 = fr[f], td = n - 1, k = 0, jend = -1;
            for (int t = first[i0]; t < first[i0 + 1]; ++t) {
                int j = kk[t];
                int64_t dj = cc[t] - v[j];
                dd[j] = dj;
                lab[j] = i0;
                if (dj <= mn) {
                    if (dj < mn) {
                        mn = dj;
                        k = 0;
                    }
                    todo[k++] = j;
                }
            }
            for (int h = 0; h < k; ++h) {
                int j = todo[h];
                if (y[j] < 0) { jend = j; goto augment; }
                ok[j] = 1;
            }
            for (;;) {
                if (k == 0) { rc = 4; goto done; }
                int jc = todo[--k];
                int i = y[jc];
                todo[td--] = jc;
                int t = first[i];
                while (t < first[i + 1] && kk[t] != jc) ++t;
                if (t == first[i + 1]) { rc = 5; goto done; }
                int64_t h = cc[t] - v[jc] - mn;
                for (t = first[i]; t < first[i + 1]; ++t) {
                    int j = kk[t];
                    if (ok[j]) continue;
                    int64_t vj = cc[t] - h - v[j];
                    if (vj < dd[j]) {
                        dd[j] = vj;
                        lab[j] = i;
                        if (vj == mn) {
                            if (y[j] < 0) { jend = j; goto price; }
                            todo[k++] = j;
                            ok[j] = 1;
                        }
                    }
                }
                if (k != 0) continue;
                mn = ORC_BIG - 1;
                for (int j = 0; j < n; ++j) {
                    if (dd[j] <= mn && !ok[j]) {
                        if (dd[j] < mn) {
                            mn = dd[j];
                            k = 0;
                        }
                        todo[k++] = j;
                    }
                }
                for (int h2 = 0; h2 < k; ++h2) {
                    int j = todo[h2];
                    if (y[j] < 0) { jend = j; goto price; }
                    ok[j] = 1;
                }
            }
        price:
            if (mn != 0)
                for (int q = td + 1; q < n; ++q) {
                    int jj = todo[q];
                    v[jj] += dd[jj] - mn;
                }
        augment:
            for (;;) {
                int i = lab[jend];
                y[jend] = i;
                int kswap = jend;
                jend = x[i];
                x[i] = kswap;
                if (i == i0) break;
            }
        }
    }
done:
    free(v); free(dd); free(lab); free(fr); free(todo); free(ok); free(multi);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* FINDBESTPERM (alignutils.f90:482-580): per group, integer costs
 * INT(d^2 * 1e6) (truncation), sparse JV, permutation
 * newperm[group[j]] = group[y_j], exact summed d^2 of the assignment.
 * Returns the summed d^2; *fail counts clamped entries.                    */
static double orc_findbestperm(const double *B, const double *A, int n, const int *perm,
                               const int *gsize, int ngroups, int bulk, const double box[3],
                               int *newperm, int *fail) {
    double dist = 0;
    int off = 0;
    for (int j = 0; j < n; ++j) newperm[j] = j;
    for (int g = 0; g < ngroups; ++g) {
        int ns = gsize[g];
        if (ns == 0) continue;
        int m = ns <= ORC_MAXNEI ? ns : ORC_MAXNEI;
        double *pb = malloc(sizeof(double) * 3 * ns), *qa = malloc(sizeof(double) * 3 * ns);
        for (int j = 0; j < ns; ++j)
            for (int c = 0; c < 3; ++c) {
                pb[3 * j + c] = B[3 * perm[off + j] + c];
                qa[3 * j + c] = A[3 * perm[off + j] + c];
            }
        double *nd = malloc(sizeof(double) * (size_t)ns * m);
        int *kk = malloc(sizeof(int) * (size_t)ns * m), *first = malloc(sizeof(int) * (ns + 1));
        int64_t *cc = malloc(sizeof(int64_t) * (size_t)ns * m);
        orc_pairdists(ns, pb, qa, bulk, box, ORC_MAXNEI, nd, kk);
        for (int i = 0; i <= ns; ++i) first[i] = i * m;
        for (size_t t = 0; t < (size_t)ns * m; ++t) cc[t] = (int64_t)(nd[t] * ORC_PSCALE);
        int *xr = malloc(sizeof(int) * ns), *yc = malloc(sizeof(int) * ns);
        orc_jv(ns, cc, kk, first, xr, yc);
        for (int j = 0; j < ns; ++j) {
            int col = xr[j];
            if (col >= ns) { col = ns - 1; ++*fail; }
            if (col < 0) { col = 0; ++*fail; }
            newperm[perm[off + j]] = perm[off + col];
            int t = j * m, found = -1;
            for (int q = 0; q < m; ++q)
                if (kk[t + q] == col) { found = t + q; break; }
            dist += (found >= 0) ? nd[found] : orc_pairdist(pb + 3 * j, qa + 3 * col, bulk, box);
        }
        free(pb); free(qa); free(nd); free(kk); free(first); free(cc); free(xr); free(yc);
        off += ns;
    }
    return dist;
}

/* ------------------------------------------------------------------------ */
/* Eigen-decomposition of a symmetric 4x4 matrix by cyclic Jacobi rotations
 * (Jacobi 1846; Golub & Van Loan sec. 8.5), standing in for LAPACK DSYEV. */
static void orc_jacobi4(double a[4][4], double w[4], double V[4][4]) {
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) V[i][j] = (i == j);
    /* an off-diagonal element below 1e-17 sqrt(|a_pp a_qq|) is zero at double
     * precision: zero it; a sweep without rotations ends the iteration */
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

/* FINDROTATION (alignutils.f90:304-379): Kearsley quaternion matrix of
 * B - A / B + A, smallest eigenpair -> rotation R (A -> B), distance. */
double orc_findrotation(const double *B, const double *A, int n, double R[9]) {
    double Q[4][4];
    memset(Q, 0, sizeof Q);
    for (int j = 0; j < n; ++j) {
        double xm = B[3 * j] - A[3 * j], ym = B[3 * j + 1] - A[3 * j + 1], zm = B[3 * j + 2] - A[3 * j + 2];
        double xp = B[3 * j] + A[3 * j], yp = B[3 * j + 1] + A[3 * j + 1], zp = B[3 * j + 2] + A[3 * j + 2];
        Q[0][0] += xm * xm + ym * ym + zm * zm;
        Q[0][1] += yp * zm - ym * zp;
        Q[0][2] += xm * zp - xp * zm;
        Q[0][3] += xp * ym - xm * yp;
        Q[1][1] += yp * yp + zp * zp + xm * xm;
        Q[1][2] += xm * ym - xp * yp;
        Q[1][3] += xm * zm - xp * zp;
        Q[2][2] += xp * xp + zp * zp + ym * ym;
        Q[2][3] += ym * zm - yp * zp;
        Q[3][3] += xp * xp + yp * yp + zm * zm;
    }
    Q[1][0] = Q[0][1]; Q[2][0] = Q[0][2]; Q[2][1] = Q[1][2];
    Q[3][0] = Q[0][3]; Q[3][1] = Q[1][3]; Q[3][2] = Q[2][3];
    double w[4], V[4][4];
    orc_jacobi4(Q, w, V);
    int jmin = 0;
    double minv = 1.0e100;
    for (int j = 0; j < 4; ++j)
        if (w[j] < minv) {
            minv = w[j];
            jmin = j;
        }
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

/* FINDDISPLACEMENT (alignutils.f90:381-419): mean minimum-image B - A. */
static double orc_finddisplacement(const double *B, const double *A, int n, const double box[3], double disp[3]) {
    disp[0] = disp[1] = disp[2] = 0;
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < 3; ++k) {
            double t = B[3 * j + k] - A[3 * j + k];
            disp[k] += t - box[k] * round(t / box[k]);
        }
    for (int k = 0; k < 3; ++k) disp[k] /= n;
    double d = 0;
    for (int j = 0; j < n; ++j) {
        double a[3] = {A[3 * j] + disp[0], A[3 * j + 1] + disp[1], A[3 * j + 2] + disp[2]};
        d += orc_pairdist(B + 3 * j, a, 1, box);
    }
    return sqrt(d);
}

static void orc_matmul3(const double X[9], const double Y[9], double Z[9]) {
    double T[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[3 * i + j] = X[3 * i] * Y[j] + X[3 * i + 1] * Y[3 + j] + X[3 * i + 2] * Y[6 + j];
    memcpy(Z, T, sizeof T);
}

/* ITERATIVEALIGN (alignutils.f90:111-286): alternate LAP permutation and
 * rotation (cluster) or mean displacement (bulk) until no atom moves, the
 * distance grows, or after 20 tries.  A is overwritten by the aligned,
 * permuted copy.  Returns the final distance.                               */
double orc_iterative_align(const double *Bin, double *A, int n, const int *perm,
                           const int *gsize, int ngroups, int bulk,
                           const double box[3], double R[9], double disp[3],
                           int *permbest, int *niter) {
    double *DA = malloc(sizeof(double) * 3 * n), *DB = malloc(sizeof(double) * 3 * n);
    double *DUM = malloc(sizeof(double) * 3 * n);
    int *newperm = malloc(sizeof(int) * n), *saveperm = malloc(sizeof(int) * n);
    double cma[3] = {0, 0, 0}, cmb[3] = {0, 0, 0};
    double Rb[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, Rn[9], dn[3] = {0, 0, 0}, db[3] = {0, 0, 0};
    if (bulk) {
        memcpy(DA, A, sizeof(double) * 3 * n);
        memcpy(DB, Bin, sizeof(double) * 3 * n);
    } else {
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < 3; ++k) {
                cma[k] += A[3 * j + k];
                cmb[k] += Bin[3 * j + k];
            }
        for (int k = 0; k < 3; ++k) {
            cma[k] /= n;
            cmb[k] /= n;
        }
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < 3; ++k) {
                DA[3 * j + k] = A[3 * j + k] - cma[k];
                DB[3 * j + k] = Bin[3 * j + k] - cmb[k];
            }
    }
    for (int j = 0; j < n; ++j) permbest[j] = j;
    int ntries = 0, nperm = n, fail = 0;
    double newdist = 0;
    while (nperm > 0) {
        memcpy(DUM, DA, sizeof(double) * 3 * n);
        memcpy(saveperm, permbest, sizeof(int) * n);
        double pd = sqrt(orc_findbestperm(DB, DA, n, perm, gsize, ngroups, bulk, box, newperm, &fail));
        nperm = 0;
        for (int j = 0; j < n; ++j) {
            for (int k = 0; k < 3; ++k) DA[3 * j + k] = DUM[3 * newperm[j] + k];
            permbest[j] = saveperm[newperm[j]];
            if (j != newperm[j]) ++nperm;
        }
        if (bulk) {
            newdist = orc_finddisplacement(DB, DA, n, box, dn);
            for (int k = 0; k < 3; ++k) db[k] += dn[k];
            for (int j = 0; j < n; ++j)
                for (int k = 0; k < 3; ++k) DA[3 * j + k] = A[3 * permbest[j] + k] + db[k];
        } else {
            newdist = orc_findrotation(DB, DA, n, Rn);
            orc_matmul3(Rn, Rb, Rb);
            for (int j = 0; j < n; ++j) {
                double t[3];
                for (int k = 0; k < 3; ++k) t[k] = A[3 * permbest[j] + k] - cma[k];
                for (int k = 0; k < 3; ++k)
                    DA[3 * j + k] = Rb[3 * k] * t[0] + Rb[3 * k + 1] * t[1] + Rb[3 * k + 2] * t[2];
            }
        }
        ++ntries;
        if ((newdist - pd) / newdist > sqrt((double)n) / ORC_PSCALE) break;
        if (ntries > ORC_MAXTRIES) break;
    }
    if (bulk) {
        newdist = orc_finddisplacement(DB, DA, n, box, dn);
        for (int k = 0; k < 3; ++k) db[k] += dn[k];
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < 3; ++k) DA[3 * j + k] += dn[k];
        memcpy(A, DA, sizeof(double) * 3 * n);
    } else {
        newdist = orc_findrotation(DB, DA, n, Rn);
        orc_matmul3(Rn, Rb, Rb);
        for (int j = 0; j < n; ++j) {
            double t[3] = {DA[3 * j], DA[3 * j + 1], DA[3 * j + 2]};
            for (int k = 0; k < 3; ++k)
                A[3 * j + k] = Rn[3 * k] * t[0] + Rn[3 * k + 1] * t[1] + Rn[3 * k + 2] * t[2] + cmb[k];
        }
    }
    if (R) memcpy(R, Rb, sizeof Rb);
    if (disp) memcpy(disp, db, sizeof db);
    if (niter) *niter = ntries;
    free(DA); free(DB); free(DUM); free(newperm); free(saveperm);
    return newdist;
}

/* ------------------------------------------------------------------------ */
/* ALIGNCOEFFS (cluster, fastclusters.f90:393-470): overlap grid from the
 * coefficients, candidate rotations from its peaks (FINDROTATIONS :962-988),
 * ITERATIVEALIGN from each, keep the smallest distance (first wins ties).  */
static int orc_align_coeffs(const double *B, const double *A, int n, const int *perm,
                            const int *gsize, int ngroups, int L, const double *ilmm, int nrot,
                            double *best_aligned, int *best_perm, double Rbest[9],
                            double *best_dist, double *omax, int *ncand) {
    int bw = L + 1, G = 2 * bw;
    double *grid = malloc(sizeof(double) * (size_t)G * G * G);
    orc_isoft(bw, ilmm, grid);
    double mx = grid[0];
    for (size_t i = 0; i < (size_t)G * G * G; ++i)
        if (grid[i] > mx) mx = grid[i];
    *omax = mx;
    double *peaks = malloc(sizeof(double) * 3 * nrot), *amps = malloc(sizeof(double) * nrot);
    int np = orc_findpeaks(grid, G, G, G, nrot, peaks, amps);
    free(grid);
    if (np < 0) {
        free(peaks); free(amps);
        return -2;
    }
    double conv = ORC_PI / G;
    double *DA = malloc(sizeof(double) * 3 * n);
    int *pb = malloc(sizeof(int) * n);
    *best_dist = HUGE_VAL;
    for (int c = 0; c < np; ++c) {
        double a = (peaks[3 * c] - 1.0) * 2 * conv, b = (peaks[3 * c + 1] - 0.5) * conv,
               g = (peaks[3 * c + 2] - 1.0) * 2 * conv;
        double Rs[9], Rr[9];
        orc_eulerm(a, b, g, Rs);
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < 3; ++k)
                DA[3 * j + k] = Rs[3 * k] * A[3 * j] + Rs[3 * k + 1] * A[3 * j + 1] + Rs[3 * k + 2] * A[3 * j + 2];
        double d = orc_iterative_align(B, DA, n, perm, gsize, ngroups, 0, NULL, Rr, NULL, pb, NULL);
        if (d < *best_dist) {
            *best_dist = d;
            memcpy(best_aligned, DA, sizeof(double) * 3 * n);
            memcpy(best_perm, pb, sizeof(int) * n);
            orc_matmul3(Rr, Rs, Rbest);
        }
    }
    *ncand += np;
    free(DA); free(pb); free(peaks); free(amps);
    return 0;
}

static void orc_coeffs_groups(const double *B, const double *A, int n, const int *perm,
                              const int *gsize, int ngroups, int L, double sigma, int cutoff,
                              double sign_a, double *ilmm) {
    int W = 2 * L + 1, off = 0;
    memset(ilmm, 0, sizeof(double) * 2 * (size_t)(L + 1) * W * W);
    for (int g = 0; g < ngroups; ++g) {
        int ns = gsize[g];
        double *pb = malloc(sizeof(double) * 3 * (ns ? ns : 1)), *pa = malloc(sizeof(double) * 3 * (ns ? ns : 1));
        for (int j = 0; j < ns; ++j)
            for (int k = 0; k < 3; ++k) {
                pb[3 * j + k] = B[3 * perm[off + j] + k];
                pa[3 * j + k] = sign_a * A[3 * perm[off + j] + k];
            }
        orc_cluster_coeffs(pb, pa, ns, L, sigma, cutoff, ilmm);
        free(pb); free(pa);
        off += ns;
    }
}

/* ALIGN (fastclusters.f90:129-269): centre both, coefficients per
 * permutation group, ALIGNCOEFFS, then (PERMINVOPT) the same for -A and keep
 * the smaller distance (non-inverted wins ties).                           */
int orc_cluster_align(const double *pos1, const double *pos2, int n,
                      const int *perm, const int *gsize, int ngroups,
                      int L, double sigma, int nrot, int invert, int cutoff,
                      double *aligned, int *permbest, orc_result *res) {
    memset(res, 0, sizeof *res);
    double *B = malloc(sizeof(double) * 3 * n), *A = malloc(sizeof(double) * 3 * n);
    memcpy(B, pos1, sizeof(double) * 3 * n);
    memcpy(A, pos2, sizeof(double) * 3 * n);
    if (sigma <= 0.0) sigma = orc_choose_kwidth(A, B, n);
    res->sigma = sigma;
    double ca[3] = {0, 0, 0}, cb[3] = {0, 0, 0};
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < 3; ++k) {
            ca[k] += A[3 * j + k];
            cb[k] += B[3 * j + k];
        }
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < 3; ++k) {
            A[3 * j + k] -= ca[k] / n;
            B[3 * j + k] -= cb[k] / n;
        }
    int W = 2 * L + 1;
    double *ilmm = malloc(sizeof(double) * 2 * (size_t)(L + 1) * W * W);
    orc_coeffs_groups(B, A, n, perm, gsize, ngroups, L, sigma, cutoff, 1.0, ilmm);
    double *al = malloc(sizeof(double) * 3 * n);
    int *pb = malloc(sizeof(int) * n);
    double Rb[9], dist, omax;
    int rc = orc_align_coeffs(B, A, n, perm, gsize, ngroups, L, ilmm, nrot, aligned, permbest,
                              res->rmat, &res->dist, &res->overlap_max, &res->ncand);
    if (rc == 0 && invert) {
        double *Ainv = malloc(sizeof(double) * 3 * n);
        for (int j = 0; j < 3 * n; ++j) Ainv[j] = -A[j];
        orc_coeffs_groups(B, A, n, perm, gsize, ngroups, L, sigma, cutoff, -1.0, ilmm);
        rc = orc_align_coeffs(B, Ainv, n, perm, gsize, ngroups, L, ilmm, nrot, al, pb, Rb, &dist,
                              &omax, &res->ncand);
        if (rc == 0 && dist < res->dist) {
            res->dist = dist;
            memcpy(aligned, al, sizeof(double) * 3 * n);
            memcpy(permbest, pb, sizeof(int) * n);
            memcpy(res->rmat, Rb, sizeof Rb);
            res->inverted = 1;
            res->overlap_max = omax;
        }
        free(Ainv);
    }
    res->status = rc;
    free(B); free(A); free(ilmm); free(al); free(pb);
    return rc;
}

/* ------------------------------------------------------------------------ */
/* Harmonic-oscillator basis (HARMONICNL fastclusters.f90:492-540): the
 * overlap integral of the Gaussian kernel at distance rj with the basis
 * function of order (i, j), by the recurrence in i that starts from the
 * closed form at i = 0.                                                    */
void orc_harmonic_nl(int nmax, int lmax, double rj, double sigma, double r0, double *ret) {
    const int w = lmax + 1;
    memset(ret, 0, sizeof(double) * (size_t)(nmax + 1) * w);
    double rs = 1.0 / (r0 * r0 + sigma * sigma);
    ret[0] = sqrt(2.0 * sqrt(ORC_PI) * pow(r0 * rs, 3)) * sigma * sigma * sigma * exp(-0.5 * rj * rj * rs) * 4 * ORC_PI;
    const double f = sqrt(2.0) * r0 * rj * rs;
    for (int j = 1; j <= lmax; ++j) ret[j] = f / sqrt(1.0 + 2.0 * j) * ret[j - 1];
    const double q = sigma * sigma / rj / r0;
    if (nmax >= 1)
        for (int j = 0; j <= lmax - 2; ++j)
            ret[w + j] = sqrt(1 + j + 0.5) * ret[j] - (2.0 * j + 3.0) * q * ret[j + 1] - sqrt(1 + j + 1.5) * ret[j + 2];
    for (int i = 2; i <= nmax; ++i) {
        const double si = sqrt((double)i);
        for (int j = 0; j <= lmax - 2 * i; ++j)
            ret[i * w + j] = (sqrt(i + j + 0.5) * ret[(i - 1) * w + j] - (2.0 * j + 3.0) * q * ret[(i - 1) * w + j + 1] -
                              sqrt(i + j + 1.5) * ret[(i - 1) * w + j + 2] + sqrt(i - 1.0) * ret[(i - 2) * w + j + 2]) / si;
    }
}

/* HARMONICCOEFFS (fastclusters.f90:654-687): c_nlm = sum_atoms d_nl conj(Y_lm),
 * d from HARMONICNL with lmax = L + 2 nmax.                                */
void orc_harmonic_coeffs(const double *X, int natoms, int nmax, int L, double hwidth,
                         double kwidth, double *cnml) {
    const int W = 2 * L + 1, lw = L + 2 * nmax + 1;
    memset(cnml, 0, sizeof(double) * 2 * (size_t)(nmax + 1) * (L + 1) * W);
    double *yr = malloc(sizeof(double) * (L + 1) * W), *yi = malloc(sizeof(double) * (L + 1) * W);
    double *d = malloc(sizeof(double) * (size_t)(nmax + 1) * lw);
    for (int k = 0; k < natoms; ++k) {
        const double *x = X + 3 * k;
        orc_ylm(x, L, yr, yi);
        orc_harmonic_nl(nmax, L + 2 * nmax, sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]), kwidth, hwidth, d);
        for (int l = 0; l <= L; ++l)
            for (int m = -l; m <= l; ++m) {
                const double ar = yr[l * W + L + m], ai = yi[l * W + L + m];
                const int im = (m + W) % W;
                for (int i = 0; i <= nmax; ++i) {
                    double *c = cnml + 2 * (((size_t)i * (L + 1) + l) * W + im);
                    c[0] += d[i * lw + l] * ar;
                    c[1] -= d[i * lw + l] * ai;
                }
            }
    }
    free(yr); free(yi); free(d);
}

/* DOTHARMONICCOEFFS (fastclusters.f90:740-759), added into the ilmm layout */
void orc_dot_harmonic(const double *c1, const double *c2, int nmax, int L, double *ilmm) {
    const int W = 2 * L + 1;
    for (int l = 0; l <= L; ++l)
        for (int m1 = -l; m1 <= l; ++m1)
            for (int m2 = -l; m2 <= l; ++m2) {
                const int i1 = (m1 + W) % W, i2 = (m2 + W) % W;
                double re = 0, im = 0;
                for (int i = 0; i <= nmax; ++i) {
                    const double *a = c1 + 2 * (((size_t)i * (L + 1) + l) * W + i1);
                    const double *b = c2 + 2 * (((size_t)i * (L + 1) + l) * W + i2);
                    re += a[0] * b[0] + a[1] * b[1];   /* conj(a) b */
                    im += a[0] * b[1] - a[1] * b[0];
                }
                double *o = ilmm + 2 * (((size_t)l * W + i1) * W + i2);
                o[0] += re;
                o[1] += im;
            }
}

/* IMML = sum over groups of DOTHARMONICCOEFFS(coefficients of B's group,
 * coefficients of sign_a * A's group); parity (-1)^l for the inversion is
 * the same as negating A.                                                  */
static void orc_harm_groups(const double *B, const double *A, int n, const int *perm, const int *gsize,
                            int ngroups, int nmax, int L, double hwidth, double kwidth, double sign_a,
                            double *ilmm) {
    const int W = 2 * L + 1;
    const size_t nc = 2 * (size_t)(nmax + 1) * (L + 1) * W;
    memset(ilmm, 0, sizeof(double) * 2 * (size_t)(L + 1) * W * W);
    double *cb = malloc(sizeof(double) * nc), *ca = malloc(sizeof(double) * nc);
    double *pb = malloc(sizeof(double) * 3 * (n ? n : 1)), *pa = malloc(sizeof(double) * 3 * (n ? n : 1));
    int off = 0;
    for (int g = 0; g < ngroups; ++g) {
        const int ns = gsize[g];
        for (int j = 0; j < ns; ++j)
            for (int k = 0; k < 3; ++k) {
                pb[3 * j + k] = B[3 * perm[off + j] + k];
                pa[3 * j + k] = A[3 * perm[off + j] + k];
            }
        orc_harmonic_coeffs(pb, ns, nmax, L, hwidth, kwidth, cb);
        orc_harmonic_coeffs(pa, ns, nmax, L, hwidth, kwidth, ca);
        if (sign_a < 0)
            for (int i = 0; i <= nmax; ++i)
                for (int l = 1; l <= L; l += 2)
                    for (int m = 0; m < 2 * W; ++m) ca[2 * (((size_t)i * (L + 1) + l) * W) + m] *= -1.0;
        orc_dot_harmonic(cb, ca, nmax, L, ilmm);
        off += ns;
    }
    free(cb); free(ca); free(pb); free(pa);
}

/* ALIGNHARM (fastclusters.f90:271-391) with ALIGN's coordinate handling (see
 * the header): coefficients of the coordinates as given, ALIGNCOEFFS, and
 * with invert the same for -A, the smaller distance winning (ties: the
 * non-inverted alignment).                                                 */
int orc_harm_align(const double *pos1, const double *pos2, int n, const int *perm, const int *gsize,
                   int ngroups, int nmax, int L, double hwidth, double kwidth, int nrot, int invert,
                   double *aligned, int *permbest, orc_result *res) {
    memset(res, 0, sizeof *res);
    res->sigma = kwidth;
    const int W = 2 * L + 1;
    double *ilmm = malloc(sizeof(double) * 2 * (size_t)(L + 1) * W * W);
    orc_harm_groups(pos1, pos2, n, perm, gsize, ngroups, nmax, L, hwidth, kwidth, 1.0, ilmm);
    double *al = malloc(sizeof(double) * 3 * n), *Ainv = malloc(sizeof(double) * 3 * n);
    int *pb = malloc(sizeof(int) * n);
    double Rb[9], dist, omax;
    int rc = orc_align_coeffs(pos1, pos2, n, perm, gsize, ngroups, L, ilmm, nrot, aligned, permbest, res->rmat,
                              &res->dist, &res->overlap_max, &res->ncand);
    if (rc == 0 && invert) {
        for (int j = 0; j < 3 * n; ++j) Ainv[j] = -pos2[j];
        orc_harm_groups(pos1, pos2, n, perm, gsize, ngroups, nmax, L, hwidth, kwidth, -1.0, ilmm);
        rc = orc_align_coeffs(pos1, Ainv, n, perm, gsize, ngroups, L, ilmm, nrot, al, pb, Rb, &dist, &omax,
                              &res->ncand);
        if (rc == 0 && dist < res->dist) {
            res->dist = dist;
            memcpy(aligned, al, sizeof(double) * 3 * n);
            memcpy(permbest, pb, sizeof(int) * n);
            memcpy(res->rmat, Rb, sizeof Rb);
            res->inverted = 1;
            res->overlap_max = omax;
        }
    }
    res->status = rc;
    free(ilmm); free(al); free(Ainv); free(pb);
    return rc;
}

/* CALCSIMILARITY (fastclusters.f90:790-815): IMML summed over the groups,
 * its squared norm, and the maximum of the overlap grid CALCOVERLAP forms. */
void orc_calc_similarity(const double *c1, const double *c2, int ngroups, int nmax, int L, double *norm,
                         double *maxover) {
    const int W = 2 * L + 1, G = 2 * (L + 1);
    const size_t nc = 2 * (size_t)(nmax + 1) * (L + 1) * W, ni = 2 * (size_t)(L + 1) * W * W;
    double *ilmm = calloc(ni, sizeof(double));
    for (int g = 0; g < ngroups; ++g) orc_dot_harmonic(c1 + g * nc, c2 + g * nc, nmax, L, ilmm);
    double s = 0;
    for (int l = 0; l <= L; ++l)
        for (int m1 = -l; m1 <= l; ++m1)
            for (int m2 = -l; m2 <= l; ++m2) {
                const double *o = ilmm + 2 * (((size_t)l * W + (m1 + W) % W) * W + (m2 + W) % W);
                s += o[0] * o[0] + o[1] * o[1];
            }
    *norm = s;
    double *grid = malloc(sizeof(double) * (size_t)G * G * G);
    orc_isoft(L + 1, ilmm, grid);
    double mx = grid[0];
    for (size_t i = 1; i < (size_t)G * G * G; ++i)
        if (grid[i] > mx) mx = grid[i];
    *maxover = mx;
    free(grid); free(ilmm);
}

/* ------------------------------------------------------------------------ */
/* Branch and bound over rotations (the upstream Python BranchandBoundMaster
 * with BranchNodeCluster, fastoverlap/bnbAlignment.py:23-104,204-277): nodes
 * are cubes of angle-axis vectors; a node's lower bound is the assignment
 * over the smallest squared distances any rotation in the cube can reach
 * (angular bound on the atom-pair angle), its upper bound the assignment
 * distance at the cube's centre.  Best-first by lower bound until the lower
 * bound is within rtol * best + atol of the best upper bound.              */

/* Dense linear assignment on double costs (shortest augmenting paths with
 * row and column potentials, Jonker & Volgenant 1987): col[i] = column of
 * row i; returns the optimal cost.                                          */
static double orc_lap_dense(int n, const double *c, int *col) {
    double *u = calloc(n + 1, sizeof(double)), *v = calloc(n + 1, sizeof(double));
    double *minv = malloc(sizeof(double) * (n + 1));
    int *p = calloc(n + 1, sizeof(int)), *way = calloc(n + 1, sizeof(int));
    char *used = malloc(n + 1);
    for (int i = 1; i <= n; ++i) {   /* 1-based, column 0 is the virtual start */
        p[0] = i;
        int j0 = 0;
        for (int j = 0; j <= n; ++j) { minv[j] = HUGE_VAL; used[j] = 0; }
        do {
            used[j0] = 1;
            const int i0 = p[j0];
            double delta = HUGE_VAL;
            int j1 = 0;
            for (int j = 1; j <= n; ++j)
                if (!used[j]) {
                    const double cur = c[(size_t)(i0 - 1) * n + (j - 1)] - u[i0] - v[j];
                    if (cur < minv[j]) { minv[j] = cur; way[j] = j0; }
                    if (minv[j] < delta) { delta = minv[j]; j1 = j; }
                }
            for (int j = 0; j <= n; ++j)
                if (used[j]) { u[p[j]] += delta; v[j] -= delta; }
                else minv[j] -= delta;
            j0 = j1;
        } while (p[j0] != 0);
        do {
            const int j1 = way[j0];
            p[j0] = p[j1];
            j0 = j1;
        } while (j0);
    }
    double tot = 0;
    for (int j = 1; j <= n; ++j) {
        col[p[j] - 1] = j - 1;
        tot += c[(size_t)(p[j] - 1) * n + (j - 1)];
    }
    free(u); free(v); free(minv); free(p); free(way); free(used);
    return tot;
}

/* angle-axis vector -> rotation matrix (row-major), Rodrigues' formula    */
static void orc_angle_axis(const double w[3], double M[9]) {
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

typedef struct {
    double rot[3], width, lower, upper;
    int sign;        /* +1: pos2, -1: the inverted pos2 */
    int id;
} orc_bnb_node;

/* binary min-heap on (lower) with the sift rules of Python's heapq: a push
 * sifts the new item up past strictly larger parents; a pop moves the last
 * item to the root, walks it down to a leaf along the smaller child (the
 * right one only when strictly smaller) and then sifts it up.            */
typedef struct { orc_bnb_node *a; int n, cap; } orc_heap;
static void heap_up(orc_heap *h, int start, int pos) {
    orc_bnb_node it = h->a[pos];
    while (pos > start) {
        const int par = (pos - 1) >> 1;
        if (it.lower < h->a[par].lower) { h->a[pos] = h->a[par]; pos = par; }
        else break;
    }
    h->a[pos] = it;
}
static void heap_push(orc_heap *h, orc_bnb_node x) {
    if (h->n == h->cap) { h->cap = h->cap ? 2 * h->cap : 64; h->a = realloc(h->a, sizeof(orc_bnb_node) * h->cap); }
    h->a[h->n++] = x;
    heap_up(h, 0, h->n - 1);
}
static orc_bnb_node heap_pop(orc_heap *h) {
    orc_bnb_node last = h->a[--h->n];
    if (h->n == 0) return last;
    orc_bnb_node top = h->a[0];
    h->a[0] = last;
    int pos = 0;
    const int end = h->n;
    orc_bnb_node it = h->a[0];
    int child = 1;
    while (child < end) {
        const int right = child + 1;
        if (right < end && !(h->a[child].lower < h->a[right].lower)) child = right;
        h->a[pos] = h->a[child];
        pos = child;
        child = 2 * pos + 1;
    }
    h->a[pos] = it;
    heap_up(h, 0, pos);
    return top;
}

typedef struct {
    int n;
    const double *X1, *X2;      /* centred pos1, centred pos2 */
    double *r1, *r2, *d2, *lb, *rp;
    int *col;
} orc_bnb_ws;

/* BranchNodeCluster.calcbounds (bnbAlignment.py:232-277) */
static void orc_bnb_bounds(orc_bnb_ws *w, orc_bnb_node *nd, double bestupper, int force, double *rpos_out) {
    const int n = w->n;
    double M[9];
    orc_angle_axis(nd->rot, M);
    double *rp = w->rp;
    for (int j = 0; j < n; ++j)   /* rpos2 = (sign * pos2) . M, row vectors */
        for (int c = 0; c < 3; ++c)
            rp[3 * j + c] = nd->sign * (w->X2[3 * j] * M[c] + w->X2[3 * j + 1] * M[3 + c] + w->X2[3 * j + 2] * M[6 + c]);
    if (rpos_out) memcpy(rpos_out, rp, sizeof(double) * 3 * n);
    const double theta = fmin(sqrt(3.0) * nd->width / 2, ORC_PI), cosd = cos(theta), sind = fabs(sin(theta));
    double upper = 0.0;
    if (!force) {   /* nearest atom of pos1 to each rotated pos2 atom */
        double s = 0.0;
        for (int j = 0; j < n; ++j) {
            double best = HUGE_VAL;
            int bi = 0;
            for (int i = 0; i < n; ++i) {
                double t = 0;
                for (int c = 0; c < 3; ++c) {
                    const double e = w->X1[3 * i + c] - rp[3 * j + c];
                    t += e * e;
                }
                if (t < best) { best = t; bi = i; }
            }
            w->col[j] = bi;
            w->lb[j] = best;
            s += best;
        }
        upper = sqrt(s);
    }
    if (force || upper < bestupper) {
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                double t = 0;
                for (int c = 0; c < 3; ++c) {
                    const double e = w->X1[3 * i + c] - rp[3 * j + c];
                    t += e * e;
                }
                const double rr = w->r1[i] * w->r2[j], rs = w->r1[i] * w->r1[i] + w->r2[j] * w->r2[j];
                const double cosa = 0.5 * (rs - t) / rr, sina = sqrt(fmin(fmax(1.0 - cosa * cosa, 0.0), 1.0));
                const double cdm = (cosa > cosd) ? 1.0 : cosa * cosd + sina * sind;
                w->d2[(size_t)i * n + j] = t;
                w->lb[(size_t)i * n + j] = fmax(rs - 2 * rr * cdm, 0.0);
            }
        nd->lower = sqrt(orc_lap_dense(n, w->lb, w->col));
        if (nd->lower < bestupper) {
            orc_lap_dense(n, w->d2, w->col);
            double s = 0;
            for (int i = 0; i < n; ++i)
                for (int c = 0; c < 3; ++c) {
                    const double e = w->X1[3 * i + c] - rp[3 * w->col[i] + c];
                    s += e * e;
                }
            nd->upper = sqrt(s);
        } else {
            nd->upper = HUGE_VAL;
        }
    } else {   /* quick bounds from the nearest neighbours */
        double s = 0;
        for (int j = 0; j < n; ++j) {
            const double r1 = w->r1[w->col[j]], r2 = w->r2[j], dd = w->lb[j];
            const double cosa = 0.5 * (r1 * r1 + r2 * r2 - dd) / r1 / r2;
            const double sina = sqrt(fmin(fmax(1.0 - cosa * cosa, 0.0), 1.0));
            const double cdm = (cosa > cosd) ? 1.0 : cosa * cosd + sina * sind;
            s += fmax(r1 * r1 + r2 * r2 - 2 * r1 * r2 * cdm, 0.0);
        }
        nd->lower = sqrt(s);
        nd->upper = upper;
    }
}

int orc_bnb_cluster(const double *pos1, const double *pos2, int n, int invert, long long niter, double rtol,
                    double atol, double *dist, double *aligned, long long *nodes_out) {
    double *X1 = malloc(sizeof(double) * 3 * n), *X2 = malloc(sizeof(double) * 3 * n);
    double c1[3] = {0, 0, 0}, c2[3] = {0, 0, 0};
    for (int j = 0; j < n; ++j)
        for (int c = 0; c < 3; ++c) { c1[c] += pos1[3 * j + c]; c2[c] += pos2[3 * j + c]; }
    for (int c = 0; c < 3; ++c) { c1[c] /= n; c2[c] /= n; }
    for (int j = 0; j < n; ++j)
        for (int c = 0; c < 3; ++c) { X1[3 * j + c] = pos1[3 * j + c] - c1[c]; X2[3 * j + c] = pos2[3 * j + c] - c2[c]; }
    orc_bnb_ws w;
    w.n = n; w.X1 = X1; w.X2 = X2;
    w.r1 = malloc(sizeof(double) * n); w.r2 = malloc(sizeof(double) * n);
    w.d2 = malloc(sizeof(double) * n * n); w.lb = malloc(sizeof(double) * n * n);
    w.rp = malloc(sizeof(double) * 3 * n); w.col = malloc(sizeof(int) * n);
    for (int j = 0; j < n; ++j) {
        w.r1[j] = sqrt(X1[3 * j] * X1[3 * j] + X1[3 * j + 1] * X1[3 * j + 1] + X1[3 * j + 2] * X1[3 * j + 2]);
        w.r2[j] = sqrt(X2[3 * j] * X2[3 * j] + X2[3 * j + 1] * X2[3 * j + 1] + X2[3 * j + 2] * X2[3 * j + 2]);
    }
    orc_heap h = {NULL, 0, 0};
    orc_bnb_node start[2];
    int nstart = invert ? 2 : 1;
    for (int k = 0; k < nstart; ++k) {
        orc_bnb_node s0 = {{0, 0, 0}, 2 * ORC_PI, 0, 0, k ? -1 : 1, k};
        orc_bnb_bounds(&w, &s0, HUGE_VAL, 1, NULL);
        start[k] = s0;
    }
    orc_bnb_node best = start[0];
    heap_push(&h, start[0]);
    for (int k = 1; k < nstart; ++k) {
        if (start[k].upper < best.upper) best = start[k];
        if (start[k].lower < best.upper) heap_push(&h, start[k]);
    }
    long long nodes = 0;
    int next_id = nstart;
    while (h.n > 0) {
        orc_bnb_node nd = heap_pop(&h);
        ++nodes;
        if (nd.lower < best.upper - rtol * best.upper - atol) {
            for (int a = 0; a < 2; ++a)       /* children in numpy.indices order */
                for (int b = 0; b < 2; ++b)
                    for (int c = 0; c < 2; ++c) {
                        orc_bnb_node ch = nd;
                        const double q = 0.25 * nd.width;
                        ch.rot[0] = (2 * a - 1) * q + nd.rot[0];
                        ch.rot[1] = (2 * b - 1) * q + nd.rot[1];
                        ch.rot[2] = (2 * c - 1) * q + nd.rot[2];
                        ch.width = 0.5 * nd.width;
                        ch.id = next_id++;
                        orc_bnb_bounds(&w, &ch, best.upper, 0, NULL);
                        if (ch.lower < best.upper) {
                            if (ch.upper < best.upper) best = ch;
                            heap_push(&h, ch);
                        }
                    }
            if (nodes > niter) break;
        }
    }
    *dist = best.upper;
    if (aligned) {   /* best node's rotated pos2, moved onto pos1's centroid */
        orc_bnb_bounds(&w, &best, HUGE_VAL, 1, aligned);
        for (int j = 0; j < n; ++j)
            for (int c = 0; c < 3; ++c) aligned[3 * j + c] += c1[c];
    }
    if (nodes_out) *nodes_out = nodes;
    free(h.a); free(X1); free(X2); free(w.r1); free(w.r2); free(w.d2); free(w.lb); free(w.rp); free(w.col);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* SETWAVEK / PERIODICFOURIERPERM / damping / DOTFOURIERCOEFFS / FFT3D / ABS
 * (fastbulk.f90:414-454,522-523,567-683; fastutils.f90:554-569):
 *   F(k) = sum_s C^B_s(k) conj(C^A_s(k)) exp(-k^2 s^2),
 *   C_s(k) = sum_{j in s} exp(-i k.r_j), k = 2 pi/L (i - K), i = 0..2K,
 * placed at the low corner of an nf^3 array, forward 3-D DFT, modulus.
 * fspace is stored x fastest.                                              */
void orc_bulk_fspace(const double *B, const double *A, int n, const int *perm,
                     const int *gsize, int ngroups, const double box[3],
                     double sigma, int nwave, int nf, double *fspace) {
    int K = nwave, nk = 2 * K + 1;
    size_t N3 = (size_t)nf * nf * nf;
    double *F = calloc(2 * N3, sizeof(double));
    double *ca = malloc(sizeof(double) * 2 * nk * nk * nk), *cbv = malloc(sizeof(double) * 2 * nk * nk * nk);
    int off = 0;
    for (int g = 0; g < ngroups; ++g) {
        int ns = gsize[g];
        memset(ca, 0, sizeof(double) * 2 * nk * nk * nk);
        memset(cbv, 0, sizeof(double) * 2 * nk * nk * nk);
        for (int ix = 0; ix < nk; ++ix)
            for (int iy = 0; iy < nk; ++iy)
                for (int iz = 0; iz < nk; ++iz) {
                    double kx = 2 * ORC_PI / box[0] * (ix - K), ky = 2 * ORC_PI / box[1] * (iy - K),
                           kz = 2 * ORC_PI / box[2] * (iz - K);
                    size_t o = 2 * (ix + (size_t)nk * (iy + (size_t)nk * iz));
                    for (int j = 0; j < ns; ++j) {
                        const double *a = A + 3 * perm[off + j], *b = B + 3 * perm[off + j];
                        double kra = kx * a[0] + ky * a[1] + kz * a[2];
                        double krb = kx * b[0] + ky * b[1] + kz * b[2];
                        ca[o] += cos(kra);
                        ca[o + 1] -= sin(kra);
                        cbv[o] += cos(krb);
                        cbv[o + 1] -= sin(krb);
                    }
                }
        for (int ix = 0; ix < nk; ++ix)
            for (int iy = 0; iy < nk; ++iy)
                for (int iz = 0; iz < nk; ++iz) {
                    double kx = 2 * ORC_PI / box[0] * (ix - K), ky = 2 * ORC_PI / box[1] * (iy - K),
                           kz = 2 * ORC_PI / box[2] * (iz - K);
                    double damp = exp(-0.5 * (kx * kx + ky * ky + kz * kz) * sigma * sigma);
                    size_t o = 2 * (ix + (size_t)nk * (iy + (size_t)nk * iz));
                    double br = cbv[o] * damp, bi = cbv[o + 1] * damp;
                    double ar = ca[o] * damp, ai = -ca[o + 1] * damp; /* conj */
                    size_t q = 2 * (ix + (size_t)nf * (iy + (size_t)nf * iz));
                    F[q] += br * ar - bi * ai;
                    F[q + 1] += br * ai + bi * ar;
                }
        off += ns;
    }
    double *line = malloc(sizeof(double) * 2 * nf);
    for (int ax = 0; ax < 3; ++ax) {
        size_t st = ax == 0 ? 1 : (ax == 1 ? (size_t)nf : (size_t)nf * nf);
        for (int u = 0; u < nf; ++u)
            for (int w = 0; w < nf; ++w) {
                size_t base;
                if (ax == 0) base = (size_t)nf * (u + (size_t)nf * w);
                else if (ax == 1) base = u + (size_t)nf * nf * w;
                else base = u + (size_t)nf * w;
                for (int t = 0; t < nf; ++t) {
                    line[2 * t] = F[2 * (base + st * t)];
                    line[2 * t + 1] = F[2 * (base + st * t) + 1];
                }
                orc_fft1d(nf, line, -1);
                for (int t = 0; t < nf; ++t) {
                    F[2 * (base + st * t)] = line[2 * t];
                    F[2 * (base + st * t) + 1] = line[2 * t + 1];
                }
            }
    }
    for (size_t i = 0; i < N3; ++i) fspace[i] = sqrt(F[2 * i] * F[2 * i] + F[2 * i + 1] * F[2 * i + 1]);
    free(line); free(F); free(ca); free(cbv);
}

/* ALIGN / ALIGN1 / ALIGNCOEFFS (bulk, fastbulk.f90:279-334,414-565):
 * defaults NWAVE = ceil(1.3 N^{1/3}), NFSPACE = FASTLEN(4 NWAVE + 3),
 * width (V/N)^{1/3}/3, 10 displacements; peaks -> displacements
 * (peak - 1) L / NFSPACE; ITERATIVEALIGN (bulk) from A - disp for each;
 * keep the smallest distance.                                              */
int orc_bulk_align(const double *pos1, const double *pos2, int n,
                   const int *perm, const int *gsize, int ngroups,
                   const double box[3], double sigma, int nwave, int nfspace,
                   int ndisps, double *aligned, int *permbest, orc_result *res) {
    memset(res, 0, sizeof *res);
    if (sigma <= 0.0) sigma = cbrt(box[0] * box[1] * box[2] / n) / 3.0;
    if (nwave <= 0) nwave = (int)ceil(1.3 * cbrt((double)n));
    if (nfspace <= 0) nfspace = orc_fastlen(4 * nwave + 3);
    if (ndisps <= 0) ndisps = 10;
    res->sigma = sigma;
    size_t N3 = (size_t)nfspace * nfspace * nfspace;
    double *fs = malloc(sizeof(double) * N3);
    orc_bulk_fspace(pos1, pos2, n, perm, gsize, ngroups, box, sigma, nwave, nfspace, fs);
    double mx = fs[0];
    for (size_t i = 0; i < N3; ++i)
        if (fs[i] > mx) mx = fs[i];
    res->overlap_max = mx;
    double *peaks = malloc(sizeof(double) * 3 * ndisps), *amps = malloc(sizeof(double) * ndisps);
    int np = orc_findpeaks(fs, nfspace, nfspace, nfspace, ndisps, peaks, amps);
    free(fs);
    if (np < 0) {
        free(peaks); free(amps);
        res->status = -2;
        return -2;
    }
    double *DA = malloc(sizeof(double) * 3 * n);
    int *pb = malloc(sizeof(int) * n);
    res->dist = HUGE_VAL;
    for (int c = 0; c < np; ++c) {
        double d0[3];
        for (int k = 0; k < 3; ++k) d0[k] = (peaks[3 * c + k] - 1.0) * box[k] / nfspace;
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < 3; ++k) DA[3 * j + k] = pos2[3 * j + k] - d0[k];
        double db[3];
        double d = orc_iterative_align(pos1, DA, n, perm, gsize, ngroups, 1, box, NULL, db, pb, NULL);
        if (d < res->dist) {
            res->dist = d;
            memcpy(aligned, DA, sizeof(double) * 3 * n);
            memcpy(permbest, pb, sizeof(int) * n);
            for (int k = 0; k < 3; ++k) res->disp[k] = db[k] - d0[k];
        }
    }
    res->ncand = np;
    res->rmat[0] = res->rmat[4] = res->rmat[8] = 1.0;
    free(DA); free(pb); free(peaks); free(amps);
    return 0;
}

/* ------------------------------------------------------------------------ */
typedef struct {
    int npairs, next, nrot, invert, cutoff;
    const double *pos1, *pos2, *sigma;
    const int64_t *coord_off, *perm_off;
    const int *natoms, *perm, *gsize, *gsize_off, *ngroups, *L;
    double *dist;
    int *perm_out;   /* optional: permutations at atom offset coord_off / 3 */
    pthread_mutex_t mu;
} orc_many_job;

static void *orc_many_worker(void *arg) {
    orc_many_job *J = (orc_many_job *)arg;
    for (;;) {
        pthread_mutex_lock(&J->mu);
        int p = J->next++;
        pthread_mutex_unlock(&J->mu);
        if (p >= J->npairs) break;
        int n = J->natoms[p];
        double *al = malloc(sizeof(double) * 3 * n);
        int *pb = malloc(sizeof(int) * n);
        orc_result r;
        orc_cluster_align(J->pos1 + J->coord_off[p], J->pos2 + J->coord_off[p], n,
                          J->perm + J->perm_off[p], J->gsize + J->gsize_off[p], J->ngroups[p],
                          J->L[p], J->sigma[p], J->nrot, J->invert, J->cutoff, al, pb, &r);
        J->dist[p] = r.dist;
        if (J->perm_out) memcpy(J->perm_out + J->coord_off[p] / 3, pb, sizeof(int) * n);
        free(al);
        free(pb);
    }
    return NULL;
}

int orc_cluster_align_many(int npairs, const double *pos1, const double *pos2,
                           const int64_t *coord_off, const int *natoms,
                           const int *perm, const int64_t *perm_off,
                           const int *gsize, const int *gsize_off,
                           const int *ngroups, const int *L,
                           const double *sigma, int nrot, int invert,
                           int cutoff, int nthreads, double *dist_out, int *perm_out) {
    orc_many_job J = {npairs, 0, nrot, invert, cutoff, pos1, pos2, sigma, coord_off, perm_off,
                      natoms, perm, gsize, gsize_off, ngroups, L, dist_out, perm_out};
    pthread_mutex_init(&J.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = malloc(sizeof(pthread_t) * nthreads);
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, orc_many_worker, &J);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&J.mu);
    return 0;
}
