/*
 * fo_oracle.h -- CPU FP64 restatement of the FASTOVERLAP alignment path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * CUDA library in fastoverlap_gb300/.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg may load it; the product never calls it.
 *
 * It restates, in plain sequential C, the Fortran cluster and bulk pipelines
 * of the upstream project (fastoverlap/f90/fastclusters.f90, fastbulk.f90,
 * DSOFT.f90, fastutils.f90, alignutils.f90).  Each function below names the
 * upstream routine (path:line) it follows.  Parity is pinned by the upstream
 * known answers (LJ38 -> 1.4767, BLJ256 -> 1.559) and by fixtures produced
 * from the upstream Python path (tests/golden/make_golden.py).
 *
 * Conventions (shared with the CUDA library):
 *   coordinates  : flat xyz, atom-major, double[3*n]
 *   groups       : permutation groups ("species"): perm[] holds 0-based atom
 *                  indices, group g owns perm[off_g .. off_g+size_g)
 *   coefficients : "ilmm" layout [l][m1 mod (2L+1)][m2 mod (2L+1)], complex
 *                  as interleaved (re, im) pairs, L = Jmax.  m1 indexes the
 *                  target structure (pos1 / COORDSB), m2 the moved one.
 *   SO(3) grid   : G = 2(L+1) per axis, stored alpha fastest:
 *                  grid[a + G*(b + G*g)]  (Fortran OUTPUT(alpha,beta,gamma))
 *   rotation     : row-major R, aligned_a = R * a (column-vector convention)
 *   permutation  : 0-based, aligned atom j of A came from original atom perm[j]
 */
#ifndef FO_ORACLE_H
#define FO_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double dist;        /* best Euclidean distance after alignment          */
    double rmat[9];     /* best rotation (cluster), row-major               */
    double disp[3];     /* best displacement (bulk): aligned = a + disp      */
    int    inverted;    /* 1 if the inverted copy of A aligned best         */
    int    ncand;       /* candidates refined (all orientations)            */
    int    status;      /* 0 ok, <0 error                                   */
    double sigma;       /* Gaussian width actually used                     */
    double overlap_max; /* max of the overlap grid of the winning orientation */
} orc_result;

/* ---- special functions ---- */
int    orc_fastlen(int n);                      /* smallest 2^a3^b5^c >= n   */
void   orc_ylm(const double xyz[3], int L, double *re, double *im);
void   orc_sphi(int L, double x, double *out);  /* i_l(x), l = 0..L          */

/* ---- spherical (cluster) stages ---- */
double orc_choose_kwidth(const double *A, const double *B, int n);
void   orc_cluster_coeffs(const double *B, const double *A, int n, int L,
                          double sigma, int cutoff, double *ilmm /*2*(L+1)(2L+1)^2*/);
void   orc_wigner_d(int bw, double *d /* bw*(2bw-1)^2*(2bw) */);
void   orc_isoft(int bw, const double *ilmm, double *grid_re /* (2bw)^3 */);
int    orc_findpeaks(const double *grid, int n1, int n2, int n3, int npeaks,
                     double *peaks /* npeaks*3, 1-based fractional */,
                     double *amps);
int    orc_findpeaks_w(const double *grid, int n1, int n2, int n3, int npeaks, int width0,
                       double *peaks, double *amps);
void   orc_eulerm(double a, double b, double g, double R[9]);

/* ---- refinement ---- */
int    orc_jv(int n, const int64_t *cc, const int *kk, const int *first,
              int *x /* col of row */, int *y /* row of col */);
void   orc_pairdists(int n, const double *p, const double *q, int bulk,
                     const double box[3], int maxnei, double *cc, int *kk);
double orc_findrotation(const double *B, const double *A, int n, double R[9]);
double orc_iterative_align(const double *B, double *A, int n, const int *perm,
                           const int *gsize, int ngroups, int bulk,
                           const double box[3], double R[9], double disp[3],
                           int *permbest, int *niter);

/* ---- full pipelines ---- */
int    orc_cluster_align(const double *pos1, const double *pos2, int n,
                         const int *perm, const int *gsize, int ngroups,
                         int L, double sigma, int nrot, int invert, int cutoff,
                         double *aligned /*3n*/, int *permbest, orc_result *res);
void   orc_bulk_fspace(const double *B, const double *A, int n, const int *perm,
                       const int *gsize, int ngroups, const double box[3],
                       double sigma, int nwave, int nf, double *fspace /* nf^3 */);
int    orc_bulk_align(const double *pos1, const double *pos2, int n,
                      const int *perm, const int *gsize, int ngroups,
                      const double box[3], double sigma, int nwave, int nfspace,
                      int ndisps, double *aligned, int *permbest, orc_result *res);

/* Harmonic-oscillator basis (the SphericalHarmonicAlignFortran path).
 * HARMONICNL fastoverlap/f90/fastclusters.f90:492-540: ret[i*(lmax+1)+j],
 * i <= nmax, j <= lmax - 2i (j <= lmax - 2 for i = 1).                    */
void   orc_harmonic_nl(int nmax, int lmax, double rj, double sigma, double r0, double *ret);
/* HARMONICCOEFFS :654-687 (coordinates as given, not centred):
 * cnml[((n*(L+1) + l)*W + m mod W)] complex interleaved, W = 2L+1.        */
void   orc_harmonic_coeffs(const double *X, int natoms, int nmax, int L, double hwidth,
                           double kwidth, double *cnml);
/* DOTHARMONICCOEFFS :740-759 added into ilmm:
 * IMML(m1,m2,l) += sum_n conj(c1(n,m1,l)) c2(n,m2,l).                     */
void   orc_dot_harmonic(const double *c1, const double *c2, int nmax, int L, double *ilmm);
/* ALIGNHARM :271-391: per-group harmonic coefficients of the coordinates
 * as given, ALIGNCOEFFS, then (invert) the same for -A.  The refinement
 * takes the coordinates in their own order and the inverted winner keeps
 * its own rotation, as ALIGN does (ALIGNHARM leaves its per-group copies
 * in place and returns the non-inverted rotation; the two agree for one
 * permutation group in index order and for non-inverted winners).         */
int    orc_harm_align(const double *pos1, const double *pos2, int n,
                      const int *perm, const int *gsize, int ngroups, int nmax, int L,
                      double hwidth, double kwidth, int nrot, int invert,
                      double *aligned, int *permbest, orc_result *res);
/* CALCSIMILARITY :790-815 over stacked per-group coefficients
 * c[g][n][l][m]: norm = sum |IMML|^2, maxover = max of the overlap grid.    */
void   orc_calc_similarity(const double *c1, const double *c2, int ngroups, int nmax, int L,
                           double *norm, double *maxover);

/* Branch and bound over rotations (the upstream Python BranchandBoundMaster,
 * fastoverlap/bnbAlignment.py:23-104,204-277): both structures centred,
 * best-first search over angle-axis cubes (start width 2 pi, 8 children of
 * half width) ordered by the lower bound, until the lower bound is within
 * rtol * best + atol of the best upper bound or `niter` nodes; invert also
 * starts from -pos2.  dist: the best upper bound; aligned (optional): that
 * node's rotated pos2 on pos1's centroid, in pos2's order (as upstream). */
int    orc_bnb_cluster(const double *pos1, const double *pos2, int n, int invert, long long niter,
                       double rtol, double atol, double *dist, double *aligned, long long *nodes);

/* batch helper for the CPU baseline and the tests: runs pairs on nthreads OS
 * threads; perm_out (optional, NULL for none) receives each pair's best
 * permutation at atom offset coord_off / 3 */
int    orc_cluster_align_many(int npairs, const double *pos1, const double *pos2,
                              const int64_t *coord_off, const int *natoms,
                              const int *perm, const int64_t *perm_off,
                              const int *gsize, const int *gsize_off,
                              const int *ngroups, const int *L,
                              const double *sigma, int nrot, int invert,
                              int cutoff, int nthreads, double *dist_out, int *perm_out);

#ifdef __cplusplus
}
#endif
#endif
