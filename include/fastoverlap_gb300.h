/*
 * fastoverlap_gb300.h -- C ABI of the GB300 (sm_103a) FASTOVERLAP alignment
 * library (libfastoverlap_gb300.so).
 *
 * Plain C types only: host pointers, sizes, POD structs.  Every call returns
 * an fo_status and never exits the process.  All coordinates are flat
 * (x, y, z) per atom in float64.  Permutation groups ("species") are given as
 * a concatenated list of atom indices plus the size of each group, as the
 * upstream Fortran takes them (fastoverlaputils.setperm); the index base is a
 * parameter so Fortran callers can pass their 1-based PERMGROUP unchanged.
 *
 * Upstream interfaces replaced (paths inside matthewghgriffiths/fastoverlap):
 *   fo_setperm             <- SETPERM            fastoverlap/f90/fastutils.f90:117-167
 *   fo_cluster_align       <- CLUSTERFASTOVERLAP::ALIGN  fastoverlap/f90/fastclusters.f90:129-269
 *                             (f2py clusterfastoverlap.align, sphericalAlignment.py:531-532)
 *   fo_bulk_align          <- BULKFASTOVERLAP::ALIGN      fastoverlap/f90/fastbulk.f90:279-334
 *                             and ALIGN1 (:414-499) when nwave/nfspace are given
 *                             (f2py bulkfastoverlap.align, periodicAlignment.py:562-565)
 *   fo_bulk_calcdefaults   <- BULKFASTOVERLAP::CALCDEFAULTS fastoverlap/f90/fastbulk.f90:253-277
 *   fo_cluster_align_harm  <- CLUSTERFASTOVERLAP::ALIGNHARM fastoverlap/f90/fastclusters.f90:271-391
 *                             (f2py clusterfastoverlap.alignharm, sphericalAlignment.py:617)
 *   fo_calc_overlap_matrices <- CLUSTERFASTOVERLAP::CALCOVERLAPMATRICES
 *                             fastoverlap/f90/fastclusters.f90:846-866 (compareList, :622-663)
 *   fo_cluster_harm_*      <- the same harmonic-basis alignment for many pairs
 *   fo_bnb_cluster(_batch) <- BranchandBoundMaster (branch and bound over rotations),
 *                             fastoverlap/bnbAlignment.py:23-104,204-277
 *   fo_bulk_align_group    <- BULKFASTOVERLAP::ALIGNGROUP fastoverlap/f90/fastbulk.f90:336-412
 *                             (f2py bulkfastoverlap.aligngroup, periodicAlignment.py:570-605)
 *   fo_cluster_align_batch <- SphericalAlign.__call__ / SphericalAlignFortran.__call__
 *                             applied to many pairs (sphericalAlignment.py:237-247,491-533)
 *   fo_bulk_align_batch    <- PeriodicAlignFortran.align applied to many pairs
 *                             (periodicAlignment.py:526-568)
 *   flags in fo_cluster_pair/fo_bulk_pair replace the COMMONS globals
 *   PERMINVOPT / OHCELLT (fastoverlap/f90/commons.f90:375-380)
 */
#ifndef FASTOVERLAP_GB300_H
#define FASTOVERLAP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    FO_OK = 0,
    FO_ERR_BAD_ARGS = 1,      /* invalid sizes, groups, widths ...           */
    FO_ERR_NO_PEAKS = 2,      /* peak search found nothing (upstream: STOP)  */
    FO_ERR_LAP_FAILED = 3,    /* assignment failed for some atoms            */
    FO_ERR_TIMEOUT = 4,       /* a bounded device wait gave up               */
    FO_ERR_OOM_BUDGET = 5,    /* request does not fit the HBM budget         */
    FO_ERR_CUDA = 6,          /* CUDA runtime error (see fo_last_error)      */
    FO_ERR_UNIMPLEMENTED = 7,
    FO_ERR_QUEUE_FULL = 8,    /* serving queue full                          */
    FO_ERR_NOT_READY = 9      /* serving request still in flight             */
} fo_status;

typedef enum {
    FO_PREC_FP64 = 0,   /* plain form: every stage in FP64                     */
    FO_PREC_MIXED = 1   /* coefficients, SO(3)/translation grids and peak fits
                           in FP32; Wigner-d generation, Kabsch and distances
                           in FP64; assignment integer                         */
} fo_precision;

typedef struct fo_ctx fo_ctx;

typedef struct {
    int    device;            /* CUDA device ordinal                          */
    int    precision;         /* fo_precision                                 */
    size_t hbm_budget_bytes;  /* admission budget for batches / serving; 0 = 80% of free */
    int    cutoff;            /* 1: skip atom pairs with |r_a - r_b| >= 4 sigma
                                 (fastclusters.f90:901); 0: full pair sum as in
                                 sphericalAlignment.py:260-273                 */
    int    profile;           /* 1: record per-kernel CUDA-event times        */
} fo_opts;

/* per-pair description for the spherical (cluster) batch */
typedef struct {
    int     natoms;      /* atoms in each structure                           */
    int     ngroups;     /* permutation groups                                */
    int     jmax;        /* L: SO(3) bandwidth L+1, grid 2(L+1) per axis      */
    int     nrot;        /* candidate rotations per orientation (peaks)       */
    int     invert;      /* 1: also align the inverted copy (PERMINVOPT)      */
    int     reserved;
    double  sigma;       /* Gaussian width; <= 0 picks CHOOSE_KWIDTH's value  */
    int64_t coord_off;   /* first atom of this pair in the packed coordinates */
    int64_t perm_off;    /* first entry in the packed permutation list        */
    int64_t group_off;   /* first entry in the packed group-size list         */
} fo_cluster_pair;

/* per-pair description for the periodic (bulk) batch */
typedef struct {
    int     natoms;
    int     ngroups;
    int     nwave;       /* K: (2K+1)^3 wave vectors; <= 0 -> ceil(1.3 N^1/3) */
    int     nfspace;     /* M: M^3 translation grid; <= 0 -> FASTLEN(4K+3)    */
    int     ndisps;      /* candidate displacements; <= 0 -> 10               */
    int     ohcell;      /* 1: also the 48 cubic-cell operations (OHCELLT)    */
    double  sigma;       /* <= 0 -> (V/N)^(1/3)/3                             */
    double  box[3];      /* orthorhombic box lengths                          */
    int64_t coord_off;
    int64_t perm_off;
    int64_t group_off;
} fo_bulk_pair;

/* per-pair result of either batch */
typedef struct {
    double dist;         /* aligned Euclidean distance (RMSD * sqrt(N))       */
    double rmat[9];      /* row-major R: aligned = R * (+/-)centred pos2      */
    double disp[3];      /* bulk: aligned = pos2[perm] + disp                 */
    double overlap_max;  /* maximum of the winning overlap grid               */
    double sigma;        /* width used                                        */
    int    inverted;     /* 1 if -pos2 aligned best                           */
    int    ncand;        /* candidates refined                                */
    int    status;       /* fo_status of this pair                            */
    int    niter;        /* assignment/rotation iterations of the winner      */
} fo_pair_result;

/* ---- context ---- */
fo_status   fo_ctx_create(const fo_opts *opts, fo_ctx **out);
void        fo_ctx_destroy(fo_ctx *ctx);
const char *fo_status_string(fo_status s);
const char *fo_last_error(const fo_ctx *ctx);
fo_status   fo_set_precision(fo_ctx *ctx, int precision);
/* Mixed form: 1 (default) runs the coefficient contraction (FOURIERCOEFFS,
 * fastoverlap/f90/fastclusters.f90:905-911) and the Wigner-d contraction of
 * the inverse SO(3) transform (ISOFT, fastoverlap/f90/DSOFT.f90:286-299) on
 * the tcgen05 tensor cores in split TF32 (3xTF32, FP32 accumulation); 0 on
 * the FP32 CUDA cores.  Applies to plans created afterwards; the FP64 form
 * never uses it.                                                             */
fo_status   fo_set_tensor_cores(fo_ctx *ctx, int on);
/* No counterpart in the reference.  1 (default): a mixed-form plan of at
 * least 256 pairs whose shape (distinct Jmax values, pair count rounded up
 * to a power of two) this context has not seen picks its tensor-core tile
 * shape -- (m1, m2) combinations per contraction CTA in {16, 32, 64, 128},
 * pairs per FFT block in {1, 2, 4} -- by timing every shape once at plan
 * creation; the choice is kept in the context for later plans of the shape.
 * 0: the default shape (64, 1).  fo_plan_tile_shape reports a plan's shape
 * (0, 0 when it does not use the tensor cores).                             */
fo_status   fo_set_autotune(fo_ctx *ctx, int on);
/* No counterpart in the reference.  Page-lock a caller's host buffer of
 * `bytes` bytes (cudaHostRegister) so that the batched entry points copy it
 * to and from the device by DMA; fo_host_unregister releases it.  The buffer
 * stays the caller's memory throughout.                                      */
fo_status   fo_host_register(fo_ctx *ctx, void *ptr, size_t bytes);
fo_status   fo_host_unregister(fo_ctx *ctx, void *ptr);

/* ---- batched entry points (host buffers in, host buffers out) ----
 * pos1 = target structures (COORDSB), pos2 = structures moved onto them
 * (COORDSA); both packed as pairs[i].coord_off.. (+natoms) atoms.
 * perm: concatenated permutation groups, `index_base` 0 or 1.
 * aligned (optional, may be NULL): 3*sum(natoms) doubles, the aligned copy of
 *   pos2 in pos1's centred frame (cluster) or pos1's frame (bulk), in pos1's
 *   atom order: aligned atom j is matched with pos1 atom j.
 * permbest (optional): sum(natoms) ints, pos2 atom matched with pos1 atom j
 *   (same index base as perm).                                                */
fo_status fo_cluster_align_batch(fo_ctx *ctx, int npairs, const fo_cluster_pair *pairs,
                                 const double *pos1, const double *pos2,
                                 const int *perm, const int *group_sizes, int index_base,
                                 double *aligned, int *permbest, fo_pair_result *results);

/* A pair with ohcell = 1 is aligned for each of the 48 operations of the
 * cubic point group applied to pos2 (signed permutations of x, y, z; ALIGN1
 * with OHCELLT, fastoverlap/f90/fastbulk.f90:458-481) and the smallest
 * distance wins (the first operation on ties, the identity first).  Its
 * result's rmat is that operation (row-major; aligned = op(pos2)[perm] +
 * disp), its ncand counts all 48 searches.  Resident plans take no ohcell
 * pairs. */
fo_status fo_bulk_align_batch(fo_ctx *ctx, int npairs, const fo_bulk_pair *pairs,
                              const double *pos1, const double *pos2,
                              const int *perm, const int *group_sizes, int index_base,
                              double *aligned, int *permbest, fo_pair_result *results);

/* The cluster batch in the harmonic-oscillator basis (SphericalHarmonicAlign,
 * ALIGNHARM): coefficients c_nlm of the coordinates as given (not centred),
 * orders n <= nmax (<= 40) at length scale hwidth; every pair's sigma is the
 * kernel width KWIDTH (> 0).  Outputs as fo_cluster_align_batch, aligned in
 * pos1's own frame. */
fo_status fo_cluster_harm_align_batch(fo_ctx *ctx, int npairs, const fo_cluster_pair *pairs,
                                      const double *pos1, const double *pos2,
                                      const int *perm, const int *group_sizes, int index_base,
                                      int nmax, double hwidth, double *aligned, int *permbest,
                                      fo_pair_result *results);

/* ---- resident plans: upload once, run many times (inputs stay in HBM) ----
 * fo_plan_run launches the whole pipeline on the context's stream and
 * returns without synchronising; fo_plan_wait blocks until it is done.
 * A plan's device memory is one block.  When a plan is destroyed the context
 * keeps its block (up to four blocks, the largest; freed by fo_ctx_destroy)
 * and hands the smallest one that fits to a later plan, so repeated batches
 * allocate no device memory.  A caller's hbm_budget_bytes bounds every plan;
 * the automatic budget (80% of free memory) applies to new allocations only. */
typedef struct fo_plan fo_plan;
fo_status fo_cluster_plan_create(fo_ctx *ctx, int npairs, const fo_cluster_pair *pairs,
                                 const double *pos1, const double *pos2,
                                 const int *perm, const int *group_sizes, int index_base,
                                 fo_plan **out);
fo_status fo_bulk_plan_create(fo_ctx *ctx, int npairs, const fo_bulk_pair *pairs,
                              const double *pos1, const double *pos2,
                              const int *perm, const int *group_sizes, int index_base,
                              fo_plan **out);
fo_status fo_cluster_harm_plan_create(fo_ctx *ctx, int npairs, const fo_cluster_pair *pairs,
                                      const double *pos1, const double *pos2,
                                      const int *perm, const int *group_sizes, int index_base,
                                      int nmax, double hwidth, fo_plan **out);
fo_status fo_plan_run(fo_plan *plan);
/* on = 1: the next fo_plan_run runs eagerly and captures its launch sequence
 * (all streams) as a CUDA graph; later runs replay the graph with one launch.
 * Per-stage profile times are not recorded while graphs are used.  on = 0
 * drops the graph. */
fo_status fo_plan_set_graph(fo_plan *plan, int on);
fo_status fo_plan_wait(fo_plan *plan);
fo_status fo_plan_results(fo_plan *plan, double *aligned, int *permbest,
                          fo_pair_result *results);
size_t    fo_plan_device_bytes(const fo_plan *plan);
fo_status fo_plan_tile_shape(const fo_plan *plan, int *chunk, int *group);
int       fo_plan_launches(const fo_plan *plan);   /* kernel launches per fo_plan_run */
void      fo_plan_destroy(fo_plan *plan);

/* ---- stage outputs of one pair (parity checks, diagnostics) ----
 * fo_cluster_overlap: SO(3) coefficients (layout [l][m1 mod W][m2 mod W],
 * W = 2L+1, complex as interleaved re/im, (L+1)W^2 complex values; the
 * inverted copy's are (-1)^l times these) and the real overlap grid of the
 * non-inverted orientation, G = 2(L+1), grid[a + G(b + G g)] -- CALCOVERLAP,
 * fastoverlap/f90/fastclusters.f90:918-960, after FOURIERCOEFFS :868-916.
 * fo_bulk_overlap: the modulus of the translation cross-correlation,
 * M^3 values, grid[x + M(y + M z)] -- CALCFSPACE,
 * fastoverlap/f90/fastbulk.f90:685-734 (without its k = 0 zeroing, as ALIGN1
 * computes it at :437-454,522-523).  Either pointer may be NULL.            */
fo_status fo_cluster_overlap(fo_ctx *ctx, const fo_cluster_pair *pair, const double *pos1,
                             const double *pos2, const int *perm, const int *group_sizes,
                             int index_base, double *coeffs, double *grid);
fo_status fo_bulk_overlap(fo_ctx *ctx, const fo_bulk_pair *pair, const double *pos1,
                          const double *pos2, const int *perm, const int *group_sizes,
                          int index_base, double *grid);

/* ---- peak search on one periodic n^3 grid ----
 * FINDPEAKS, fastoverlap/f90/fastutils.f90:475-548 (with FINDPEAK :401-444
 * and FIT :353-397): up to npeaks Gaussian peaks, each fitted in the
 * (2w+1)^3 window around the current first maximum and subtracted from a
 * copy of the grid; w starts at `width` (the module variable WIDTH, 2 by
 * default) and grows while no peak is found, up to min(n/2, 7).  grid: n^3
 * host doubles, a fastest (left unchanged).  peaks[3k..3k+2]: 1-based
 * fractional grid coordinates of peak k; amps[k] (may be NULL): its
 * amplitude X(1).  *nfound: number of peaks.  Mixed precision fits in FP32.
 * Returns FO_ERR_NO_PEAKS with *nfound = 0 where FINDPEAKS stops.
 * Limits: 2 <= n <= 256, 1 <= npeaks <= 64, 1 <= width <= 7.               */
fo_status fo_findpeaks(fo_ctx *ctx, const double *grid, int n, int npeaks, int width,
                       double *peaks, double *amps, int *nfound);

/* ---- periodic overlap grid without device allocation ----
 * No counterpart in the reference.  For callers that cannot let a library
 * allocate device memory (their own pool owns it, or an allocation in the
 * middle of a request is not allowed): same result as fo_bulk_overlap in
 * FP64, but inputs and output are DEVICE pointers and the only scratch is a
 * fixed file-scope device array (fo_bulk_overlap_noalloc_scratch_bytes(),
 * about 4 MiB, held by every GPU that loads the library until exit).
 * Limits: nfspace (M) <= 64, at most 64 permutation groups; larger requests
 * return FO_ERR_BAD_ARGS.  The atoms of group g must be the contiguous range
 * [sum of earlier sizes, + group_sizes[g]) of d_pos1/d_pos2 (3 doubles each);
 * group_sizes is a host array.  d_grid receives M^3 doubles, x fastest.
 * Work is queued on `stream` (a cudaStream_t, NULL = default stream) and the
 * call returns without waiting.  The first call on a device looks up the
 * scratch array's address; make that first call before any stream capture.
 * All calls share the array (it keeps the previous contents; the kernel
 * clears what must start at zero): calls that overlap on the GPU race and
 * must be serialised by the caller.  If an error from earlier CUDA work is
 * pending on the calling thread (cudaPeekAtLastError), the call queues
 * nothing, returns FO_ERR_CUDA and leaves that error for the caller to read. */
fo_status fo_bulk_overlap_noalloc(const double *d_pos1, const double *d_pos2, int natoms,
                                  const int *group_sizes, int ngroups, double boxlx,
                                  double boxly, double boxlz, double kwidth, int nwave,
                                  int nfspace, double *d_grid, void *stream);
size_t    fo_bulk_overlap_noalloc_scratch_bytes(void);

/* ---- Fortran-compatible single-pair entry points ----
 * fo_setperm keeps the permutation groups in the context, as SETPERM keeps
 * them in module storage; permgroup is 1-based like the Fortran array.      */
fo_status fo_setperm(fo_ctx *ctx, int natoms, const int *permgroup, const int *npermsize,
                     int npermgroup);
fo_status fo_get_bestperm(const fo_ctx *ctx, int *bestperm /* natoms, 1-based */);
/* COMMONS OHCELLT for fo_bulk_align: 1 searches the 48 cubic operations. */
fo_status fo_set_ohcell(fo_ctx *ctx, int ohcell);

/* CLUSTERFASTOVERLAP::ALIGN: coordsb is centred in place, coordsa becomes the
 * aligned, permuted copy; kwidth <= 0 is replaced by the chosen width;
 * rmatbest is column-major 3x3 as in Fortran.  perminvopt = PERMINVOPT.     */
fo_status fo_cluster_align(fo_ctx *ctx, double *coordsb, double *coordsa, int natoms,
                           int debug, int l, double *kwidth, int nrotations, int perminvopt,
                           double *distance, double *dist2, double *rmatbest);

/* CLUSTERFASTOVERLAP::ALIGNHARM (argument order of the Fortran routine, with
 * PERMINVOPT last): the coordinates as given (coordsb is left as it is),
 * harmonic-basis coefficients of order n at length scale hwidth, kernel
 * width kwidth (> 0); coordsa becomes the aligned, permuted copy in
 * coordsb's frame.  Every atom is refined in its own order and an inverted
 * winner returns its own rotation, as CLUSTERFASTOVERLAP::ALIGN does (the
 * Fortran ALIGNHARM keeps its per-group copies of the coordinates for the
 * refinement and returns the non-inverted rotation; the results are the
 * same for one permutation group in index order and non-inverted winners). */
fo_status fo_cluster_align_harm(fo_ctx *ctx, double *coordsb, double *coordsa, int natoms,
                                int debug, int n, int l, double hwidth, double kwidth,
                                double *distance, double *dist2, double *rmatbest,
                                int nrotations, int perminvopt);

/* CLUSTERFASTOVERLAP::CALCOVERLAPMATRICES: for every pair of structures of
 * coordslist(3*natoms, nlist) (column-major), the squared norm of the
 * harmonic-basis SO(3) coefficients (norms) and the maximum of the overlap
 * grid (maxovers), both (nlist, nlist) and symmetric; groups of fo_setperm. */
fo_status fo_calc_overlap_matrices(fo_ctx *ctx, const double *coordslist, int natoms, int nlist,
                                   int n, int l, double hwidth, double kwidth,
                                   double *norms, double *maxovers);

/* BULKFASTOVERLAP::ALIGN (nwave = nfspace = 0) or ALIGN1 (both given). */
fo_status fo_bulk_align(fo_ctx *ctx, double *coordsb, double *coordsa, int natoms,
                        int debug, double boxlx, double boxly, double boxlz,
                        double kwidth, int ndisplacements, int nwave, int nfspace,
                        double *distance, double *dist2);

/* BULKFASTOVERLAP::ALIGNGROUP: structure j of coords2list aligned onto
 * structure i of coords1list for every (i, j) -- or, with sym, for i >= j
 * only, the list-2 structures standing for list 1's (the reference reuses
 * list 1's coefficients there).  Fortran (column-major) layouts:
 * coords1list(3*natoms, n1list), coords2list(3*natoms, n2list),
 * distmat(n1list, n2list), alignedcoords2(3*natoms, n1list, n2list) (may be
 * NULL); entries sym skips are 0.  The groups are those of fo_setperm; every
 * pair runs as ALIGN / ALIGN1 with the given parameters. */
fo_status fo_bulk_align_group(fo_ctx *ctx, const double *coords1list, int n1list,
                              const double *coords2list, int n2list, int natoms, int debug,
                              double boxlx, double boxly, double boxlz, double kwidth,
                              int ndisplacements, int nwave, int nfspace, double *distmat,
                              double *alignedcoords2, int sym);

/* Branch and bound over rotations (the upstream Python BranchandBoundMaster
 * with BranchNodeCluster): both structures centred; a best-first search over
 * cubes of angle-axis vectors (start width 2 pi, 8 children of half width)
 * by lower bound until it is within rtol * best + atol of the best upper
 * bound, or after niter expanded nodes; invert also starts from -pos2.
 * dist: the best upper bound (the assignment distance at that node's
 * rotation); aligned (optional): that node's rotated pos2 on pos1's centroid,
 * in pos2's atom order; nodes (optional): nodes taken from the queue.  One
 * species, natoms <= 256.  The batch form runs npairs searches side by side
 * (pair p's atoms follow pair p-1's in pos1, pos2 and aligned).  The children
 * of one round are evaluated in launches sized to the context's HBM budget.
 * A search whose assignment hits its step guard stops with dist (and its
 * aligned rows) NaN while the others finish; the call then returns
 * FO_ERR_LAP_FAILED. */
fo_status fo_bnb_cluster(fo_ctx *ctx, const double *pos1, const double *pos2, int natoms, int invert,
                         long long niter, double rtol, double atol, double *dist, double *aligned,
                         long long *nodes);
fo_status fo_bnb_cluster_batch(fo_ctx *ctx, int npairs, const int *natoms, const double *pos1,
                               const double *pos2, int invert, long long niter, double rtol, double atol,
                               double *dist, double *aligned, long long *nodes);

/* BULKFASTOVERLAP::CALCDEFAULTS */
fo_status fo_bulk_calcdefaults(int natoms, double boxlx, double boxly, double boxlz,
                               double *kernelwidth, int *nwave, int *nfspace);

/* ---- serving: alignment requests admitted as they arrive ----
 * No counterpart in the reference (its classes align one pair per call).
 * Spherical (SphericalAlign) and periodic (PeriodicAlign) requests of any
 * size are submitted one at a time, from any host thread; inputs are copied
 * at submission.  `workers` worker threads (the given context and contexts
 * created with its options, each on its own streams) take every request
 * pending when they are free (continuous batching, arrival order, at most
 * max_batch), run them as one resident plan per kind, and complete their
 * tickets; one batch's last large pairs overlap the next batch.  The
 * context's HBM budget is shared evenly by the workers: a plan larger than a
 * share is split in halves, and a request that does not fit alone completes
 * with FO_ERR_OOM_BUDGET.  The server owns the context while it lives: make
 * no other call on it.                                                       */
typedef struct fo_server fo_server;

enum { FO_KIND_CLUSTER = 0, FO_KIND_BULK = 1 };

typedef struct {
    int           kind;        /* FO_KIND_CLUSTER or FO_KIND_BULK                  */
    int           natoms;
    int           ngroups;
    int           jmax;        /* cluster: L                                       */
    int           nrot;        /* cluster: peaks per orientation; bulk: displacements
                                  (<= 0: 10)                                        */
    int           invert;      /* cluster: also align the inverted copy            */
    int           nwave;       /* bulk: K (<= 0: default)                          */
    int           nfspace;     /* bulk: M (<= 0: default)                          */
    double        sigma;       /* <= 0: default width                              */
    double        box[3];      /* bulk: box lengths                                */
    const double *pos1;        /* 3*natoms, target structure                       */
    const double *pos2;        /* 3*natoms, structure moved onto it                */
    const int    *perm;        /* natoms atom indices (0-based) grouped by species */
    const int    *group_sizes; /* ngroups                                          */
} fo_request;

typedef struct {
    int    max_batch;     /* requests per plan; <= 0: 4096                         */
    int    max_queue;     /* pending requests before FO_ERR_QUEUE_FULL; <= 0: 1<<20 */
    double max_wait_ms;   /* once a worker is free, wait up to this long for more
                             requests before launching; 0: launch at once           */
    int    workers;       /* concurrent batches (contexts); <= 0: 2                */
    int    reserved;
} fo_server_opts;

typedef struct {
    int64_t submitted, completed, failed, batches;
    double  latency_p50_ms, latency_p99_ms, latency_max_ms;  /* submit -> complete */
    double  mean_batch;   /* requests per batch                                    */
    double  busy_ms;      /* summed over workers: time with a batch being prepared or run */
} fo_server_stats;

fo_status fo_server_create(fo_ctx *ctx, const fo_server_opts *opts, fo_server **out);
/* FO_ERR_BAD_ARGS for an invalid request (nothing queued). */
fo_status fo_server_submit(fo_server *srv, const fo_request *req, int64_t *ticket);
/* FO_ERR_NOT_READY while the request is in flight; otherwise the request's own
 * status, with result, aligned (3*natoms, may be NULL) and permbest (natoms,
 * 0-based, may be NULL) filled as by the batch entry points, and the ticket
 * released.  fo_server_wait blocks up to timeout_ms (< 0: no limit) and
 * returns FO_ERR_TIMEOUT when the time runs out.  A ticket that was never
 * issued, or whose result was already collected (by poll or by another
 * wait), gives FO_ERR_BAD_ARGS at once.  Latency percentiles in the stats
 * come from a log-scale histogram with 1% bins (within 0.5%).               */
fo_status fo_server_poll(fo_server *srv, int64_t ticket, fo_pair_result *result, double *aligned,
                         int *permbest);
fo_status fo_server_wait(fo_server *srv, int64_t ticket, double timeout_ms, fo_pair_result *result,
                         double *aligned, int *permbest);
fo_status fo_server_stats_get(fo_server *srv, fo_server_stats *stats);
void      fo_server_destroy(fo_server *srv);   /* completes every queued request first */

/* ---- timing helpers on the context's stream (benchmarks) ----
 * fo_ctx_record records CUDA event `slot` (0..63) on the context stream;
 * fo_ctx_elapsed_ms reads the device time between two recorded slots (it
 * synchronises on the later one); fo_ctx_flush_l2 writes `bytes` of
 * scratch memory on the stream so the next launch starts with a cold L2.   */
fo_status fo_ctx_record(fo_ctx *ctx, int slot);
fo_status fo_ctx_elapsed_ms(fo_ctx *ctx, int slot_a, int slot_b, float *ms);
fo_status fo_ctx_flush_l2(fo_ctx *ctx, size_t bytes);
fo_status fo_ctx_synchronize(fo_ctx *ctx);

/* ---- profiling: per-kernel CUDA-event time of the last fo_plan_run ----
 * names[i] receives a static string; returns the number of kernels.         */
int fo_profile_kernels(const fo_ctx *ctx, const char **names, double *ms_total,
                       int *launches, int cap);
void fo_profile_reset(fo_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif
