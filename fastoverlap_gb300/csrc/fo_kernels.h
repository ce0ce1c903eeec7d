// fo_kernels.h -- host-side launch wrappers exported by the kernel files and
// used by the C-ABI layer (fo_api.cu).  All launches are asynchronous on the
// given stream.
#pragma once
#include <cuda.h>   // CUtensorMap (types only; the driver entry point is looked up at run time)
#include <cuda_runtime.h>
#include <mutex>
#include <vector>
#include "../../include/fastoverlap_gb300.h"
#include "fo_common.cuh"

namespace fo {

// Raise kernel K's dynamic shared-memory limit to the device's opt-in maximum,
// once per kernel.  The limit is a process-wide attribute of the kernel: a
// thread that lowered it for a small launch would make another thread's
// larger launch of the same kernel fail, so it is only ever set to the
// maximum (the launch's own size still decides occupancy).  Set on the device
// current at the first launch.
template <auto K>
inline void allow_max_smem() {
    static std::once_flag once;
    std::call_once(once, [] {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncAttributes fa{};
        cudaFuncGetAttributes(&fa, K);
        cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    });
}

struct SphBuffers {
    const PairDev *pairs;
    const GroupDev *groups;
    const int *slot2orig;   // per slot: original atom index within the pair
    const int *slot2pair;   // per slot
    const double *pos1, *pos2;  // packed original-order inputs (3 per atom)
    double *xa, *xb;        // slot-ordered centred coordinates (3 per slot)
    double *ra, *rb;        // per slot radii
    void *ylmA, *ylmB;      // complex T per (slot, lm)
    void *W;                // radial weights (T)
    void *coef;             // complex T coefficients (ilmm layout)
    void *grid;             // real T overlap grids
    const void *const *dtab;  // per bandwidth: Wigner table (T), layout [k][l][m1][m2]
    int npairs, ngroups, nslots, maxL, maxG, maxgroup;
    int harm_n = -1;          // >= 0: harmonic-oscillator basis of this order (all pairs)
    double *hd = nullptr;     // its radial overlaps d_nl, FP64 [side][slot][n][l <= maxL]
    bool tc_layout = false;   // mixed form on the tensor cores: Y_lm as [lm][atom] per pair and
                              // radial weights as [l][a][b] per group (read by launch_coef_tc)
};

constexpr int kMaxHarmN = 40;   // largest harmonic order nmax

// spherical stages
void launch_sph_center(const SphBuffers &b, cudaStream_t s);
void init_sph_tables();   // constant tables of the current device; before the first launch
void launch_sph_ylm(const SphBuffers &b, bool fp32, cudaStream_t s);
void launch_sph_radial(const SphBuffers &b, bool fp32, int cutoff, cudaStream_t s);
void launch_sph_coeff(const SphBuffers &b, bool fp32, cudaStream_t s);
// the same contraction on the tcgen05 tensor cores (FP32 data in 3xTF32, the
// tc_layout layouts); *err is set when a pipeline wait timed out
void launch_coef_tc(const SphBuffers &b, int *err, cudaStream_t s);
void launch_isoft(const SphBuffers &b, bool fp32, cudaStream_t s);
void launch_pair_stats(const SphBuffers &b, bool fp32, double *out, cudaStream_t s);
void launch_wigner_table(int bw, double *d64, float *d32, cudaStream_t s);

// periodic stages
struct BulkBuffers {
    const PairDev *pairs;
    const GroupDev *groups;
    const int *slot2orig;
    const double *pos1, *pos2;
    double *xa, *xb;
    void *fgrid;            // complex T, M^3 per pair
    void *grid;             // real T, M^3 per pair
    int npairs, maxK, maxM;
};
void launch_bulk_prep(const BulkBuffers &b, cudaStream_t s);
void launch_bulk_sf(const BulkBuffers &b, bool fp32, cudaStream_t s);
void launch_bulk_fft(const BulkBuffers &b, bool fp32, cudaStream_t s);

// peaks and refinement (shared)
struct RefineBucket {
    int offset, count;  // slice of cand_list
    size_t smem;        // dynamic shared memory per candidate
    int ct64;           // 64-bit integer costs
    int nw;             // warps per candidate (> 1: helpers for the neighbour lists, mixed form)
};
int refine_block_warps(bool bulk, bool ct64, size_t smem);

struct RefineBuffers {
    const PairDev *pairs;
    const GroupDev *groups;
    const int *slot2orig;
    const int *cand2pair;
    const double *xa, *xb;
    void *grid;             // real T, consumed (peaks are subtracted)
    double *overlap_max;    // [pair][2]
    double *peaks;          // [cand][3] 1-based fractional grid coordinates
    int *npeaks;            // [pair][2]
    int *pstatus;           // [pair]
    unsigned char *lap;     // LAP scratch
    double *cdist, *cR, *cdisp, *cxyz;
    int *cperm, *cniter, *cstat;
    float *cthr;            // per candidate atom: its neighbour-list threshold (mixed form)
    float4 *b4;             // per slot: the fixed structure's FP32 copy (mixed form)
    int *cscr;              // per candidate atom: two permutation working entries and the
                            // assignment's free list (mixed form)
    // final outputs
    void *results;          // fo_pair_result[npairs]
    double *aligned;        // 3 per atom, original order
    int *permbest;          // per atom, original order
    int npairs, ncand, maxG, maxn;
    const int *cand_list;          // device: candidate ids grouped by bucket
    const RefineBucket *buckets;   // host
    int nbuckets;
    bool fp32;
    bool recomp;   // costs recomputed from FP32 coordinates (mixed form)
    bool bulk;     // periodic pairs (minimum-image distances)
};
void launch_findpeaks(const RefineBuffers &b, bool fp32, cudaStream_t s);
void launch_findpeaks_from(const PairDev *pairs, int npairs, void *grid, double *omax, double *peaks,
                           double *amps, int *npeaks, int *pstatus, bool fp32, int width0, cudaStream_t s);
void launch_refine(const RefineBuffers &b, cudaStream_t main, cudaStream_t *aux, int naux,
                   cudaEvent_t fork, cudaEvent_t *join);
void launch_select(const RefineBuffers &b, cudaStream_t s);

// tensor-core Wigner contraction (mixed form), fo_wigner_tc.cu
constexpr int kTcTile = 64;        // pairs per tile: 128 MMA rows (real parts, then imaginary parts)
constexpr int kTcMaxBuckets = 8;   // bandwidths (Wigner tables) per launch
constexpr int kTcChunk = 64;       // (m1, m2) combinations per work item

struct TcTile {
    int L;            // Jmax of every pair of the tile
    int bucket;       // index of its table in the launch's TcMaps
    int npairs;       // pairs in the tile (<= kTcTile)
    int pad;
    long long s0;     // offset (floats) of the tile's sums in S: [col < 2G][mm < W^2][row < 2 npairs]
    long long coef0[kTcTile];   // complex offset of each pair's coefficients (ilmm layout)
};
struct TcItem { int tile, mm0, mm1, pad; };
// Pairs per block of the FFT stage: at most kTcFftGroup, one when G = 64
// (the autotuner picks the group size per plan shape).
constexpr int kTcFftGroup = 4;
__host__ __device__ inline int tc_fft_group(int G, int group) {
    return G <= 32 ? (group < kTcFftGroup ? group : kTcFftGroup) : 1;
}
struct TcFftGroup {
    long long s0;   // its tile's S offset
    int L;          // Jmax of the tile
    int ntile;      // pairs in the tile (rows: 2 ntile per column and mm)
    int p0, npg;    // first pair (row) of the group in the tile, pairs in the group
    int pair[kTcFftGroup];   // plan index of each pair of the group
};
struct TcMaps {
    CUtensorMap map[kTcMaxBuckets];   // Wigner tables [hi|lo][mm][Nr][32] (TMA, 128-byte swizzle)
    int nr[kTcMaxBuckets];            // rows per mm: 2G rounded up to 16
};
struct TcLaunch {
    TcMaps maps;
    int item0, nitems, nrmax;
};
struct TcBuffers {
    const PairDev *pairs = nullptr;
    const TcTile *tiles = nullptr;
    const TcItem *items = nullptr;
    const TcFftGroup *groups = nullptr;   // FFT-stage blocks
    int ngroups = 0;
    size_t fft_smem = 0;                  // dynamic shared memory of the FFT stage
    const void *coef = nullptr;   // complex FP32 coefficients
    float *S = nullptr;           // contraction sums
    void *grid = nullptr;         // FP32 overlap grids
    int *err = nullptr;           // set when a wait timed out
    int npairs = 0, maxG = 0;
    std::vector<TcLaunch> launches;
};
int tc_rows(int bw);                 // Nr of a bandwidth
size_t tc_table_floats(int bw);      // floats of its table
// fills `out` (tc_table_floats(bw) floats) from the FP64 Wigner table and
// encodes its tensor map; false when the tensor-map encoder is unavailable
bool tc_make_table(int bw, const double *d64, float *out, CUtensorMap *map, cudaStream_t s);
void launch_wigner_tc(const TcBuffers &b, cudaStream_t s);   // the contraction (tcgen05)
void launch_isoft_tc(const TcBuffers &b, cudaStream_t s);    // the FFT stage after it
size_t tc_fft_smem(int G, int npg);  // its dynamic shared memory: npg pairs of planes of edge G

// context options (library-internal; the server creates worker contexts)
fo_opts ctx_opts(const fo_ctx *ctx);
void ctx_set_budget(fo_ctx *ctx, size_t bytes);
cudaStream_t ctx_stream(fo_ctx *ctx);
fo_status ctx_error(fo_ctx *ctx, fo_status s, const char *msg);   // sets the message fo_last_error returns

}  // namespace fo
