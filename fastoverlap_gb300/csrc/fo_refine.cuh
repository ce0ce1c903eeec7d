// fo_refine.cuh -- shared-memory / scratch layout of one refinement
// candidate, computed identically on the host (bucketing) and the device.
#pragma once
#include <cuda_runtime.h>

namespace fo {

struct RefLayout {
    size_t DBf, DAf, perm, nperm, ptmp, coord_end;
    size_t lap_cc, lap_kk, lap_heap, lap_v, lap_d, lap_x, lap_y, lap_lab, lap_fr, lap_todo, lap_ok, lap_end;
    size_t lap_small;   // bytes of the assignment block before the costs and neighbour lists
    int kkbytes;   // bytes per neighbour-list column index
};

// Neighbour lists of groups with more than 60 atoms (mixed form): rows of at
// most kHeapMaxRow columns are selected a row per lane (nearest_lane), longer
// rows by the whole warp on one row at a time (one row of distances as
// scratch) or by all warps of a multi-warp block.
constexpr int kHeapMaxRow = 256;

// Mixed form, groups of more than kHeapMaxRow atoms: blocks of up to
// kRefMaxWarps warps per candidate, where the warps beyond the first only
// help with the neighbour lists (one row per warp at a time, the row's
// distances in registers: at most 32 * kNearRegMW columns).  The rest of the
// refinement stays on the first warp.
constexpr int kRefMaxWarps = 8;
constexpr int kNearRegMW = 32;
__host__ __device__ inline bool ref_multiwarp(int maxg) {
    return maxg > kHeapMaxRow && maxg <= 32 * kNearRegMW;
}

__host__ __device__ inline size_t ref_a16(size_t b) { return (b + 15) & ~(size_t)15; }

// Column indices of the neighbour lists fit one byte when no group has more
// than 256 atoms.
__host__ __device__ inline int ref_kkbytes(int maxg) { return maxg <= 256 ? 1 : 2; }

// n atoms, largest permutation group maxg, FP32 coordinate copies (float4
// per atom) when fp32, ctsize = bytes per integer cost (4 or 8), recomp =
// costs recomputed from the FP32 coordinates instead of stored (only the
// neighbour lists of groups with more than 60 atoms are kept, selected
// through a per-lane heap or one-row distance scratch).  The FP64 coordinates are not held here: the
// refinement keeps them in global memory.
__host__ __device__ inline void ref_layout(int n, int maxg, bool fp32, int ctsize, bool recomp,
                                           RefLayout &L) {
    // recomp (mixed form): the fixed structure's FP32 copy and the
    // permutations live in global memory, only the moved structure's FP32
    // copy and the assignment arrays on chip
    size_t o = 0;
    L.DBf = o; o += (fp32 && !recomp) ? 16 * (size_t)n : 0;
    L.DAf = o; o += fp32 ? 16 * (size_t)n : 0;
    const size_t pn = recomp ? 0 : ref_a16(4 * (size_t)n);
    L.perm = o; o += pn;
    L.nperm = o; o += pn;
    L.ptmp = o; o += pn;
    L.coord_end = o;
    const int m = maxg < 60 ? maxg : 60;
    const bool sparse = maxg > 60;
    L.kkbytes = ref_kkbytes(maxg);
    // the assignment's working arrays first, then the stored costs and the
    // neighbour lists (the large part, which may live apart from the rest)
    size_t p = 0;
    L.lap_v = p; p += ref_a16(8 * (size_t)maxg);
    L.lap_d = p; p += ref_a16(8 * (size_t)maxg);
    L.lap_x = p; p += ref_a16(4 * (size_t)maxg);
    L.lap_y = p; p += ref_a16(4 * (size_t)maxg);
    L.lap_lab = p; p += ref_a16(4 * (size_t)maxg);
    L.lap_fr = p; p += recomp ? 0 : ref_a16(4 * (size_t)maxg);   // mixed form: free list in global scratch
    L.lap_todo = p; p += ref_a16(4 * (size_t)maxg);
    L.lap_ok = p; p += ref_a16((size_t)maxg);
    // the neighbour-selection scratch is only used before a group's
    // assignment starts, so it overlays the working arrays (and never the
    // neighbour lists it is filling)
    L.lap_heap = L.lap_v;
    size_t scratch = 0;
    if (recomp && sparse && maxg > kHeapMaxRow) {
        // one row of distances for the one-warp selector of rows longer than
        // kHeapMaxRow; shorter rows are selected a row per lane, in registers
        scratch = ref_a16(4 * (size_t)maxg);
    }
    const size_t heap_end = L.lap_heap + scratch;
    if (heap_end > p) p = heap_end;
    L.lap_small = p;
    L.lap_cc = p; p += recomp ? 0 : ref_a16((size_t)ctsize * maxg * m);
    L.lap_kk = p; p += sparse ? ref_a16((size_t)L.kkbytes * maxg * m) : 0;
    L.lap_end = p;
}

}  // namespace fo
