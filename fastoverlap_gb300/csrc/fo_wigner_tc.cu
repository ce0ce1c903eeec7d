// fo_wigner_tc.cu -- the Wigner-d contraction of the inverse SO(3) transform
// on the tcgen05 tensor cores (mixed form), and the FFT stage that follows it.
//
// Reference behaviour (matthewghgriffiths/fastoverlap): ISOFT
// fastoverlap/f90/DSOFT.f90:265-329 (soft.py:115-125 in the Python path):
//   T[m1, beta_k, m2] = sum_{l >= max(|m1|,|m2|)} d^l_{m1 m2}(beta_k) I^l_{m1 m2}
// followed by inverse FFTs over m2 -> gamma and m1 -> alpha.
//
// GEMM form.  Pairs of one bandwidth are grouped into tiles of 64.  For each
// (m1, m2) -- "mm", W^2 of them -- the contraction over l of all pairs of a
// tile and all beta_k is one product
//   D[row][col] = sum_l A[row][l] B[col][l]
//     row < 128: real parts of the 64 pairs' I^l_{m1m2}, then imaginary parts
//     col < 2G : beta_k of the direct orientation, then of the inverted one
//                (B[G + k][l] = (-1)^l d^l(beta_k), since I_inv^l = (-1)^l I^l)
//     l   < 32 : zero beyond the bandwidth
// issued as tcgen05.mma kind::tf32 with M = 128, N = Nr (2G rounded up to 16),
// K = 8 per instruction, the FP32 accumulator in tensor memory.  Precision is
// FP32-like by 3xTF32 splitting: x = hi + lo with hi the operand rounded to
// TF32, and D = A_hi B_hi + A_hi B_lo + A_lo B_hi (the dropped A_lo B_lo term
// is ~2^-22 relative).
//
// Data movement.  B (the Wigner tables, split into hi/lo once per bandwidth
// from the FP64 recurrence, layout [hi|lo][mm][Nr rows][32 l]) arrives by TMA
// (cp.async.bulk.tensor, 128-byte swizzle) into shared memory.  A is read from
// the coefficient array by four producer warps, split into hi/lo in registers
// and written to shared memory in the same 128-byte-swizzled K-major layout.
// A single thread issues the MMAs; four epilogue warps read the accumulators
// (tcgen05.ld, warp w owns TMEM lanes 32w..32w+31) for four mm at a time and
// write the sums to S[tile][col][mm][row] (rows fastest: the real parts of
// the tile's pairs, then their imaginary parts, 2 npairs rows), so each warp
// store covers 128 contiguous bytes; the FFT kernel below reads the rows of a
// group of pairs for every mm of one beta_k.
//
// Every wait on an mbarrier is bounded (about two seconds on the global
// timer); a wait that runs out sets *err, the CTA leaves its loops, frees its
// tensor memory and returns, and the host reports FO_ERR_CUDA.
#include <cuda.h>   // CUtensorMap and the tensor-map enums (no driver library link)

#include "fo_common.cuh"
#include "fo_kernels.h"
#include "fo_tc.cuh"

#include <mutex>

namespace fo {

namespace {

constexpr int kTcStages = 2;
constexpr int kTcThreads = 288;          // warps 0-3 epilogue, 4-7 A producers, 8 MMA
constexpr int kTcBatch = 4;              // mm per accumulator group
constexpr int kTcRowBytes = 128;         // 32 FP32 values of l per row
constexpr int kTcABytes = 128 * kTcRowBytes;

using namespace tc;
__device__ __forceinline__ void tc_fence_before() { fence_before(); }
__device__ __forceinline__ void tc_fence_after() { fence_after(); }

}  // namespace

// ---------------------------------------------------------------------------
// Wigner tables in the MMA layout, from the FP64 table d64 ([k][l][i1][i2],
// k < G, l < bw): out[h][mm][row][l] (h = 0 hi, 1 lo; row < Nr; l < 32) with
// row = o G + k (o = 1: times (-1)^l), zero for l >= bw and rows >= 2G.
__global__ void k_wigner_tc_table(int bw, const double *__restrict__ d64, float *__restrict__ out, int Nr) {
    const int W = 2 * bw - 1, W2 = W * W, G = 2 * bw;
    const long long n = (long long)W2 * Nr * 32;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const int l = (int)(t % 32), row = (int)((t / 32) % Nr), mm = (int)(t / (32LL * Nr));
    double x = 0.0;
    if (l < bw && row < 2 * G) {
        const int o = row / G, k = row % G;
        x = d64[((long long)k * bw + l) * W2 + mm];
        if (o && (l & 1)) x = -x;
    }
    const float hi = tf32_round((float)x);
    out[t] = hi;
    out[n + t] = (float)(x - (double)hi);
}

// ---------------------------------------------------------------------------
// The contraction.  One CTA per work item (a tile and a range of mm).
__global__ void __launch_bounds__(kTcThreads, 2)
    k_wigner_tc(const __grid_constant__ TcMaps maps, const TcTile *__restrict__ tiles,
                const TcItem *__restrict__ items, const float2 *__restrict__ coef, float *__restrict__ S,
                int tmem_cols, int nrmax, int *err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t bars[3 * kTcStages + 2];
    __shared__ uint32_t tmem_base_sh;
    __shared__ int abort_sh;
    __shared__ long long coef0_sh[kTcTile];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const TcItem it = items[blockIdx.x];
    const TcTile &T = tiles[it.tile];
    const int L = T.L, bw = L + 1, G = 2 * bw, W = 2 * L + 1;
    const int Nr = maps.nr[T.bucket], nks = (bw + 7) / 8, nmm = it.mm1 - it.mm0;
    const int npairs = T.npairs;
    const CUtensorMap *map = &maps.map[T.bucket];
    const uint32_t idesc = tf32_idesc(128, Nr);

    // 1024-aligned carve: A[stage][hi|lo] (16 KB each), B[stage][hi|lo] (nrmax x 128 B)
    const uint32_t sbase = (smem_u32(smem_raw) + 1023u) & ~1023u;
    unsigned char *gbase = smem_raw + (sbase - smem_u32(smem_raw));
    auto a_addr = [&](int s, int h) { return sbase + (uint32_t)((2 * s + h) * kTcABytes); };
    const uint32_t bsz = (uint32_t)nrmax * kTcRowBytes;
    auto b_addr = [&](int s, int h) { return sbase + 2u * kTcStages * kTcABytes + (uint32_t)(2 * s + h) * bsz; };
    auto full_a = [&](int s) { return smem_u32(&bars[s]); };
    auto full_b = [&](int s) { return smem_u32(&bars[kTcStages + s]); };
    auto empty = [&](int s) { return smem_u32(&bars[2 * kTcStages + s]); };
    const uint32_t acc_full = smem_u32(&bars[3 * kTcStages]), acc_empty = smem_u32(&bars[3 * kTcStages + 1]);

    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(full_a(s), 128);
            mbar_init(full_b(s), 1);
            mbar_init(empty(s), 1);
        }
        mbar_init(acc_full, 1);
        mbar_init(acc_empty, 128);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int p = tid; p < kTcTile; p += kTcThreads) coef0_sh[p] = T.coef0[p];
    if (warp == 8) {   // tensor memory: four accumulators of Nr columns
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = tmem_base_sh;
    volatile int *abort = &abort_sh;
    auto give_up = [&]() {
        *abort = 1;
        atomicOr(err, 1);
    };

    if (warp >= 4 && warp < 8) {
        // ---- A producers: row r = pair (r & 63), real (r < 64) or imaginary part
        const int r = tid - 128, p = r & 63, part = r >> 6;
        const bool valid = p < npairs;
        const float2 *cp = coef + (valid ? coef0_sh[p] : 0);
        const int nchunk = 2 * nks;   // 16-byte chunks (4 values of l) the MMAs read
        for (int j = 0; j < nmm; ++j) {
            const int s = j % kTcStages;
            if (j >= kTcStages && !mbar_wait(empty(s), ((j / kTcStages) - 1) & 1, abort)) { give_up(); break; }
            const int mm = it.mm0 + j;
            if (r == 0) {   // B by TMA: the hi and lo tables of this mm
                mbar_expect_tx(full_b(s), 2u * (uint32_t)Nr * kTcRowBytes);
                tma_load_2d(b_addr(s, 0), map, 0, mm * Nr, full_b(s));
                tma_load_2d(b_addr(s, 1), map, 0, (W * W + mm) * Nr, full_b(s));
            }
            const int i1 = mm / W, i2 = mm % W;
            float v[32];
#pragma unroll
            for (int l = 0; l < 32; ++l) {
                v[l] = 0.f;
                if (valid && l < bw) {
                    const float2 c = cp[((long long)l * W + i1) * W + i2];
                    v[l] = part ? c.y : c.x;
                }
            }
            unsigned char *ah = gbase + (a_addr(s, 0) - sbase), *al = gbase + (a_addr(s, 1) - sbase);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                if (c < nchunk) {
                    float4 h, lo;
                    h.x = tf32_round(v[4 * c]);     lo.x = v[4 * c] - h.x;
                    h.y = tf32_round(v[4 * c + 1]); lo.y = v[4 * c + 1] - h.y;
                    h.z = tf32_round(v[4 * c + 2]); lo.z = v[4 * c + 2] - h.z;
                    h.w = tf32_round(v[4 * c + 3]); lo.w = v[4 * c + 3] - h.w;
                    const int off = r * kTcRowBytes + ((c ^ (r & 7)) << 4);
                    *reinterpret_cast<float4 *>(ah + off) = h;
                    *reinterpret_cast<float4 *>(al + off) = lo;
                }
            }
            fence_async_smem();   // generic-proxy stores -> visible to the tensor cores
            mbar_arrive(full_a(s));
        }
    } else if (warp == 8) {
        // ---- MMA issuer (one thread)
        if (lane == 0) {
            for (int j = 0; j < nmm; ++j) {
                const int s = j % kTcStages, slot = j % kTcBatch, q = j / kTcBatch;
                if (slot == 0 && q > 0) {
                    if (!mbar_wait(acc_empty, (q - 1) & 1, abort)) { give_up(); break; }
                }
                const uint32_t ph = (j / kTcStages) & 1;
                if (!mbar_wait(full_a(s), ph, abort) || !mbar_wait(full_b(s), ph, abort)) { give_up(); break; }
                tc_fence_after();
                const uint32_t d = tbase + (uint32_t)(slot * Nr);
                for (int ks = 0; ks < nks; ++ks) {
                    const uint64_t ah = sw128_desc(a_addr(s, 0) + 32u * ks), alo = sw128_desc(a_addr(s, 1) + 32u * ks);
                    const uint64_t bh = sw128_desc(b_addr(s, 0) + 32u * ks), blo = sw128_desc(b_addr(s, 1) + 32u * ks);
                    mma_tf32(d, ah, bh, idesc, ks > 0 ? 1u : 0u);
                    mma_tf32(d, ah, blo, idesc, 1u);
                    mma_tf32(d, alo, bh, idesc, 1u);
                }
                mma_commit(empty(s));
                if (slot == kTcBatch - 1 || j == nmm - 1) mma_commit(acc_full);
            }
        }
        __syncwarp();
    } else {
        // ---- epilogue: warp w reads TMEM lanes 32w..32w+31 (rows)
        const int row = 32 * warp + lane, p = row & 63, part = row >> 6;
        const bool valid = p < npairs;
        const uint32_t lrow = tbase + ((uint32_t)(32 * warp) << 16);
        const int ncol = 2 * G, W2 = W * W;
        const long long R = 2LL * npairs;   // rows per (col, mm)
        float *base = S + T.s0 + (part * npairs + p);
        const int nbatch = (nmm + kTcBatch - 1) / kTcBatch;
        for (int q = 0; q < nbatch; ++q) {
            if (!mbar_wait(acc_full, q & 1, abort)) { give_up(); break; }
            tc_fence_after();
            const int nb = min(kTcBatch, nmm - kTcBatch * q), mmq = it.mm0 + kTcBatch * q;
            for (int cc = 0; cc < ncol; cc += 16) {
                uint32_t v0[16], v1[16], v2[16], v3[16];
                tmem_ld16(lrow + (uint32_t)(0 * Nr + cc), v0);
                tmem_ld16(lrow + (uint32_t)(1 * Nr + cc), v1);
                tmem_ld16(lrow + (uint32_t)(2 * Nr + cc), v2);
                tmem_ld16(lrow + (uint32_t)(3 * Nr + cc), v3);
                tmem_ld_wait();
                if (valid) {
#pragma unroll
                    for (int c = 0; c < 16; ++c) {
                        const int col = cc + c;
                        if (col < ncol) {
                            float *dst = base + ((long long)col * W2 + mmq) * R;
                            dst[0] = __uint_as_float(v0[c]);
                            if (nb > 1) dst[R] = __uint_as_float(v1[c]);
                            if (nb > 2) dst[2 * R] = __uint_as_float(v2[c]);
                            if (nb > 3) dst[3 * R] = __uint_as_float(v3[c]);
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(acc_empty);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 8) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tbase), "r"(tmem_cols) : "memory");
    }
}

// ---------------------------------------------------------------------------
// FFT stage: one block per (beta index k, group of up to four pairs of a
// tile).  For every mm the group's real and imaginary rows of both
// orientations' columns are contiguous (4 runs of npg floats); they are
// scattered into each pair's (m1, m2) planes, then each pair goes through the
// transform tail shared with k_isoft.
__global__ void __launch_bounds__(256) k_isoft_tc(const PairDev *pairs, const TcFftGroup *groups, const float *S,
                                                  float *grid) {
    extern __shared__ __align__(16) unsigned char smem_fft[];
    const int k = blockIdx.x;
    const TcFftGroup Gr = groups[blockIdx.y];
    const int L = Gr.L, G = 2 * (L + 1), Wc = 2 * L + 1, W2 = Wc * Wc, npg = Gr.npg;
    if (k >= G) return;
    const int PL = isoft_plane(G), ld = isoft_ld(G);
    float2 *planes = (float2 *)smem_fft;   // pair q: A at 3q PL, Z at (3q + 1) PL, C at (3q + 2) PL
    float2 *tw = planes + 3 * npg * PL;
    for (int t = threadIdx.x; t < G; t += blockDim.x) {
        float sn, cs;
        sincospif(2.0f * t / G, &sn, &cs);
        tw[t] = make_float2(cs, sn);
    }
    for (int q = 0; q < npg; ++q)
        for (int t = threadIdx.x; t < PL; t += blockDim.x) {
            planes[3 * q * PL + t] = make_float2(0.f, 0.f);
            planes[(3 * q + 2) * PL + t] = make_float2(0.f, 0.f);
        }
    __syncthreads();
    const long long R = 2LL * Gr.ntile;
    const float *c0 = S + Gr.s0 + (long long)k * W2 * R + Gr.p0;        // column k (direct)
    const float *c1 = S + Gr.s0 + (long long)(G + k) * W2 * R + Gr.p0;  // column G + k (inverted)
    for (int t = threadIdx.x; t < W2 * npg; t += blockDim.x) {
        const int mm = t / npg, q = t % npg;
        const int i1 = mm / Wc, i2 = mm % Wc;
        const int m1 = (i1 <= L) ? i1 : i1 - Wc, m2 = (i2 <= L) ? i2 : i2 - Wc;
        const int dst = ((m1 + G) % G) * ld + (m2 + G) % G;
        const long long o = (long long)mm * R + q;
        planes[3 * q * PL + dst] = make_float2(c0[o], c0[o + Gr.ntile]);
        planes[(3 * q + 2) * PL + dst] = make_float2(c1[o], c1[o + Gr.ntile]);
    }
    __syncthreads();
    for (int q = 0; q < npg; ++q) {
        const PairDev &P = pairs[Gr.pair[q]];
        isoft_tail<float, float2>(planes + 3 * q * PL, planes + (3 * q + 1) * PL, planes + (3 * q + 2) * PL, tw, G,
                                  k, P.norient == 2, grid + P.grid0);
    }
}

// ---------------------------------------------------------------------------
// host side

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    return fn;
}

int pow2_at_least(int x) {
    int p = 32;
    while (p < x) p *= 2;
    return p;
}

// Dynamic shared memory of one CTA and its tensor-memory columns; the shared
// memory is raised when needed so that the CTAs resident on an SM never ask
// for more than the 512 columns there are.
void tc_footprint(int nrmax, size_t *smem, int *cols) {
    *cols = pow2_at_least(kTcBatch * nrmax);
    size_t sm = 1024 + 2ull * kTcStages * kTcABytes + 2ull * kTcStages * nrmax * kTcRowBytes;
    const size_t per_sm = 228 * 1024, reserved = 1024 + 4096;   // per-CTA reservation and static smem
    while ((int)(per_sm / (sm + reserved)) * (*cols) > 512) sm += 8 * 1024;
    *smem = sm;
}

}  // namespace

int tc_rows(int bw) { return ((4 * bw + 15) / 16) * 16; }

size_t tc_table_floats(int bw) {
    const int W = 2 * bw - 1;
    return 2ull * W * W * tc_rows(bw) * 32;
}

bool tc_make_table(int bw, const double *d64, float *out, CUtensorMap *map, cudaStream_t s) {
    const int Nr = tc_rows(bw), W = 2 * bw - 1;
    const long long n = (long long)W * W * Nr * 32;
    k_wigner_tc_table<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(bw, d64, out, Nr);
    EncodeTiledFn enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[2] = {32, (cuuint64_t)2 * W * W * Nr};
    const cuuint64_t strides[1] = {32 * sizeof(float)};
    const cuuint32_t box[2] = {32, (cuuint32_t)Nr};
    const cuuint32_t estr[2] = {1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, out, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

void launch_wigner_tc(const TcBuffers &b, cudaStream_t s) {
    allow_max_smem<k_wigner_tc>();
    for (const TcLaunch &lg : b.launches) {
        size_t sm;
        int cols;
        tc_footprint(lg.nrmax, &sm, &cols);
        k_wigner_tc<<<lg.nitems, kTcThreads, sm, s>>>(lg.maps, b.tiles, b.items + lg.item0, (const float2 *)b.coef,
                                                       b.S, cols, lg.nrmax, b.err);
    }
}

size_t tc_fft_smem(int G, int npg) { return sizeof(float2) * (3ull * npg * isoft_plane(G) + G); }

void launch_isoft_tc(const TcBuffers &b, cudaStream_t s) {
    allow_max_smem<k_isoft_tc>();
    k_isoft_tc<<<dim3(b.maxG, b.ngroups), 256, b.fft_smem, s>>>(b.pairs, b.groups, b.S, (float *)b.grid);
}

}  // namespace fo
