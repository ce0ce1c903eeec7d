// fo_coef_tc.cu -- the SO(3) overlap-coefficient contraction on the tcgen05
// tensor cores (mixed form).
//
// Reference behaviour (matthewghgriffiths/fastoverlap): FOURIERCOEFFS
// fastoverlap/f90/fastclusters.f90:868-916, the pair loop :905-911
// (calcSO3Coeffs sphericalAlignment.py:260-273 in the Python path):
//   I^l[m1][m2] = sum_groups sum_{a, b} YB_l[m1](b) W_l(b, a) conj(YA_l[m2](a))
// with W_l(b, a) the radial weight of atom a of structure A and atom b of
// structure B in the same permutation group.
//
// GEMM form, one CTA per (l, pair).  For every group of the pair and every
// tile of 32 atoms a of structure A:
//   GEMM1   D1[c][a] = sum_b A1[c][b] B1[a][b]          P = YB_l W_l
//           c = 2i + p: i = m1 + l, p = 0 real / 1 imaginary part of YB_l[m1](b)
//           (M = 128 rows, 2(2l+1) of them live), N = 32 atoms a, K = atoms b
//           in stages of 32
//   GEMM2   D2[c][c'] += sum_a P_c(a) YA_c'(a)             I = P YA_l^H
//           A operand: P itself, read from tensor memory; B operand: YA_l
//           (c' = 2i' + p' as above) from shared memory; D2 accumulates over
//           all tiles and groups of the pair
//   Re I[i][i'] = D2[2i][2i'] + D2[2i+1][2i'+1],  Im I[i][i'] = D2[2i+1][2i'] - D2[2i][2i'+1]
// Both products run as kind::tf32 MMAs in 3xTF32 (x = hi + lo with hi the
// value rounded to TF32; D += hi*hi + hi*lo + lo*hi), FP32 accumulators in
// tensor memory, so the sums keep FP32-like accuracy.
//
// Inputs come in the layouts the mixed form's producers write for this
// kernel: Y_lm per pair as [lm][atom] (atom fastest), radial weights per
// group as [l][a][b] (b fastest), so every staged row of K values is a
// contiguous run in global memory.
//
// Roles (288 threads): warps 0-3 convert D1 into the TF32 hi/lo halves of P
// (warp w owns tensor-memory lanes 32w..32w+31), stage YA_l for GEMM2 and
// write the coefficients at the end; warps 4-7 stage A1 (YB_l) and B1
// (W_l) per K stage; one thread of warp 8 issues the MMAs.  Rows of A1 past
// 2(2l+1) feed only rows of D1 and D2 that are never read, so for Jmax <= 15
// the A1 buffers hold 64 rows and the MMA's other 64 rows read whatever lies
// next in shared memory.  Every mbarrier wait is bounded (about two
// seconds); a wait that runs out sets *err, the CTA drains its MMAs, frees
// its tensor memory and returns, and the host reports FO_ERR_CUDA.
#include "fo_common.cuh"
#include "fo_kernels.h"
#include "fo_tc.cuh"

namespace fo {

namespace {

using namespace tc;

constexpr int kCtThreads = 288;
constexpr int kCtTile = 32;          // atoms a per tile (GEMM1 N, GEMM2 K)
constexpr int kCtK = 32;             // atoms b per GEMM1 stage
constexpr int kCtB1Bytes = kCtTile * 128;
constexpr int kCtAUnits = 4;        // A1 staging units per producer thread: (2l+1) rows x 8 chunks <= 4 x 128
constexpr int kCtCols = 256;         // tensor memory per CTA
constexpr int kD2 = 0, kD1 = 128, kH = 192, kLo = 224;   // columns: D2 (<= 128), D1 [2] (32 each), P hi, P lo

// x = hi + lo with both halves rounded to TF32 (the tensor cores would
// otherwise truncate lo), so each product of the split keeps about 2^-22 of
// relative error.
__device__ __forceinline__ void split4(const float (&v)[4], float4 &h, float4 &lo) {
    h.x = tf32_round(v[0]); lo.x = tf32_round(v[0] - h.x);
    h.y = tf32_round(v[1]); lo.y = tf32_round(v[1] - h.y);
    h.z = tf32_round(v[2]); lo.z = tf32_round(v[2] - h.z);
    h.w = tf32_round(v[3]); lo.w = tf32_round(v[3] - h.w);
}

// Rows 2i (real parts) and 2i+1 (imaginary parts) of a Y_l operand for the
// K values k0..k0+3 (chunk q of the 128-byte row): four complex values of
// one lm, consecutive atoms; atoms at or past n are zero.
__device__ __forceinline__ void stage_y(const float2 *__restrict__ y, int k0, int n, int i, int q,
                                        unsigned char *hi, unsigned char *lo) {
    float re[4], im[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        float2 v = make_float2(0.f, 0.f);
        if (k0 + e < n) v = y[k0 + e];
        re[e] = v.x;
        im[e] = v.y;
    }
    float4 h, l;
    split4(re, h, l);
    *reinterpret_cast<float4 *>(hi + sw128_off(2 * i, q)) = h;
    *reinterpret_cast<float4 *>(lo + sw128_off(2 * i, q)) = l;
    split4(im, h, l);
    *reinterpret_cast<float4 *>(hi + sw128_off(2 * i + 1, q)) = h;
    *reinterpret_cast<float4 *>(lo + sw128_off(2 * i + 1, q)) = l;
}

}  // namespace

__global__ void __launch_bounds__(kCtThreads, 2)
    k_coef_tc(const PairDev *__restrict__ pairs, const GroupDev *__restrict__ groups, const float2 *__restrict__ ytA,
              const float2 *__restrict__ ytB, const float *__restrict__ wt, float2 *__restrict__ coef, int n2max,
              int a1bytes, int *err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t bars[11];
    __shared__ uint32_t tmem_base_sh;
    __shared__ int abort_sh;

    const int l = blockIdx.x;
    const PairDev P = pairs[blockIdx.y];
    if (l > P.L) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ni = 2 * l + 1, live = 2 * ni, N2 = ((live + 15) / 16) * 16, Wc = 2 * P.L + 1;
    const long long yoff = P.ylm0 + (long long)(l * l) * P.n;   // row i of Y_l: yoff + i * n_pair + atom
    const uint32_t idesc1 = tf32_idesc(128, kCtTile), idesc2 = tf32_idesc(128, N2);

    // 1024-aligned carve: A1[stage][hi|lo], B1[stage][hi|lo], B2[hi|lo], then
    // the converters' FP32 sums of D2, [column][thread]
    const uint32_t sbase = (smem_u32(smem_raw) + 1023u) & ~1023u;
    unsigned char *gbase = smem_raw + (sbase - smem_u32(smem_raw));
    const uint32_t b1base = sbase + 4u * (uint32_t)a1bytes, b2base = b1base + 4u * kCtB1Bytes;
    const uint32_t b2bytes = (uint32_t)n2max * 128u;
    auto a1_addr = [&](int s, int h) { return sbase + (uint32_t)(2 * s + h) * (uint32_t)a1bytes; };
    auto b1_addr = [&](int s, int h) { return b1base + (uint32_t)(2 * s + h) * kCtB1Bytes; };
    auto b2_addr = [&](int h) { return b2base + (uint32_t)h * b2bytes; };
    auto gen = [&](uint32_t a) { return gbase + (a - sbase); };
    float *accs = reinterpret_cast<float *>(gen(b2base + 2u * b2bytes));
    auto full = [&](int s) { return smem_u32(&bars[s]); };
    auto empty = [&](int s) { return smem_u32(&bars[2 + s]); };
    auto d1full = [&](int s) { return smem_u32(&bars[4 + s]); };
    auto d1free = [&](int s) { return smem_u32(&bars[6 + s]); };
    const uint32_t conv = smem_u32(&bars[8]), d2full = smem_u32(&bars[9]), drain = smem_u32(&bars[10]);

    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            mbar_init(full(s), 128);
            mbar_init(empty(s), 1);
            mbar_init(d1full(s), 1);
            mbar_init(d1free(s), 128);
        }
        mbar_init(conv, 128);
        mbar_init(d2full, 1);
        mbar_init(drain, 1);
        abort_sh = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // rows of A1 at and past `live` (up to the 64 or 128 rows a buffer holds) are zero
    {
        const int rows = a1bytes / 128;
        for (int t = tid; t < 4 * (rows - live) * 8; t += kCtThreads) {
            const int buf = t / ((rows - live) * 8), r = live + (t / 8) % (rows - live), q = t % 8;
            *reinterpret_cast<float4 *>(gen(sbase + (uint32_t)buf * a1bytes) + sw128_off(r, q)) =
                make_float4(0.f, 0.f, 0.f, 0.f);
        }
        fence_async_smem();
    }
    if (warp == 8) tmem_alloc(smem_u32(&tmem_base_sh), kCtCols);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tbase = tmem_base_sh;
    volatile int *abort = &abort_sh;
    auto give_up = [&]() {
        *abort = 1;
        atomicOr(err, 1);
    };

    if (warp >= 4 && warp < 8) {
        // ---- producers: A1 = YB_l rows, B1 = W_l rows of the a tile, per K
        // stage of 32 atoms b.  The next stage's values are loaded into
        // registers before the wait for its buffer, so the global loads of
        // one stage overlap the hand-over of the previous one.
        const int r = tid - 128;
        int j = 0;
        float2 ya[kCtAUnits][4];
        float wb[2][4];
        // stage (group gi, tile a0, chunk kc) -> registers
        auto load = [&](const GroupDev &g, int a0, int kc) {
            const int n = g.n, k0 = kc * kCtK;
            const float2 *yb = ytB + yoff + (g.slot0 - P.atom0);
            const float *w = wt + g.w0 + (long long)l * n * n;
#pragma unroll
            for (int x = 0; x < kCtAUnits; ++x) {
                const int u = r + 128 * x, i = u >> 3, b = k0 + 4 * (u & 7);
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    ya[x][e] = (u < ni * 8 && b + e < n) ? yb[(long long)i * P.n + b + e] : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                const int u = r + 128 * x, a = a0 + (u >> 3), b = k0 + 4 * (u & 7);
#pragma unroll
                for (int e = 0; e < 4; ++e) wb[x][e] = (a < n && b + e < n) ? w[(long long)a * n + b + e] : 0.f;
            }
        };
        // the stage sequence: groups, a tiles, K chunks
        int gi = 0, a0 = 0, kc = 0;
        GroupDev g = groups[P.group0];
        load(g, a0, kc);
        for (;;) {
            const int s = j & 1;
            if (j >= 2 && !mbar_wait(empty(s), ((j >> 1) - 1) & 1, abort)) { give_up(); break; }
            unsigned char *ah = gen(a1_addr(s, 0)), *al = gen(a1_addr(s, 1));
#pragma unroll
            for (int x = 0; x < kCtAUnits; ++x) {
                const int u = r + 128 * x, i = u >> 3, q = u & 7;
                if (u < ni * 8) {
                    float re[4], im[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) { re[e] = ya[x][e].x; im[e] = ya[x][e].y; }
                    float4 h, lo;
                    split4(re, h, lo);
                    *reinterpret_cast<float4 *>(ah + sw128_off(2 * i, q)) = h;
                    *reinterpret_cast<float4 *>(al + sw128_off(2 * i, q)) = lo;
                    split4(im, h, lo);
                    *reinterpret_cast<float4 *>(ah + sw128_off(2 * i + 1, q)) = h;
                    *reinterpret_cast<float4 *>(al + sw128_off(2 * i + 1, q)) = lo;
                }
            }
            unsigned char *bh = gen(b1_addr(s, 0)), *bl = gen(b1_addr(s, 1));
#pragma unroll
            for (int x = 0; x < 2; ++x) {
                const int u = r + 128 * x;
                float4 h, lo;
                split4(wb[x], h, lo);
                *reinterpret_cast<float4 *>(bh + sw128_off(u >> 3, u & 7)) = h;
                *reinterpret_cast<float4 *>(bl + sw128_off(u >> 3, u & 7)) = lo;
            }
            fence_async_smem();   // generic-proxy stores -> visible to the tensor cores
            mbar_arrive(full(s));
            ++j;
            // advance to the next stage and prefetch it
            if (++kc == (g.n + kCtK - 1) / kCtK) {
                kc = 0;
                a0 += kCtTile;
                if (a0 >= g.n) {
                    a0 = 0;
                    if (++gi == P.ngroups) break;
                    g = groups[P.group0 + gi];
                }
            }
            load(g, a0, kc);
        }
    } else if (warp == 8) {
        // ---- MMA issuer (one thread).  Each accumulator in tensor memory takes
        // one K stage (GEMM1) or one a tile (GEMM2), at most 12 MMAs; the
        // longer sums are carried in FP32 by the converters.
        if (lane == 0) {
            int j = 0, t = 0;
            bool ok = true;
            for (int gi = 0; gi < P.ngroups && ok; ++gi) {
                const int n = groups[P.group0 + gi].n, nk = (n + kCtK - 1) / kCtK;
                for (int a0 = 0; a0 < n && ok; a0 += kCtTile, ++t) {
                    for (int kc = 0; kc < nk; ++kc, ++j) {
                        const int s = j & 1;
                        if (!mbar_wait(full(s), (j >> 1) & 1, abort) ||
                            (j >= 2 && !mbar_wait(d1free(s), ((j >> 1) - 1) & 1, abort))) {
                            give_up();
                            ok = false;
                            break;
                        }
                        fence_after();
                        const uint32_t d1 = tbase + kD1 + 32u * s;
                        const int nks = min(4, (n - kc * kCtK + 7) / 8);
                        for (int ks = 0; ks < nks; ++ks) {
                            const uint64_t ah = sw128_desc(a1_addr(s, 0) + 32u * ks);
                            const uint64_t al = sw128_desc(a1_addr(s, 1) + 32u * ks);
                            const uint64_t bh = sw128_desc(b1_addr(s, 0) + 32u * ks);
                            const uint64_t bl = sw128_desc(b1_addr(s, 1) + 32u * ks);
                            mma_tf32(d1, ah, bh, idesc1, ks > 0 ? 1u : 0u);
                            mma_tf32(d1, ah, bl, idesc1, 1u);
                            mma_tf32(d1, al, bh, idesc1, 1u);
                        }
                        mma_commit(empty(s));
                        mma_commit(d1full(s));
                    }
                    if (!ok) break;
                    // GEMM2 of this tile, once the converters have P in H/Lo and YA_l in B2
                    if (!mbar_wait(conv, t & 1, abort)) { give_up(); ok = false; break; }
                    fence_after();
                    const int nks = (min(kCtTile, n - a0) + 7) / 8;
                    for (int ks = 0; ks < nks; ++ks) {
                        const uint32_t ah = tbase + kH + 8u * ks, alo = tbase + kLo + 8u * ks;
                        const uint64_t bh = sw128_desc(b2_addr(0) + 32u * ks);
                        const uint64_t bl = sw128_desc(b2_addr(1) + 32u * ks);
                        mma_tf32_ts(tbase + kD2, ah, bh, idesc2, ks > 0 ? 1u : 0u);
                        mma_tf32_ts(tbase + kD2, ah, bl, idesc2, 1u);
                        mma_tf32_ts(tbase + kD2, alo, bh, idesc2, 1u);
                    }
                }
            }
            if (ok) mma_commit(d2full);
            // drain: every MMA issued has completed before the tensor memory is freed
            mma_commit(drain);
            const unsigned long long t0 = gtimer();
            while (!mbar_try(drain, 0) && (long long)(gtimer() - t0) < kWaitNs) {
            }
        }
        __syncwarp();
    } else {
        // ---- converters (thread = tensor-memory lane = row c of D1 and D2):
        // P summed over the K stages in FP32 registers, split into TF32 hi/lo
        // in tensor memory for GEMM2; YA_l into B2; D2 of each tile summed in
        // FP32 in shared memory; the coefficients at the end.
        const uint32_t lrow = (uint32_t)(32 * warp) << 16;
        const bool rows_live = 32 * warp < live;
        int t = 0, j = 0;
        bool ok = true;
        auto fold_d2 = [&](bool first) {   // accs (+)= D2 of the tile GEMM2 has just finished
            for (int c0 = 0; c0 < N2; c0 += 16) {
                uint32_t v[16];
                tmem_ld16(tbase + lrow + kD2 + (uint32_t)c0, v);
                tmem_ld_wait();
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    float *a = accs + (c0 + e) * 128 + tid;
                    *a = first ? __uint_as_float(v[e]) : *a + __uint_as_float(v[e]);
                }
            }
        };
        for (int gi = 0; gi < P.ngroups && ok; ++gi) {
            const GroupDev g = groups[P.group0 + gi];
            const int n = g.n, nk = (n + kCtK - 1) / kCtK;
            const float2 *ya = ytA + yoff + (g.slot0 - P.atom0);
            for (int a0 = 0; a0 < n && ok; a0 += kCtTile, ++t) {
                float acc1[32];
                for (int kc = 0; kc < nk; ++kc, ++j) {
                    const int s = j & 1;
                    if (!mbar_wait(d1full(s), (j >> 1) & 1, abort)) { give_up(); ok = false; break; }
                    fence_after();
                    if (rows_live) {
                        uint32_t v0[16], v1[16];
                        tmem_ld16(tbase + lrow + kD1 + 32u * s, v0);
                        tmem_ld16(tbase + lrow + kD1 + 32u * s + 16u, v1);
                        tmem_ld_wait();
#pragma unroll
                        for (int e = 0; e < 16; ++e) {
                            acc1[e] = kc ? acc1[e] + __uint_as_float(v0[e]) : __uint_as_float(v0[e]);
                            acc1[16 + e] = kc ? acc1[16 + e] + __uint_as_float(v1[e]) : __uint_as_float(v1[e]);
                        }
                    }
                    fence_before();
                    mbar_arrive(d1free(s));
                }
                if (!ok) break;
                // GEMM2 of the previous tile was issued before this tile's
                // stages, so it has completed: fold its D2, then hand over P
                if (rows_live) {
                    if (t > 0) fold_d2(t == 1);
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        uint32_t vh[16], vl[16];
#pragma unroll
                        for (int e = 0; e < 16; ++e) {
                            const float x = acc1[16 * h + e], hi = tf32_round(x);
                            vh[e] = __float_as_uint(hi);
                            vl[e] = __float_as_uint(tf32_round(x - hi));
                        }
                        tmem_st16(tbase + lrow + kH + 16u * h, vh);
                        tmem_st16(tbase + lrow + kLo + 16u * h, vl);
                    }
                    tmem_st_wait();
                }
                unsigned char *bh = gen(b2_addr(0)), *bl = gen(b2_addr(1));
                for (int u = tid; u < ni * 8; u += 128) {
                    const int i = u >> 3, q = u & 7;
                    stage_y(ya + (long long)i * P.n, a0 + 4 * q, n, i, q, bh, bl);
                }
                fence_async_smem();
                fence_before();
                mbar_arrive(conv);
            }
        }
        if (ok && mbar_wait(d2full, 0, abort)) {
            fence_after();
            if (rows_live) {
                fold_d2(t == 1);
                __syncwarp();
                const int c = 32 * warp + lane, i = c >> 1, p = c & 1;
                const float sgn = p ? -1.f : 1.f;
                if (c < live) {
                    const int i1 = (i - l + Wc) % Wc;
                    float *out = reinterpret_cast<float *>(coef + P.coef0 + (long long)(l * Wc + i1) * Wc);
                    for (int ip = 0; ip < ni; ++ip)
                        out[2 * ((ip - l + Wc) % Wc) + p] =
                            accs[(2 * ip) * 128 + tid] + sgn * accs[(2 * ip + 1) * 128 + (tid ^ 1)];
                }
            }
        } else if (ok) {
            give_up();
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 8) {
        fence_after();
        tmem_dealloc(tbase, kCtCols);
    }
}

// Launch over (l, pair); the plan's Jmax decides the shared-memory carve.
void launch_coef_tc(const SphBuffers &b, int *err, cudaStream_t s) {
    const int n2max = ((2 * (2 * b.maxL + 1) + 15) / 16) * 16;
    const int a1bytes = b.maxL <= 15 ? 64 * 128 : 128 * 128;
    const size_t sm = 1024 + 4ull * a1bytes + 4ull * kCtB1Bytes + 2ull * n2max * 128 + 128ull * n2max * 4;
    allow_max_smem<k_coef_tc>();
    k_coef_tc<<<dim3(b.maxL + 1, b.npairs), kCtThreads, sm, s>>>(b.pairs, b.groups, (const float2 *)b.ylmA,
                                                                (const float2 *)b.ylmB, (const float *)b.W,
                                                                (float2 *)b.coef, n2max, a1bytes, err);
}

}  // namespace fo
