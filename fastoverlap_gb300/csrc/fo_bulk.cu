// fo_bulk.cu -- periodic (bulk) front end: structure factors on the
// (2K+1)^3 wave-vector grid, damped cross product summed over permutation
// groups, 3-D forward FFT of the zero-padded M^3 array and its modulus.
//
// Reference behaviour (matthewghgriffiths/fastoverlap):
//   SETWAVEK            fastoverlap/f90/fastbulk.f90:567-597
//   PERIODICFOURIER(PERM) fastoverlap/f90/fastbulk.f90:599-665
//   damping + DOTFOURIERCOEFFS fastoverlap/f90/fastbulk.f90:441-454,667-683
//   FFT3D + ABS         fastoverlap/f90/fastutils.f90:554-569, fastbulk.f90:522-523
//   (Python: PeriodicAlign.setPos, fastoverlap/periodicAlignment.py:408-440)
#include "fo_common.cuh"
#include "fo_kernels.h"

namespace fo {

// gather slot-ordered copies of both structures (no centring for bulk)
__global__ void k_bulk_prep(const PairDev *pairs, const int *slot2orig, const double *pos1,
                            const double *pos2, double *xa, double *xb) {
    const PairDev &P = pairs[blockIdx.x];
    for (int s = threadIdx.x; s < P.n; s += blockDim.x) {
        int o = slot2orig[P.atom0 + s];
        for (int k = 0; k < 3; ++k) {
            xa[3LL * (P.atom0 + s) + k] = pos2[3LL * (P.atom0 + o) + k];
            xb[3LL * (P.atom0 + s) + k] = pos1[3LL * (P.atom0 + o) + k];
        }
    }
}

// F(k) = sum_groups C^B(k) conj(C^A(k)) exp(-|k|^2 s^2), C(k) = sum_j exp(-i k.r_j),
// written at [ix + M(iy + M iz)] of the M^3 grid.  The phase factor separates,
// exp(-i k.r) = e_x(ix) e_y(iy) e_z(iz) with e_a(i) = exp(-i 2 pi (i-K) r_a / L_a),
// so a block -- one z wave number iz and a slab of up to kSfPer*256 (ix, iy)
// wave vectors -- computes each atom's 2(2K+1)+1 axis factors once into
// shared memory (chunks of atoms) and every wave vector then costs two complex
// products per atom.  Factors come from sincos in the grid precision T.
constexpr int kSfThreads = 256, kSfPer = 4, kSfSlab = kSfThreads * kSfPer;
constexpr int kSfSmem = 48 * 1024;   // dynamic shared memory of every k_bulk_sf block

__host__ __device__ inline int sf_chunk(int nk, int tsize) {
    // atoms per shared-memory chunk: both structures, 2nk+1 complex factors
    // each, within kSfSmem for every nk (so pairs of any K share one launch)
    int c = kSfSmem / (2 * (2 * nk + 1) * 2 * tsize);
    return c < 1 ? 1 : (c > 64 ? 64 : c);
}

template <typename T, typename T2>
__global__ void __launch_bounds__(kSfThreads) k_bulk_sf(const PairDev *pairs, const GroupDev *groups,
                                                        const double *xa, const double *xb, T2 *fgrid,
                                                        int nslab) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const PairDev &P = pairs[blockIdx.y];
    const int K = P.L, nk = 2 * K + 1, M = P.G, nf = 2 * nk + 1;
    const int iz = blockIdx.x / nslab, slab = blockIdx.x % nslab;
    if (iz >= nk || slab * kSfSlab >= nk * nk) return;
    const int chunk = sf_chunk(nk, (int)sizeof(T));
    T2 *fac = (T2 *)smem_raw;   // [side][atom][factor]: x factors 0..nk-1, y nk..2nk-1, z 2nk
    const double twopi_l[3] = {2.0 * FO_PI / P.box[0], 2.0 * FO_PI / P.box[1], 2.0 * FO_PI / P.box[2]};
    int ixy[kSfPer];
#pragma unroll
    for (int q = 0; q < kSfPer; ++q) {
        const int w = slab * kSfSlab + q * kSfThreads + threadIdx.x;
        ixy[q] = w < nk * nk ? w : -1;
    }
    T fr[kSfPer], fi[kSfPer];
#pragma unroll
    for (int q = 0; q < kSfPer; ++q) fr[q] = fi[q] = 0;
    for (int gi = 0; gi < P.ngroups; ++gi) {
        const GroupDev g = groups[P.group0 + gi];
        T ar[kSfPer], ai[kSfPer], br[kSfPer], bi[kSfPer];
#pragma unroll
        for (int q = 0; q < kSfPer; ++q) ar[q] = ai[q] = br[q] = bi[q] = 0;
        for (int j0 = 0; j0 < g.n; j0 += chunk) {
            const int nj = min(chunk, g.n - j0);
            __syncthreads();   // the previous chunk's factors are no longer read
            for (int t = threadIdx.x; t < 2 * nj * nf; t += blockDim.x) {
                const int side = t / (nj * nf), r = t % (nj * nf), jj = r / nf, w = r % nf;
                const double *X = (side ? xb : xa) + 3LL * (g.slot0 + j0 + jj);
                const int axis = w < nk ? 0 : (w < 2 * nk ? 1 : 2);
                const int m = (axis == 0 ? w : (axis == 1 ? w - nk : iz)) - K;
                const double ph = twopi_l[axis] * m * X[axis];
                T sn, cs;
                if constexpr (sizeof(T) == 4) sincosf((float)ph, &sn, &cs);
                else sincos(ph, &sn, &cs);
                fac[(side * chunk + jj) * nf + w] = pack2<T2, T>(cs, -sn);
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < kSfPer; ++q) {
                if (ixy[q] < 0) continue;
                const int ix = ixy[q] % nk, iy = ixy[q] / nk;
                for (int jj = 0; jj < nj; ++jj) {
                    const T2 *fa = fac + jj * nf, *fb = fac + (chunk + jj) * nf;
                    const T2 ea = cmul(cmul(fa[ix], fa[nk + iy]), fa[2 * nk]);
                    const T2 eb = cmul(cmul(fb[ix], fb[nk + iy]), fb[2 * nk]);
                    ar[q] += ea.x; ai[q] += ea.y;
                    br[q] += eb.x; bi[q] += eb.y;
                }
            }
        }
        // C^B * conj(C^A)
#pragma unroll
        for (int q = 0; q < kSfPer; ++q) {
            fr[q] += br[q] * ar[q] + bi[q] * ai[q];
            fi[q] += bi[q] * ar[q] - br[q] * ai[q];
        }
    }
#pragma unroll
    for (int q = 0; q < kSfPer; ++q) {
        if (ixy[q] < 0) continue;
        const int ix = ixy[q] % nk, iy = ixy[q] / nk;
        const double kx = twopi_l[0] * (ix - K), ky = twopi_l[1] * (iy - K), kz = twopi_l[2] * (iz - K);
        const double damp = exp(-(kx * kx + ky * ky + kz * kz) * P.sigma * P.sigma);
        fgrid[P.coef0 + ix + (long long)M * (iy + (long long)M * iz)] =
            pack2<T2, T>(T(fr[q] * damp), T(fi[q] * damp));
    }
}

// One pass of the 3-D FFT: forward 1-D transforms along `axis` for a batch
// of kLines lines per block; the last pass writes the modulus to the real grid.
constexpr int kLines = 16;

template <typename T, typename T2>
__global__ void __launch_bounds__(256) k_bulk_fft_axis(const PairDev *pairs, T2 *fgrid, T *grid,
                                                       int axis, int last) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const PairDev &P = pairs[blockIdx.y];
    const int M = P.G;
    const int l0 = blockIdx.x * kLines;
    if (l0 >= M * M) return;
    const int nl = min(kLines, M * M - l0);
    T2 *bufA = (T2 *)smem_raw, *bufB = bufA + kLines * M, *tw = bufB + kLines * M;
    for (int t = threadIdx.x; t < M; t += blockDim.x) {
        double sn, cs;
        sincospi(2.0 * t / M, &sn, &cs);
        tw[t] = mk2<T2>(cs, sn);
    }
    T2 *F = fgrid + P.coef0;
    const long long st = axis == 0 ? 1 : (axis == 1 ? M : (long long)M * M);
    auto base_of = [&](int line) -> long long {
        int u = line % M, w = line / M;
        if (axis == 0) return (long long)M * (u + (long long)M * w);
        if (axis == 1) return u + (long long)M * M * w;
        return u + (long long)M * w;
    };
    for (int t = threadIdx.x; t < nl * M; t += blockDim.x) {
        int l = t / M, e = t % M;
        bufA[l * M + e] = F[base_of(l0 + l) + st * e];
    }
    __syncthreads();
    T2 *r = fft_lines(bufA, bufB, M, nl, M, 1, -1, tw);
    for (int t = threadIdx.x; t < nl * M; t += blockDim.x) {
        int l = t / M, e = t % M;
        long long idx = base_of(l0 + l) + st * e;
        T2 v = r[l * M + e];
        if (last) grid[P.grid0 + idx] = sqrt(v.x * v.x + v.y * v.y);
        else F[idx] = v;
    }
}

void launch_bulk_prep(const BulkBuffers &b, cudaStream_t s) {
    k_bulk_prep<<<b.npairs, 256, 0, s>>>(b.pairs, b.slot2orig, b.pos1, b.pos2, b.xa, b.xb);
}

void launch_bulk_sf(const BulkBuffers &b, bool fp32, cudaStream_t s) {
    const int nk = 2 * b.maxK + 1, nslab = (nk * nk + kSfSlab - 1) / kSfSlab;
    dim3 grid(nk * nslab, b.npairs);
    // one chunk of any pair's factors fits kSfSmem (nk <= 2K+1 <= M <= 256, so
    // even a single atom's 2(2nk+1) FP64 factors take at most 16 KB)
    if (fp32)
        k_bulk_sf<float, float2><<<grid, kSfThreads, kSfSmem, s>>>(b.pairs, b.groups, b.xa, b.xb,
                                                                  (float2 *)b.fgrid, nslab);
    else
        k_bulk_sf<double, double2><<<grid, kSfThreads, kSfSmem, s>>>(b.pairs, b.groups, b.xa, b.xb,
                                                                    (double2 *)b.fgrid, nslab);
}

void launch_bulk_fft(const BulkBuffers &b, bool fp32, cudaStream_t s) {
    dim3 grid((b.maxM * b.maxM + kLines - 1) / kLines, b.npairs);
    for (int axis = 0; axis < 3; ++axis) {
        if (fp32) {
            size_t sm = sizeof(float2) * (2 * kLines * b.maxM + b.maxM);
            allow_max_smem<k_bulk_fft_axis<float, float2>>();
            k_bulk_fft_axis<float, float2><<<grid, 256, sm, s>>>(b.pairs, (float2 *)b.fgrid,
                                                                (float *)b.grid, axis, axis == 2);
        } else {
            size_t sm = sizeof(double2) * (2 * kLines * b.maxM + b.maxM);
            allow_max_smem<k_bulk_fft_axis<double, double2>>();
            k_bulk_fft_axis<double, double2><<<grid, 256, sm, s>>>(b.pairs, (double2 *)b.fgrid,
                                                                  (double *)b.grid, axis, axis == 2);
        }
    }
}

}  // namespace fo
