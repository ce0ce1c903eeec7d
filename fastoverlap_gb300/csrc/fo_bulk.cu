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
// one thread per wave vector; written at [ix + M(iy + M iz)] of the M^3 grid.
template <typename T, typename T2>
__global__ void k_bulk_sf(const PairDev *pairs, const GroupDev *groups, const double *xa,
                          const double *xb, T2 *fgrid) {
    const PairDev &P = pairs[blockIdx.y];
    const int K = P.L, nk = 2 * K + 1, M = P.G;
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nk * nk * nk) return;
    const int ix = t % nk, iy = (t / nk) % nk, iz = t / (nk * nk);
    const double kx = 2.0 * FO_PI / P.box[0] * (ix - K), ky = 2.0 * FO_PI / P.box[1] * (iy - K),
                 kz = 2.0 * FO_PI / P.box[2] * (iz - K);
    const double damp = exp(-(kx * kx + ky * ky + kz * kz) * P.sigma * P.sigma);
    T fr = 0, fi = 0;
    for (int gi = 0; gi < P.ngroups; ++gi) {
        const GroupDev g = groups[P.group0 + gi];
        T ar = 0, ai = 0, br = 0, bi = 0;
        for (int j = 0; j < g.n; ++j) {
            const double *a = xa + 3LL * (g.slot0 + j), *b = xb + 3LL * (g.slot0 + j);
            double sa, ca, sb, cb;
            sincos(kx * a[0] + ky * a[1] + kz * a[2], &sa, &ca);
            sincos(kx * b[0] + ky * b[1] + kz * b[2], &sb, &cb);
            ar += T(ca); ai -= T(sa);
            br += T(cb); bi -= T(sb);
        }
        // C^B * conj(C^A)
        fr += br * ar + bi * ai;
        fi += bi * ar - br * ai;
    }
    fgrid[P.coef0 + ix + (long long)M * (iy + (long long)M * iz)] = mk2<T2>(fr * damp, fi * damp);
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
    int nk = 2 * b.maxK + 1, nk3 = nk * nk * nk;
    dim3 grid((nk3 + 127) / 128, b.npairs);
    if (fp32)
        k_bulk_sf<float, float2><<<grid, 128, 0, s>>>(b.pairs, b.groups, b.xa, b.xb, (float2 *)b.fgrid);
    else
        k_bulk_sf<double, double2><<<grid, 128, 0, s>>>(b.pairs, b.groups, b.xa, b.xb, (double2 *)b.fgrid);
}

void launch_bulk_fft(const BulkBuffers &b, bool fp32, cudaStream_t s) {
    dim3 grid((b.maxM * b.maxM + kLines - 1) / kLines, b.npairs);
    for (int axis = 0; axis < 3; ++axis) {
        if (fp32) {
            size_t sm = sizeof(float2) * (2 * kLines * b.maxM + b.maxM);
            k_bulk_fft_axis<float, float2><<<grid, 256, sm, s>>>(b.pairs, (float2 *)b.fgrid,
                                                                (float *)b.grid, axis, axis == 2);
        } else {
            size_t sm = sizeof(double2) * (2 * kLines * b.maxM + b.maxM);
            k_bulk_fft_axis<double, double2><<<grid, 256, sm, s>>>(b.pairs, (double2 *)b.fgrid,
                                                                  (double *)b.grid, axis, axis == 2);
        }
    }
}

}  // namespace fo
