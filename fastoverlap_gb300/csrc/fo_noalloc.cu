// fo_noalloc.cu -- periodic overlap grid without any device allocation.
//
// For callers that cannot let a library allocate device memory: programs that
// hand all device memory to their own pool allocator up front (a cudaMalloc
// would fail or fragment the pool), serving loops that must not pay
// allocation latency or risk an out-of-memory failure in the middle of a
// request, and embedders that forbid hidden allocations.  The caller passes
// device pointers for the inputs and the
// output; the one scratch buffer the computation needs -- the complex M^3
// structure-factor product and the descriptors the kernels read -- is a
// file-scope __device__ array of fixed size that every GPU loading this
// library holds until the process exits (kNoAllocScratchBytes, about 4 MiB).
//
// Set-up: the first call on each device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress; do that first call
// before any stream capture.  All calls on a device share the array and it
// keeps the previous call's contents, so the product grid is cleared at the
// start of every call; calls that overlap on the GPU (different streams, or
// host threads issuing concurrently) race on the array and must be ordered
// by the caller.  The pair and group descriptors reach the array through the
// parameters of a small kernel (copied at launch), so no host buffer has to
// outlive the call.
#include "../../include/fastoverlap_gb300.h"
#include "fo_common.cuh"
#include "fo_kernels.h"

#include <cmath>
#include <cstring>
#include <mutex>

namespace {

constexpr int kNoAllocMaxM = 64;       // translation grid at most 64^3
constexpr int kNoAllocMaxGroups = 64;  // permutation groups
constexpr size_t kNoAllocDescBytes = 8192;
constexpr size_t kNoAllocGridBytes = sizeof(double2) * kNoAllocMaxM * kNoAllocMaxM * kNoAllocMaxM;
constexpr size_t kNoAllocScratchBytes = kNoAllocDescBytes + kNoAllocGridBytes;

static_assert(sizeof(fo::PairDev) + kNoAllocMaxGroups * sizeof(fo::GroupDev) <= kNoAllocDescBytes,
              "descriptor region too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once).
cudaError_t scratch_address(unsigned char **out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = (unsigned char *)p;
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

// Descriptors of one call, passed by value to k_noalloc_desc (kernel
// parameters are copied when the launch is queued).
struct NoAllocDesc {
    fo::PairDev pair;
    fo::GroupDev groups[kNoAllocMaxGroups];
    int ngroups;
};
static_assert(sizeof(NoAllocDesc) <= 4000, "descriptor parameter above the classic launch limit");

// Writes the pair descriptor and the ngroups group descriptors to the head of
// the scratch array (PairDev, then GroupDev[ngroups]).
__global__ void k_noalloc_desc(const NoAllocDesc d, unsigned char *dst) {
    const unsigned char *src = (const unsigned char *)&d.pair;
    const int pbytes = (int)sizeof(fo::PairDev);
    const int gbytes = d.ngroups * (int)sizeof(fo::GroupDev);
    const unsigned char *gsrc = (const unsigned char *)d.groups;
    for (int i = threadIdx.x; i < pbytes + gbytes; i += blockDim.x)
        dst[i] = i < pbytes ? src[i] : gsrc[i - pbytes];
}

int fastlen(int n) {
    if (n <= 1) return 1;
    for (int m = n;; ++m) {
        int k = m;
        while (k % 2 == 0) k /= 2;
        while (k % 3 == 0) k /= 3;
        while (k % 5 == 0) k /= 5;
        if (k == 1) return m;
    }
}

}  // namespace

extern "C" fo_status fo_bulk_overlap_noalloc(const double *d_pos1, const double *d_pos2, int natoms,
                                             const int *group_sizes, int ngroups, double boxlx,
                                             double boxly, double boxlz, double kwidth, int nwave,
                                             int nfspace, double *d_grid, void *stream) {
    if (!d_pos1 || !d_pos2 || !d_grid || !group_sizes || natoms < 1) return FO_ERR_BAD_ARGS;
    if (ngroups < 1 || ngroups > kNoAllocMaxGroups) return FO_ERR_BAD_ARGS;
    long long tot = 0;
    for (int g = 0; g < ngroups; ++g) {
        if (group_sizes[g] < 0) return FO_ERR_BAD_ARGS;
        tot += group_sizes[g];
    }
    if (tot != natoms) return FO_ERR_BAD_ARGS;
    const double box[3] = {boxlx, boxly, boxlz};
    for (int k = 0; k < 3; ++k)
        if (!(box[k] > 0.0) || !std::isfinite(box[k])) return FO_ERR_BAD_ARGS;
    const int K = nwave > 0 ? nwave : (int)std::ceil(1.3 * std::cbrt((double)natoms));
    const int M = nfspace > 0 ? nfspace : fastlen(4 * K + 3);
    if (M < 2 * K + 1 || M > kNoAllocMaxM) return FO_ERR_BAD_ARGS;  // scratch holds M <= 64
    const double sigma = kwidth > 0 ? kwidth : std::cbrt(boxlx * boxly * boxlz / natoms) / 3.0;

    // an error left pending by earlier work on this thread is not ours to
    // clear or to report as this call's: refuse, and leave it for the caller
    if (cudaPeekAtLastError() != cudaSuccess) return FO_ERR_CUDA;
    unsigned char *base = nullptr;
    if (scratch_address(&base) != cudaSuccess) return FO_ERR_CUDA;
    cudaStream_t st = (cudaStream_t)stream;

    NoAllocDesc desc{};
    fo::PairDev &P = desc.pair;
    P.n = natoms;
    P.ngroups = ngroups;
    P.group0 = 0;
    P.L = K;
    P.G = M;
    P.nrot = 1;
    P.norient = 1;
    P.bulk = 1;
    P.coef0 = 0;
    P.grid0 = 0;
    P.sigma = sigma;
    for (int k = 0; k < 3; ++k) P.box[k] = box[k];
    desc.ngroups = ngroups;
    int off = 0;
    for (int g = 0; g < ngroups; ++g) {
        fo::GroupDev &G = desc.groups[g];
        G.pair = 0;
        G.slot0 = off;  // atoms of group g are the contiguous range [off, off + size)
        G.n = group_sizes[g];
        G.m = group_sizes[g] < fo::kMaxNei ? group_sizes[g] : fo::kMaxNei;
        off += group_sizes[g];
    }
    unsigned char *d_desc = base, *d_fgrid = base + kNoAllocDescBytes;
    k_noalloc_desc<<<1, 256, 0, st>>>(desc, d_desc);
    if (cudaGetLastError() != cudaSuccess) return FO_ERR_CUDA;
    // the product grid must start at zero outside the (2K+1)^3 corner
    if (cudaMemsetAsync(d_fgrid, 0, sizeof(double2) * (size_t)M * M * M, st) != cudaSuccess)
        return FO_ERR_CUDA;
    fo::BulkBuffers b{};
    b.pairs = (const fo::PairDev *)d_desc;
    b.groups = (const fo::GroupDev *)(d_desc + sizeof(fo::PairDev));
    b.xa = const_cast<double *>(d_pos2);
    b.xb = const_cast<double *>(d_pos1);
    b.fgrid = d_fgrid;
    b.grid = d_grid;
    b.npairs = 1;
    b.maxK = K;
    b.maxM = M;
    fo::launch_bulk_sf(b, false, st);
    if (cudaGetLastError() != cudaSuccess) return FO_ERR_CUDA;
    fo::launch_bulk_fft(b, false, st);
    return cudaGetLastError() == cudaSuccess ? FO_OK : FO_ERR_CUDA;
}

extern "C" size_t fo_bulk_overlap_noalloc_scratch_bytes(void) { return kNoAllocScratchBytes; }
