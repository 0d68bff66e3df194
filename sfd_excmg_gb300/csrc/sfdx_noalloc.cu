// sfdx_noalloc.cu -- an entry point that allocates no memory: the residual
// r = b - K x and the relative residual norms of ns interleaved systems on
// device buffers owned by the caller.
//
// Why: some callers cannot call cudaMalloc at all -- for example a host
// code whose device memory is handed out by its own pool or by another
// runtime (a Fortran or C++ application that owns all GPU memory), or code
// that must not allocate inside a time-critical loop.  Such a caller owns the
// conductivity, right-hand side, solution and residual buffers; everything
// else the kernel needs (spacing tables, per-system state, the partial sums
// of the reductions and their arrival counter) lives in one file-scope device
// array of fixed size.  The array is reserved on a device when this file's
// device code is loaded there: with CUDA's default lazy module loading that is
// the first call of this entry point on the device (its address look-up loads
// the module).  A caller that hands all device memory to its own pool therefore
// makes one call (any small case) before filling the pool, or runs with
// CUDA_MODULE_LOADING=EAGER.  Every GPU that loaded the library holds the
// array until the process exits.
//
// Limits: nx, ny, nz <= SFDX_NOALLOC_MAX_N cells per axis, ns <=
// SFDX_NOALLOC_MAX_NS systems; larger sizes are rejected with
// SFDX_ERR_NOMEM.  Calls share the array and leave their contents in it, so
// calls that overlap on the GPU (different streams or threads at the same
// time) race and must be serialised by the caller.
#include <cstdint>
#include <cuda_runtime.h>

#include "sfdx.h"
#include "sfdx_kernels.cuh"

namespace sfdx {
namespace {

constexpr int kMaxN = SFDX_NOALLOC_MAX_N;
constexpr int kMaxNS = SFDX_NOALLOC_MAX_NS;
constexpr int kMaxBlocks = 2048;
constexpr int kStride = kMaxN + 2;
// layout of the scratch array (byte offsets, each 256-aligned)
constexpr size_t kTabBytes = sizeof(double) * 18 * kStride;             // 3 axes x 6 tables
constexpr size_t kSpacBytes = sizeof(double) * 3 * kMaxN;               // a, b, c
constexpr size_t kFreqBytes = sizeof(double) * kMaxNS;                  // frequencies
constexpr size_t kStateBytes = sizeof(KState) * kMaxNS;                 // per-system state
constexpr size_t kPartBytes = sizeof(double2) * kMaxBlocks * 2 * kMaxNS;  // block partial sums
constexpr size_t kRelBytes = sizeof(double) * kMaxNS;                   // relative residuals
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kOffTab = 0;
constexpr size_t kOffSpac = kOffTab + align256(kTabBytes);
constexpr size_t kOffFreq = kOffSpac + align256(kSpacBytes);
constexpr size_t kOffState = kOffFreq + align256(kFreqBytes);
constexpr size_t kOffPart = kOffState + align256(kStateBytes);
constexpr size_t kOffRel = kOffPart + align256(kPartBytes);
constexpr size_t kOffCounter = kOffRel + align256(kRelBytes);
constexpr size_t kScratchBytes = kOffCounter + 256;

}  // namespace

// The scratch itself (about 4.5 MB).  Host code never passes this symbol to a
// kernel: on the host it names a stand-in, not a device address.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

// Device address of the scratch on the current device.  Looked up on every
// call (cheap once the module is loaded) rather than cached: a cudaDeviceReset
// by the caller reloads the module, possibly at another address.  The first
// look-up on a device loads the module there; it must not happen inside a
// stream capture.
int scratch_address(unsigned char** out) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SFDX_ERR_CUDA;
    *out = static_cast<unsigned char*>(p);
    return SFDX_OK;
}

// Spacing tables of the operator from a, b, c (same formulas as the host
// builder of the regular entry points).
__global__ void k_tables(int nx, int ny, int nz, const double* __restrict__ spac, double* __restrict__ tab, int stride) {
    const int n3[3] = {nx, ny, nz};
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 3 * stride; t += gridDim.x * blockDim.x) {
        const int ax = t / stride, m = t % stride, n = n3[ax];
        const double* h = spac + (ax == 0 ? 0 : (ax == 1 ? nx : nx + ny));
        double* base = tab + (size_t)ax * 6 * stride;
        double rh = 0, lo = 0, hi = 0, rs = 0, wl = 0, wh = 0;
        if (m < n) rh = 1.0 / h[m];
        if (m >= 1 && m < n) {
            double s = h[m - 1] + h[m];
            lo = -2 / (h[m - 1] * (h[m - 1] + h[m]));
            hi = -2 / (h[m] * (h[m - 1] + h[m]));
            rs = 1.0 / s;
            wl = h[m - 1] / s;
            wh = h[m] / s;
        }
        base[m] = rh;
        base[stride + m] = lo;
        base[2 * stride + m] = hi;
        base[3 * stride + m] = rs;
        base[4 * stride + m] = wl;
        base[5 * stride + m] = wh;
    }
}

__global__ void k_init_states(KState* st, int ns, const double* __restrict__ freqs) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    KState S;
    memset(&S, 0, sizeof(S));
    S.wm = 2.0 * 3.141592653589793238462643 * freqs[s] * (4.0 * 3.141592653589793238462643 * 1e-7);
    S.active = 1;
    st[s] = S;
}

__global__ void k_relres(const KState* st, int ns, double* rel) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < ns) rel[s] = st[s].babs > 0 ? st[s].err / st[s].babs : st[s].err;
}

__global__ void k_any_offdiag_dev(int64_t ncell, const double* __restrict__ sig, int* flag) {
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * ncell; q += (int64_t)gridDim.x * blockDim.x)
        if (sig[3 * ncell + q] != 0.0) {
            *flag = 1;
            return;
        }
}

}  // namespace
}  // namespace sfdx

using namespace sfdx;

extern "C" int sfdx_residual_noalloc(int nx, int ny, int nz, const double* a, const double* b, const double* c,
                                     const double* d_sigma, int ns, const double* freqs, const double* d_rhs,
                                     const double* d_x, double* d_r, double* relres, void* stream) {
    if (!a || !b || !c || !d_sigma || !freqs || !d_rhs || !d_x || !d_r || !relres) return SFDX_ERR_ARG;
    if (nx < 2 || ny < 2 || nz < 2 || ns < 1) return SFDX_ERR_ARG;
    // the kernels read and write the caller's complex vectors as 16-byte
    // double2 and sigma as double: refuse pointers that would fault
    if ((reinterpret_cast<uintptr_t>(d_rhs) | reinterpret_cast<uintptr_t>(d_x) | reinterpret_cast<uintptr_t>(d_r)) & 15)
        return SFDX_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(d_sigma) & 7) return SFDX_ERR_ARG;
    if (nx > kMaxN || ny > kMaxN || nz > kMaxN || ns > kMaxNS) return SFDX_ERR_NOMEM;
    unsigned char* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    double* tab = reinterpret_cast<double*>(base + kOffTab);
    double* spac = reinterpret_cast<double*>(base + kOffSpac);
    double* fr = reinterpret_cast<double*>(base + kOffFreq);
    KState* state = reinterpret_cast<KState*>(base + kOffState);
    double2* part = reinterpret_cast<double2*>(base + kOffPart);
    double* rel = reinterpret_cast<double*>(base + kOffRel);
    unsigned int* counter = reinterpret_cast<unsigned int*>(base + kOffCounter);
    int* flag = reinterpret_cast<int*>(base + kOffCounter + 64);
    // inputs into the scratch (copies, no allocation); what must start at zero is cleared
    if (cudaMemcpyAsync(spac, a, sizeof(double) * nx, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(spac + nx, b, sizeof(double) * ny, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(spac + nx + ny, c, sizeof(double) * nz, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(fr, freqs, sizeof(double) * ns, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(counter, 0, 128, st) != cudaSuccess)
        return SFDX_ERR_CUDA;
    k_tables<<<(3 * kStride + 255) / 256, 256, 0, st>>>(nx, ny, nz, spac, tab, kStride);
    k_init_states<<<(ns + 63) / 64, 64, 0, st>>>(state, ns, fr);
    Lev<double> L;
    L.nx = nx;
    L.ny = ny;
    L.nz = nz;
    L.xnl = (int64_t)nx * (ny + 1) * (nz + 1);
    L.ynl = (int64_t)(nx + 1) * ny * (nz + 1);
    L.nl = L.xnl + L.ynl + (int64_t)(nx + 1) * (ny + 1) * nz;
    L.ncell = (int64_t)nx * ny * nz;
    for (int ax = 0; ax < 3; ax++) {
        const double* p = tab + (size_t)ax * 6 * kStride;
        AxisT<double> A{p, p + kStride, p + 2 * kStride, p + 3 * kStride, p + 4 * kStride, p + 5 * kStride};
        (ax == 0 ? L.ax : (ax == 1 ? L.ay : L.az)) = A;
    }
    L.sig = d_sigma;
    int aniso = 0;
    k_any_offdiag_dev<<<128, 256, 0, st>>>(L.ncell, d_sigma, flag);
    if (cudaMemcpyAsync(&aniso, flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return SFDX_ERR_CUDA;
    L.aniso = aniso;
    L.rc = nullptr;
    int B = ns;
    while (B < 128 || B < 2 * ns) B *= 2;
    int dev = 0, nsm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    int64_t G = (L.nl * ns + B - 1) / B;
    if (G > (int64_t)nsm * 8) G = (int64_t)nsm * 8;
    if (G > kMaxBlocks) G = kMaxBlocks;
    RedBuf rb{part, counter};
    k_residual<double, double, 2><<<(int)G, B, 2 * B * sizeof(double2), st>>>(
        L, state, ns, reinterpret_cast<const double2*>(d_rhs), reinterpret_cast<const double2*>(d_x),
        reinterpret_cast<double2*>(d_r), nullptr, rb, nullptr, 0);
    k_relres<<<(ns + 63) / 64, 64, 0, st>>>(state, ns, rel);
    if (cudaGetLastError() != cudaSuccess) return SFDX_ERR_CUDA;
    if (cudaMemcpyAsync(relres, rel, sizeof(double) * ns, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return SFDX_ERR_CUDA;
    return SFDX_OK;
}
