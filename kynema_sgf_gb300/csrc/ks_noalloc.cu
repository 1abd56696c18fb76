// Allocation-free entry point for the tensor diffusion term.
//
// Some callers of this library cannot call cudaMalloc at the point where they
// need the viscous term: hosts whose device memory is reserved up front by
// another allocator or framework and must not grow, plug-in code that runs
// inside an application that owns every device allocation, and
// latency-critical loops that cannot afford the device-wide synchronisation
// an allocation may cause.  For them, ks_divtau_noalloc evaluates
// div(mu (grad u + grad u^T) - 2/3 mu div(u) I) on caller-owned device
// buffers, and keeps the nine face-flux scratch arrays it needs in the
// file-scope device array below instead of allocating them.
//
// The scratch array holds KS_NOALLOC_MAX_CELLS cells' worth of face fluxes
// (about 24 MB of FP64).  Every GPU that loads the library holds it until the
// process exits.  All calls share it: calls whose kernels overlap on the GPU
// (different streams, or different host threads on one device) race on it, so
// callers must order them.  Each call writes every scratch value it reads
// before reading it, so nothing carries over from the previous call.
//
// The first call on a device looks up the array's device address with that
// device current (cudaGetSymbolAddress) and caches it; make that first call
// before any stream capture.  A device reset (cudaDeviceReset) unloads the
// module that holds the array, so calls after a reset are not supported.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/ks.h"
#include "ks_launch.hpp"

namespace {

constexpr long long kMaxCells = KS_NOALLOC_MAX_CELLS;
// three face directions x three components; z faces carry one extra layer
// (nx*ny <= cells/4 because nz >= 4)
constexpr long long kScratchValues = 9 * (kMaxCells + kMaxCells / 4);

static __device__ __align__(256) double g_divtau_scratch[kScratchValues];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once
// per device, with that device current).
int scratch_on_current_device(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return KS_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_divtau_scratch);
        if (e != cudaSuccess || !p) return KS_ERR_CUDA;
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return KS_OK;
}

}  // namespace

extern "C" int ks_divtau_noalloc(const double* vel, const double* mueff, const double* wall_grad, double* divtau, int nx, int ny,
                                 int nz, double dx, double dy, double dz, int z_periodic, int zlo_wall_model, void* stream) {
    if (!vel || !mueff || !divtau) return KS_ERR_ARG;
    if (nx < 4 || ny < 4 || nz < 4 || nx % 2 || ny % 2 || nz % 2) return KS_ERR_ARG;
    if (!(dx > 0.0) || !(dy > 0.0) || !(dz > 0.0)) return KS_ERR_ARG;
    const long long cells = (long long)nx * ny * nz;
    if (cells > kMaxCells) return KS_ERR_ARG;  // beyond the static scratch: use the allocating path
    if (zlo_wall_model && (z_periodic || !wall_grad)) return KS_ERR_ARG;
    double* scratch = nullptr;
    const int rc = scratch_on_current_device(&scratch);
    if (rc != KS_OK) return rc;

    ks::Grid g{};
    g.nx = nx;
    g.ny = ny;
    g.nz = nz;
    g.zper = z_periodic ? 1 : 0;
    g.zlo = z_periodic ? ks::ZPER : (zlo_wall_model ? ks::ZWALLMODEL : ks::ZSLIP);
    g.zhi = z_periodic ? ks::ZPER : ks::ZSLIP;
    g.dx = dx;
    g.dy = dy;
    g.dz = dz;
    g.idx = 1.0 / dx;
    g.idy = 1.0 / dy;
    g.idz = 1.0 / dz;
    g.N = cells;
    g.NFz = (long long)nx * ny * (nz + 1);

    double* fl[9];
    double* q = scratch;
    for (int d = 0; d < 3; ++d)
        for (int n = 0; n < 3; ++n) {
            fl[3 * d + n] = q;
            q += (d == 2) ? g.NFz : g.N;
        }
    // A CUDA error already pending on this thread belongs to the caller: it is
    // left in place for the caller's own check, and nothing is launched.
    if (cudaPeekAtLastError() != cudaSuccess) return KS_ERR_CUDA;
    ks::Ctx ctx;
    ctx.stream = static_cast<cudaStream_t>(stream);
    ks::launch_divtau_faces(ctx, g, vel, mueff, wall_grad, divtau, 0, nullptr, nullptr, nullptr, nullptr, 0.0, 1.0, fl);
    // a launch failure stays pending (as the runtime leaves it) for the caller to read
    return cudaPeekAtLastError() == cudaSuccess ? KS_OK : KS_ERR_CUDA;
}
