// pbte_transport_residual_noalloc: the transport residual without any device
// allocation on the call path.
//
// Who needs it.  pbte_transport_residual keeps its per-element moment sources
// in scratch owned by the context.  Some callers cannot allocate device
// memory at all where they call from -- a host that hands the whole device to
// its own memory pool, where a cudaMalloc behind the pool's back fails or
// breaks its accounting -- and some must not touch the context's scratch
// because a sweep may be using it.  This entry point allocates nothing: its scratch is a file-scope
// __device__ array of kScratchDoubles doubles (4 MiB) that every GPU loading
// the library holds until the process exits.
//
// Rules of use (also in include/pbte_gb300.h):
//  - 3 * ndof * n_tris must not exceed kScratchDoubles (PBTE_ERR_ARG if it
//    does): 29127 triangles at P2, 58254 at P1, 17476 at P3.
//  - The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (with that device current); under lazy module
//    loading that is also when the runtime commits the array's 4 MiB.  Make
//    that first call before any stream capture begins.
//  - Call it with the context's device current: the array's address is per
//    device, so a call on another device is refused (PBTE_ERR_ARG).
//  - Periodic faces are refused (PBTE_ERR_UNSUPPORTED).
//  - All calls share the one array: calls whose kernels overlap on the GPU
//    race.  The array carries nothing from one call to the next (each call
//    overwrites all of it that it reads), so nothing needs clearing.
#include <cuda_runtime.h>

#include <mutex>

#include "pbte_internal.cuh"

namespace {

constexpr long long kScratchDoubles = 1LL << 19;   // 4 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

std::mutex g_mu;
double *g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device (looked up once
// per device); nullptr on failure.
double *scratch_address() {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_addr[dev] == nullptr) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess) return nullptr;
        g_addr[dev] = static_cast<double *>(p);
    }
    return g_addr[dev];
}

}  // namespace

extern "C" int pbte_transport_residual_noalloc(pbte_ctx *c, const double *ts, const double *qxs,
                                               const double *qys, const double *vdf, const double *flux_wall,
                                               double *num, double *den, void *stream) {
    if (!c || !ts || !qxs || !qys || !vdf || !num || !den) return PBTE_ERR_ARG;
    if (c->n_wall_ad && !flux_wall) return PBTE_ERR_ARG;
    if (3LL * c->nd * c->n_tris > kScratchDoubles) return PBTE_ERR_ARG;
    if (c->has_periodic) return PBTE_ERR_UNSUPPORTED;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return PBTE_ERR_CUDA;
    if (dev != c->device) return PBTE_ERR_ARG;
    double *S = scratch_address();
    if (!S) return PBTE_ERR_CUDA;
    return pbte::launch_transport_residual_scratch(c, ts, qxs, qys, vdf, flux_wall, num, den, S,
                                                   reinterpret_cast<cudaStream_t>(stream));
}
