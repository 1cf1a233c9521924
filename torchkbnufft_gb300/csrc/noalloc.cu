// Forward table interpolation that allocates no device memory.
//
// tkbn_interp_fwd builds on a trajectory layout whose workspace the caller
// allocates (tkbn_points_workspace_size / tkbn_points_build). Some callers
// cannot do that: runtimes that hand out a fixed device-memory budget at start
// and forbid any later cudaMalloc (real-time reconstruction loops, embedded
// pipelines that pre-reserve all memory), and plain-C hosts that only hold
// raw device pointers from another framework and have no allocator of their
// own. For them, tkbn_interp_fwd_noalloc keeps the layout in a file-scope
// device array of kScratchBytes, which every GPU that loads this library holds
// until the process exits.
//
// Set-up: the first call on each device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress; make that first call
// before any stream capture. The address is cached per device together with
// the CUDA context it belongs to: when the device's context changes (after
// cudaDeviceReset, or when the primary context is released and created
// again) the next call looks the address up again, so that call too should
// come before any stream capture. Every call shares the one array and
// overwrites it, so calls that overlap on the GPU (other streams, other host
// threads) race; serialise them. The layout build clears everything that
// must start at zero on each call.

#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "tkbn_common.cuh"

namespace tkbn_host {
int points_layout(const tkbn_geometry* g, const tkbn_points_desc* p, PointsLayout* L);
int points_build(const tkbn_geometry* g, const tkbn_points_desc* p, const void* omega, void* ws, size_t bytes,
                 cudaStream_t s);
int interp_fwd(const tkbn_geometry* g, const tkbn_points_desc* p, const void* ws, const void* const* tables,
               const void* grid, int64_t B, int64_t C, void* kdata, cudaStream_t s);
}  // namespace tkbn_host

namespace {

constexpr size_t kScratchBytes = TKBN_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
struct ScratchAddress {
  CUcontext ctx;  // the context the address belongs to
  void* addr;
};
ScratchAddress g_addr[kMaxDevices] = {};

// The calling thread's current context (null when none is current or the
// driver entry point is unavailable), through the runtime's driver entry
// point, so the library needs no link against libcuda.
CUcontext current_context() {
  static PFN_cuCtxGetCurrent_v4000 get = []() -> PFN_cuCtxGetCurrent_v4000 {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    return (PFN_cuCtxGetCurrent_v4000)fn;
  }();
  CUcontext c = nullptr;
  if (!get || get(&c) != CUDA_SUCCESS) return nullptr;
  return c;
}

int scratch_address(void** out) {
  int dev = 0;
  int rc = tkbn_host::check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
  if (rc) return rc;
  if (dev < 0 || dev >= kMaxDevices) return tkbn_host::set_error(TKBN_ERR_UNSUPPORTED, "device index %d too large", dev);
  std::lock_guard<std::mutex> lock(g_mu);
  CUcontext ctx = current_context();
  if (!ctx || ctx != g_addr[dev].ctx || !g_addr[dev].addr) {
    // also makes the device's primary context current when none is yet
    void* p = nullptr;
    rc = tkbn_host::check_cuda(cudaGetSymbolAddress(&p, g_noalloc_scratch), "cudaGetSymbolAddress(scratch)");
    if (rc) return rc;
    ctx = current_context();
    g_addr[dev].ctx = ctx;       // null: no context to key on, so look it up on every call
    g_addr[dev].addr = ctx ? p : nullptr;
    *out = p;
    return TKBN_OK;
  }
  *out = g_addr[dev].addr;
  return TKBN_OK;
}

}  // namespace

extern "C" int tkbn_interp_fwd_noalloc(const tkbn_geometry* g, const void* const* tables, const void* omega,
                                       int64_t npts, const void* grid, int64_t nbatch, int64_t ncoil, void* kdata,
                                       void* stream) {
  try {
    if (!g || !tables) return tkbn_host::set_error(TKBN_ERR_INVALID, "null geometry or tables");
    if (npts < 0) return tkbn_host::set_error(TKBN_ERR_INVALID, "npts must be >= 0");
    tkbn_points_desc p{};
    p.npts = npts;
    p.ntraj = 1;
    // forward only: the layout needs none of the adjoint's per-tile lists
    tkbn_geometry gf = *g;
    gf.flags |= TKBN_LAYOUT_FORWARD_ONLY;
    g = &gf;
    tkbn_host::PointsLayout L;
    int rc = tkbn_host::points_layout(g, &p, &L);
    if (rc) return rc;
    if (L.total > kScratchBytes)
      return tkbn_host::set_error(TKBN_ERR_INVALID,
                                  "trajectory needs %zu bytes of layout scratch; tkbn_interp_fwd_noalloc holds %zu "
                                  "(use tkbn_points_build with a caller-allocated workspace)",
                                  L.total, kScratchBytes);
    void* ws = nullptr;
    if ((rc = scratch_address(&ws))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (npts > 0 && (rc = tkbn_host::points_build(g, &p, omega, ws, kScratchBytes, s))) return rc;
    return tkbn_host::interp_fwd(g, &p, ws, tables, grid, nbatch, ncoil, kdata, s);
  } catch (...) {
    return tkbn_host::set_error(TKBN_ERR_INVALID, "internal error");
  }
}
