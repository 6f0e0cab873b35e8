// Allocation-free variant of the spline adjoint.
//
// Some callers cannot allocate device memory at the moment they need a
// gradient. A solver embedded in a host application with a fixed device-memory
// budget is one. A real-time loop that must not enter the CUDA allocator (its
// calls can block and synchronise the device) is another. So is code that runs
// while another component owns every allocation.
// topo_spline_adjoint_noalloc serves them. It runs the same three separable
// passes as topo_spline_adjoint. The caller passes the sensitivity input and
// the gradient output as device pointers. The two intermediate planes live in
// a fixed device array declared in this file, so the call allocates nothing.
#include <mutex>

#include "topo_internal.h"

namespace topo {

// Scratch for the two intermediate planes of the separable adjoint:
// nb_x * ny * nz + nb_x * nb_y * nz doubles must fit.  16 MiB per device,
// held by every GPU that loads the library until the process exits.
constexpr int64_t kNoallocScratchDoubles = 2 * 1024 * 1024;
static __device__ __align__(256) double g_adjoint_scratch[kNoallocScratchDoubles];

// Device address of g_adjoint_scratch per device, looked up once per device
// (the host-side name is only a stand-in for the symbol, not a device address).
constexpr int kMaxDevices = 64;
static double* g_scratch_ptr[kMaxDevices] = {nullptr};
static std::mutex g_scratch_mutex;

static int scratch_for_device(int dev, double** out) {
  if (dev < 0 || dev >= kMaxDevices) return TOPO_E_BAD_INPUT;
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) return TOPO_E_CUDA;
    if (cur != dev && cudaSetDevice(dev) != cudaSuccess) return TOPO_E_CUDA;
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_adjoint_scratch);
    if (cur != dev) cudaSetDevice(cur);
    if (e != cudaSuccess || !p) return TOPO_E_CUDA;
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return TOPO_OK;
}

}  // namespace topo

using namespace topo;

extern "C" int topo_spline_adjoint_noalloc(topo_handle* h, const double* sens_dev, double* csens_dev) {
  if (!h || !sens_dev || !csens_dev) return TOPO_E_BAD_INPUT;
  SplineView sv;
  const int rc = handle_spline_view(h, &sv);
  if (rc != TOPO_OK) return rc;
  DeviceScope device_scope(sv.device);
  const int64_t n1 = (int64_t)sv.sp.nb[0] * sv.d.ey * sv.d.ez;
  const int64_t n2 = (int64_t)sv.sp.nb[0] * sv.sp.nb[1] * sv.d.ez;
  if (n1 + n2 > kNoallocScratchDoubles)
    return handle_fail(h, TOPO_E_BAD_INPUT,
                       "topo_spline_adjoint_noalloc: intermediate planes need more than the fixed "
                       "2097152-double scratch; use topo_spline_adjoint");
  double* scratch = nullptr;
  if (scratch_for_device(sv.device, &scratch) != TOPO_OK)
    return handle_fail(h, TOPO_E_CUDA, "topo_spline_adjoint_noalloc: cudaGetSymbolAddress failed");
  // Every element of both planes is written by the first two passes before it
  // is read, so nothing needs clearing between calls.
  launch_spline_adjoint(sv.stream, sv.d, sv.eactive, sv.sp, sens_dev, csens_dev, scratch, scratch + n1);
  count_launch(3);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return handle_fail(h, TOPO_E_CUDA, cudaGetErrorString(e));
  return TOPO_OK;
}
