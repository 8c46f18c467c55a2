// vec_dot_nabla without a caller-provided workspace.
//
// Some callers cannot allocate device memory at the point where they need
// the nonlinear term: code that runs inside a framework which owns every
// device allocation and hands a kernel only its operands and results, or a
// real-time section where allocating is not allowed.  This entry point
// gives them mgb_vec_dot_nabla with its transform scratch taken from a
// fixed array in the library's own device memory, so the call itself
// allocates nothing.
//
// The array is a file-scope __device__ object of MGB_NOALLOC_SCRATCH_BYTES;
// every GPU that loads the library holds it until the process exits.  All
// calls on a device share it, so calls that overlap on the GPU (different
// streams, or host threads racing on one stream) race on the scratch and
// must be serialised by the caller.  Each call writes every scratch element
// it later reads, so nothing needs clearing between calls.  The call must
// run with the plan's device current: the scratch address is per device.
#include <mutex>

#include "internal.h"

namespace mgb {
namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[MGB_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
void* g_noalloc_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The name
// g_noalloc_scratch in host code is a host-side stand-in, not a device
// address, so the address is looked up once per device with that device
// current.
int noalloc_scratch(void** out) {
  int dev = 0;
  MGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(MGB_ERR_UNSUPPORTED, "device index %d beyond %d", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress(noalloc scratch)");
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return MGB_OK;
}

}  // namespace
}  // namespace mgb

using namespace mgb;

extern "C" int mgb_vec_dot_nabla_noalloc(const mgb_plan* p, const void* q_spec, double* q_phys, const double* ux,
                                         const double* uz, void* out_spec, void* stream) {
  if (!p) return fail(MGB_ERR_INVALID, "%s: null plan", __func__);
  if (!q_spec || !q_phys || !ux || !uz || !out_spec) return fail(MGB_ERR_INVALID, "%s: null array", __func__);
  if (int st = need_exp_ffts(p, __func__)) return st;
  int dev = -1;
  MGB_CUDA(cudaGetDevice(&dev));
  if (dev != p->device)
    return fail(MGB_ERR_INVALID, "%s: the plan belongs to device %d but device %d is current; make the plan's "
                "device current first", __func__, p->device, dev);
  const GridC& g = p->g;
  // scratch: two x-pass intermediates (fully spectral) or one physical field (FDM z)
  const size_t need = g.fdm ? (size_t)g.nx * g.nz * sizeof(double) : 2 * inter_bytes(g, MGB_PREC_DOUBLE);
  if (need > (size_t)MGB_NOALLOC_SCRATCH_BYTES)
    return fail(MGB_ERR_UNSUPPORTED,
                "%s: grid %dx%d needs %zu bytes of scratch, above the built-in %u; use mgb_vec_dot_nabla with a "
                "caller workspace",
                __func__, g.nx, g.nz, need, (unsigned)MGB_NOALLOC_SCRATCH_BYTES);
  void* work = nullptr;
  int st = noalloc_scratch(&work);
  if (st) return st;
  if (g.fdm)
    return fd_vec_dot_nabla(p, (const zd*)q_spec, q_phys, ux, uz, (zd*)out_spec, work, (cudaStream_t)stream);
  return fs_vec_dot_nabla(p, (const zd*)q_spec, q_phys, ux, uz, (zd*)out_spec, work, (cudaStream_t)stream);
}
