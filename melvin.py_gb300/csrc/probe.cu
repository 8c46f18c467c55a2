// Throughput probe of the FP64 FMA pipe.
//
// The FP64 step is bound by the FP64 pipe, not by HBM, so its roofline needs
// the rate at which this GPU retires FP64 FMAs.  This kernel measures it:
// every thread runs kProbeChains independent chains a = a*b + c, enough
// warps per SM to cover the FMA latency, so the pipe is the only limit.
// A launch of `blocks` CTAs of kProbeThreads threads retires
// 2 * kProbeChains * iters * kProbeThreads * blocks FP64 flops (an FMA
// counts two); the caller times it with CUDA events.
#include "internal.h"

namespace mgb {
namespace {

constexpr int kProbeThreads = 256;
constexpr int kProbeChains = 8;

__global__ void __launch_bounds__(kProbeThreads) k_fp64_fma_probe(double* sink, int iters, double b, double c,
                                                                  double sentinel) {
  double a[kProbeChains];
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) a[k] = 1e-3 * threadIdx.x + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < kProbeChains; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kProbeChains; ++k) s += a[k];
  // the chains converge to c / (1 - b) > 0, never to the negative sentinel:
  // the store keeps the work alive without writing anything
  if (s == sentinel) sink[blockIdx.x] = s;
}

}  // namespace
}  // namespace mgb

using namespace mgb;

extern "C" int mgb_fp64_fma_probe(double* sink, int32_t blocks, int32_t iters, double* flops, void* stream) {
  if (!sink || !flops) return fail(MGB_ERR_INVALID, "%s: null pointer", __func__);
  if (blocks < 1 || blocks > (1 << 20) || iters < 1)
    return fail(MGB_ERR_INVALID, "%s: blocks %d iters %d out of range", __func__, blocks, iters);
  k_fp64_fma_probe<<<blocks, kProbeThreads, 0, (cudaStream_t)stream>>>(sink, iters, 1.0 - 0x1p-30, 1e-3, -1.0);
  MGB_LAUNCH_CHECK();
  *flops = 2.0 * kProbeChains * (double)iters * kProbeThreads * (double)blocks;
  return MGB_OK;
}
