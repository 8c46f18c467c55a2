// Fully spectral fused-step kernels for length 1024 in FP32 (every tile variant).
#include "spectral2d_impl.cuh"

namespace mgb {
void fill_fs_f32_1024(FsLaunchers& L) { fill_step_kernels<float, 1024>(L, MGB_PREC_SPLIT); }
}  // namespace mgb
