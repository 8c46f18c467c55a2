// Fully spectral fused-step kernels for length 2048 in FP32 (every tile variant).
#include "spectral2d_impl.cuh"

namespace mgb {
void fill_fs_f32_2048(FsLaunchers& L) { fill_step_kernels<float, 2048>(L, MGB_PREC_SPLIT); }
}  // namespace mgb
