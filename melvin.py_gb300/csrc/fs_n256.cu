// Fully spectral kernels for length 256: the FP64 fused-step kernels (every
// tile variant), the FP64 per-verb kernels, and the launcher table that also
// takes the FP32 and double-float kernels of fs_n256_f32.cu / fs_n256_df64.cu.
#include "spectral2d_impl.cuh"

namespace mgb {
void fill_fs_f32_256(FsLaunchers& L);
void fill_fs_df64_256(FsLaunchers& L);

const FsLaunchers* fs_launchers_256() {
  static const FsLaunchers L = [] {
    FsLaunchers l{};
    fill_step_kernels<double, 256>(l, MGB_PREC_DOUBLE);
    fill_fs_f32_256(l);
    fill_fs_df64_256(l);
    fill_verb_kernels<256>(l);
    return l;
  }();
  return &L;
}
}  // namespace mgb
