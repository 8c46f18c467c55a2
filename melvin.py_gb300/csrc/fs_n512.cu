// Fully spectral kernels for length 512: the FP64 fused-step kernels (every
// tile variant), the FP64 per-verb kernels, and the launcher table that also
// takes the FP32 and double-float kernels of fs_n512_f32.cu / fs_n512_df64.cu.
#include "spectral2d_impl.cuh"

namespace mgb {
void fill_fs_f32_512(FsLaunchers& L);
void fill_fs_df64_512(FsLaunchers& L);

const FsLaunchers* fs_launchers_512() {
  static const FsLaunchers L = [] {
    FsLaunchers l{};
    fill_step_kernels<double, 512>(l, MGB_PREC_DOUBLE);
    fill_fs_f32_512(l);
    fill_fs_df64_512(l);
    fill_verb_kernels<512>(l);
    return l;
  }();
  return &L;
}
}  // namespace mgb
