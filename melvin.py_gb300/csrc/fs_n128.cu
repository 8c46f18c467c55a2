// Fully spectral kernels for length 128: the FP64 fused-step kernels (every
// tile variant), the FP64 per-verb kernels, and the launcher table that also
// takes the FP32 and double-float kernels of fs_n128_f32.cu / fs_n128_df64.cu.
#include "spectral2d_impl.cuh"

namespace mgb {
void fill_fs_f32_128(FsLaunchers& L);
void fill_fs_df64_128(FsLaunchers& L);

const FsLaunchers* fs_launchers_128() {
  static const FsLaunchers L = [] {
    FsLaunchers l{};
    fill_step_kernels<double, 128>(l, MGB_PREC_DOUBLE);
    fill_fs_f32_128(l);
    fill_fs_df64_128(l);
    fill_verb_kernels<128>(l);
    return l;
  }();
  return &L;
}
}  // namespace mgb
