// Fully spectral fused-step kernels for length 256 in double-float (default tile).
#include "spectral2d_impl.cuh"

namespace mgb {
void fill_fs_df64_256(FsLaunchers& L) { fill_step_kernels<df64, 256, 0x1>(L, MGB_PREC_DFLOAT); }
}  // namespace mgb
