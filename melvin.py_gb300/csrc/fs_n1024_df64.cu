// Fully spectral fused-step kernels for length 1024 in double-float (default tile).
#include "spectral2d_impl.cuh"

namespace mgb {
void fill_fs_df64_1024(FsLaunchers& L) { fill_step_kernels<df64, 1024, 0x1>(L, MGB_PREC_DFLOAT); }
}  // namespace mgb
