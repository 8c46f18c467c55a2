// Fourier-x / finite-difference-z kernels for length 16 (all precisions).
#include "fdm_impl.cuh"

namespace mgb {
const FdLaunchers* fd_launchers_16() {
  static const FdLaunchers L = make_fd_launchers<16>();
  return &L;
}
}  // namespace mgb
