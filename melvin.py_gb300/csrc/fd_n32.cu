// Fourier-x / finite-difference-z kernels for length 32 (all precisions).
#include "fdm_impl.cuh"

namespace mgb {
const FdLaunchers* fd_launchers_32() {
  static const FdLaunchers L = make_fd_launchers<32>();
  return &L;
}
}  // namespace mgb
