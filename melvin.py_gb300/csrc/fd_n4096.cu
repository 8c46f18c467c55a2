// Fourier-x / finite-difference-z kernels for length 4096 (all precisions).
#include "fdm_impl.cuh"

namespace mgb {
const FdLaunchers* fd_launchers_4096() {
  static const FdLaunchers L = make_fd_launchers<4096>();
  return &L;
}
}  // namespace mgb
