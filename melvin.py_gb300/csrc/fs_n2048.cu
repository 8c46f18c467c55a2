// Transform kernels instantiated for length 2048.
#include "fdm_impl.cuh"

namespace mgb {
const FsLaunchers* fs_launchers_2048() {
  static const FsLaunchers L = make_fs_launchers<2048>();
  return &L;
}
const FdLaunchers* fd_launchers_2048() {
  static const FdLaunchers L = make_fd_launchers<2048>();
  return &L;
}
}  // namespace mgb
