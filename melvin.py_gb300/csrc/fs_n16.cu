// Transform kernels instantiated for length 16.
#include "fdm_impl.cuh"

namespace mgb {
const FsLaunchers* fs_launchers_16() {
  static const FsLaunchers L = make_fs_launchers<16>();
  return &L;
}
const FdLaunchers* fd_launchers_16() {
  static const FdLaunchers L = make_fd_launchers<16>();
  return &L;
}
}  // namespace mgb
