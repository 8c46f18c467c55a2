// Transform kernels instantiated for length 1024.
#include "fdm_impl.cuh"

namespace mgb {
const FsLaunchers* fs_launchers_1024() {
  static const FsLaunchers L = make_fs_launchers<1024>();
  return &L;
}
const FdLaunchers* fd_launchers_1024() {
  static const FdLaunchers L = make_fd_launchers<1024>();
  return &L;
}
}  // namespace mgb
