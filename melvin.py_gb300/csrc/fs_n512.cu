// Transform kernels instantiated for length 512.
#include "fdm_impl.cuh"

namespace mgb {
const FsLaunchers* fs_launchers_512() {
  static const FsLaunchers L = make_fs_launchers<512>();
  return &L;
}
const FdLaunchers* fd_launchers_512() {
  static const FdLaunchers L = make_fd_launchers<512>();
  return &L;
}
}  // namespace mgb
