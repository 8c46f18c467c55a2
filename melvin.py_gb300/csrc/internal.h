// Host-side plan object and internal launchers shared by the .cu files.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <map>
#include <mutex>

#include "common.cuh"

// What the last mgb_step_prepare computed into a step workspace (used to
// reject a fused step whose coefficients were prepared for another dt or
// equation).
struct PrepRecord {
  const void* work = nullptr;
  double dt = 0, alpha = 0;
  double kappa[3] = {0, 0, 0};
  int nfields = 0, integrator = -1, order = 0;
  bool valid = false;
  bool driven = false;  // a driven run may have refreshed the coefficients for its device dt
};

struct mgb_plan {
  mgb_grid grid;
  mgb::GridC g;
  // Twiddle tables exp(-2*pi*i*t/N), t in [0, N): x axis and (fully
  // spectral) z axis, in double and float.
  void* tw_x_d = nullptr;
  void* tw_x_f = nullptr;
  void* tw_x_df = nullptr;  // double-float
  void* tw_z_d = nullptr;
  void* tw_z_f = nullptr;
  void* tw_z_df = nullptr;
  // FDM-z: Thomas factors of the per-mode Dirichlet Poisson matrices,
  // [nn][nz] each (inverse pivots and modified upper diagonals).
  double* th_inv = nullptr;
  double* th_cp = nullptr;
  double* th_ps = nullptr;  // segment products of the segmented Thomas sweeps
  double* th_qs = nullptr;
  // Fully spectral: per-mode inversion factors tux, tuz, rlap (double,
  // 3 x rows*cols) and tux, tuz (float, 2 x rows*cols).
  double* tab_d = nullptr;
  float* tab_f = nullptr;
  void* tab_df = nullptr;  // tux, tuz as double-float
  int device = 0;
  // Both axes are power-of-two lengths, so the complex-exponential kernels
  // (the fused step, vec_dot_nabla, the velocity) can run.  A fully spectral
  // plan with another axis length (9..4096 points) has the transforms of
  // every basis (Bluestein for lengths that are not powers of two) and the
  // pointwise spectral verbs.
  bool exp_ok = true;
  // Twiddle tables of other transform lengths (cosine/sine bases), by length
  // (guarded by mu).
  mutable std::map<int, void*> tw_extra;
  // Bluestein tables of non-power-of-two transform lengths: chirp, forward
  // and inverse kernel transforms (device), by length (guarded by mu).
  mutable std::map<int, std::array<void*, 3>> blue;
  // Fused-step tile variants [nfields-1][mgb_family] (guarded by mu).
  int tiles[3][3] = {};
  mutable std::mutex mu;
  mutable PrepRecord prep;
};

namespace mgb {

constexpr int NT = 256;  // threads per CTA for every transform kernel

// Record a one-line error for mgb_last_error and return `status`.
int fail(int status, const char* fmt, ...);
int cuda_check(cudaError_t e, const char* what);
#define MGB_CUDA(call)                                       \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return ::mgb::cuda_check(e_, #call); \
  } while (0)
#define MGB_LAUNCH_CHECK() MGB_CUDA(cudaGetLastError())

// Bytes of one transform intermediate (nx rows x ld cols) of complex T:
// complex64 for the split precision, 16 bytes (complex128 or double-float
// pairs) otherwise.
inline size_t inter_bytes(const GridC& g, int prec) {
  return (size_t)g.nx * (size_t)g.cols * (prec == MGB_PREC_SPLIT ? 8 : 16);
}

// Twiddle table of the x or z axis for a precision.
inline const void* twiddles_for(const mgb_plan* p, bool zaxis, int prec) {
  if (prec == MGB_PREC_SPLIT) return zaxis ? p->tw_z_f : p->tw_x_f;
  if (prec == MGB_PREC_DFLOAT) return zaxis ? p->tw_z_df : p->tw_x_df;
  return zaxis ? p->tw_z_d : p->tw_x_d;
}

// ---- fully spectral family (spectral2d.cu) ----
int fs_to_physical(const mgb_plan* p, const zd* spec, double* phys, void* work, cudaStream_t s);
int fs_to_spectral(const mgb_plan* p, const double* phys, zd* spec, void* work, cudaStream_t s);
int fs_vec_dot_nabla(const mgb_plan* p, const zd* q, double* q_phys, const double* ux,
                     const double* uz, zd* out, void* work, cudaStream_t s);
int fs_velocity(const mgb_plan* p, const zd* w, zd* psi, zd* ux_s, zd* uz_s, double* ux,
                double* uz, void* work, cudaStream_t s);
// Optional per-kernel events: ev[0] is recorded before the first kernel and
// ev[k] after kernel k, for k < nev; kernel k waits for wait[k] (when not
// null, k < nwait) before it starts.
struct EventTrack {
  cudaEvent_t* ev = nullptr;
  int nev = 0;
  const cudaEvent_t* wait = nullptr;
  int nwait = 0;
  int k = 0;
  void mark(cudaStream_t s) {
    if (ev && k < nev) cudaEventRecord(ev[k], s);
    if (wait && k < nwait && wait[k]) cudaStreamWaitEvent(s, wait[k], 0);
    ++k;
  }
};

// Members of a batched fused step: field f of slot k has its state at
// q[f] + k * q_stride and its history at hist[f] + k * h_stride (elements).
// A single simulation is count = 1, members = null, zero strides.
struct StepBatch {
  int count = 1;
  const int* members = nullptr;  // device slot list or null (slots 0..count-1)
  zd* q[3] = {nullptr, nullptr, nullptr};
  zd* hist[3] = {nullptr, nullptr, nullptr};
  size_t q_stride = 0, h_stride = 0;
  const double* tcoef = nullptr;  // optional device [slot][3][4] term coefficients
  Gate gate;                      // run control (open unless driven by mgb_run_step)
};

// Twiddles exp(-2 pi i t/L) in double for transform length L (the plan's own
// tables, or one made on first use); null when it cannot be made.
const void* mirror_twiddles(const mgb_plan* p, int L);
// Cosine/sine-basis transforms (csrc/mirror.cu); basis 0 exp, 1 cosine, 2 sine.
int mirror_to_physical(const mgb_plan* p, int bx, int bz, const zd* spec, double* phys, void* work, cudaStream_t s);
int mirror_to_spectral(const mgb_plan* p, int bx, int bz, const double* phys, zd* spec, void* work, cudaStream_t s);
int basis_length(int basis, int n);
// Pointwise spectral verbs with per-axis bases (csrc/pointwise.cu).
int pw_spectral_derivative_basis(const mgb_plan* p, int kind, int bx, int bz, const zd* in, zd* out, cudaStream_t s);
int pw_laplacian_basis(const mgb_plan* p, int bx, int bz, double* lap, cudaStream_t s);
int pw_poisson_basis(const mgb_plan* p, int bx, int bz, const zd* rhs, zd* out, cudaStream_t s);
// MGB_ERR_UNSUPPORTED unless both axes can take complex-exponential FFTs.
int need_exp_ffts(const mgb_plan* p, const char* fn);

// Shape of tile variant `v` of a fused-step kernel family (fully spectral).
int fs_tile_info(const mgb_plan* p, int family, int nfields, int v, mgb_tile_info* out);
int fs_batch_step(const mgb_plan* p, const mgb_equation* eq, const StepBatch& sb, int curr, double dt, void* work,
                  double* diag, cudaStream_t s, EventTrack* et = nullptr);
size_t fs_step_workspace(const mgb_plan* p, int nfields);
size_t fs_batch_workspace(const mgb_plan* p, int nfields, int count);
int fs_prepare(const mgb_plan* p, const mgb_equation* eq, double dt, void* work, cudaStream_t s,
               const mgb_run_state* run = nullptr);
// Tick of a driven run (csrc/driver.cu).
int run_tick(const mgb_plan* p, mgb_run_state* st, const mgb_run_config* cfg, long long upto, int flags,
             cudaStream_t s);
int fs_plan_init(mgb_plan* p);

// ---- Fourier-x / Dirichlet-z family (fdm.cu) ----
int fd_to_physical(const mgb_plan* p, const zd* spec, double* phys, cudaStream_t s);
int fd_to_spectral(const mgb_plan* p, const double* phys, zd* spec, cudaStream_t s);
int fd_poisson(const mgb_plan* p, const zd* rhs, zd* out, cudaStream_t s);
int fd_vec_dot_nabla(const mgb_plan* p, const zd* q, double* q_phys, const double* ux,
                     const double* uz, zd* out, void* work, cudaStream_t s);
int fd_velocity(const mgb_plan* p, const zd* w, zd* psi, zd* uz_s, double* psi_phys, double* ux,
                double* uz, void* work, cudaStream_t s);
int fd_batch_step(const mgb_plan* p, const mgb_equation* eq, const StepBatch& sb, int curr, double dt, void* work,
                  double* diag, cudaStream_t s, EventTrack* et = nullptr);
size_t fd_step_workspace(const mgb_plan* p, int nfields);
size_t fd_batch_workspace(const mgb_plan* p, int nfields, int count);
size_t fd_verb_workspace(const mgb_plan* p);
int fd_plan_init(mgb_plan* p);

// ---- pointwise family (pointwise.cu) ----
int pw_pddx(const mgb_plan* p, const double* in, double* out, cudaStream_t s);
int pw_pddz(const mgb_plan* p, const double* in, double* out, cudaStream_t s);
int pw_spectral_derivative(const mgb_plan* p, int kind, const zd* in, zd* out, cudaStream_t s);
int pw_laplacian(const mgb_plan* p, double* lap, cudaStream_t s);
int pw_poisson_spectral(const mgb_plan* p, const zd* rhs, zd* out, cudaStream_t s);
int pw_integrate_semi_implicit(const mgb_plan* p, zd* var, zd* hist, int order, int curr,
                               double dt, double alpha, const double* lin_op, cudaStream_t s);
int pw_integrate_explicit(const mgb_plan* p, zd* var, zd* hist, int order, int curr, double dt,
                          const zd* diffusion, cudaStream_t s);
int pw_adams(const mgb_plan* p, int corrector, const zd* hist, int order, int curr, double dt,
             zd* out, cudaStream_t s);
int pw_diagnostics(const mgb_plan* p, const double* ux, const double* uz, double* out, void* work,
                   cudaStream_t s);
// Fold per-CTA partials [count][n][3] (sum, max, max) into
// out[count][3] = {0.5*sum/(nx*nz), max, max}.
// Per-CTA diagnostics partials are kDiagW doubles: sum of ux^2 + uz^2, max ux,
// max uz, sum of uz * q for the flux field (0 when none).  The fold writes
// ow = 3 or 4 values per member.
constexpr int kDiagW = 4;
int pw_finish_diag(const double* partial, int n, int count, double inv_npts, double* out, cudaStream_t s,
                   int ow = 3);

}  // namespace mgb
