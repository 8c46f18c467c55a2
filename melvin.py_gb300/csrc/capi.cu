// The extern "C" entry points declared in include/melvin_gb300.h.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>

#include <map>
#include <mutex>
#include <new>
#include <vector>

#include "internal.h"

namespace mgb {

static thread_local char g_last_error[512] = "";

int fail(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return status;
}

int cuda_check(cudaError_t e, const char* what) {
  return fail(MGB_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

// Shared-memory opt-ins already made: (kernel, device) -> largest size set.
static std::mutex g_optin_mu;
static std::map<std::pair<const void*, int>, size_t> g_optin;

bool smem_optin_done(const void* kernel, int device, size_t smem) {
  std::lock_guard<std::mutex> lock(g_optin_mu);
  auto it = g_optin.find({kernel, device});
  return it != g_optin.end() && it->second >= smem;
}

void smem_optin_record(const void* kernel, int device, size_t smem) {
  std::lock_guard<std::mutex> lock(g_optin_mu);
  size_t& v = g_optin[{kernel, device}];
  if (smem > v) v = smem;
}

static bool pow2_in_range(int n) { return n >= 16 && n <= 4096 && (n & (n - 1)) == 0; }

// exp(-2*pi*i*t/n), t in [0, n), evaluated in long double (the values on
// the axes exact), then rounded to double, float and double-float.
static void twiddle_ld(int n, std::vector<long double>& re, std::vector<long double>& im) {
  re.resize(n);
  im.resize(n);
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int t = 0; t < n; ++t) {
    long double c, s;
    if (t == 0) c = 1.0L, s = 0.0L;
    else if (4 * t == n) c = 0.0L, s = 1.0L;
    else if (2 * t == n) c = -1.0L, s = 0.0L;
    else if (4 * t == 3 * n) c = 0.0L, s = -1.0L;
    else {
      const long double ang = 2.0L * pi * (long double)t / (long double)n;
      c = cosl(ang);
      s = sinl(ang);
    }
    re[t] = c;
    im[t] = -s;
  }
}

static df64 to_df64(long double v) {
  const float h = (float)v;
  return df64(h, (float)(v - (long double)h));
}

static int upload_twiddles(int n, void** td, void** tf, void** tdf) {
  std::vector<long double> re, im;
  twiddle_ld(n, re, im);
  std::vector<double> d(2 * (size_t)n);
  std::vector<float> f(2 * (size_t)n);
  std::vector<df64> q(2 * (size_t)n);
  for (int t = 0; t < n; ++t) {
    d[2 * t] = (double)re[t];
    d[2 * t + 1] = (double)im[t];
    f[2 * t] = (float)re[t];
    f[2 * t + 1] = (float)im[t];
    q[2 * t] = to_df64(re[t]);
    q[2 * t + 1] = to_df64(im[t]);
  }
  MGB_CUDA(cudaMalloc(td, d.size() * sizeof(double)));
  MGB_CUDA(cudaMalloc(tf, f.size() * sizeof(float)));
  MGB_CUDA(cudaMalloc(tdf, q.size() * sizeof(df64)));
  MGB_CUDA(cudaMemcpy(*td, d.data(), d.size() * sizeof(double), cudaMemcpyHostToDevice));
  MGB_CUDA(cudaMemcpy(*tf, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
  MGB_CUDA(cudaMemcpy(*tdf, q.data(), q.size() * sizeof(df64), cudaMemcpyHostToDevice));
  return MGB_OK;
}

static void release(mgb_plan* p) {
  if (!p) return;
  for (auto& kv : p->tw_extra) cudaFree(kv.second);
  for (auto& kv : p->blue)
    for (void* q : kv.second) cudaFree(q);
  cudaFree(p->tw_x_d);
  cudaFree(p->tw_x_f);
  cudaFree(p->tw_x_df);
  cudaFree(p->tw_z_d);
  cudaFree(p->tw_z_f);
  cudaFree(p->tw_z_df);
  cudaFree(p->tab_df);
  cudaFree(p->th_inv);
  cudaFree(p->th_cp);
  cudaFree(p->th_ps);
  cudaFree(p->th_qs);
  cudaFree(p->tab_d);
  cudaFree(p->tab_f);
  delete p;
}

const void* mirror_twiddles(const mgb_plan* p, int L) {
  if (L == p->g.nx && p->tw_x_d) return p->tw_x_d;
  if (!p->g.fdm && L == p->g.nz && p->tw_z_d) return p->tw_z_d;
  std::lock_guard<std::mutex> lock(p->mu);
  auto it = p->tw_extra.find(L);
  if (it != p->tw_extra.end()) return it->second;
  void *td = nullptr, *tf = nullptr, *tdf = nullptr;
  const int st = upload_twiddles(L, &td, &tf, &tdf);
  cudaFree(tf);
  cudaFree(tdf);
  if (st != MGB_OK) {
    cudaFree(td);
    return nullptr;
  }
  p->tw_extra[L] = td;
  return td;
}

int need_exp_ffts(const mgb_plan* p, const char* fn) {
  if (p->exp_ok) return MGB_OK;
  return fail(MGB_ERR_UNSUPPORTED,
              "%s: the fused complex-exponential kernels need power-of-two nx and nz; this plan has another axis "
              "length, which the transforms and the pointwise verbs support", fn);
}

// A fully spectral axis of n points: its transforms run for transform
// lengths 16 <= L <= 4096, L = n (complex exponential) or 2(n-1) (cosine,
// sine).
static bool spectral_len(int n) { return n >= 9 && n <= 4096; }

}  // namespace mgb

using namespace mgb;

#define CHECK_PLAN(p) \
  if (!(p)) return fail(MGB_ERR_INVALID, "%s: null plan", __func__)
#define CHECK_PTR(x) \
  if (!(x)) return fail(MGB_ERR_INVALID, "%s: null pointer '%s'", __func__, #x)

extern "C" {

const char* mgb_last_error(void) { return g_last_error; }

const char* mgb_status_string(int32_t status) {
  switch (status) {
    case MGB_OK: return "ok";
    case MGB_ERR_INVALID: return "invalid argument";
    case MGB_ERR_UNSUPPORTED: return "unsupported configuration";
    case MGB_ERR_CUDA: return "CUDA error";
    case MGB_ERR_NONFINITE: return "non-finite value";
    case MGB_ERR_CFL: return "CFL condition breached";
    case MGB_ERR_NOMEM: return "out of device memory";
    default: return "unknown status";
  }
}

int mgb_plan_create(const mgb_grid* grid, mgb_plan** out) {
  CHECK_PTR(grid);
  CHECK_PTR(out);
  *out = nullptr;
  const mgb_grid& G = *grid;
  const bool px = pow2_in_range(G.nx), pz = pow2_in_range(G.nz);
  if (!px && (G.fdm_z || !spectral_len(G.nx)))
    return fail(MGB_ERR_UNSUPPORTED,
                "nx=%d: x transforms need 9..4096 points on a fully spectral grid, a power of two in [16, 4096] "
                "with a Dirichlet z axis", G.nx);
  if (!G.fdm_z && !pz && !spectral_len(G.nz))
    return fail(MGB_ERR_UNSUPPORTED, "nz=%d: fully spectral z transforms need 9..4096 points", G.nz);
  if (G.fdm_z && (G.nz < 5 || G.nz > 1800))
    return fail(MGB_ERR_UNSUPPORTED, "nz=%d: FDM z axis needs 5 <= nz <= 1800", G.nz);
  if (G.sdo != 2 && G.sdo != 4)
    return fail(MGB_ERR_INVALID, "spatial_derivative_order=%d (2 or 4)", G.sdo);
  if (G.precision != MGB_PREC_DOUBLE && G.precision != MGB_PREC_SPLIT && G.precision != MGB_PREC_DFLOAT)
    return fail(MGB_ERR_INVALID, "precision=%d", G.precision);
  if (!(G.lx > 0) || !(G.lz > 0)) return fail(MGB_ERR_INVALID, "box lengths must be positive");
  mgb_plan* p = new (std::nothrow) mgb_plan();
  if (!p) return fail(MGB_ERR_NOMEM, "plan allocation");
  p->grid = G;
  GridC& g = p->g;
  g.nx = G.nx;
  g.nz = G.nz;
  g.nn = (G.nx - 1) / 3;
  g.fdm = G.fdm_z ? 1 : 0;
  g.nm = G.fdm_z ? G.nz : (G.nz - 1) / 3;
  g.rows = G.fdm_z ? g.nn : 2 * g.nn + 1;
  g.cols = g.nm;
  g.sdo = G.sdo;
  g.dx = G.lx / G.nx;
  g.dz = G.lz / G.nz;
  const double tp = 2.0 * M_PI;
  g.dfx = tp / G.lx;
  g.dfz = tp / G.lz;
  g.d2x = -((tp * tp) / (G.lx * G.lx));
  g.d2z = -((tp * tp) / (G.lz * G.lz));
  cudaGetDevice(&p->device);
  p->exp_ok = px && (G.fdm_z || pz);
  int st = px ? upload_twiddles(G.nx, &p->tw_x_d, &p->tw_x_f, &p->tw_x_df) : MGB_OK;
  if (!st && !G.fdm_z && pz) st = upload_twiddles(G.nz, &p->tw_z_d, &p->tw_z_f, &p->tw_z_df);
  if (!st && !G.fdm_z) st = fs_plan_init(p);
  if (!st && G.fdm_z) st = fd_plan_init(p);
  if (st) {
    release(p);
    return st;
  }
  *out = p;
  return MGB_OK;
}

int mgb_plan_destroy(mgb_plan* plan) {
  release(plan);
  return MGB_OK;
}

int mgb_plan_shapes(const mgb_plan* p, int32_t* spec_rows, int32_t* spec_cols, int32_t* phys_rows,
                    int32_t* phys_cols) {
  CHECK_PLAN(p);
  if (spec_rows) *spec_rows = p->g.rows;
  if (spec_cols) *spec_cols = p->g.cols;
  if (phys_rows) *phys_rows = p->g.nx;
  if (phys_cols) *phys_cols = p->g.nz;
  return MGB_OK;
}

int mgb_workspace_bytes(const mgb_plan* p, int32_t family, int32_t nfields, size_t* bytes) {
  CHECK_PLAN(p);
  CHECK_PTR(bytes);
  const size_t diag = 152 * 4 * kDiagW * sizeof(double) + 256;
  if (family == 0) {
    size_t b = p->g.fdm ? fd_verb_workspace(p) : 2 * inter_bytes(p->g, MGB_PREC_DOUBLE);
    *bytes = (b > diag ? b : diag) + 256;
    return MGB_OK;
  }
  if (family == 1) {
    if (nfields < 1 || nfields > 3) return fail(MGB_ERR_INVALID, "nfields=%d (1..3)", nfields);
    *bytes = (p->g.fdm ? fd_step_workspace(p, nfields) : fs_step_workspace(p, nfields)) + 256;
    return MGB_OK;
  }
  return fail(MGB_ERR_INVALID, "workspace family %d", family);
}

int mgb_to_physical(const mgb_plan* p, const void* spec, double* phys, void* work, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(spec);
  CHECK_PTR(phys);
  // an axis that is not a power of two: the basis path with both axes
  // complex exponential (Bluestein transforms)
  if (!p->exp_ok && !p->g.fdm) {
    CHECK_PTR(work);
    return mirror_to_physical(p, 0, 0, (const zd*)spec, phys, work, (cudaStream_t)stream);
  }
  if (int st = need_exp_ffts(p, __func__)) return st;
  if (p->g.fdm) return fd_to_physical(p, (const zd*)spec, phys, (cudaStream_t)stream);
  CHECK_PTR(work);
  return fs_to_physical(p, (const zd*)spec, phys, work, (cudaStream_t)stream);
}

int mgb_to_spectral(const mgb_plan* p, const double* phys, void* spec, void* work, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(spec);
  CHECK_PTR(phys);
  if (!p->exp_ok && !p->g.fdm) {
    CHECK_PTR(work);
    return mirror_to_spectral(p, 0, 0, phys, (zd*)spec, work, (cudaStream_t)stream);
  }
  if (int st = need_exp_ffts(p, __func__)) return st;
  if (p->g.fdm) return fd_to_spectral(p, phys, (zd*)spec, (cudaStream_t)stream);
  CHECK_PTR(work);
  return fs_to_spectral(p, phys, (zd*)spec, work, (cudaStream_t)stream);
}

int mgb_to_physical_basis(const mgb_plan* p, int32_t bx, int32_t bz, const void* spec, double* phys, void* work,
                          void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(spec);
  CHECK_PTR(phys);
  CHECK_PTR(work);
  if (bx == MGB_BASIS_COMPLEX_EXP && bz == MGB_BASIS_COMPLEX_EXP) return mgb_to_physical(p, spec, phys, work, stream);
  return mirror_to_physical(p, bx, bz, (const zd*)spec, phys, work, (cudaStream_t)stream);
}

int mgb_to_spectral_basis(const mgb_plan* p, int32_t bx, int32_t bz, const double* phys, void* spec, void* work,
                          void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(spec);
  CHECK_PTR(phys);
  CHECK_PTR(work);
  if (bx == MGB_BASIS_COMPLEX_EXP && bz == MGB_BASIS_COMPLEX_EXP) return mgb_to_spectral(p, phys, spec, work, stream);
  return mirror_to_spectral(p, bx, bz, phys, (zd*)spec, work, (cudaStream_t)stream);
}

int mgb_spectral_derivative_basis(const mgb_plan* p, int32_t kind, int32_t bx, int32_t bz, const void* in, void* out,
                                  void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(in);
  CHECK_PTR(out);
  return pw_spectral_derivative_basis(p, kind, bx, bz, (const zd*)in, (zd*)out, (cudaStream_t)stream);
}

int mgb_laplacian_basis(const mgb_plan* p, int32_t bx, int32_t bz, double* lap, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(lap);
  return pw_laplacian_basis(p, bx, bz, lap, (cudaStream_t)stream);
}

int mgb_poisson_solve_basis(const mgb_plan* p, int32_t bx, int32_t bz, const void* rhs, void* out, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(rhs);
  CHECK_PTR(out);
  return pw_poisson_basis(p, bx, bz, (const zd*)rhs, (zd*)out, (cudaStream_t)stream);
}

int mgb_pddx(const mgb_plan* p, const double* in, double* out, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(in);
  CHECK_PTR(out);
  if (in == out) return fail(MGB_ERR_INVALID, "pddx: input and output must differ");
  return pw_pddx(p, in, out, (cudaStream_t)stream);
}

int mgb_pddz(const mgb_plan* p, const double* in, double* out, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(in);
  CHECK_PTR(out);
  if (in == out) return fail(MGB_ERR_INVALID, "pddz: input and output must differ");
  return pw_pddz(p, in, out, (cudaStream_t)stream);
}

int mgb_spectral_derivative(const mgb_plan* p, int32_t kind, const void* in, void* out, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(in);
  CHECK_PTR(out);
  return pw_spectral_derivative(p, kind, (const zd*)in, (zd*)out, (cudaStream_t)stream);
}

int mgb_laplacian(const mgb_plan* p, double* lap, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(lap);
  return pw_laplacian(p, lap, (cudaStream_t)stream);
}

int mgb_poisson_solve(const mgb_plan* p, const void* rhs, void* out, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(rhs);
  CHECK_PTR(out);
  if (p->g.fdm) return fd_poisson(p, (const zd*)rhs, (zd*)out, (cudaStream_t)stream);
  return pw_poisson_spectral(p, (const zd*)rhs, (zd*)out, (cudaStream_t)stream);
}

int mgb_vec_dot_nabla(const mgb_plan* p, const void* q_spec, double* q_phys, const double* ux, const double* uz,
                      void* out_spec, void* work, void* stream) {
  CHECK_PLAN(p);
  if (int st = need_exp_ffts(p, __func__)) return st;
  CHECK_PTR(q_spec);
  CHECK_PTR(q_phys);
  CHECK_PTR(ux);
  CHECK_PTR(uz);
  CHECK_PTR(out_spec);
  CHECK_PTR(work);
  if (p->g.fdm)
    return fd_vec_dot_nabla(p, (const zd*)q_spec, q_phys, ux, uz, (zd*)out_spec, work, (cudaStream_t)stream);
  return fs_vec_dot_nabla(p, (const zd*)q_spec, q_phys, ux, uz, (zd*)out_spec, work, (cudaStream_t)stream);
}

int mgb_velocity_from_vorticity(const mgb_plan* p, const void* w_spec, void* psi_spec, void* ux_spec, void* uz_spec,
                                double* psi_phys, double* ux_phys, double* uz_phys, void* work, void* stream) {
  CHECK_PLAN(p);
  if (int st = need_exp_ffts(p, __func__)) return st;
  CHECK_PTR(w_spec);
  CHECK_PTR(psi_spec);
  CHECK_PTR(ux_phys);
  CHECK_PTR(uz_phys);
  CHECK_PTR(work);
  if (p->g.fdm)
    return fd_velocity(p, (const zd*)w_spec, (zd*)psi_spec, (zd*)uz_spec, psi_phys, ux_phys, uz_phys, work,
                       (cudaStream_t)stream);
  return fs_velocity(p, (const zd*)w_spec, (zd*)psi_spec, (zd*)ux_spec, (zd*)uz_spec, ux_phys, uz_phys, work,
                     (cudaStream_t)stream);
}

int mgb_integrate_semi_implicit(const mgb_plan* p, void* var, void* hist, int32_t order, int32_t curr, double dt,
                                double alpha, const double* lin_op, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(var);
  CHECK_PTR(hist);
  CHECK_PTR(lin_op);
  if (order != 2 && order != 4) return fail(MGB_ERR_INVALID, "integrator_order=%d (2 or 4)", order);
  if (curr < 0 || curr >= order) return fail(MGB_ERR_INVALID, "curr_idx=%d out of range", curr);
  return pw_integrate_semi_implicit(p, (zd*)var, (zd*)hist, order, curr, dt, alpha, lin_op, (cudaStream_t)stream);
}

int mgb_integrate_explicit(const mgb_plan* p, void* var, void* hist, int32_t order, int32_t curr, double dt,
                           const void* diffusion, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(var);
  CHECK_PTR(hist);
  CHECK_PTR(diffusion);
  if (order != 2 && order != 4) return fail(MGB_ERR_INVALID, "integrator_order=%d (2 or 4)", order);
  if (curr < 0 || curr >= order) return fail(MGB_ERR_INVALID, "curr_idx=%d out of range", curr);
  return pw_integrate_explicit(p, (zd*)var, (zd*)hist, order, curr, dt, (const zd*)diffusion, (cudaStream_t)stream);
}

int mgb_adams(const mgb_plan* p, int32_t corrector, const void* hist, int32_t order, int32_t curr, double dt,
              void* out, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(hist);
  CHECK_PTR(out);
  if (order != 2 && order != 4) return fail(MGB_ERR_INVALID, "integrator_order=%d (2 or 4)", order);
  if (curr < 0 || curr >= order) return fail(MGB_ERR_INVALID, "curr_idx=%d out of range", curr);
  return pw_adams(p, corrector, (const zd*)hist, order, curr, dt, (zd*)out, (cudaStream_t)stream);
}

int mgb_diagnostics(const mgb_plan* p, const double* ux, const double* uz, double* out, void* work, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(ux);
  CHECK_PTR(uz);
  CHECK_PTR(out);
  CHECK_PTR(work);
  return pw_diagnostics(p, ux, uz, out, work, (cudaStream_t)stream);
}

static int check_equation(const mgb_equation* eq, int32_t curr) {
  const int F = eq->nfields;
  if (F < 1 || F > 3) return fail(MGB_ERR_INVALID, "nfields=%d (1..3)", F);
  if (eq->order != 2 && eq->order != 4) return fail(MGB_ERR_INVALID, "integrator_order=%d (2 or 4)", eq->order);
  if (curr < 0 || curr >= eq->order) return fail(MGB_ERR_INVALID, "curr_idx=%d out of range", curr);
  if (eq->diag_flux < 0 || eq->diag_flux > F)
    return fail(MGB_ERR_INVALID, "diag_flux=%d (0 for none, or 1..nfields)", eq->diag_flux);
  for (int f = 0; f < F; ++f) {
    const mgb_field_eq& fe = eq->f[f];
    if (fe.nterms < 0 || fe.nterms > 4) return fail(MGB_ERR_INVALID, "field %d: nterms=%d (0..4)", f, fe.nterms);
    for (int t = 0; t < fe.nterms; ++t) {
      if (fe.terms[t].src < -1 || fe.terms[t].src >= F)
        return fail(MGB_ERR_INVALID, "field %d term %d: src=%d", f, t, fe.terms[t].src);
      if (fe.terms[t].op < 0 || fe.terms[t].op > 2)
        return fail(MGB_ERR_INVALID, "field %d term %d: op=%d", f, t, fe.terms[t].op);
    }
  }
  return MGB_OK;
}

static int dispatch_step(const mgb_plan* p, const mgb_equation* eq, const StepBatch& sb, int32_t curr, double dt,
                         void* work, double* diag, void* stream, EventTrack* et) {
  if (int st = need_exp_ffts(p, "mgb_step")) return st;
  if (p->g.fdm) return fd_batch_step(p, eq, sb, curr, dt, work, diag, (cudaStream_t)stream, et);
  if (eq->integrator != MGB_INT_SEMI_IMPLICIT && eq->integrator != MGB_INT_EXPLICIT)
    return fail(MGB_ERR_UNSUPPORTED, "fully spectral step: integrator %d", eq->integrator);
  return fs_batch_step(p, eq, sb, curr, dt, work, diag, (cudaStream_t)stream, et);
}

static int step_impl(const mgb_plan* p, const mgb_equation* eq, void* const* q, void* const* hist, int32_t curr,
                     double dt, void* work, double* diag, void* stream, EventTrack* et, Gate gate = Gate()) {
  CHECK_PLAN(p);
  CHECK_PTR(eq);
  CHECK_PTR(q);
  CHECK_PTR(hist);
  CHECK_PTR(work);
  const int F = eq->nfields;
  int st = check_equation(eq, curr);
  if (st) return st;
  for (int f = 0; f < F; ++f) {
    if (!q[f] || !hist[f]) return fail(MGB_ERR_INVALID, "null state or history for field %d", f);
    const mgb_field_eq& fe = eq->f[f];
    if (fe.nterms < 0 || fe.nterms > 4) return fail(MGB_ERR_INVALID, "field %d: nterms=%d (0..4)", f, fe.nterms);
    for (int t = 0; t < fe.nterms; ++t) {
      if (fe.terms[t].src < -1 || fe.terms[t].src >= F)
        return fail(MGB_ERR_INVALID, "field %d term %d: src=%d", f, t, fe.terms[t].src);
      if (fe.terms[t].op < 0 || fe.terms[t].op > 2)
        return fail(MGB_ERR_INVALID, "field %d term %d: op=%d", f, t, fe.terms[t].op);
    }
  }
  StepBatch sb;
  sb.count = 1;
  sb.gate = gate;
  for (int f = 0; f < F; ++f) {
    sb.q[f] = (zd*)q[f];
    sb.hist[f] = (zd*)hist[f];
  }
  return dispatch_step(p, eq, sb, curr, dt, work, diag, stream, et);
}

int mgb_step(const mgb_plan* p, const mgb_equation* eq, void* const* q, void* const* hist, int32_t curr, double dt,
             void* work, double* diag, void* stream) {
  return step_impl(p, eq, q, hist, curr, dt, work, diag, stream, nullptr);
}

int mgb_batch_workspace_bytes(const mgb_plan* p, int32_t nfields, int32_t count, size_t* bytes) {
  CHECK_PLAN(p);
  CHECK_PTR(bytes);
  if (nfields < 1 || nfields > 3) return fail(MGB_ERR_INVALID, "nfields=%d (1..3)", nfields);
  if (count < 1) return fail(MGB_ERR_INVALID, "count=%d", count);
  *bytes = (p->g.fdm ? fd_batch_workspace(p, nfields, count) : fs_batch_workspace(p, nfields, count)) + 256;
  return MGB_OK;
}

int mgb_batch_step(const mgb_plan* p, const mgb_equation* eq, const mgb_batch* batch, int32_t curr, double dt,
                   void* work, double* diag, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(eq);
  CHECK_PTR(batch);
  CHECK_PTR(work);
  CHECK_PTR(batch->q);
  CHECK_PTR(batch->hist);
  int st = check_equation(eq, curr);
  if (st) return st;
  if (batch->count < 1 || batch->count > 65535) return fail(MGB_ERR_INVALID, "batch count=%d", batch->count);
  const int F = eq->nfields;
  const size_t S = (size_t)p->g.rows * p->g.cols;
  StepBatch sb;
  sb.count = batch->count;
  sb.members = batch->members;
  sb.q_stride = (size_t)F * S;
  sb.h_stride = (size_t)F * eq->order * S;
  sb.tcoef = batch->term_coef;
  for (int f = 0; f < F; ++f) {
    sb.q[f] = (zd*)batch->q + (size_t)f * S;
    sb.hist[f] = (zd*)batch->hist + (size_t)f * eq->order * S;
  }
  return dispatch_step(p, eq, sb, curr, dt, work, diag, stream, nullptr);
}

int mgb_step_prepare(const mgb_plan* p, const mgb_equation* eq, double dt, void* work, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(eq);
  CHECK_PTR(work);
  const int F = eq->nfields;
  if (F < 1 || F > 3) return fail(MGB_ERR_INVALID, "nfields=%d (1..3)", F);
  if (eq->order != 2 && eq->order != 4) return fail(MGB_ERR_INVALID, "integrator_order=%d (2 or 4)", eq->order);
  if (p->g.fdm) return MGB_OK;  // the Dirichlet update needs no per-mode coefficients
  int st = fs_prepare(p, eq, dt, work, (cudaStream_t)stream);
  std::lock_guard<std::mutex> lock(p->mu);
  PrepRecord& pr = p->prep;
  pr.valid = st == MGB_OK;
  pr.work = work;
  pr.dt = dt;
  pr.alpha = eq->alpha;
  pr.nfields = F;
  pr.integrator = eq->integrator;
  pr.order = eq->order;
  pr.driven = false;
  for (int f = 0; f < 3; ++f) pr.kappa[f] = f < F ? eq->f[f].kappa : 0.0;
  return st;
}

int mgb_step_kernel_count(const mgb_plan* p, const mgb_equation* eq, int32_t* count) {
  CHECK_PLAN(p);
  CHECK_PTR(eq);
  CHECK_PTR(count);
  if (!p->g.fdm) *count = 3;
  else *count = eq->integrator == MGB_INT_PECE ? 8 : 4;
  return MGB_OK;
}

int mgb_step_events(const mgb_plan* p, const mgb_equation* eq, void* const* q, void* const* hist, int32_t curr,
                    double dt, void* work, double* diag, void* stream, void* const* events, int32_t nevents) {
  CHECK_PTR(events);
  EventTrack et;
  et.ev = (cudaEvent_t*)events;
  et.nev = nevents;
  return step_impl(p, eq, q, hist, curr, dt, work, diag, stream, &et);
}

int mgb_step_waits(const mgb_plan* p, const mgb_equation* eq, void* const* q, void* const* hist, int32_t curr,
                   double dt, void* work, double* diag, void* stream, void* const* waits, int32_t nwaits) {
  CHECK_PTR(waits);
  if (nwaits < 0) return fail(MGB_ERR_INVALID, "mgb_step_waits: nwaits=%d", nwaits);
  EventTrack et;
  et.wait = (const cudaEvent_t*)waits;
  et.nwait = nwaits;
  return step_impl(p, eq, q, hist, curr, dt, work, diag, stream, &et);
}

static int check_run_config(const mgb_run_config* cfg, const char* fn) {
  if (cfg->horizon < 1) return fail(MGB_ERR_INVALID, "%s: horizon=%d (>= 1)", fn, cfg->horizon);
  if (cfg->cfl_cadence < 0 || cfg->tracker_cadence < 0 || cfg->capacity < 0)
    return fail(MGB_ERR_INVALID, "%s: negative cadence or capacity", fn);
  if (cfg->capacity > 0 && (!cfg->tracker_t || !cfg->tracker_ke))
    return fail(MGB_ERR_INVALID, "%s: tracker buffers missing", fn);
  return MGB_OK;
}

int mgb_run_begin(const mgb_plan* p, mgb_run_state* state, const mgb_run_config* cfg, void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(state);
  CHECK_PTR(cfg);
  if (int st = check_run_config(cfg, __func__)) return st;
  // no iteration since the last tick: only the stop point is computed
  return run_tick(p, state, cfg, -1, 0, (cudaStream_t)stream);
}

int mgb_run_step(const mgb_plan* p, const mgb_equation* eq, void* const* q, void* const* hist, int32_t curr,
                 int64_t loop, int32_t flags, void* work, mgb_run_state* state, const mgb_run_config* cfg,
                 void* stream) {
  CHECK_PLAN(p);
  CHECK_PTR(eq);
  CHECK_PTR(state);
  CHECK_PTR(cfg);
  if (int st = check_run_config(cfg, __func__)) return st;
  if (loop < 0) return fail(MGB_ERR_INVALID, "%s: loop=%lld", __func__, (long long)loop);
  if ((flags & MGB_RUN_CFL) && cfg->cfl_cadence < 1)
    return fail(MGB_ERR_INVALID, "%s: CFL tick without a CFL cadence", __func__);
  if ((flags & MGB_RUN_TRACK) && cfg->tracker_cadence < 1)
    return fail(MGB_ERR_INVALID, "%s: tracker tick without a tracker cadence", __func__);
  if (cfg->tracker_flux && !eq->diag_flux)
    return fail(MGB_ERR_INVALID, "%s: a flux tracker needs eq->diag_flux", __func__);
  double dt = 0.0;
  if (!p->g.fdm) {
    std::lock_guard<std::mutex> lock(p->mu);
    dt = p->prep.dt;  // the coefficients follow the device dt from here on
  }
  Gate gate;
  gate.stop_at = (const long long*)&state->stop_loop;
  gate.loop = loop;
  gate.dt = &state->dt;
  const bool diagnose = (flags & (MGB_RUN_CFL | MGB_RUN_TRACK)) != 0;
  int st = step_impl(p, eq, q, hist, curr, dt, work, diagnose ? state->diag : nullptr, stream, nullptr, gate);
  if (st) return st;
  if (!p->g.fdm) {
    std::lock_guard<std::mutex> lock(p->mu);
    p->prep.driven = true;
  }
  if (!flags) return MGB_OK;
  st = run_tick(p, state, cfg, (long long)loop + 1, flags, (cudaStream_t)stream);
  if (st) return st;
  if ((flags & MGB_RUN_CFL) && !p->g.fdm) return fs_prepare(p, eq, dt, work, (cudaStream_t)stream, state);
  return MGB_OK;
}

static int check_tile_args(const mgb_plan* p, const char* fn, int32_t nfields) {
  if (p->g.fdm) return fail(MGB_ERR_UNSUPPORTED, "%s: tile variants exist for fully spectral plans only", fn);
  if (int st = need_exp_ffts(p, fn)) return st;
  if (nfields < 1 || nfields > 3) return fail(MGB_ERR_INVALID, "%s: nfields=%d outside 1..3", fn, nfields);
  return MGB_OK;
}

int mgb_tile_info_get(const mgb_plan* p, int32_t family, int32_t nfields, int32_t variant, mgb_tile_info* info) {
  CHECK_PLAN(p);
  CHECK_PTR(info);
  if (int st = check_tile_args(p, __func__, nfields)) return st;
  if (family < 0 || family > 2) return fail(MGB_ERR_INVALID, "%s: family=%d outside 0..2", __func__, family);
  if (variant < 0 || variant >= MGB_TILE_VARIANTS)
    return fail(MGB_ERR_INVALID, "%s: variant=%d outside 0..%d", __func__, variant, MGB_TILE_VARIANTS - 1);
  return fs_tile_info(p, family, nfields, variant, info);
}

int mgb_plan_set_tiles(mgb_plan* p, int32_t nfields, const int32_t* tiles) {
  CHECK_PLAN(p);
  CHECK_PTR(tiles);
  if (int st = check_tile_args(p, __func__, nfields)) return st;
  for (int k = 0; k < 3; ++k) {
    mgb_tile_info info;
    if (tiles[k] < 0 || tiles[k] >= MGB_TILE_VARIANTS)
      return fail(MGB_ERR_INVALID, "%s: tiles[%d]=%d outside 0..%d", __func__, k, tiles[k], MGB_TILE_VARIANTS - 1);
    fs_tile_info(p, k, nfields, tiles[k], &info);
    if (!info.available)
      return fail(MGB_ERR_INVALID, "%s: variant %d of family %d does not fit shared memory on this grid", __func__,
                  tiles[k], k);
  }
  std::lock_guard<std::mutex> lock(p->mu);
  for (int k = 0; k < 3; ++k) p->tiles[nfields - 1][k] = tiles[k];
  return MGB_OK;
}

int mgb_plan_get_tiles(const mgb_plan* p, int32_t nfields, int32_t* tiles) {
  CHECK_PLAN(p);
  CHECK_PTR(tiles);
  if (int st = check_tile_args(p, __func__, nfields)) return st;
  std::lock_guard<std::mutex> lock(p->mu);
  for (int k = 0; k < 3; ++k) tiles[k] = p->tiles[nfields - 1][k];
  return MGB_OK;
}

}  // extern "C"
