// Host orchestration of the fully spectral (doubly periodic) kernels.
#include <vector>

#include "spectral2d_impl.cuh"

namespace mgb {

const FsLaunchers* fs_launchers_16();
const FsLaunchers* fs_launchers_32();
const FsLaunchers* fs_launchers_64();
const FsLaunchers* fs_launchers_128();
const FsLaunchers* fs_launchers_256();
const FsLaunchers* fs_launchers_512();
const FsLaunchers* fs_launchers_1024();
const FsLaunchers* fs_launchers_2048();
const FsLaunchers* fs_launchers_4096();

const FsLaunchers* fs_launchers(int N) {
  switch (N) {
    case 16: return fs_launchers_16();
    case 32: return fs_launchers_32();
    case 64: return fs_launchers_64();
    case 128: return fs_launchers_128();
    case 256: return fs_launchers_256();
    case 512: return fs_launchers_512();
    case 1024: return fs_launchers_1024();
    case 2048: return fs_launchers_2048();
    case 4096: return fs_launchers_4096();
    default: return nullptr;
  }
}

static inline double fd_inv(int sdo, double h) { return sdo == 2 ? 1.0 / (2.0 * h) : 1.0 / (3.0 * h); }

static int launched(cudaError_t e, const char* what) {
  if (e == cudaErrorInvalidConfiguration)
    return fail(MGB_ERR_UNSUPPORTED, "%s: shared-memory footprint too large for this size", what);
  if (e != cudaSuccess) return cuda_check(e, what);
  return MGB_OK;
}

static void set_tables(const mgb_plan* p, XinvArgs& xa, int prec) {
  const size_t S = (size_t)p->g.rows * p->g.cols;
  if (prec == MGB_PREC_SPLIT) {
    xa.tux = p->tab_f;
    xa.tuz = p->tab_f + S;
  } else if (prec == MGB_PREC_DFLOAT) {
    xa.tux = (const df64*)p->tab_df;
    xa.tuz = (const df64*)p->tab_df + S;
  } else {
    xa.tux = p->tab_d;
    xa.tuz = p->tab_d + S;
  }
  xa.rlap = p->tab_d + 2 * S;
}

int fs_to_physical(const mgb_plan* p, const zd* spec, double* phys, void* work, cudaStream_t s) {
  const GridC& g = p->g;
  const FsLaunchers* Lx = fs_launchers(g.nx);
  const FsLaunchers* Lz = fs_launchers(g.nz);
  XinvArgs xa = {};
  xa.g = g;
  xa.ld = g.cols;
  xa.tw = p->tw_x_d;
  set_tables(p, xa, MGB_PREC_DOUBLE);
  xa.job[0] = XinvJob{spec, SRC_COPY, work, nullptr, nullptr};
  int st = launched(Lx->xinv[0][0](xa, 1, 1, s), "to_physical x pass");
  if (st) return st;
  ZinvArgs za = {};
  za.g = g;
  za.ld = g.cols;
  za.in[0] = work;
  za.out[0] = phys;
  za.tw = p->tw_z_d;
  return launched(Lz->zinv_phys[0](za, s), "to_physical z pass");
}

int fs_to_spectral(const mgb_plan* p, const double* phys, zd* spec, void* work, cudaStream_t s) {
  const GridC& g = p->g;
  const FsLaunchers* Lx = fs_launchers(g.nx);
  const FsLaunchers* Lz = fs_launchers(g.nz);
  ZfwdArgs za = {};
  za.g = g;
  za.ld = g.cols;
  za.in = phys;
  za.out = work;
  za.tw = p->tw_z_d;
  int st = launched(Lz->zfwd_phys(za, s), "to_spectral z pass");
  if (st) return st;
  XfOutArgs xa = {};
  xa.g = g;
  xa.ld = g.cols;
  xa.ain = work;
  xa.cin = nullptr;
  xa.out = spec;
  xa.scale = 1.0 / ((double)g.nx * (double)g.nz);
  xa.fdx = fd_inv(g.sdo, g.dx);
  xa.tw = p->tw_x_d;
  return launched(Lx->xf_out(xa, s), "to_spectral x pass");
}

int fs_vec_dot_nabla(const mgb_plan* p, const zd* q, double* q_phys, const double* ux,
                     const double* uz, zd* out, void* work, cudaStream_t s) {
  const GridC& g = p->g;
  const FsLaunchers* Lx = fs_launchers(g.nx);
  const FsLaunchers* Lz = fs_launchers(g.nz);
  char* w0 = (char*)work;
  char* w1 = w0 + inter_bytes(g, MGB_PREC_DOUBLE);
  XinvArgs xa = {};
  xa.g = g;
  xa.ld = g.cols;
  xa.tw = p->tw_x_d;
  set_tables(p, xa, MGB_PREC_DOUBLE);
  xa.job[0] = XinvJob{q, SRC_COPY, w0, nullptr, nullptr};
  int st = launched(Lx->xinv[0][0](xa, 1, 1, s), "vec_dot_nabla x pass");
  if (st) return st;
  ZvdnArgs za = {};
  za.g = g;
  za.ld = g.cols;
  za.qin = w0;
  za.qphys = q_phys;
  za.ux = ux;
  za.uz = uz;
  za.aout = w0;
  za.cout = w1;
  za.fdz = fd_inv(g.sdo, g.dz);
  za.tw = p->tw_z_d;
  st = launched(Lz->zz_vdn(za, s), "vec_dot_nabla z pass");
  if (st) return st;
  XfOutArgs fa = {};
  fa.g = g;
  fa.ld = g.cols;
  fa.ain = w0;
  fa.cin = w1;
  fa.out = out;
  fa.scale = 1.0 / ((double)g.nx * (double)g.nz);
  fa.fdx = fd_inv(g.sdo, g.dx);
  fa.tw = p->tw_x_d;
  return launched(Lx->xf_out(fa, s), "vec_dot_nabla forward x pass");
}

int fs_velocity(const mgb_plan* p, const zd* w, zd* psi, zd* ux_s, zd* uz_s, double* ux,
                double* uz, void* work, cudaStream_t s) {
  const GridC& g = p->g;
  const FsLaunchers* Lx = fs_launchers(g.nx);
  const FsLaunchers* Lz = fs_launchers(g.nz);
  char* w0 = (char*)work;
  char* w1 = w0 + inter_bytes(g, MGB_PREC_DOUBLE);
  XinvArgs xa = {};
  xa.g = g;
  xa.ld = g.cols;
  xa.tw = p->tw_x_d;
  set_tables(p, xa, MGB_PREC_DOUBLE);
  xa.job[0] = XinvJob{w, SRC_UX, w0, ux_s, psi};
  xa.job[1] = XinvJob{w, SRC_UZ, w1, uz_s, nullptr};
  int st = launched(Lx->xinv[0][0](xa, 2, 1, s), "velocity x pass");
  if (st) return st;
  ZinvArgs za = {};
  za.g = g;
  za.ld = g.cols;
  za.in[0] = w0;
  za.in[1] = w1;
  za.out[0] = ux;
  za.out[1] = uz;
  za.tw = p->tw_z_d;
  return launched(Lz->zinv_phys[1](za, s), "velocity z pass");
}

static inline size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

// Step scratch: per-field update coefficients (a, b) per mode (shared by
// all members, at a fixed offset), then per member the diagnostics partials
// and the transform intermediates.
struct FsWork {
  zd* coef[3];
  double* partial;        // [count][nx/2][kDiagW]
  char* inter[6];         // member 0's intermediates
  size_t inter_stride;    // bytes between members' intermediate blocks
  size_t bytes;
};

static FsWork fs_carve(const mgb_plan* p, int F, int count, void* base) {
  const int nin = 2 + F, nout = 2 * F;
  const int ninter = nin > nout ? nin : nout;
  const size_t ib = al256(inter_bytes(p->g, p->grid.precision));
  FsWork w = {};
  char* c = (char*)base;
  size_t off = 0;
  for (int f = 0; f < 3; ++f) {
    w.coef[f] = (zd*)(c + off);
    if (f < F) off += al256((size_t)p->g.rows * p->g.cols * sizeof(zd));
  }
  w.partial = (double*)(c + off);
  off += al256((size_t)count * (p->g.nx / 2) * kDiagW * sizeof(double));
  for (int i = 0; i < 6; ++i) w.inter[i] = c + off + (size_t)(i < ninter ? i : ninter - 1) * ib;
  w.inter_stride = (size_t)ninter * ib;
  off += (size_t)count * w.inter_stride;
  w.bytes = off;
  return w;
}

size_t fs_step_workspace(const mgb_plan* p, int nfields) { return fs_carve(p, nfields, 1, nullptr).bytes; }
size_t fs_batch_workspace(const mgb_plan* p, int nfields, int count) {
  return fs_carve(p, nfields, count, nullptr).bytes;
}

// Per-mode update coefficients of one field, with L = kappa * lap(n, m):
//   semi-implicit (melvin/Integrator.py:58-63):
//     a = (1 + (1-alpha) dt L) / (1 - alpha dt L),  b = c_AB / (1 - alpha dt L)
//   explicit (melvin/Integrator.py:53-56):  a = L,  b = c_AB
// with c_AB = dt/2 (AB2) or dt/24 (AB4).
// With `run` set (a driven run), the coefficients follow the run's device
// dt and are recomputed only after a tick that changed it.
__global__ void k_update_coefs(GridC g, double kappa, int semi, double dt, double alpha, double cab,
                               zd* __restrict__ out, const mgb_run_state* run, int order) {
  if (run) {
    if (!run->dt_changed) return;
    dt = run->dt;
    cab = order == 2 ? dt / 2 : dt / 24;
  }
  const size_t total = (size_t)g.rows * g.cols;
  for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < total; i += (size_t)gridDim.x * NT) {
    const int r = (int)(i / g.cols), m = (int)(i - (size_t)r * g.cols);
    const int n = row_mode(r, g.nn);
    const double L = kappa * lap_symbol(g, n, m);
    if (semi) {
      const double c1 = 1 + ((1 - alpha) * dt) * L;
      const double den = 1 - (alpha * dt) * L;
      out[i] = mk(c1 / den, cab / den);
    } else {
      out[i] = mk(L, cab);
    }
  }
}

int fs_prepare(const mgb_plan* p, const mgb_equation* eq, double dt, void* work, cudaStream_t s,
               const mgb_run_state* run) {
  const GridC& g = p->g;
  FsWork w = fs_carve(p, eq->nfields, 1, work);
  const double cab = eq->order == 2 ? dt / 2 : dt / 24;
  const size_t total = (size_t)g.rows * g.cols;
  size_t nb = (total + NT - 1) / NT;
  nb = nb > 152 * 8 ? 152 * 8 : nb;
  for (int f = 0; f < eq->nfields; ++f) {
    k_update_coefs<<<(int)nb, NT, 0, s>>>(g, eq->f[f].kappa, eq->integrator == MGB_INT_SEMI_IMPLICIT ? 1 : 0, dt,
                                          eq->alpha, cab, w.coef[f], run, eq->order);
    MGB_LAUNCH_CHECK();
  }
  return MGB_OK;
}

int fs_plan_init(mgb_plan* p) {
  const GridC& g = p->g;
  // The fused inverse transforms skip the inputs 3N/8 .. 5N/8 - 1 as removed
  // modes: true of the 2/3 rule (nn = (nx - 1) / 3) at every power of two.
  if ((fs_launchers(g.nx) && 8 * (g.nn + 1) > 3 * g.nx) || (fs_launchers(g.nz) && 8 * g.nm > 3 * g.nz))
    return MGB_ERR_INVALID;
  const size_t S = (size_t)g.rows * g.cols;
  std::vector<double> td(3 * S);
  std::vector<float> tf(2 * S);
  for (int r = 0; r < g.rows; ++r) {
    const int n = row_mode(r, g.nn);
    for (int m = 0; m < g.cols; ++m) {
      const size_t i = (size_t)r * g.cols + m;
      const double a = g.d2x * (double)(n * n);
      const double b = g.d2z * (double)(m * m);
      const double lap = (i == 0) ? 1.0 : a + b;
      const double tux = (g.dfz * (double)m) / lap;
      const double tuz = (g.dfx * (double)n) / lap;
      td[i] = tux;
      td[S + i] = tuz;
      td[2 * S + i] = 1.0 / lap;
      tf[i] = (float)tux;
      tf[S + i] = (float)tuz;
    }
  }
  std::vector<df64> tdf(2 * S);
  for (size_t i = 0; i < 2 * S; ++i) tdf[i] = df64(td[i]);
  MGB_CUDA(cudaMalloc(&p->tab_df, tdf.size() * sizeof(df64)));
  MGB_CUDA(cudaMemcpy(p->tab_df, tdf.data(), tdf.size() * sizeof(df64), cudaMemcpyHostToDevice));
  MGB_CUDA(cudaMalloc(&p->tab_d, td.size() * sizeof(double)));
  MGB_CUDA(cudaMalloc(&p->tab_f, tf.size() * sizeof(float)));
  MGB_CUDA(cudaMemcpy(p->tab_d, td.data(), td.size() * sizeof(double), cudaMemcpyHostToDevice));
  MGB_CUDA(cudaMemcpy(p->tab_f, tf.data(), tf.size() * sizeof(float), cudaMemcpyHostToDevice));
  // default z pass: the register-resident kernel where it exists (FP32;
  // 2048^2 split step: z pass 55 -> 37 us), else variant 0
  if (p->exp_ok && fs_launchers(g.nz) != nullptr && fs_launchers(g.nx) != nullptr) {
    for (int F = 1; F <= 3; ++F) {
      mgb_tile_info info;
      fs_tile_info(p, MGB_FAMILY_ZSTEP, F, 4, &info);
      if (info.available) p->tiles[F - 1][MGB_FAMILY_ZSTEP] = 4;
    }
  }
  return MGB_OK;
}


int fs_batch_step(const mgb_plan* p, const mgb_equation* eq, const StepBatch& sb, int curr, double dt, void* work,
                  double* diag, cudaStream_t s, EventTrack* et) {
  EventTrack none;
  if (!et) et = &none;
  const GridC& g = p->g;
  const int F = eq->nfields;
  const int nb = sb.count;
  int tile[3];
  {
    // the update coefficients in `work` must be the ones for (eq, dt)
    std::lock_guard<std::mutex> lock(p->mu);
    const PrepRecord& pr = p->prep;
    // a driven step reads dt from the run state (coefficients refreshed on
    // the device); a plain step needs coefficients prepared for its own dt
    const bool driven = sb.gate.stop_at != nullptr;
    bool ok = pr.valid && pr.work == work && (driven || (pr.dt == dt && !pr.driven)) && pr.nfields == F &&
              pr.integrator == eq->integrator &&
              pr.order == eq->order && (eq->integrator != MGB_INT_SEMI_IMPLICIT || pr.alpha == eq->alpha);
    for (int f = 0; ok && f < F; ++f) ok = pr.kappa[f] == eq->f[f].kappa;
    if (!ok) return fail(MGB_ERR_INVALID, "mgb_step: call mgb_step_prepare for this equation, dt and workspace first");
    for (int k = 0; k < 3; ++k) tile[k] = p->tiles[F - 1][k];
  }
  et->mark(s);
  const int prec = p->grid.precision;
  const FsLaunchers* Lx = fs_launchers(g.nx);
  const FsLaunchers* Lz = fs_launchers(g.nz);
  FsWork w = fs_carve(p, F, nb, work);
  const void* twx = twiddles_for(p, false, prec);
  const void* twz = twiddles_for(p, true, prec);
  BatchC bc = {};
  bc.members = sb.members;
  bc.q_stride = sb.q_stride;
  bc.h_stride = sb.h_stride;
  bc.inter_stride = w.inter_stride;
  bc.tcoef = sb.tcoef;
  bc.gate = sb.gate;

  XinvArgs xa = {};
  xa.g = g;
  xa.ld = g.cols;
  xa.tw = twx;
  xa.b = bc;
  set_tables(p, xa, prec);
  xa.job[0] = XinvJob{sb.q[0], SRC_UX, w.inter[0], nullptr, nullptr};
  xa.job[1] = XinvJob{sb.q[0], SRC_UZ, w.inter[1], nullptr, nullptr};
  for (int f = 0; f < F; ++f) xa.job[2 + f] = XinvJob{sb.q[f], SRC_COPY, w.inter[2 + f], nullptr, nullptr};
  int st = launched(Lx->xinv[prec][tile[MGB_FAMILY_XINV]](xa, 2 + F, nb, s), "step x pass");
  if (st) return st;
  et->mark(s);

  ZzArgs za = {};
  za.g = g;
  za.ld = g.cols;
  za.b = bc;
  for (int i = 0; i < 2 + F; ++i) za.in[i] = w.inter[i];
  for (int f = 0; f < F; ++f) {
    za.aout[f] = w.inter[f];
    za.cout[f] = w.inter[F + f];
  }
  za.partial = diag ? w.partial : nullptr;
  za.flux_f = eq->diag_flux - 1;
  za.fdz = fd_inv(g.sdo, g.dz);
  // the forward x pass needs N = -J / (nx nz): the z pass leaves 2 A and
  // -C / (nx nz), and the x stencil factor takes -1 / (2 nx nz)
  const double out_scale = -0.5 / ((double)g.nx * (double)g.nz);
  za.cscale = out_scale;
  za.tw = twz;
  st = launched(Lz->zz_step[prec][F - 1][tile[MGB_FAMILY_ZSTEP]](za, nb, s), "step z pass");
  if (st) return st;
  et->mark(s);

  XfArgs fa = {};
  fa.g = g;
  fa.ld = g.cols;
  fa.b = bc;
  fa.need_psi = 0;
  fa.rlap = p->tab_d + 2 * (size_t)g.rows * g.cols;
  for (int f = 0; f < F; ++f) {
    fa.ain[f] = w.inter[f];
    fa.cin[f] = w.inter[F + f];
    fa.q[f] = sb.q[f];
    fa.hist[f] = sb.hist[f];
    fa.coef[f] = w.coef[f];
    const mgb_field_eq& fe = eq->f[f];
    fa.eq[f].nterms = fe.nterms;
    fa.eq[f].bc = fe.bc;
    for (int t = 0; t < fe.nterms; ++t) {
      fa.eq[f].tsrc[t] = fe.terms[t].src;
      fa.eq[f].top[t] = fe.terms[t].op;
      fa.eq[f].tcoef[t] = fe.terms[t].coef;
      if (fe.terms[t].src < 0) fa.need_psi = 1;
    }
  }
  fa.order = eq->order;
  fa.curr = curr;
  fa.integrator = eq->integrator;
  fa.fdx = fd_inv(g.sdo, g.dx) * out_scale;
  fa.tw = twx;
  st = launched(Lx->xf_step[prec][F - 1][tile[MGB_FAMILY_XFWD]](fa, nb, s), "step forward x pass");
  if (st) return st;
  et->mark(s);
  if (diag) {
    const int pairs = Lz->zz_shape[prec][F - 1][tile[MGB_FAMILY_ZSTEP]].shape;
    return pw_finish_diag(w.partial, g.nx / (2 * pairs), nb, 1.0 / ((double)g.nx * (double)g.nz), diag, s,
                          eq->diag_flux ? 4 : 3);
  }
  return MGB_OK;
}

int fs_tile_info(const mgb_plan* p, int family, int nfields, int v, mgb_tile_info* out) {
  const GridC& g = p->g;
  const int prec = p->grid.precision;
  const FsLaunchers* L = fs_launchers(family == MGB_FAMILY_ZSTEP ? g.nz : g.nx);
  const TileShape* ts = nullptr;
  bool have = false;
  if (family == MGB_FAMILY_XINV) {
    ts = &L->xinv_shape[prec][v];
    have = L->xinv[prec][v] != nullptr;
  } else if (family == MGB_FAMILY_ZSTEP) {
    ts = &L->zz_shape[prec][nfields - 1][v];
    have = L->zz_step[prec][nfields - 1][v] != nullptr;
  } else {
    ts = &L->xf_shape[prec][nfields - 1][v];
    have = L->xf_step[prec][nfields - 1][v] != nullptr;
  }
  // a z pass that covers several row pairs per CTA needs whole CTAs of rows
  // (its diagnostics partials are folded per CTA)
  if (family == MGB_FAMILY_ZSTEP && have && g.nx % (2 * ts->shape) != 0) have = false;
  out->available = have ? 1 : 0;
  out->shape = ts->shape;
  out->radix = ts->radix;
  out->kind = ts->kind;
  out->smem_bytes = ts->smem;
  return MGB_OK;
}

}  // namespace mgb
