// Host orchestration of the fully spectral (doubly periodic) kernels.
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

int fs_to_physical(const mgb_plan* p, const zd* spec, double* phys, void* work, cudaStream_t s) {
  const GridC& g = p->g;
  const FsLaunchers* Lx = fs_launchers(g.nx);
  const FsLaunchers* Lz = fs_launchers(g.nz);
  XinvArgs xa = {};
  xa.g = g;
  xa.ld = g.cols;
  xa.tw = p->tw_x_d;
  xa.job[0] = XinvJob{spec, SRC_COPY, work, nullptr, nullptr};
  int st = launched(Lx->xinv[0](xa, 1, s), "to_physical x pass");
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
  char* w1 = w0 + inter_bytes(g, false);
  XinvArgs xa = {};
  xa.g = g;
  xa.ld = g.cols;
  xa.tw = p->tw_x_d;
  xa.job[0] = XinvJob{q, SRC_COPY, w0, nullptr, nullptr};
  int st = launched(Lx->xinv[0](xa, 1, s), "vec_dot_nabla x pass");
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
  char* w1 = w0 + inter_bytes(g, false);
  XinvArgs xa = {};
  xa.g = g;
  xa.ld = g.cols;
  xa.tw = p->tw_x_d;
  xa.job[0] = XinvJob{w, SRC_UX, w0, ux_s, psi};
  xa.job[1] = XinvJob{w, SRC_UZ, w1, uz_s, nullptr};
  int st = launched(Lx->xinv[0](xa, 2, s), "velocity x pass");
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

size_t fs_step_workspace(const mgb_plan* p, int nfields) {
  const bool split = p->grid.precision == MGB_PREC_SPLIT;
  const int nin = 2 + nfields, nout = 2 * nfields;
  const int ninter = nin > nout ? nin : nout;
  return (size_t)ninter * inter_bytes(p->g, split) + (size_t)(p->g.nx / 2) * 3 * sizeof(double) + 256;
}

int fs_step(const mgb_plan* p, const mgb_equation* eq, void* const* q, void* const* hist, int curr,
            double dt, void* work, double* diag, cudaStream_t s, EventTrack* et) {
  EventTrack none;
  if (!et) et = &none;
  et->mark(s);
  const GridC& g = p->g;
  const int F = eq->nfields;
  const int split = p->grid.precision == MGB_PREC_SPLIT ? 1 : 0;
  const FsLaunchers* Lx = fs_launchers(g.nx);
  const FsLaunchers* Lz = fs_launchers(g.nz);
  const size_t ib = inter_bytes(g, split);
  const int nin = 2 + F, nout = 2 * F;
  const int ninter = nin > nout ? nin : nout;
  char* inter[6];
  for (int i = 0; i < 6; ++i) inter[i] = (char*)work + (size_t)i * ib;
  double* partial = (double*)((char*)work + (size_t)ninter * ib);
  partial = (double*)(((uintptr_t)partial + 255) & ~(uintptr_t)255);
  const void* twx = split ? p->tw_x_f : p->tw_x_d;
  const void* twz = split ? p->tw_z_f : p->tw_z_d;

  XinvArgs xa = {};
  xa.g = g;
  xa.ld = g.cols;
  xa.tw = twx;
  xa.job[0] = XinvJob{(const zd*)q[0], SRC_UX, inter[0], nullptr, nullptr};
  xa.job[1] = XinvJob{(const zd*)q[0], SRC_UZ, inter[1], nullptr, nullptr};
  for (int f = 0; f < F; ++f) xa.job[2 + f] = XinvJob{(const zd*)q[f], SRC_COPY, inter[2 + f], nullptr, nullptr};
  int st = launched(Lx->xinv[split](xa, 2 + F, s), "step x pass");
  if (st) return st;
  et->mark(s);

  ZzArgs za = {};
  za.g = g;
  za.ld = g.cols;
  for (int i = 0; i < 2 + F; ++i) za.in[i] = inter[i];
  for (int f = 0; f < F; ++f) {
    za.aout[f] = inter[f];
    za.cout[f] = inter[F + f];
  }
  za.partial = diag ? partial : nullptr;
  za.fdz = fd_inv(g.sdo, g.dz);
  za.tw = twz;
  st = launched(Lz->zz_step[split][F - 1](za, s), "step z pass");
  if (st) return st;
  et->mark(s);

  XfArgs fa = {};
  fa.g = g;
  fa.ld = g.cols;
  fa.need_psi = 0;
  for (int f = 0; f < F; ++f) {
    fa.ain[f] = inter[f];
    fa.cin[f] = inter[F + f];
    fa.q[f] = (zd*)q[f];
    fa.hist[f] = (zd*)hist[f];
    const mgb_field_eq& fe = eq->f[f];
    fa.eq[f].kappa = fe.kappa;
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
  fa.dt = dt;
  fa.alpha = eq->alpha;
  fa.fdx = fd_inv(g.sdo, g.dx);
  fa.inv_norm = 1.0 / ((double)g.nx * (double)g.nz);
  fa.tw = twx;
  st = launched(Lx->xf_step[split][F - 1](fa, s), "step forward x pass");
  if (st) return st;
  et->mark(s);
  if (diag) return pw_finish_diag(partial, g.nx / 2, 1.0 / ((double)g.nx * (double)g.nz), diag, s);
  return MGB_OK;
}

}  // namespace mgb
