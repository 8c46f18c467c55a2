// Host orchestration of the Fourier-x / Dirichlet-z kernels, plus the two
// small physical stencil kernels of the per-verb API.
#include <algorithm>
#include <utility>
#include <vector>

#include "fdm_impl.cuh"

namespace mgb {

const FdLaunchers* fd_launchers_16();
const FdLaunchers* fd_launchers_32();
const FdLaunchers* fd_launchers_64();
const FdLaunchers* fd_launchers_128();
const FdLaunchers* fd_launchers_256();
const FdLaunchers* fd_launchers_512();
const FdLaunchers* fd_launchers_1024();
const FdLaunchers* fd_launchers_2048();
const FdLaunchers* fd_launchers_4096();

const FdLaunchers* fd_launchers(int N) {
  switch (N) {
    case 16: return fd_launchers_16();
    case 32: return fd_launchers_32();
    case 64: return fd_launchers_64();
    case 128: return fd_launchers_128();
    case 256: return fd_launchers_256();
    case 512: return fd_launchers_512();
    case 1024: return fd_launchers_1024();
    case 2048: return fd_launchers_2048();
    case 4096: return fd_launchers_4096();
    default: return nullptr;
  }
}

namespace {

inline double fd_inv(int sdo, double h) { return sdo == 2 ? 1.0 / (2.0 * h) : 1.0 / (3.0 * h); }

int launched(cudaError_t e, const char* what) {
  if (e == cudaErrorInvalidConfiguration)
    return fail(MGB_ERR_UNSUPPORTED, "%s: shared-memory footprint too large for this size", what);
  if (e != cudaSuccess) return cuda_check(e, what);
  return MGB_OK;
}

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// ux = -pddz(psi) on the physical streamfunction, Dirichlet z
// (melvin/utility.py:66-69).
__global__ void k_fd_vel(GridC g, const double* __restrict__ psi, double* __restrict__ ux, double fdz) {
  const size_t total = (size_t)g.nx * g.nz;
  const int h = g.sdo / 2;
  for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < total; i += (size_t)gridDim.x * NT) {
    const int x = (int)(i / g.nz), z = (int)(i - (size_t)x * g.nz);
    const double* row = psi + (size_t)x * g.nz;
    double u = 0.0;
    if (z >= h && z < g.nz - h)
      u = st1(h == 2 ? row[z + 2] : 0.0, row[z + 1], row[z - 1], h == 2 ? row[z - 2] : 0.0, g.sdo, fdz);
    ux[i] = -u;
  }
}

// J = pddx(ux q) + pddz(uz q) with z Dirichlet (melvin/Variable.py:125-127).
__global__ void k_fd_vdn_phys(GridC g, const double* __restrict__ q, const double* __restrict__ ux,
                              const double* __restrict__ uz, double* __restrict__ J, double fdx, double fdz) {
  const size_t total = (size_t)g.nx * g.nz;
  const int h = g.sdo / 2;
  for (size_t i = blockIdx.x * (size_t)NT + threadIdx.x; i < total; i += (size_t)gridDim.x * NT) {
    const int x = (int)(i / g.nz), z = (int)(i - (size_t)x * g.nz);
    auto px = [&](int dx) {
      int xx = x + dx;
      xx = xx < 0 ? xx + g.nx : (xx >= g.nx ? xx - g.nx : xx);
      const size_t k = (size_t)xx * g.nz + z;
      return ux[k] * q[k];
    };
    double jx = st1(px(2), px(1), px(-1), px(-2), g.sdo, fdx);
    double jz = 0.0;
    if (z >= h && z < g.nz - h) {
      auto pz = [&](int dz) {
        const size_t k = (size_t)x * g.nz + z + dz;
        return uz[k] * q[k];
      };
      jz = st1(h == 2 ? pz(2) : 0.0, pz(1), pz(-1), h == 2 ? pz(-2) : 0.0, g.sdo, fdz);
    }
    J[i] = jx + jz;
  }
}

inline int grid_for(size_t n) {
  size_t b = (n + NT - 1) / NT;
  return (int)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

template <int G>
void launch_thomas(const mgb_plan* p, Mptr rhs, double sign, Mptr out, const int* members, int nb, cudaStream_t s,
                   Gate gate) {
  const GridC& g = p->g;
  const int blocks = (g.nn * G + TH_THREADS - 1) / TH_THREADS;
  k_thomas<G><<<dim3(blocks, nb), TH_THREADS, 0, s>>>(g, rhs, sign, out, members, p->th_inv, p->th_cp, p->th_ps,
                                                     p->th_qs, gate);
}

int thomas(const mgb_plan* p, Mptr rhs, double sign, Mptr out, const int* members, int nb, cudaStream_t s,
           Gate gate) {
  switch (thomas_lanes(p->g.nz)) {
    case 1: launch_thomas<1>(p, rhs, sign, out, members, nb, s, gate); break;
    case 2: launch_thomas<2>(p, rhs, sign, out, members, nb, s, gate); break;
    case 4: launch_thomas<4>(p, rhs, sign, out, members, nb, s, gate); break;
    case 8: launch_thomas<8>(p, rhs, sign, out, members, nb, s, gate); break;
    case 16: launch_thomas<16>(p, rhs, sign, out, members, nb, s, gate); break;
    default: launch_thomas<32>(p, rhs, sign, out, members, nb, s, gate); break;
  }
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

}  // namespace

int fd_plan_init(mgb_plan* p) {
  const GridC& g = p->g;
  // The inverse x transforms skip the inputs 3N/8 .. 5N/8 - 1 as removed
  // modes: true of the 2/3 rule (nn = (nx - 1) / 3).
  if (8 * g.nn > 3 * g.nx) return MGB_ERR_INVALID;
  const size_t n = (size_t)g.nn * g.nz;
  std::vector<double> ip(n, 0.0), cp(n, 0.0), ps(n, 0.0), qs(n, 0.0);
  const double a = 1.0 / (g.dz * g.dz);
  const double kx = g.dfx;  // |2*pi*i/lx|
  for (int m = 0; m < g.nn; ++m) {
    // diagonal -((n*|ddx|)^2 + 2/dz^2), off-diagonals 1/dz^2, identity end rows
    // (melvin/LaplacianSolver.py:25-52)
    const double nk = (double)m * kx;
    const double b = -(nk * nk + 2.0 / (g.dz * g.dz));
    double* ipm = ip.data() + (size_t)m * g.nz;
    double* cpm = cp.data() + (size_t)m * g.nz;
    ipm[0] = 1.0;
    cpm[0] = 0.0;
    for (int j = 1; j < g.nz - 1; ++j) {
      const double piv = b - a * cpm[j - 1];
      ipm[j] = 1.0 / piv;
      cpm[j] = a / piv;
    }
    ipm[g.nz - 1] = 1.0;
    cpm[g.nz - 1] = 0.0;
    // the segment products of the segmented sweeps: P_j = prod_{i=s..j}
    // (-a ip_i) forward, Q_j = prod_{i=j..e-1} (-cp_i) backward, per segment
    // [s, e) of TH_SEG interior rows
    double* psm = ps.data() + (size_t)m * g.nz;
    double* qsm = qs.data() + (size_t)m * g.nz;
    for (int s0 = 1; s0 < g.nz - 1; s0 += TH_SEG) {
      const int s1 = std::min(s0 + TH_SEG, g.nz - 1);
      double pr = 1.0, qr = 1.0;
      for (int j = s0; j < s1; ++j) psm[j] = pr *= -a * ipm[j];
      for (int j = s1 - 1; j >= s0; --j) qsm[j] = qr *= -cpm[j];
    }
  }
  const std::pair<double**, const std::vector<double>*> arrays[] = {
      {&p->th_inv, &ip}, {&p->th_cp, &cp}, {&p->th_ps, &ps}, {&p->th_qs, &qs}};
  for (const auto& [dst, src] : arrays) {
    MGB_CUDA(cudaMalloc(dst, n * sizeof(double)));
    MGB_CUDA(cudaMemcpy(*dst, src->data(), n * sizeof(double), cudaMemcpyHostToDevice));
  }
  return MGB_OK;
}

int fd_poisson(const mgb_plan* p, const zd* rhs, zd* out, cudaStream_t s) {
  return thomas(p, mp(rhs), 1.0, mp(out), nullptr, 1, s, Gate());
}

int fd_to_physical(const mgb_plan* p, const zd* spec, double* phys, cudaStream_t s) {
  const GridC& g = p->g;
  FdXinvArgs xa = {};
  xa.g = g;
  xa.tw = p->tw_x_d;
  xa.job[0] = FdXinvJob{mp(spec), mp(phys), mp(nullptr), 0.0, FD_COPY, nullptr};
  return launched(fd_launchers(g.nx)->xinv[0](xa, 1, 1, s), "fdm to_physical");
}

int fd_to_spectral(const mgb_plan* p, const double* phys, zd* spec, cudaStream_t s) {
  const GridC& g = p->g;
  FdXfArgs fa = {};
  fa.g = g;
  fa.jin[0] = mp(phys);
  fa.out = spec;
  fa.nf = 1;
  fa.mode = FD_OUT;
  fa.inv_nx = 1.0 / (double)g.nx;
  fa.tw = p->tw_x_d;
  return launched(fd_launchers(g.nx)->xfwd[0][0](fa, 1, s), "fdm to_spectral");
}

size_t fd_verb_workspace(const mgb_plan* p) {
  return align256((size_t)p->g.nx * p->g.nz * sizeof(double)) + align256(152 * 4 * 3 * sizeof(double));
}

int fd_vec_dot_nabla(const mgb_plan* p, const zd* q, double* q_phys, const double* ux, const double* uz, zd* out,
                     void* work, cudaStream_t s) {
  const GridC& g = p->g;
  int st = fd_to_physical(p, q, q_phys, s);
  if (st) return st;
  double* J = (double*)work;
  k_fd_vdn_phys<<<grid_for((size_t)g.nx * g.nz), NT, 0, s>>>(g, q_phys, ux, uz, J, fd_inv(g.sdo, g.dx),
                                                            fd_inv(g.sdo, g.dz));
  MGB_LAUNCH_CHECK();
  return fd_to_spectral(p, J, out, s);
}

int fd_velocity(const mgb_plan* p, const zd* w, zd* psi, zd* uz_s, double* psi_phys, double* ux, double* uz,
                void* work, cudaStream_t s) {
  const GridC& g = p->g;
  int st = thomas(p, mp(w), -1.0, mp(psi), nullptr, 1, s, Gate());
  if (st) return st;
  double* pp = psi_phys ? psi_phys : (double*)work;
  FdXinvArgs xa = {};
  xa.g = g;
  xa.fdz = fd_inv(g.sdo, g.dz);
  xa.inv_dz2 = 1.0 / (g.dz * g.dz);
  xa.tw = p->tw_x_d;
  xa.job[0] = FdXinvJob{mp(psi), mp(pp), mp(nullptr), 0.0, FD_COPY, nullptr};
  xa.job[1] = FdXinvJob{mp(psi), mp(uz), mp(nullptr), 0.0, FD_UZ, uz_s};
  st = launched(fd_launchers(g.nx)->xinv[0](xa, 2, 1, s), "fdm velocity x pass");
  if (st) return st;
  k_fd_vel<<<grid_for((size_t)g.nx * g.nz), NT, 0, s>>>(g, pp, ux, fd_inv(g.sdo, g.dz));
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

// Scratch of the fused FDM step, per member: psi_hat, physical ux, uz and
// fields, J per field, predicted states (PECE), diagnostics partials.
struct FdWork {
  size_t psi, phys[5], J[3], qpred[3], partial;  // byte offsets in a member block
  size_t member_bytes;
  char* base;
};

static FdWork fd_carve(const mgb_plan* p, int F, void* base) {
  const GridC& g = p->g;
  const bool split = p->grid.precision == MGB_PREC_SPLIT;
  const size_t S = align256((size_t)g.nn * g.nz * sizeof(zd));
  const size_t P = align256((size_t)g.nx * g.nz * (split ? sizeof(float) : sizeof(double)));  // df64 is 8 bytes
  const int nctas = ((g.nz + FD_TZ - 1) / FD_TZ) * ((g.nx + FD_TX - 1) / FD_TX);
  FdWork w = {};
  size_t off = 0;
  w.psi = off;
  off += S;
  for (int i = 0; i < 2 + F; ++i) {
    w.phys[i] = off;
    off += P;
  }
  for (int f = 0; f < F; ++f) {
    w.J[f] = off;
    off += P;
  }
  for (int f = 0; f < F; ++f) {
    w.qpred[f] = off;
    off += S;
  }
  w.partial = off;
  off += align256((size_t)nctas * kDiagW * sizeof(double));
  w.member_bytes = off;
  w.base = (char*)base;
  return w;
}

static inline Mptr wmp(const FdWork& w, size_t off) { return mp(w.base + off, w.member_bytes, 0); }

size_t fd_step_workspace(const mgb_plan* p, int nfields) { return fd_carve(p, nfields, nullptr).member_bytes; }
size_t fd_batch_workspace(const mgb_plan* p, int nfields, int count) {
  return fd_carve(p, nfields, nullptr).member_bytes * (size_t)count;
}

// One evaluation of the right-hand side at the states `qeval` (the members'
// own states, or their predicted states in scratch) followed by the update
// selected by `mode`.
static int fd_stage(const mgb_plan* p, const mgb_equation* eq, const FdWork& w, const StepBatch& sb, bool eval_pred,
                    int curr, double dt, int mode, bool diag, cudaStream_t s, EventTrack* et) {
  const GridC& g = p->g;
  const int F = eq->nfields;
  const int nb = sb.count;
  const int prec = p->grid.precision;
  const FdLaunchers* L = fd_launchers(g.nx);
  const size_t qs = sb.q_stride * sizeof(zd), hs = sb.h_stride * sizeof(zd);
  Mptr qev[3], qown[3], hist[3], hslot[3];
  for (int f = 0; f < F; ++f) {
    qown[f] = mp(sb.q[f], qs, 1);
    qev[f] = eval_pred ? wmp(w, w.qpred[f]) : qown[f];
    hist[f] = mp(sb.hist[f], hs, 1);
    hslot[f] = mp(sb.hist[f] + (size_t)curr * g.nn * g.nz, hs, 1);
  }
  int st = thomas(p, qev[0], -1.0, wmp(w, w.psi), sb.members, nb, s, sb.gate);
  if (st) return st;
  et->mark(s);
  FdXinvArgs xa = {};
  xa.gate = sb.gate;
  xa.g = g;
  xa.fdz = fd_inv(g.sdo, g.dz);
  xa.inv_dz2 = 1.0 / (g.dz * g.dz);
  xa.tw = twiddles_for(p, false, prec);
  xa.members = sb.members;
  xa.job[0] = FdXinvJob{wmp(w, w.psi), wmp(w, w.phys[0]), mp(nullptr), 0.0, FD_UX, nullptr};
  xa.job[1] = FdXinvJob{wmp(w, w.psi), wmp(w, w.phys[1]), mp(nullptr), 0.0, FD_UZ, nullptr};
  for (int f = 0; f < F; ++f)
    xa.job[2 + f] = FdXinvJob{qev[f], wmp(w, w.phys[2 + f]), hslot[f], eq->f[f].kappa, FD_COPY, nullptr};
  st = launched(L->xinv[prec](xa, 2 + F, nb, s), "fdm step x pass");
  if (st) return st;
  et->mark(s);
  FdPhysArgs pa = {};
  pa.g = g;
  pa.ux = wmp(w, w.phys[0]);
  pa.uz = wmp(w, w.phys[1]);
  for (int f = 0; f < F; ++f) {
    pa.q[f] = wmp(w, w.phys[2 + f]);
    pa.jout[f] = wmp(w, w.J[f]);
  }
  pa.nf = F;
  pa.partial = diag ? wmp(w, w.partial) : mp(nullptr);
  pa.flux_f = eq->diag_flux - 1;
  pa.fdx = fd_inv(g.sdo, g.dx);
  pa.fdz = fd_inv(g.sdo, g.dz);
  pa.gate = sb.gate;
  dim3 grid((g.nz + FD_TZ - 1) / FD_TZ, (g.nx + FD_TX - 1) / FD_TX, nb);
  if (prec == MGB_PREC_SPLIT)
    k_fd_phys<float><<<grid, NT, 0, s>>>(pa);
  else if (prec == MGB_PREC_DFLOAT)
    k_fd_phys<df64><<<grid, NT, 0, s>>>(pa);
  else
    k_fd_phys<double><<<grid, NT, 0, s>>>(pa);
  MGB_LAUNCH_CHECK();
  et->mark(s);
  FdXfArgs fa = {};
  fa.g = g;
  fa.members = sb.members;
  fa.tcoef = sb.tcoef;
  for (int f = 0; f < F; ++f) {
    fa.jin[f] = wmp(w, w.J[f]);
    fa.q[f] = qown[f];
    fa.qsrc[f] = qev[f];
    fa.qpred[f] = wmp(w, w.qpred[f]);
    fa.hist[f] = hist[f];
    const mgb_field_eq& fe = eq->f[f];
    fa.eq[f].nterms = fe.nterms;
    fa.eq[f].bc = fe.bc;
    for (int t = 0; t < fe.nterms; ++t) {
      fa.eq[f].tsrc[t] = fe.terms[t].src;
      fa.eq[f].top[t] = fe.terms[t].op;
      fa.eq[f].tcoef[t] = fe.terms[t].coef;
    }
  }
  fa.psi = wmp(w, w.psi);
  fa.nf = F;
  fa.mode = mode;
  fa.order = eq->order;
  fa.curr = curr;
  fa.dt = dt;
  fa.gate = sb.gate;
  fa.inv_nx = 1.0 / (double)g.nx;
  fa.tw = twiddles_for(p, false, prec);
  st = launched(L->xfwd[prec][F - 1](fa, nb, s), "fdm step forward x pass");
  if (st) return st;
  et->mark(s);
  return MGB_OK;
}

int fd_batch_step(const mgb_plan* p, const mgb_equation* eq, const StepBatch& sb, int curr, double dt, void* work,
                  double* diag, cudaStream_t s, EventTrack* et) {
  EventTrack none;
  if (!et) et = &none;
  et->mark(s);
  const GridC& g = p->g;
  const int F = eq->nfields;
  for (int f = 0; f < F; ++f)
    for (int t = 0; t < eq->f[f].nterms; ++t)
      if (eq->f[f].terms[t].op == 2)
        return fail(MGB_ERR_UNSUPPORTED, "d/dz linear terms are not pointwise on an FDM z axis");
  FdWork w = fd_carve(p, F, work);
  const int nctas = ((g.nz + FD_TZ - 1) / FD_TZ) * ((g.nx + FD_TX - 1) / FD_TX);
  int st;
  if (eq->integrator == MGB_INT_EXPLICIT) {
    st = fd_stage(p, eq, w, sb, false, curr, dt, FD_EXPLICIT, diag != nullptr, s, et);
  } else if (eq->integrator == MGB_INT_PECE) {
    // predict into scratch, then evaluate there and correct the states in
    // place; the corrector's f* goes to the next slot, which the caller's
    // advance makes the next step's f0 slot.
    st = fd_stage(p, eq, w, sb, false, curr, dt, FD_PREDICT, diag != nullptr, s, et);
    if (st) return st;
    const int next = (curr + 1) % eq->order;
    st = fd_stage(p, eq, w, sb, true, next, dt, FD_CORRECT, false, s, et);
  } else {
    return fail(MGB_ERR_UNSUPPORTED,
                "semi-implicit integration needs a fully spectral grid (melvin/Integrator.py:78-81)");
  }
  if (st) return st;
  if (diag) {
    // per-member partials sit member_bytes apart: fold each member's block
    for (int z = 0; z < sb.count; ++z) {
      const int ow = eq->diag_flux ? 4 : 3;
      st = pw_finish_diag((const double*)(w.base + (size_t)z * w.member_bytes + w.partial), nctas, 1,
                          1.0 / ((double)g.nx * (double)g.nz), diag + ow * z, s, ow);
      if (st) return st;
    }
  }
  return MGB_OK;
}

}  // namespace mgb
