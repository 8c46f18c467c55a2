// Pointwise and stencil kernels of the per-verb API: physical finite
// differences, spectral derivative verbs, the spectral Poisson divide, the
// Adams-Bashforth/Moulton updates and the diagnostic reductions.
#include <math.h>

#include "internal.h"

namespace mgb {

namespace {

constexpr int PT = 256;

inline int nblocks(size_t n, int per = PT) {
  size_t b = (n + per - 1) / per;
  return (int)(b > 152 * 16 ? 152 * 16 : (b < 1 ? 1 : b));
}

__device__ __forceinline__ double lap_sym(const GridC& g, int n, int m) {
  return __dadd_rn(__dmul_rn(g.d2x, (double)(n * n)), __dmul_rn(g.d2z, (double)(m * m)));
}

// Signed x mode and z mode of spectral element (r, c).
__device__ __forceinline__ void modes(const GridC& g, int r, int c, int& n, int& m) {
  n = g.fdm ? r : row_mode(r, g.nn);
  m = c;
}

// pddx: periodic central difference along x (melvin/SpatialDifferentiator.py:76-89, 130-155).
__global__ void k_pddx(GridC g, const double* __restrict__ in, double* __restrict__ out, double inv) {
  const size_t total = (size_t)g.nx * g.nz;
  for (size_t i = blockIdx.x * (size_t)PT + threadIdx.x; i < total; i += (size_t)gridDim.x * PT) {
    const int x = (int)(i / g.nz), z = (int)(i - (size_t)x * g.nz);
    auto at = [&](int dx) {
      int xx = x + dx;
      xx = xx < 0 ? xx + g.nx : (xx >= g.nx ? xx - g.nx : xx);
      return in[(size_t)xx * g.nz + z];
    };
    double v;
    if (g.sdo == 2)
      v = (at(1) - at(-1)) * inv;
    else
      v = (((-0.25 * at(2) + 2 * at(1)) - 2 * at(-1)) + 0.25 * at(-2)) * inv;
    out[i] = v;
  }
}

// pddz: central difference along z, periodic (spectral z) or Dirichlet
// with the outer sdo/2 points left 0 (FDM z) (:91-104, 157-185).
template <typename V>
__device__ __forceinline__ V zstencil1(const V* row, int z, int nz, int sdo, bool periodic, double inv,
                                       bool& inside) {
  const int h = sdo / 2;
  inside = periodic || (z >= h && z < nz - h);
  if (!inside) return V();
  auto at = [&](int dz) {
    int zz = z + dz;
    if (periodic) zz = zz < 0 ? zz + nz : (zz >= nz ? zz - nz : zz);
    return row[zz];
  };
  if (sdo == 2) return (at(1) - at(-1)) * inv;
  return (((at(2) * -0.25 + at(1) * 2.0) - at(-1) * 2.0) + at(-2) * 0.25) * inv;
}

__global__ void k_pddz(GridC g, int rows, int periodic, const double* __restrict__ in,
                       double* __restrict__ out, double inv) {
  const size_t total = (size_t)rows * g.nz;
  for (size_t i = blockIdx.x * (size_t)PT + threadIdx.x; i < total; i += (size_t)gridDim.x * PT) {
    const int x = (int)(i / g.nz), z = (int)(i - (size_t)x * g.nz);
    bool inside;
    const double v = zstencil1(in + (size_t)x * g.nz, z, g.nz, g.sdo, periodic != 0, inv, inside);
    out[i] = inside ? v : 0.0;
  }
}

// Complex value helpers for the spectral FD stencils.
struct Zc {
  double x, y;
  __device__ Zc() : x(0), y(0) {}
  __device__ Zc(double a, double b) : x(a), y(b) {}
  __device__ Zc(zd v) : x(v.x), y(v.y) {}
  __device__ Zc operator+(Zc o) const { return Zc(x + o.x, y + o.y); }
  __device__ Zc operator-(Zc o) const { return Zc(x - o.x, y - o.y); }
  __device__ Zc operator*(double s) const { return Zc(x * s, y * s); }
};

// pd2dz2 on a complex spectral array (melvin/SpatialDifferentiator.py:106-128).
__device__ __forceinline__ Zc d2z_stencil(const zd* row, int z, int nz, int sdo, double inv_dz2, bool& inside) {
  const int h = sdo / 2;
  inside = z >= h && z < nz - h;
  if (!inside) return Zc();
  const Zc p1 = row[z + 1], c0 = row[z], m1 = row[z - 1];
  if (sdo == 2) return ((p1 - c0 * 2.0) + m1) * inv_dz2;
  const Zc p2 = row[z + 2], m2 = row[z - 2];
  return ((((p2 * (-1.0 / 12) + p1 * (4.0 / 3)) - c0 * (5.0 / 2)) + m1 * (4.0 / 3)) - m2 * (1.0 / 12)) * inv_dz2;
}

__global__ void k_spec_deriv(GridC g, int kind, const zd* __restrict__ in, zd* __restrict__ out) {
  const size_t total = (size_t)g.rows * g.cols;
  const double inv_dz2 = 1.0 / (g.dz * g.dz);
  const double inv_fd = g.sdo == 2 ? 1.0 / (2.0 * g.dz) : 1.0 / (3.0 * g.dz);
  for (size_t i = blockIdx.x * (size_t)PT + threadIdx.x; i < total; i += (size_t)gridDim.x * PT) {
    const int r = (int)(i / g.cols), c = (int)(i - (size_t)r * g.cols);
    int n, m;
    modes(g, r, c, n, m);
    const zd v = in[i];
    zd o = mk(0.0, 0.0);
    if (kind == MGB_DDX) {
      const double b = g.dfx * (double)n;
      o = g.bx ? mk(b * v.x, b * v.y) : mk(-(b * v.y), b * v.x);
    } else if (kind == MGB_DDZ) {
      if (g.fdm) {
        bool inside;
        const Zc d = zstencil1<Zc>(reinterpret_cast<const Zc*>(in + (size_t)r * g.cols), c, g.nz, g.sdo, false,
                                   inv_fd, inside);
        o = inside ? mk(d.x, d.y) : mk(0.0, 0.0);
      } else {
        const double b = g.dfz * (double)m;
        o = g.bz ? mk(b * v.x, b * v.y) : mk(-(b * v.y), b * v.x);
      }
    } else {
      zd dx2 = mk(0.0, 0.0), dz2 = mk(0.0, 0.0);
      if (kind == MGB_D2DX2 || kind == MGB_NABLA2) {
        const double f = g.d2x * (double)(n * n);
        dx2 = mk(f * v.x, f * v.y);
      }
      if (kind == MGB_D2DZ2 || kind == MGB_NABLA2) {
        if (g.fdm) {
          bool inside;
          const Zc d = d2z_stencil(in + (size_t)r * g.cols, c, g.nz, g.sdo, inv_dz2, inside);
          dz2 = mk(d.x, d.y);
        } else {
          const double f = g.d2z * (double)(m * m);
          dz2 = mk(f * v.x, f * v.y);
        }
      }
      if (kind == MGB_D2DX2) o = dx2;
      else if (kind == MGB_D2DZ2) o = dz2;
      else o = mk(dx2.x + dz2.x, dx2.y + dz2.y);
    }
    out[i] = o;
  }
}

__global__ void k_laplacian(GridC g, double* __restrict__ lap) {
  const size_t total = (size_t)g.rows * g.cols;
  for (size_t i = blockIdx.x * (size_t)PT + threadIdx.x; i < total; i += (size_t)gridDim.x * PT) {
    const int r = (int)(i / g.cols), c = (int)(i - (size_t)r * g.cols);
    int n, m;
    modes(g, r, c, n, m);
    // FDM z contributes -|0|^2/lz^2 = 0 (melvin/BasisFunctions.py:26-42)
    lap[i] = g.fdm ? g.d2x * (double)(n * n) : lap_sym(g, n, m);
  }
}

__global__ void k_poisson_spectral(GridC g, const zd* __restrict__ rhs, zd* __restrict__ out) {
  const size_t total = (size_t)g.rows * g.cols;
  for (size_t i = blockIdx.x * (size_t)PT + threadIdx.x; i < total; i += (size_t)gridDim.x * PT) {
    const int r = (int)(i / g.cols), c = (int)(i - (size_t)r * g.cols);
    int n, m;
    modes(g, r, c, n, m);
    const double l = (i == 0) ? 1.0 : lap_sym(g, n, m);
    const zd v = rhs[i];
    out[i] = mk(v.x / l, v.y / l);
  }
}

__device__ __forceinline__ zd hget(const zd* h, size_t slot, int order, int curr, int k) {
  // TimeDerivative.get(k): data[curr + k] with Python negative wrap
  int s = curr + k;
  s = s < 0 ? s + order : s;
  return h[(size_t)s * slot];
}

__device__ __forceinline__ zd ab_value(const zd* h, size_t slot, int order, int curr, double dt) {
  const zd f0 = hget(h, slot, order, curr, 0), f1 = hget(h, slot, order, curr, -1);
  if (order == 2) {
    const double c = dt / 2;
    return mk(c * (3 * f0.x - f1.x), c * (3 * f0.y - f1.y));
  }
  const zd f2 = hget(h, slot, order, curr, -2), f3 = hget(h, slot, order, curr, -3);
  const double c = dt / 24;
  return mk(c * (((55 * f0.x - 59 * f1.x) + 37 * f2.x) - 9 * f3.x),
            c * (((55 * f0.y - 59 * f1.y) + 37 * f2.y) - 9 * f3.y));
}

__device__ __forceinline__ zd am_value(const zd* h, size_t slot, int order, int curr, double dt) {
  const zd f0 = hget(h, slot, order, curr, 0), f1 = hget(h, slot, order, curr, -1);
  if (order == 2) {
    const double c = dt / 2;
    return mk(c * (f0.x + f1.x), c * (f0.y + f1.y));
  }
  const zd f2 = hget(h, slot, order, curr, -2), f3 = hget(h, slot, order, curr, -3);
  const double c = dt / 24;
  return mk(c * (((9 * f0.x + 19 * f1.x) - 5 * f2.x) + f3.x), c * (((9 * f0.y + 19 * f1.y) - 5 * f2.y) + f3.y));
}

__global__ void k_semi_implicit(size_t total, zd* __restrict__ var, const zd* __restrict__ hist, int order,
                                int curr, double dt, double alpha, const double* __restrict__ lin) {
  for (size_t i = blockIdx.x * (size_t)PT + threadIdx.x; i < total; i += (size_t)gridDim.x * PT) {
    const double L = lin[i];
    const zd ab = ab_value(hist + i, total, order, curr, dt);
    const zd q = var[i];
    const double c1 = 1 + ((1 - alpha) * dt) * L;
    const double den = 1 - (alpha * dt) * L;
    var[i] = mk((c1 * q.x + ab.x) / den, (c1 * q.y + ab.y) / den);
  }
}

__global__ void k_explicit(size_t total, zd* __restrict__ var, zd* __restrict__ hist, int order, int curr,
                           double dt, const zd* __restrict__ diff) {
  for (size_t i = blockIdx.x * (size_t)PT + threadIdx.x; i < total; i += (size_t)gridDim.x * PT) {
    zd* h0 = hist + (size_t)curr * total + i;
    const zd d = diff[i], f = *h0;
    *h0 = mk(f.x + d.x, f.y + d.y);
    const zd ab = ab_value(hist + i, total, order, curr, dt);
    const zd q = var[i];
    var[i] = mk(q.x + ab.x, q.y + ab.y);
  }
}

__global__ void k_adams(size_t total, int corrector, const zd* __restrict__ hist, int order, int curr, double dt,
                        zd* __restrict__ out) {
  for (size_t i = blockIdx.x * (size_t)PT + threadIdx.x; i < total; i += (size_t)gridDim.x * PT)
    out[i] = corrector ? am_value(hist + i, total, order, curr, dt) : ab_value(hist + i, total, order, curr, dt);
}

__device__ __forceinline__ double nmax(double m, double v) { return (v != v || v > m) ? v : m; }

template <int THREADS>
__device__ __forceinline__ void reduce4(double& s, double& mx, double& mz, double& fl) {
  __shared__ double red[4][THREADS / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    mx = nmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mz = nmax(mz, __shfl_xor_sync(0xffffffffu, mz, o));
    fl += __shfl_xor_sync(0xffffffffu, fl, o);
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[0][w] = s;
    red[1][w] = mx;
    red[2][w] = mz;
    red[3][w] = fl;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    s = 0;
    mx = -INFINITY;
    mz = -INFINITY;
    fl = 0;
    for (int i = 0; i < THREADS / 32; ++i) {
      s += red[0][i];
      mx = nmax(mx, red[1][i]);
      mz = nmax(mz, red[2][i]);
      fl += red[3][i];
    }
  }
}


// Per-CTA partial sums of ux^2 + uz^2 and signed maxima (fixed assignment
// of elements to CTAs, so the result does not depend on scheduling).
__global__ void k_diag_partial(size_t total, const double* __restrict__ ux, const double* __restrict__ uz,
                               double* __restrict__ partial) {
  double s = 0, mx = -INFINITY, mz = -INFINITY;
  for (size_t i = blockIdx.x * (size_t)PT + threadIdx.x; i < total; i += (size_t)gridDim.x * PT) {
    const double a = ux[i], b = uz[i];
    s += b * b + a * a;
    mx = nmax(mx, a);
    mz = nmax(mz, b);
  }
  double fl = 0;
  reduce4<PT>(s, mx, mz, fl);
  if (threadIdx.x == 0) {
    partial[kDiagW * blockIdx.x + 0] = s;
    partial[kDiagW * blockIdx.x + 1] = mx;
    partial[kDiagW * blockIdx.x + 2] = mz;
    partial[kDiagW * blockIdx.x + 3] = fl;
  }
}

// Per member (blockIdx.x): fold n partials into kinetic energy
// (calc_kinetic_energy, melvin/utility.py:42-59), max ux, max uz and, for
// ow = 4, the mean convective flux.
__global__ void k_diag_finish(const double* __restrict__ partial, int n, double inv_npts, int ow,
                              double* __restrict__ out) {
  partial += (size_t)blockIdx.x * n * kDiagW;
  out += (size_t)blockIdx.x * ow;
  double s = 0, mx = -INFINITY, mz = -INFINITY, fl = 0;
  for (int i = threadIdx.x; i < n; i += PT) {
    s += partial[kDiagW * i];
    mx = nmax(mx, partial[kDiagW * i + 1]);
    mz = nmax(mz, partial[kDiagW * i + 2]);
    fl += partial[kDiagW * i + 3];
  }
  reduce4<PT>(s, mx, mz, fl);
  if (threadIdx.x == 0) {
    out[0] = 0.5 * s * inv_npts;
    out[1] = mx;
    out[2] = mz;
    if (ow == 4) out[3] = fl * inv_npts;
  }
}

}  // namespace

int pw_pddx(const mgb_plan* p, const double* in, double* out, cudaStream_t s) {
  const GridC& g = p->g;
  const double inv = g.sdo == 2 ? 1.0 / (2.0 * g.dx) : 1.0 / (3.0 * g.dx);
  k_pddx<<<nblocks((size_t)g.nx * g.nz), PT, 0, s>>>(g, in, out, inv);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_pddz(const mgb_plan* p, const double* in, double* out, cudaStream_t s) {
  const GridC& g = p->g;
  const double inv = g.sdo == 2 ? 1.0 / (2.0 * g.dz) : 1.0 / (3.0 * g.dz);
  k_pddz<<<nblocks((size_t)g.nx * g.nz), PT, 0, s>>>(g, g.nx, g.fdm ? 0 : 1, in, out, inv);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_spectral_derivative(const mgb_plan* p, int kind, const zd* in, zd* out, cudaStream_t s) {
  const GridC& g = p->g;
  if (kind < MGB_DDX || kind > MGB_NABLA2) return fail(MGB_ERR_INVALID, "unknown derivative kind %d", kind);
  if (in == out && g.fdm && (kind != MGB_DDX && kind != MGB_D2DX2))
    return fail(MGB_ERR_INVALID, "z stencils on FDM-z need distinct input and output");
  k_spec_deriv<<<nblocks((size_t)g.rows * g.cols), PT, 0, s>>>(g, kind, in, out);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_laplacian(const mgb_plan* p, double* lap, cudaStream_t s) {
  const GridC& g = p->g;
  k_laplacian<<<nblocks((size_t)g.rows * g.cols), PT, 0, s>>>(g, lap);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_poisson_spectral(const mgb_plan* p, const zd* rhs, zd* out, cudaStream_t s) {
  const GridC& g = p->g;
  k_poisson_spectral<<<nblocks((size_t)g.rows * g.cols), PT, 0, s>>>(g, rhs, out);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

// The plan's grid constants with the derivative factors of bases (bx, bz)
// (melvin/BasisFunctions.py:26-59): cosine -pi/L, sine pi/L (real), second
// derivative -pi^2/L^2.
static int basis_grid(const mgb_plan* p, int bx, int bz, GridC& g, const char* fn) {
  g = p->g;
  if (bx < 0 || bx > 2 || bz < 0 || bz > 2) return fail(MGB_ERR_INVALID, "%s: basis (%d, %d)", fn, bx, bz);
  if (g.fdm && (bx || bz)) return fail(MGB_ERR_UNSUPPORTED, "%s: cosine and sine bases need a fully spectral grid", fn);
  const double pi = M_PI;
  if (bx) {
    g.bx = bx;
    g.dfx = (bx == MGB_BASIS_SINE ? pi : -pi) / p->grid.lx;
    g.d2x = -((pi * pi) / (p->grid.lx * p->grid.lx));
  }
  if (bz) {
    g.bz = bz;
    g.dfz = (bz == MGB_BASIS_SINE ? pi : -pi) / p->grid.lz;
    g.d2z = -((pi * pi) / (p->grid.lz * p->grid.lz));
  }
  return MGB_OK;
}

int pw_spectral_derivative_basis(const mgb_plan* p, int kind, int bx, int bz, const zd* in, zd* out, cudaStream_t s) {
  GridC g;
  if (int st = basis_grid(p, bx, bz, g, "mgb_spectral_derivative_basis")) return st;
  if (kind < MGB_DDX || kind > MGB_NABLA2) return fail(MGB_ERR_INVALID, "unknown derivative kind %d", kind);
  if (in == out && g.fdm && (kind != MGB_DDX && kind != MGB_D2DX2))
    return fail(MGB_ERR_INVALID, "z stencils on FDM-z need distinct input and output");
  k_spec_deriv<<<nblocks((size_t)g.rows * g.cols), PT, 0, s>>>(g, kind, in, out);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_laplacian_basis(const mgb_plan* p, int bx, int bz, double* lap, cudaStream_t s) {
  GridC g;
  if (int st = basis_grid(p, bx, bz, g, "mgb_laplacian_basis")) return st;
  k_laplacian<<<nblocks((size_t)g.rows * g.cols), PT, 0, s>>>(g, lap);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_poisson_basis(const mgb_plan* p, int bx, int bz, const zd* rhs, zd* out, cudaStream_t s) {
  GridC g;
  if (int st = basis_grid(p, bx, bz, g, "mgb_poisson_solve_basis")) return st;
  if (g.fdm) return fail(MGB_ERR_UNSUPPORTED, "mgb_poisson_solve_basis: fully spectral plans only");
  k_poisson_spectral<<<nblocks((size_t)g.rows * g.cols), PT, 0, s>>>(g, rhs, out);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_integrate_semi_implicit(const mgb_plan* p, zd* var, zd* hist, int order, int curr, double dt,
                               double alpha, const double* lin_op, cudaStream_t s) {
  const size_t total = (size_t)p->g.rows * p->g.cols;
  k_semi_implicit<<<nblocks(total), PT, 0, s>>>(total, var, hist, order, curr, dt, alpha, lin_op);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_integrate_explicit(const mgb_plan* p, zd* var, zd* hist, int order, int curr, double dt, const zd* diffusion,
                          cudaStream_t s) {
  const size_t total = (size_t)p->g.rows * p->g.cols;
  k_explicit<<<nblocks(total), PT, 0, s>>>(total, var, hist, order, curr, dt, diffusion);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_adams(const mgb_plan* p, int corrector, const zd* hist, int order, int curr, double dt, zd* out,
             cudaStream_t s) {
  const size_t total = (size_t)p->g.rows * p->g.cols;
  k_adams<<<nblocks(total), PT, 0, s>>>(total, corrector, hist, order, curr, dt, out);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_finish_diag(const double* partial, int n, int count, double inv_npts, double* out, cudaStream_t s, int ow) {
  k_diag_finish<<<count, PT, 0, s>>>(partial, n, inv_npts, ow, out);
  MGB_LAUNCH_CHECK();
  return MGB_OK;
}

int pw_diagnostics(const mgb_plan* p, const double* ux, const double* uz, double* out, void* work,
                   cudaStream_t s) {
  const GridC& g = p->g;
  const size_t total = (size_t)g.nx * g.nz;
  const int nb = 152 * 4;
  double* partial = (double*)work;
  k_diag_partial<<<nb, PT, 0, s>>>(total, ux, uz, partial);
  MGB_LAUNCH_CHECK();
  return pw_finish_diag(partial, nb, 1, 1.0 / (double)total, out, s);
}

}  // namespace mgb
