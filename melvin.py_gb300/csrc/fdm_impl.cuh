// Fourier-x / finite-difference-z (Dirichlet) kernels.
//
// Layouts (row-major): spectral zd[nn][nz] (x modes n = 0..nn-1 by z
// points), physical T/double [nx][nz].
//
// Transforms are along x only (melvin/SpectralTransformer.py:33-88): the
// x pass works on tiles of C adjacent z columns; two real z columns are
// packed into one complex transform of length nx.
//
// Timestep (examples/rayleigh_benard_convection.py:97-142):
//   k_thomas    psi = solve(-w), per-mode Dirichlet tridiagonal
//               (melvin/LaplacianSolver.py:21-56, 70-79);
//   k_fd_xinv   ux = -pddz(psi), uz = sddx(psi) and the advected fields to
//               physical (melvin/utility.py:66-79); writes the diffusion
//               term kappa * snabla2(q) into the history slot that receives f0;
//   k_fd_phys   J = pddx(ux q) + pddz(uz q) (melvin/Variable.py:119-128);
//   k_fd_xfwd   J to spectral, f = -J^ + linear terms + diffusion, explicit
//               Adams-Bashforth, AB predictor or AM corrector, boundary rules.
#pragma once

#include "spectral2d_impl.cuh"

namespace mgb {

// Complex columns (pairs of z columns) per CTA of an FDM x pass.
template <typename T, int N>
struct FdTile {
  static constexpr int E = 4096;
  static constexpr int P0 = E / N;
  static constexpr int CP = P0 < 1 ? 1 : (P0 > 32 ? 32 : P0);
  static constexpr int C = 2 * CP;  // z columns
};

// Address of a per-member array in a batched launch: member z uses
// base + k * stride bytes, with k the member's slot (arrays owned by the
// caller, e.g. states and histories) or z itself (step scratch).
struct Mptr {
  void* base;
  size_t stride;  // bytes
  int by_slot;
};
__device__ __forceinline__ char* maddr(const Mptr& p, const int* members, int z) {
  const int k = (p.by_slot && members) ? members[z] : z;
  return (char*)p.base + (size_t)k * p.stride;
}
inline Mptr mp(const void* base, size_t stride = 0, int by_slot = 0) { return Mptr{(void*)base, stride, by_slot}; }

// pd2dz2 of a complex spectral row at z (interior only), times kappa, plus
// kappa * d2x n^2 q  ==  kappa * snabla2(q) (melvin/Variable.py:111-113);
// inv = 1/dz^2, computed once on the host.
__device__ __forceinline__ zd fd_snabla2(const GridC& g, const zd* row, int n, int z, double kappa, double inv) {
  const int h = g.sdo / 2;
  double ax = 0, ay = 0;
  if (z >= h && z < g.nz - h) {
    const zd p1 = row[z + 1], c0 = row[z], m1 = row[z - 1];
    if (g.sdo == 2) {
      ax = ((p1.x - 2 * c0.x) + m1.x) * inv;
      ay = ((p1.y - 2 * c0.y) + m1.y) * inv;
    } else {
      const zd p2 = row[z + 2], m2 = row[z - 2];
      ax = ((((-1.0 / 12) * p2.x + (4.0 / 3) * p1.x) - (5.0 / 2) * c0.x) + (4.0 / 3) * m1.x - (1.0 / 12) * m2.x) * inv;
      ay = ((((-1.0 / 12) * p2.y + (4.0 / 3) * p1.y) - (5.0 / 2) * c0.y) + (4.0 / 3) * m1.y - (1.0 / 12) * m2.y) * inv;
    }
  }
  const zd q = row[z];
  const double f = g.d2x * (double)(n * n);
  return mk(kappa * (f * q.x + ax), kappa * (f * q.y + ay));
}

// ---------------------------------------------------------------------------
// Thomas solve of the per-mode Dirichlet Poisson systems, segmented.
//
// The factors (inverse pivots ip, modified upper diagonal cp) are
// precomputed per plan.  The forward sweep y_j = (r_j - a y_{j-1}) ip_j and
// the back substitution x_j = y_j - cp_j x_{j+1} are first-order linear
// recurrences, so a sweep over a segment started from zero differs from the
// true one by the carried value times a product of coefficients:
//   y_j = yh_j + P_j y_{s-1},  P_j = prod_{i=s..j} (-a ip_i)
//   x_j = xh_j + Q_j x_{e},    Q_j = prod_{i=j..e-1} (-cp_i)
// for a segment [s, e).  The interior rows 1..nz-2 are cut into segments of
// TH_SEG rows (fixed per grid; P and Q are precomputed per plan).  G lanes of
// a warp solve one mode: a round covers G consecutive segments, one per lane;
// each lane sweeps its segment from zero in registers, the segment maps
// c -> P c + yh are composed across the G lanes by a shuffle scan, and each
// lane adds its correction.  The lane that starts where the previous round
// ended sweeps from the known carry and needs no correction, so with G = 1
// this is the plain sequential sweep.  G depends on nz only, so a mode gives
// the same bits whatever the batch around it.  `out` may alias the
// right-hand side: a lane reads its rows before writing them, and rows 0 and
// nz-1 are read by every lane before the first write.
// ---------------------------------------------------------------------------

constexpr int TH_SEG = 16;
constexpr int TH_THREADS = 32;  // one warp per CTA: the modes spread over every SM

// Lanes per mode: one segment per lane per round, at most a warp.
inline int thomas_lanes(int nz) {
  const int segs = (nz - 2 + TH_SEG - 1) / TH_SEG;
  int G = 1;
  while (G < 32 && G < segs) G *= 2;
  return G;
}

// Member = blockIdx.y; mode = (blockIdx.x * TH_THREADS + threadIdx.x) / G.
template <int G>
static __global__ void __launch_bounds__(TH_THREADS)
    k_thomas(GridC g, Mptr rhs_p, double rhs_sign, Mptr out_p, const int* members, const double* __restrict__ inv_piv,
             const double* __restrict__ cp, const double* __restrict__ pseg, const double* __restrict__ qseg,
             Gate gate) {
  if (gate_closed(gate)) return;
  const int lane = threadIdx.x & 31;
  const int gl = lane & (G - 1);
  const unsigned gmask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
  const int n = (blockIdx.x * TH_THREADS + threadIdx.x) / G;
  if (n >= g.nn) return;  // whole groups leave together
  const int nz = g.nz;
  const size_t fo = (size_t)n * nz;
  const zd* rhs = (const zd*)maddr(rhs_p, members, blockIdx.y) + fo;
  zd* out = (zd*)maddr(out_p, members, blockIdx.y) + fo;
  const double* ip = inv_piv + fo;
  const double* c = cp + fo;
  const double* ps = pseg + fo;
  const double* qs = qseg + fo;
  const double a = 1.0 / (g.dz * g.dz);
  // rhs_sign is +1 or -1, applied as a negation (exact, and no multiply the
  // compiler could fuse into the sweep's FMA)
  const bool neg = rhs_sign < 0;
  zd y0 = rhs[0], yl = rhs[nz - 1];  // identity end rows
  if (neg) {
    y0 = -y0;
    yl = -yl;
  }
  __syncwarp(gmask);
  constexpr int R = G * TH_SEG;
  const int rounds = (nz - 2 + R - 1) / R;

  // forward sweep
  zd carry = y0;
  for (int rd = 0; rd < rounds; ++rd) {
    const int js = 1 + rd * R + gl * TH_SEG;
    const int cnt = min(max(nz - 1 - js, 0), TH_SEG);
    zd v[TH_SEG];
    double q[TH_SEG];
#pragma unroll
    for (int u = 0; u < TH_SEG; ++u) {
      v[u] = u < cnt ? rhs[js + u] : mk(0.0, 0.0);
      q[u] = u < cnt ? ip[js + u] : 0.0;
    }
    if (neg) {
#pragma unroll
      for (int u = 0; u < TH_SEG; ++u) v[u] = -v[u];
    }
    const bool first = gl == 0;
    zd prev = first ? carry : mk(0.0, 0.0);
#pragma unroll
    for (int u = 0; u < TH_SEG; ++u) {
      if (u < cnt) {
        prev = mk((v[u].x - a * prev.x) * q[u], (v[u].y - a * prev.y) * q[u]);
        v[u] = prev;
      }
    }
    if constexpr (G > 1) {
      double A = first ? 0.0 : (cnt > 0 ? ps[js + cnt - 1] : 1.0);
      zd B = prev;
#pragma unroll
      for (int d = 1; d < G; d <<= 1) {
        const double Ao = __shfl_up_sync(gmask, A, d, G);
        const double Bx = __shfl_up_sync(gmask, B.x, d, G);
        const double By = __shfl_up_sync(gmask, B.y, d, G);
        if (gl >= d) {
          B = mk(fma(A, Bx, B.x), fma(A, By, B.y));
          A *= Ao;
        }
      }
      // B is now y at the end of this lane's segment (lane 0's map is constant)
      const double cx = __shfl_up_sync(gmask, B.x, 1, G);
      const double cy = __shfl_up_sync(gmask, B.y, 1, G);
      carry = mk(__shfl_sync(gmask, B.x, G - 1, G), __shfl_sync(gmask, B.y, G - 1, G));
      if (!first) {
#pragma unroll
        for (int u = 0; u < TH_SEG; ++u)
          if (u < cnt) {
            const double p = ps[js + u];
            v[u] = mk(fma(p, cx, v[u].x), fma(p, cy, v[u].y));
          }
      }
    } else {
      carry = prev;
    }
#pragma unroll
    for (int u = 0; u < TH_SEG; ++u)
      if (u < cnt) out[js + u] = v[u];
  }

  // back substitution
  carry = yl;
  for (int rd = rounds - 1; rd >= 0; --rd) {
    const int js = 1 + rd * R + gl * TH_SEG;
    const int cnt = min(max(nz - 1 - js, 0), TH_SEG);
    const int jend = min(1 + (rd + 1) * R, nz - 1);
    zd v[TH_SEG];
    double cc[TH_SEG];
#pragma unroll
    for (int u = 0; u < TH_SEG; ++u) {
      v[u] = u < cnt ? out[js + u] : mk(0.0, 0.0);
      cc[u] = u < cnt ? c[js + u] : 0.0;
    }
    const bool first = cnt > 0 && js + cnt == jend;  // the lane the carry enters
    zd next = first ? carry : mk(0.0, 0.0);
#pragma unroll
    for (int u = TH_SEG - 1; u >= 0; --u) {
      if (u < cnt) {
        next = mk(v[u].x - cc[u] * next.x, v[u].y - cc[u] * next.y);
        v[u] = next;
      }
    }
    if constexpr (G > 1) {
      double A = first ? 0.0 : (cnt > 0 ? qs[js] : 1.0);
      zd B = next;
#pragma unroll
      for (int d = 1; d < G; d <<= 1) {
        const double Ao = __shfl_down_sync(gmask, A, d, G);
        const double Bx = __shfl_down_sync(gmask, B.x, d, G);
        const double By = __shfl_down_sync(gmask, B.y, d, G);
        if (gl + d < G) {
          B = mk(fma(A, Bx, B.x), fma(A, By, B.y));
          A *= Ao;
        }
      }
      // B is now x at the start of this lane's segment
      const double cx = __shfl_down_sync(gmask, B.x, 1, G);
      const double cy = __shfl_down_sync(gmask, B.y, 1, G);
      carry = mk(__shfl_sync(gmask, B.x, 0, G), __shfl_sync(gmask, B.y, 0, G));
      if (!first) {
#pragma unroll
        for (int u = 0; u < TH_SEG; ++u)
          if (u < cnt) {
            const double q = qs[js + u];
            v[u] = mk(fma(q, cx, v[u].x), fma(q, cy, v[u].y));
          }
      }
    } else {
      carry = next;
    }
#pragma unroll
    for (int u = 0; u < TH_SEG; ++u)
      if (u < cnt) out[js + u] = v[u];
  }
  if (gl == 0) {
    out[0] = y0;
    out[nz - 1] = yl;
  }
}

// ---------------------------------------------------------------------------
// x pass inverse: spectral rows n < nn of up to 3 fields -> physical.
// ---------------------------------------------------------------------------

// What an x-inverse job transforms.
enum FdKind : int {
  FD_COPY = 0,  // the spectral field itself
  FD_UX = 1,    // ux = -pddz(psi): the Dirichlet z stencil commutes with the x transform
  FD_UZ = 2     // uz = sddx(psi) = (2*pi*i/lx) n psi (melvin/utility.py:76-79)
};

struct FdXinvJob {
  Mptr src;       // zd [nn][nz]
  Mptr phys;      // T [nx][nz]
  Mptr diff_out;  // optional (base null): kappa * snabla2(src) -> history slot
  double kappa;
  int kind;       // FdKind
  zd* spec_out;   // optional, single member: the transformed spectral field (uz spectral data)
};

// First-derivative z stencil of a complex spectral row (Dirichlet: the
// outer sdo/2 points are 0), scaled by inv = 1/(2dz) or 1/(3dz).
__device__ __forceinline__ zd fd_ddz_row(const zd* row, int z, int nz, int sdo, double inv) {
  const int h = sdo / 2;
  if (z < h || z >= nz - h) return mk(0.0, 0.0);
  const zd p1 = row[z + 1], m1 = row[z - 1];
  if (sdo == 2) return mk((p1.x - m1.x) * inv, (p1.y - m1.y) * inv);
  const zd p2 = row[z + 2], m2 = row[z - 2];
  return mk((((-0.25 * p2.x + 2 * p1.x) - 2 * m1.x) + 0.25 * m2.x) * inv,
            (((-0.25 * p2.y + 2 * p1.y) - 2 * m1.y) + 0.25 * m2.y) * inv);
}

// The same two stencils evaluated in the transform precision T (split and
// double-float modes: derivatives in the precision of the transforms).
template <typename T>
__device__ __forceinline__ cx<T> fd_ddz_row_t(const zd* row, int z, int nz, int sdo, T inv) {
  const int h = sdo / 2;
  if (z < h || z >= nz - h) return mk<T>(0, 0);
  const cx<T> p1 = cvt<T>(row[z + 1]), m1 = cvt<T>(row[z - 1]);
  if (sdo == 2) return (p1 - m1) * inv;
  const cx<T> p2 = cvt<T>(row[z + 2]), m2 = cvt<T>(row[z - 2]);
  return (((p2 * (T)-0.25 + p1 * (T)2) - m1 * (T)2) + m2 * (T)0.25) * inv;
}

template <typename T>
__device__ __forceinline__ zd fd_snabla2_t(const GridC& g, const zd* row, int n, int z, T kappa, T inv) {
  const int h = g.sdo / 2;
  const cx<T> q = cvt<T>(row[z]);
  cx<T> acc = mk<T>(0, 0);
  if (z >= h && z < g.nz - h) {
    const cx<T> p1 = cvt<T>(row[z + 1]), m1 = cvt<T>(row[z - 1]);
    if (g.sdo == 2) {
      acc = ((p1 - q * (T)2) + m1) * inv;
    } else {
      const cx<T> p2 = cvt<T>(row[z + 2]), m2 = cvt<T>(row[z - 2]);
      acc = ((((p2 * (T)(-1.0 / 12) + p1 * (T)(4.0 / 3)) - q * (T)2.5) + m1 * (T)(4.0 / 3)) - m2 * (T)(1.0 / 12)) *
            inv;
    }
  }
  const T f = to_t<T>(g.d2x) * (T)(n * n);
  return cvt<double>((q * f + acc) * kappa);
}

struct FdXinvArgs {
  GridC g;
  FdXinvJob job[5];
  double fdz;    // 1/(2dz) or 1/(3dz)
  double inv_dz2;  // 1/dz^2
  const void* tw;
  const int* members;  // member = blockIdx.z
  Gate gate;
};

template <typename T, int N, int CP>
__global__ void __launch_bounds__(NT) k_fd_xinv(const FdXinvArgs a) {
  if (gate_closed(a.gate)) return;
  constexpr int C = 2 * CP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const FdXinvJob jb = a.job[blockIdx.y];
  const int z0 = blockIdx.x * C;
  const zd* src = (const zd*)maddr(jb.src, a.members, blockIdx.z);
  zd* dout = jb.diff_out.base ? (zd*)maddr(jb.diff_out, a.members, blockIdx.z) : nullptr;
  for (int e = threadIdx.x; e < sbuf_elems<T, CP>(N); e += NT) buf[e] = mk<T>(0, 0);
  __syncthreads();
  for (int e = threadIdx.x; e < g.nn * CP; e += NT) {
    const int n = e / CP, j = e - n * CP;
    const int za = z0 + 2 * j, zb = za + 1;
    const zd* row = src + (size_t)n * g.nz;
    if constexpr (std::is_same<T, double>::value) {
      zd A = mk(0.0, 0.0), B = mk(0.0, 0.0);
      if (jb.kind == FD_UX) {
        if (za < g.nz) A = fd_ddz_row(row, za, g.nz, g.sdo, a.fdz);
        if (zb < g.nz) B = fd_ddz_row(row, zb, g.nz, g.sdo, a.fdz);
        A = mk(-A.x, -A.y);
        B = mk(-B.x, -B.y);
      } else {
        if (za < g.nz) A = row[za];
        if (zb < g.nz) B = row[zb];
        if (jb.kind == FD_UZ) {
          const double b = g.dfx * (double)n;
          A = mk(-(b * A.y), b * A.x);
          B = mk(-(b * B.y), b * B.x);
        }
      }
      if (jb.spec_out) {
        if (za < g.nz) jb.spec_out[(size_t)n * g.nz + za] = A;
        if (zb < g.nz) jb.spec_out[(size_t)n * g.nz + zb] = B;
      }
      put_pair<T, N, CP>(buf, j, n, A, B);
      if (dout) {
        if (za < g.nz) dout[(size_t)n * g.nz + za] = fd_snabla2(g, row, n, za, jb.kappa, a.inv_dz2);
        if (zb < g.nz) dout[(size_t)n * g.nz + zb] = fd_snabla2(g, row, n, zb, jb.kappa, a.inv_dz2);
      }
    } else {
      // split / double-float: stencils and the i*kx factor in T, from the
      // FP64 rows (the per-verb spec_out outputs are FP64-only)
      cx<T> A = mk<T>(0, 0), B = mk<T>(0, 0);
      if (jb.kind == FD_UX) {
        const T inv = to_t<T>(a.fdz);
        if (za < g.nz) A = -fd_ddz_row_t<T>(row, za, g.nz, g.sdo, inv);
        if (zb < g.nz) B = -fd_ddz_row_t<T>(row, zb, g.nz, g.sdo, inv);
      } else {
        if (za < g.nz) A = cvt<T>(row[za]);
        if (zb < g.nz) B = cvt<T>(row[zb]);
        if (jb.kind == FD_UZ) {
          const T b = to_t<T>(g.dfx) * (T)n;
          A = mk(-(b * A.y), b * A.x);
          B = mk(-(b * B.y), b * B.x);
        }
      }
      put_pair<T, N, CP>(buf, j, n, A, B);
      if (dout) {
        const T kap = to_t<T>(jb.kappa), inv = to_t<T>(a.inv_dz2);
        if (za < g.nz) dout[(size_t)n * g.nz + za] = fd_snabla2_t<T>(g, row, n, za, kap, inv);
        if (zb < g.nz) dout[(size_t)n * g.nz + zb] = fd_snabla2_t<T>(g, row, n, zb, kap, inv);
      }
    }
  }
  __syncthreads();
  // modes nn .. N-nn are zero (the 2/3 rule: nn <= 3N/8)
  block_fft<T, N, CP, CP, NT, +1, 8, true>(buf, (const cx<T>*)a.tw);
  T* out = (T*)maddr(jb.phys, a.members, blockIdx.z);
  for (int e = threadIdx.x; e < N * CP; e += NT) {
    const int x = e / CP, j = e - x * CP;
    const int za = z0 + 2 * j;
    const cx<T> v = buf[sx<T, CP>(x, j)];
    if (za < g.nz) out[(size_t)x * g.nz + za] = v.x;
    if (za + 1 < g.nz) out[(size_t)x * g.nz + za + 1] = v.y;
  }
}

// ---------------------------------------------------------------------------
// Physical stencil pass on a 2D tile with a halo of h = sdo/2 points.
// ---------------------------------------------------------------------------

constexpr int FD_TX = 16, FD_TZ = 64;

struct FdPhysArgs {
  GridC g;
  Mptr ux;           // T [nx][nz], per member
  Mptr uz;
  Mptr q[3];
  Mptr jout[3];
  Mptr partial;      // optional (base null): per-CTA diagnostics (sum ux^2+uz^2, max ux, max uz,
                     // sum uz*q of field flux_f)
  int nf;
  int flux_f;        // -1: none
  double fdx, fdz;   // 1/(2dx) or 1/(3dx); same for z
  Gate gate;
};

// Central first difference (-f[i+2]/4 + 2 f[i+1] - 2 f[i-1] + f[i-2]/4) * inv
// of order 4 (inv = 1/(3h)), or (f[i+1] - f[i-1]) * inv of order 2, as
// (p1 - m1) * inv2 - (p2 - m2) * inv4 with inv2 = 2 inv, inv4 = inv / 4: four
// operations instead of five (powers of two, so inv2 and inv4 are exact).
template <typename T>
__device__ __forceinline__ T st1(T p2, T p1, T m1, T m2, int sdo, T inv, T inv2, T inv4) {
  if (sdo == 2) return (p1 - m1) * inv;
  return (p1 - m1) * inv2 - (p2 - m2) * inv4;
}
// The same difference in the reference's order of operations
// (melvin/SpatialDifferentiator.py:76-104; the per-verb kernels).
template <typename T>
__device__ __forceinline__ T st1(T p2, T p1, T m1, T m2, int sdo, T inv) {
  if (sdo == 2) return (p1 - m1) * inv;
  return (((p2 * (T)-0.25 + p1 * (T)2) - m1 * (T)2) + m2 * (T)0.25) * inv;
}

// J_f = pddx(ux q_f) + pddz(uz q_f) on a 2D tile (x periodic, z Dirichlet:
// the outer sdo/2 points of pddz stay 0) (melvin/Variable.py:125-127).
template <typename T>
__global__ void __launch_bounds__(NT, (std::is_same<T, float>::value ? 8 : 1)) k_fd_phys(const FdPhysArgs a) {
  if (gate_closed(a.gate)) return;
  constexpr int H = 2;  // storage halo (covers order 4)
  constexpr int SX = FD_TX + 2 * H, SZ = FD_TZ + 2 * H;
  __shared__ T s_ux[SX][FD_TZ];  // x halo
  __shared__ T s_uz[FD_TX][SZ];  // z halo
  // FP64 and double-float stage the products ux*q and uz*q once per point (as
  // the reference forms them before differentiating, melvin/Variable.py:125-127):
  // a third fewer operations on the narrow FP64 pipe (1024x513 RBC step 0.500
  // -> 0.467 ms).  FP32 multiplies inside the stencil from staged q: the extra
  // shared-memory pass costs it 2%.  The products are the same rounded values
  // either way.
  constexpr bool kStage = !std::is_same<T, float>::value;
  __shared__ T s_a[kStage ? SX : 1][kStage ? FD_TZ : 1];  // ux*q, x halo
  __shared__ T s_b[kStage ? FD_TX : SX][SZ];               // uz*q (z halo), or q (both halos)
  const GridC& g = a.g;
  const int nx = g.nx, nz = g.nz, sdo = g.sdo, h = sdo / 2;
  const int x0 = blockIdx.y * FD_TX, z0 = blockIdx.x * FD_TZ;
  const T fdx = to_t<T>(a.fdx), fdz = to_t<T>(a.fdz);
  const T fdx2 = fdx * (T)2, fdx4 = fdx * (T)0.25, fdz2 = fdz * (T)2, fdz4 = fdz * (T)0.25;
  const T* ux = (const T*)maddr(a.ux, nullptr, blockIdx.z);
  const T* uz = (const T*)maddr(a.uz, nullptr, blockIdx.z);
  for (int e = threadIdx.x; e < SX * FD_TZ; e += NT) {
    const int i = e / FD_TZ, k = e - i * FD_TZ;
    const int x = (x0 + i - H + nx) % nx, z = z0 + k;
    s_ux[i][k] = z < nz ? ux[(size_t)x * nz + z] : (T)0;
  }
  for (int e = threadIdx.x; e < FD_TX * SZ; e += NT) {
    const int i = e / SZ, k = e - i * SZ;
    const int x = x0 + i, z = z0 + k - H;
    s_uz[i][k] = (x < nx && z >= 0 && z < nz) ? uz[(size_t)x * nz + z] : (T)0;
  }
  __syncthreads();
  double ke = 0, mx = -INFINITY, mz = -INFINITY, fl = 0;
  if (a.partial.base) {
    for (int e = threadIdx.x; e < FD_TX * FD_TZ; e += NT) {
      const int i = e / FD_TZ, k = e - i * FD_TZ;
      if (x0 + i < nx && z0 + k < nz) {
        const double u = (double)s_ux[i + H][k], w = (double)s_uz[i][k + H];
        ke += w * w + u * u;
        mx = (u != u || u > mx) ? u : mx;
        mz = (w != w || w > mz) ? w : mz;
      }
    }
  }
  for (int f = 0; f < a.nf; ++f) {
    const T* q = (const T*)maddr(a.q[f], nullptr, blockIdx.z);
    const bool flux = a.partial.base && f == a.flux_f;
    if constexpr (kStage) {
      for (int e = threadIdx.x; e < SX * SZ; e += NT) {
        const int i = e / SZ, k = e - i * SZ;
        const int x = (x0 + i - H + nx) % nx, z = z0 + k - H;
        const T qv = (z >= 0 && z < nz) ? q[(size_t)x * nz + z] : (T)0;
        const bool in_z = k >= H && k < H + FD_TZ, in_x = i >= H && i < H + FD_TX;
        if (in_z) s_a[i][k - H] = s_ux[i][k - H] * qv;
        if (in_x) s_b[i - H][k] = s_uz[i - H][k] * qv;
        if (flux && in_x && in_z && x0 + i - H < nx && z < nz) fl += (double)s_uz[i - H][k] * (double)qv;
      }
      __syncthreads();
    } else {
      auto& s_q = s_b;
      for (int e = threadIdx.x; e < SX * SZ; e += NT) {
        const int i = e / SZ, k = e - i * SZ;
        const int x = (x0 + i - H + nx) % nx, z = z0 + k - H;
        s_q[i][k] = (z >= 0 && z < nz) ? q[(size_t)x * nz + z] : (T)0;
      }
      __syncthreads();
      if (flux) {
        for (int e = threadIdx.x; e < FD_TX * FD_TZ; e += NT) {
          const int i = e / FD_TZ, k = e - i * FD_TZ;
          if (x0 + i < nx && z0 + k < nz) fl += (double)s_uz[i][k + H] * (double)s_q[i + H][k + H];
        }
      }
    }
    T* jo = (T*)maddr(a.jout[f], nullptr, blockIdx.z);
    for (int e = threadIdx.x; e < FD_TX * FD_TZ; e += NT) {
      const int i = e / FD_TZ, k = e - i * FD_TZ;
      const int x = x0 + i, z = z0 + k;
      if (x >= nx || z >= nz) continue;
      const int ii = i + H, kk = k + H;
      T jx, jz = 0;
      if constexpr (kStage) {
        jx = st1(s_a[ii + 2][k], s_a[ii + 1][k], s_a[ii - 1][k], s_a[ii - 2][k], sdo, fdx, fdx2, fdx4);
        if (z >= h && z < nz - h)
          jz = st1(s_b[i][kk + 2], s_b[i][kk + 1], s_b[i][kk - 1], s_b[i][kk - 2], sdo, fdz, fdz2, fdz4);
      } else {
        const auto& s_q = s_b;
        jx = st1(s_ux[ii + 2][k] * s_q[ii + 2][kk], s_ux[ii + 1][k] * s_q[ii + 1][kk],
                 s_ux[ii - 1][k] * s_q[ii - 1][kk], s_ux[ii - 2][k] * s_q[ii - 2][kk], sdo, fdx, fdx2, fdx4);
        if (z >= h && z < nz - h)
          jz = st1(s_uz[i][kk + 2] * s_q[ii][kk + 2], s_uz[i][kk + 1] * s_q[ii][kk + 1],
                   s_uz[i][kk - 1] * s_q[ii][kk - 1], s_uz[i][kk - 2] * s_q[ii][kk - 2], sdo, fdz, fdz2, fdz4);
      }
      jo[(size_t)x * nz + z] = jx + jz;
    }
    __syncthreads();
  }
  if (a.partial.base) {
    __shared__ double red[4][NT / 32];
    for (int o = 16; o > 0; o >>= 1) {
      ke += __shfl_xor_sync(0xffffffffu, ke, o);
      fl += __shfl_xor_sync(0xffffffffu, fl, o);
      const double t1 = __shfl_xor_sync(0xffffffffu, mx, o), t2 = __shfl_xor_sync(0xffffffffu, mz, o);
      mx = (t1 != t1 || t1 > mx) ? t1 : mx;
      mz = (t2 != t2 || t2 > mz) ? t2 : mz;
    }
    if ((threadIdx.x & 31) == 0) {
      red[0][threadIdx.x >> 5] = ke;
      red[1][threadIdx.x >> 5] = mx;
      red[2][threadIdx.x >> 5] = mz;
      red[3][threadIdx.x >> 5] = fl;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double S = 0, MX = -INFINITY, MZ = -INFINITY, FL = 0;
      for (int i = 0; i < NT / 32; ++i) {
        S += red[0][i];
        FL += red[3][i];
        MX = (red[1][i] != red[1][i] || red[1][i] > MX) ? red[1][i] : MX;
        MZ = (red[2][i] != red[2][i] || red[2][i] > MZ) ? red[2][i] : MZ;
      }
      const int cta = blockIdx.y * gridDim.x + blockIdx.x;
      double* part = (double*)maddr(a.partial, nullptr, blockIdx.z);
      part[kDiagW * cta + 0] = S;
      part[kDiagW * cta + 1] = MX;
      part[kDiagW * cta + 2] = MZ;
      part[kDiagW * cta + 3] = FL;
    }
  }
}

// ---------------------------------------------------------------------------
// x pass forward: physical J_f -> spectral, then the update.
// ---------------------------------------------------------------------------

enum FdMode : int {
  FD_OUT = 0,       // plain to_spectral into `out` (per-verb API)
  FD_EXPLICIT = 1,  // q += AB(hist)
  FD_PREDICT = 2,   // qpred = q + AB(hist)
  FD_CORRECT = 3    // q = q + AM(hist)
};

struct FdXfField {
  int nterms;
  int tsrc[4];
  int top[4];
  double tcoef[4];
  int bc;
};

struct FdXfArgs {
  GridC g;
  Mptr jin[3];         // T [nx][nz]
  Mptr q[3];           // states: read (all modes); written for EXPLICIT / CORRECT
  Mptr qsrc[3];        // states the linear terms read (q, or the predicted state)
  Mptr qpred[3];       // PREDICT output
  Mptr hist[3];
  Mptr psi;            // spectral psi of the evaluated state (for src = -1 terms)
  zd* out;             // FD_OUT target (single member)
  const int* members;  // member = blockIdx.y
  const double* tcoef; // optional per-slot term coefficients [slot][3][4]
  int nf, mode, order, curr;
  double dt, inv_nx;   // dt: used unless gate.dt points at a driven run's dt
  FdXfField eq[3];
  const void* tw;
  Gate gate;
};

// History values f_{-1}, f_{-2}, f_{-3} of one element (AB2 uses the
// first) from the ring of `order` slots (melvin/TimeDerivative.py:4-65).
__device__ __forceinline__ void fd_hist_load(const zd* h, size_t slot, int order, int curr, zd hp[3]) {
  if (order == 2) {
    hp[0] = h[(size_t)((curr + 1) & 1) * slot];
    return;
  }
  hp[0] = h[(size_t)((curr + 3) & 3) * slot];
  hp[1] = h[(size_t)((curr + 2) & 3) * slot];
  hp[2] = h[(size_t)((curr + 1) & 3) * slot];
}
// Adams-Bashforth and Adams-Moulton increments (melvin/Integrator.py:5-33)
// of the newest value f0 and the history values hp.
__device__ __forceinline__ zd fd_ab(int order, zd f0, const zd hp[3], double dt) {
  if (order == 2) {
    const double c = dt / 2;
    return mk(c * (3 * f0.x - hp[0].x), c * (3 * f0.y - hp[0].y));
  }
  const double c = dt / 24;
  return mk(c * (((55 * f0.x - 59 * hp[0].x) + 37 * hp[1].x) - 9 * hp[2].x),
            c * (((55 * f0.y - 59 * hp[0].y) + 37 * hp[1].y) - 9 * hp[2].y));
}
__device__ __forceinline__ zd fd_am(int order, zd f0, const zd hp[3], double dt) {
  if (order == 2) {
    const double c = dt / 2;
    return mk(c * (f0.x + hp[0].x), c * (f0.y + hp[0].y));
  }
  const double c = dt / 24;
  return mk(c * (((9 * f0.x + 19 * hp[0].x) - 5 * hp[1].x) + hp[2].x),
            c * (((9 * f0.y + 19 * hp[0].y) - 5 * hp[1].y) + hp[2].y));
}
__device__ __forceinline__ zd fd_bc(zd v, int bc, int n, int z, int nz, int e) {
  const bool lower = z < e, upper = z >= nz - e;
  if (bc & MGB_BC_DIRICHLET_W) {
    if (n == 0 || lower || upper) return mk(0.0, 0.0);
  }
  if (bc & MGB_BC_DIRICHLET_T) {
    if (n == 0) {
      if (lower) return mk(1.0, 0.0);
      if (upper) return mk(0.0, 0.0);
    } else if (lower || upper) {
      return mk(0.0, 0.0);
    }
  }
  return v;
}

// Two resident CTAs of the x-forward pass where shared memory allows (the
// register budget then stays at 128: the update holds every load of an
// element for all fields at once).
template <typename T, int N, int F, int CP>
struct FdXfOcc {
  static constexpr size_t smem = (size_t)F * sbuf_elems<T, CP>(N) * sizeof(cx<T>);
  static constexpr int value = 233472 / (smem + 1024) >= 2 ? 2 : 1;
};

template <typename T, int N, int F, int CP>
__global__ void __launch_bounds__(NT, (FdXfOcc<T, N, F, CP>::value)) k_fd_xfwd(const FdXfArgs a) {
  if (gate_closed(a.gate)) return;
  const double dt = a.gate.dt ? *a.gate.dt : a.dt;
  constexpr int C = 2 * CP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const int z0 = blockIdx.x * C;
  const int zm = blockIdx.y;
  const int slot = a.members ? a.members[zm] : zm;
#pragma unroll
  for (int f = 0; f < F; ++f) {
    const T* J = (const T*)maddr(a.jin[f], a.members, zm);
    cx<T>* bf = buf + f * sbuf_elems<T, CP>(N);
    for (int e = threadIdx.x; e < N * CP; e += NT) {
      const int x = e / CP, j = e - x * CP;
      const int za = z0 + 2 * j;
      const T va = za < g.nz ? J[(size_t)x * g.nz + za] : (T)0;
      const T vb = za + 1 < g.nz ? J[(size_t)x * g.nz + za + 1] : (T)0;
      bf[sx<T, CP>(x, j)] = mk(va, vb);
    }
  }
  __syncthreads();
#pragma unroll
  for (int f = 0; f < F; ++f) block_fft<T, N, CP, CP, NT, -1>(buf + f * sbuf_elems<T, CP>(N), (const cx<T>*)a.tw);
  const size_t hslot = (size_t)g.nn * g.nz;
  const int e_bc = g.sdo / 2;
  zd* qf[F];
  const zd* qs_[F];
  zd* qp[F];
  zd* hf[F];
#pragma unroll
  for (int f = 0; f < F; ++f) {
    qf[f] = (zd*)maddr(a.q[f], a.members, zm);
    qs_[f] = (const zd*)maddr(a.qsrc[f], a.members, zm);
    qp[f] = a.qpred[f].base ? (zd*)maddr(a.qpred[f], a.members, zm) : nullptr;
    hf[f] = (zd*)maddr(a.hist[f], a.members, zm);
  }
  const zd* psi = a.psi.base ? (const zd*)maddr(a.psi, a.members, zm) : nullptr;
  const double* tco = a.tcoef ? a.tcoef + (size_t)slot * 12 : nullptr;
  const double hnx = 0.5 * a.inv_nx;
  for (int e = threadIdx.x; e < g.nn * C; e += NT) {
    const int n = e / C, c = e - n * C, z = z0 + c;
    if (z >= g.nz) continue;
    const size_t idx = (size_t)n * g.nz + z;
    const int j = c >> 1, part = c & 1;
    if (a.mode == FD_OUT) {
      cx<T> A, B;
      get_pair<T, N, CP>(buf, j, n, A, B);
      const zd v = cvt<double>(part ? B : A);
      a.out[idx] = mk(v.x * a.inv_nx, v.y * a.inv_nx);
      continue;
    }
    // every load of the element, for all fields, before the first store (the
    // compiler cannot reorder loads above stores through these pointers)
    zd qs[F], hd[F], q0[F], hp[F][3];
    const double kx = g.dfx * (double)n;  // d/dx factor of the linear terms (every equation here has them)
    const zd ps = psi ? psi[idx] : mk(0.0, 0.0);
#pragma unroll
    for (int f = 0; f < F; ++f) {
      qs[f] = qs_[f][idx];
      hd[f] = hf[f][(size_t)a.curr * hslot + idx];
      q0[f] = qf[f][idx];
      fd_hist_load(hf[f] + idx, hslot, a.order, a.curr, hp[f]);
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
      // column z's half spectrum, twice over: (Z(n) + conj Z(N-n)) for the
      // even column of the pair, (Z(n) - conj Z(N-n)) / i for the odd one;
      // the 1/2 rides on the 1/nx scale (a power of two: the same values)
      const cx<T>* bf = buf + f * sbuf_elems<T, CP>(N);
      const cx<T> zn = bf[sx<T, CP>(n, j)], zc = bf[sx<T, CP>((N - n) & (N - 1), j)];
      const T s0 = part ? zn.y : zn.x, s1 = part ? zc.y : zc.x;
      const T d0 = part ? zc.x : zn.y, d1 = part ? zn.x : zc.y;
      const zd v = cvt<double>(mk(s0 + s1, d0 - d1));
      // f = -vec_dot_nabla + linear terms + diffusion (already in the slot)
      const zd d = hd[f];
      zd fv = mk(d.x - v.x * hnx, d.y - v.y * hnx);
      const FdXfField& eq = a.eq[f];
      for (int t = 0; t < eq.nterms; ++t) {
        const int sidx = eq.tsrc[t];
        zd sv = sidx < 0 ? ps : qs[0];
#pragma unroll
        for (int q2 = 1; q2 < F; ++q2)
          if (sidx == q2) sv = qs[q2];
        double cc = tco ? tco[f * 4 + t] : eq.tcoef[t];
        if (eq.top[t] == 1) {  // d/dx: the factor 2 pi n / lx rides on the coefficient, i on the value
          cc *= kx;
          sv = mk(-sv.y, sv.x);
        }
        fv = mk(fv.x + cc * sv.x, fv.y + cc * sv.y);
      }
      hf[f][(size_t)a.curr * hslot + idx] = fv;
      zd qn;
      if (a.mode == FD_CORRECT) {
        const zd am = fd_am(a.order, fv, hp[f], dt);
        qn = mk(q0[f].x + am.x, q0[f].y + am.y);
      } else {
        const zd ab = fd_ab(a.order, fv, hp[f], dt);
        qn = mk(q0[f].x + ab.x, q0[f].y + ab.y);
      }
      qn = fd_bc(qn, eq.bc, n, z, g.nz, e_bc);
      if (a.mode == FD_PREDICT)
        qp[f][idx] = qn;
      else
        qf[f][idx] = qn;
    }
  }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

// Column pairs per CTA of an FDM x pass: FdTile's count, or a half or a
// quarter of it.  The arithmetic of a column does not depend on the tile, so
// the choice is free per launch (measured on GB300 over single simulations
// and 32-slot pools, 128x129 .. 1024x1025):
//  * the x-inverse pass takes tiles of at most 1024 elements in FP64 (its FFT
//    is bound by the FP64 pipe and gains from more resident warps), and in
//    FP32 tiles of 2048 elements below length 512, FdTile's from 512 on;
//  * the x-forward pass takes the widest tile that still gives 1.5 CTAs per
//    SM (a single simulation on a short z axis narrows it; pools keep it).
// Double-float follows the FP32 rules.
inline int fd_sm_count() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    return cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && v > 0 ? v : 152;
  }();
  return n;
}

template <typename T, int N>
struct FdCps {
  static constexpr int c0 = FdTile<T, N>::CP;
  static constexpr int c1 = c0 > 1 ? c0 / 2 : c0;
  static constexpr int c2 = c1 > 1 ? c1 / 2 : c1;
  static constexpr int kInvElems = std::is_same<T, double>::value ? 1024 : (N >= 512 ? 4096 : 2048);
  static int xinv() {
    for (int cp : {c0, c1}) if (cp * N <= kInvElems) return cp;
    return c2;
  }
  static int xfwd(int nz, int nb) {
    for (int cp : {c0, c1}) {
      const long long ctas = (long long)((nz + 2 * cp - 1) / (2 * cp)) * nb;
      if (2 * ctas >= 3LL * fd_sm_count()) return cp;
    }
    return c2;
  }
};

template <typename T, int N, int CP>
cudaError_t launch_fd_xinv_cp(const FdXinvArgs& a, int njobs, int nb, cudaStream_t s) {
  constexpr int C = 2 * CP;
  const size_t smem = (size_t)sbuf_elems<T, CP>(N) * sizeof(cx<T>);
  cudaError_t e = prep_smem(k_fd_xinv<T, N, CP>, smem);
  if (e != cudaSuccess) return e;
  dim3 grid((a.g.nz + C - 1) / C, njobs, nb);
  k_fd_xinv<T, N, CP><<<grid, NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int N>
cudaError_t launch_fd_xinv(const FdXinvArgs& a, int njobs, int nb, cudaStream_t s) {
  using K = FdCps<T, N>;
  const int cp = K::xinv();
  if (cp == K::c2) return launch_fd_xinv_cp<T, N, K::c2>(a, njobs, nb, s);
  if (cp == K::c1) return launch_fd_xinv_cp<T, N, K::c1>(a, njobs, nb, s);
  return launch_fd_xinv_cp<T, N, K::c0>(a, njobs, nb, s);
}

template <typename T, int N, int F, int CP>
cudaError_t launch_fd_xfwd_cp(const FdXfArgs& a, int nb, cudaStream_t s) {
  constexpr int C = 2 * CP;
  constexpr size_t smem = (size_t)F * sbuf_elems<T, CP>(N) * sizeof(cx<T>);
  if constexpr (smem > kMaxDynSmem) {
    return cudaErrorInvalidConfiguration;
  } else {
    cudaError_t e = prep_smem(k_fd_xfwd<T, N, F, CP>, smem);
    if (e != cudaSuccess) return e;
    k_fd_xfwd<T, N, F, CP><<<dim3((a.g.nz + C - 1) / C, nb), NT, smem, s>>>(a);
    return cudaGetLastError();
  }
}

template <typename T, int N, int F>
cudaError_t launch_fd_xfwd(const FdXfArgs& a, int nb, cudaStream_t s) {
  using K = FdCps<T, N>;
  const int cp = K::xfwd(a.g.nz, nb);
  if (cp == K::c2) return launch_fd_xfwd_cp<T, N, F, K::c2>(a, nb, s);
  if (cp == K::c1) return launch_fd_xfwd_cp<T, N, F, K::c1>(a, nb, s);
  return launch_fd_xfwd_cp<T, N, F, K::c0>(a, nb, s);
}

struct FdLaunchers {
  cudaError_t (*xinv[3])(const FdXinvArgs&, int, int, cudaStream_t);  // [precision](args, jobs, members)
  cudaError_t (*xfwd[3][3])(const FdXfArgs&, int, cudaStream_t);      // [precision][F-1](args, members)
};

template <int N>
FdLaunchers make_fd_launchers() {
  FdLaunchers L;
  L.xinv[0] = launch_fd_xinv<double, N>;
  L.xinv[1] = launch_fd_xinv<float, N>;
  L.xfwd[0][0] = launch_fd_xfwd<double, N, 1>;
  L.xfwd[0][1] = launch_fd_xfwd<double, N, 2>;
  L.xfwd[0][2] = launch_fd_xfwd<double, N, 3>;
  L.xfwd[1][0] = launch_fd_xfwd<float, N, 1>;
  L.xfwd[1][1] = launch_fd_xfwd<float, N, 2>;
  L.xfwd[1][2] = launch_fd_xfwd<float, N, 3>;
  L.xinv[2] = launch_fd_xinv<df64, N>;
  L.xfwd[2][0] = launch_fd_xfwd<df64, N, 1>;
  L.xfwd[2][1] = launch_fd_xfwd<df64, N, 2>;
  L.xfwd[2][2] = launch_fd_xfwd<df64, N, 3>;
  return L;
}

const FdLaunchers* fd_launchers(int N);

}  // namespace mgb
