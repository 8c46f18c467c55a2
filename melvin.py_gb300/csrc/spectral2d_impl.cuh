// Fully spectral (doubly periodic) transform kernels.
//
// Layouts (all row-major):
//   spectral state  zd  [rows = 2nn+1][cols = nm]        (reference layout)
//   intermediate    cx<T>[nx][ld = nm]   z-mode columns after an x pass
//   physical        double[nx][nz]
//
// Inverse (to_physical, melvin/SpectralTransformer.py:90-150): an x pass
// (inverse c2c of length nx over the nm kept columns, zero rows in the 2/3
// gap are never stored) then a z pass (c2r of length nz per row, two real
// rows packed into one complex transform).  Forward
// (melvin/SpectralTransformer.py:152-199): a z pass (r2c per row, two rows
// per complex transform, only the nm kept modes leave the CTA) then an x
// pass (c2c over nm columns, only the 2nn+1 kept rows leave the CTA).
// Both directions are unnormalised: the reference multiplies by nx*nz before
// irfft2, which divides by the same factor, and divides the rfft2 result by
// nx*nz (applied at the end of the forward x pass).
//
// The fused timestep (k_xinv -> k_zz_step -> k_xf_step) evaluates the loop
// body of examples/taylor_green_vortex.py:87-93 and its multi-field
// relatives in three HBM round trips.  The finite-difference stencils of
// vec_dot_nabla (melvin/Variable.py:119-128,
// melvin/SpatialDifferentiator.py:76-185) are applied in the pass that holds
// the full periodic line: d/dz of uz*q along each row inside k_zz_step, and
// d/dx of (ux*q)^ along each column inside k_xf_step (the z transform is
// linear and commutes with the x stencil).
#pragma once

#include "fft_block.cuh"
#include "internal.h"

namespace mgb {

// Resident CTAs per SM the compiler must allow for (register budget).  The
// FP32 and double-float kernels are latency bound (global loads, chains of
// dependent FP32 ops), so they ask for three and two 256-thread CTAs per SM;
// the FP64 kernels are bound by the FP64 pipe and keep the default.
template <typename T>
struct MinCTAs {
  static constexpr int value = 1;
};
template <>
struct MinCTAs<float> {
  static constexpr int value = 3;
};
template <>
struct MinCTAs<df64> {
  static constexpr int value = 2;
};

// Columns per CTA of an x pass: 4096 complex values in shared memory
// (64 KB at 16 bytes, 32 KB at 8 bytes, so more FP32 CTAs are resident).
template <typename T, int N>
struct XTile {
  static constexpr int E = 4096;
  static constexpr int C0 = E / N;
  static constexpr int C = C0 < 1 ? 1 : (C0 > 64 ? 64 : C0);
};

// Batched launches: member z of a launch (the last grid dimension) works on
// slot = members ? members[z] : z; the arrays of a slot sit at
// base + slot * stride.  A single simulation is a batch of one with zero
// strides.
struct BatchC {
  const int* members;    // device slot list, or null for slots 0..count-1
  size_t q_stride;       // zd elements between slots of a state array
  size_t h_stride;       // zd elements between slots of a history array
  size_t inter_stride;   // bytes between members' intermediate blocks
  const double* tcoef;   // optional per-slot term coefficients [slot][3][4]
};

__device__ __forceinline__ int batch_slot(const BatchC& b, int z) { return b.members ? b.members[z] : z; }

template <typename T>
__device__ __forceinline__ T nan_max(T m, T v) {
  return (v != v || v > m) ? v : m;
}

// Laplacian symbol d2x*n^2 + d2z*m^2 evaluated without contraction, as
// calc_lap does (melvin/SpatialDifferentiator.py:70-74).
__device__ __forceinline__ double lap_symbol(const GridC& g, int n, int m) {
  return __dadd_rn(__dmul_rn(g.d2x, (double)(n * n)), __dmul_rn(g.d2z, (double)(m * m)));
}

// ---------------------------------------------------------------------------
// x pass, inverse
// ---------------------------------------------------------------------------

struct XinvJob {
  const zd* src;  // spectral state
  int kind;       // SrcKind
  void* out;      // intermediate [nx][ld]
  zd* spec_out;   // optional (FP64 kernels): the derived spectral field (ux_s / uz_s)
  zd* psi_out;    // optional (FP64 kernels): psi = solve(-src)
};

// Per-mode factors of the streamfunction inversion, precomputed per plan
// (lap(0,0) := 1, melvin/LaplacianSolver.py:58-68):
//   tux = (2 pi/lz) m / lap,  tuz = (2 pi/lx) n / lap,  rlap = 1 / lap,
// so that ux = -(2 pi i/lz) m psi = i tux w and uz = (2 pi i/lx) n psi =
// -i tuz w with psi = -w / lap (melvin/utility.py:62-79).
struct XinvArgs {
  GridC g;
  XinvJob job[5];
  int ld;
  const void* tux;     // T[rows*cols]
  const void* tuz;     // T[rows*cols]
  const double* rlap;  // double[rows*cols]
  const void* tw;
  BatchC b;            // member = blockIdx.z
};

template <typename T, int N>
__global__ void __launch_bounds__(NT, MinCTAs<T>::value) k_xinv(const XinvArgs a) {
  constexpr int C = XTile<T, N>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const XinvJob jb = a.job[blockIdx.y];
  const int m0 = blockIdx.x * C;
  const T* tab = (const T*)(jb.kind == SRC_UX ? a.tux : a.tuz);
  const zd* src = jb.src + (size_t)batch_slot(a.b, blockIdx.z) * a.b.q_stride;
  for (int e = threadIdx.x; e < sbuf_elems<C>(N); e += NT) buf[e] = mk<T>(0, 0);
  __syncthreads();
  for (int e = threadIdx.x; e < g.rows * C; e += NT) {
    const int r = e / C, c = e - r * C, m = m0 + c;
    if (m >= g.cols) continue;
    const size_t idx = (size_t)r * g.cols + m;
    const zd w = src[idx];
    const cx<T> wt = cvt<T>(w);
    cx<T> v = wt;
    if (jb.kind == SRC_UX) {
      const T t = tab[idx];
      v = mk(-(t * wt.y), t * wt.x);
    } else if (jb.kind == SRC_UZ) {
      const T t = tab[idx];
      v = mk(t * wt.y, -(t * wt.x));
    }
    if (jb.spec_out) jb.spec_out[idx] = cvt<double>(v);
    if (jb.psi_out) {
      const double rl = a.rlap[idx];
      jb.psi_out[idx] = mk(-(w.x * rl), -(w.y * rl));
    }
    buf[sx<C>(row_bin(r, g.nn, N), c)] = v;
  }
  __syncthreads();
  block_fft<T, N, C, C, NT, +1>(buf, (const cx<T>*)a.tw);
  cx<T>* out = (cx<T>*)((char*)jb.out + (size_t)blockIdx.z * a.b.inter_stride);
  for (int e = threadIdx.x; e < N * C; e += NT) {
    const int x = e / C, c = e - x * C, m = m0 + c;
    if (m < g.cols) out[(size_t)x * a.ld + m] = buf[sx<C>(x, c)];
  }
}

// ---------------------------------------------------------------------------
// z pass helpers: two real rows A, B of half spectra packed as one complex
// transform W = A_h + i B_h (A_h = Hermitian extension; the imaginary part of
// the m = 0 term is dropped, as irfft does).
// ---------------------------------------------------------------------------

template <typename T, int N, int CS>
__device__ __forceinline__ void put_pair(cx<T>* buf, int col, int m, cx<T> A, cx<T> B) {
  if (m == 0) {
    buf[col] = mk(A.x, B.x);
  } else {
    buf[sx<CS>(m, col)] = mk(A.x - B.y, A.y + B.x);
    buf[sx<CS>(N - m, col)] = mk(A.x + B.y, B.x - A.y);
  }
}

// Split the forward transform Z of a + i b into the half spectra of a and b.
template <typename T, int N, int CS>
__device__ __forceinline__ void get_pair(const cx<T>* buf, int col, int m, cx<T>& A, cx<T>& B) {
  const cx<T> zm = buf[sx<CS>(m, col)];
  const cx<T> zn = buf[sx<CS>((N - m) & (N - 1), col)];
  const T h = (T)0.5;
  A = mk((zm.x + zn.x) * h, (zm.y - zn.y) * h);
  B = mk((zm.y + zn.y) * h, (zn.x - zm.x) * h);
}

// Periodic central first difference of the imaginary parts of column `col`
// at position i (melvin/SpatialDifferentiator.py:91-104, 157-185), scaled by
// inv = 1/(2h) (order 2) or 1/(3h) (order 4).
template <typename T, int N, int CS>
__device__ __forceinline__ T fd_imag(const cx<T>* buf, int col, int i, int sdo, T inv) {
  const T p1 = buf[sx<CS>((i + 1) & (N - 1), col)].y;
  const T m1 = buf[sx<CS>((i - 1) & (N - 1), col)].y;
  if (sdo == 2) return (p1 - m1) * inv;
  const T p2 = buf[sx<CS>((i + 2) & (N - 1), col)].y;
  const T m2 = buf[sx<CS>((i - 2) & (N - 1), col)].y;
  return (((T)-0.25 * p2 + (T)2 * p1) - (T)2 * m1 + (T)0.25 * m2) * inv;
}

// Replace the imaginary parts of columns [0, NCOL) by their periodic
// z-derivative (in place, staged through registers).
template <typename T, int N, int CS, int NCOL>
__device__ __forceinline__ void fd_imag_columns(cx<T>* buf, int sdo, T inv) {
  constexpr int EPT = (N + NT - 1) / NT;
#pragma unroll 1
  for (int col = 0; col < NCOL; ++col) {
    T v[EPT];
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const int z = threadIdx.x + i * NT;
      if (z < N) v[i] = fd_imag<T, N, CS>(buf, col, z, sdo, inv);
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < EPT; ++i) {
      const int z = threadIdx.x + i * NT;
      if (z < N) buf[sx<CS>(z, col)].y = v[i];
    }
  }
  __syncthreads();
}

// Deterministic CTA reduction of (sum, max, max) -> partial[blockIdx.x*3].
__device__ __forceinline__ void block_diag(double s, double mx, double mz, double* partial) {
  __shared__ double red[3][NT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    mx = nan_max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    mz = nan_max(mz, __shfl_xor_sync(0xffffffffu, mz, o));
  }
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    red[0][w] = s;
    red[1][w] = mx;
    red[2][w] = mz;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double S = 0, MX = -INFINITY, MZ = -INFINITY;
    for (int i = 0; i < NT / 32; ++i) {
      S += red[0][i];
      MX = nan_max(MX, red[1][i]);
      MZ = nan_max(MZ, red[2][i]);
    }
    partial[3 * blockIdx.x + 0] = S;
    partial[3 * blockIdx.x + 1] = MX;
    partial[3 * blockIdx.x + 2] = MZ;
  }
}

// ---------------------------------------------------------------------------
// Fused z pass of the timestep: for rows x0 = 2*blockIdx.x and x0+1,
//   inverse c2r of ux, uz and the F advected fields,
//   a_f = ux * q_f, b_f = uz * q_f, c_f = d/dz b_f (periodic stencil),
//   forward r2c of a_f + i c_f, keep the nm leading modes.
// Outputs may alias the inputs: a CTA reads only its own two rows, before it
// writes them.
// ---------------------------------------------------------------------------

struct ZzArgs {
  GridC g;
  int ld;
  const void* in[5];  // ux, uz, q_0 .. q_{F-1}
  void* aout[3];
  void* cout[3];
  double* ux_phys;    // optional physical velocity
  double* uz_phys;
  double* partial;    // optional [member][gridDim.x][3]
  double fdz;         // 1/(2dz) or 1/(3dz)
  const void* tw;
  BatchC b;           // member = blockIdx.y
};

template <typename T, int N, int F>
__global__ void __launch_bounds__(NT, MinCTAs<T>::value) k_zz_step(const ZzArgs a) {
  constexpr int NIN = 2 + F, NOUT = 2 * F;
  constexpr int CS = NIN > NOUT ? NIN : NOUT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const int x0 = 2 * blockIdx.x;
  const int nm = g.cols, ld = a.ld;
  const size_t moff = (size_t)blockIdx.y * a.b.inter_stride;
  const size_t r0 = (size_t)x0 * ld, r1 = r0 + ld;
  for (int e = threadIdx.x; e < sbuf_elems<CS>(N); e += NT) buf[e] = mk<T>(0, 0);
  __syncthreads();
  {
    const cx<T>* ux = (const cx<T>*)((const char*)a.in[0] + moff);
    const cx<T>* uz = (const cx<T>*)((const char*)a.in[1] + moff);
    for (int m = threadIdx.x; m < nm; m += NT) {
      put_pair<T, N, CS>(buf, 0, m, ux[r0 + m], uz[r0 + m]);
      put_pair<T, N, CS>(buf, 1, m, ux[r1 + m], uz[r1 + m]);
#pragma unroll
      for (int f = 0; f < F; ++f) {
        const cx<T>* q = (const cx<T>*)((const char*)a.in[2 + f] + moff);
        put_pair<T, N, CS>(buf, 2 + f, m, q[r0 + m], q[r1 + m]);
      }
    }
  }
  __syncthreads();
  block_fft<T, N, NIN, CS, NT, +1>(buf, (const cx<T>*)a.tw);

  double ke = 0.0, mx = -INFINITY, mz = -INFINITY;
  for (int z = threadIdx.x; z < N; z += NT) {
    cx<T> w[NIN];
#pragma unroll
    for (int c = 0; c < NIN; ++c) w[c] = buf[sx<CS>(z, c)];
    const T ux0 = w[0].x, uz0 = w[0].y, ux1 = w[1].x, uz1 = w[1].y;
    if (a.ux_phys) {
      a.ux_phys[(size_t)x0 * N + z] = (double)ux0;
      a.ux_phys[(size_t)(x0 + 1) * N + z] = (double)ux1;
      a.uz_phys[(size_t)x0 * N + z] = (double)uz0;
      a.uz_phys[(size_t)(x0 + 1) * N + z] = (double)uz1;
    }
    if (a.partial) {
      const double dx0 = (double)ux0, dz0 = (double)uz0, dx1 = (double)ux1, dz1 = (double)uz1;
      ke += (dz0 * dz0 + dx0 * dx0) + (dz1 * dz1 + dx1 * dx1);
      mx = nan_max(nan_max(mx, dx0), dx1);
      mz = nan_max(nan_max(mz, dz0), dz1);
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
      const T q0 = w[2 + f].x, q1 = w[2 + f].y;
      buf[sx<CS>(z, f)] = mk(ux0 * q0, uz0 * q0);
      buf[sx<CS>(z, F + f)] = mk(ux1 * q1, uz1 * q1);
    }
  }
  __syncthreads();
  fd_imag_columns<T, N, CS, NOUT>(buf, g.sdo, (T)a.fdz);
  block_fft<T, N, NOUT, CS, NT, -1>(buf, (const cx<T>*)a.tw);
  for (int m = threadIdx.x; m < nm; m += NT) {
#pragma unroll
    for (int f = 0; f < F; ++f) {
      cx<T>* ao = (cx<T>*)((char*)a.aout[f] + moff);
      cx<T>* co = (cx<T>*)((char*)a.cout[f] + moff);
#pragma unroll
      for (int rho = 0; rho < 2; ++rho) {
        cx<T> A, Cc;
        get_pair<T, N, CS>(buf, rho * F + f, m, A, Cc);
        ao[(rho ? r1 : r0) + m] = A;
        co[(rho ? r1 : r0) + m] = Cc;
      }
    }
  }
  if (a.partial) block_diag(ke, mx, mz, a.partial + (size_t)blockIdx.y * gridDim.x * 3);
}

// ---------------------------------------------------------------------------
// Fused x pass of the timestep: J_f = d/dx(A_f) + C_f along each column,
// forward c2c, keep the 2nn+1 rows, N_f = -J_f/(nx*nz) + linear terms,
// history write and the Adams-Bashforth / semi-implicit update
// (melvin/Integrator.py:5-18, 53-63), boundary rules.
// ---------------------------------------------------------------------------

struct XfField {
  int nterms;
  int tsrc[4];
  int top[4];
  double tcoef[4];
  int bc;
};

struct XfArgs {
  GridC g;
  int ld;
  const void* ain[3];
  const void* cin[3];
  zd* q[3];
  zd* hist[3];
  const zd* coef[3];   // per-mode update coefficients (a, b) from mgb_step_prepare
  const double* rlap;  // 1/lap, for linear terms of psi
  int order, curr, integrator, need_psi;
  double fdx, inv_norm;
  XfField eq[3];
  const void* tw;
  BatchC b;            // member = blockIdx.y
};

// J at (x, m): periodic x stencil of A plus C (both intermediates).
template <typename T, int N>
__device__ __forceinline__ cx<T> jac_x(const cx<T>* __restrict__ A, const cx<T>* __restrict__ Cc,
                                      int x, int m, int ld, int sdo, T inv) {
  const cx<T> p1 = A[(size_t)((x + 1) & (N - 1)) * ld + m];
  const cx<T> m1 = A[(size_t)((x - 1) & (N - 1)) * ld + m];
  cx<T> d;
  if (sdo == 2) {
    d = (p1 - m1) * inv;
  } else {
    const cx<T> p2 = A[(size_t)((x + 2) & (N - 1)) * ld + m];
    const cx<T> m2 = A[(size_t)((x - 2) & (N - 1)) * ld + m];
    d = (((p2 * (T)-0.25 + p1 * (T)2) - m1 * (T)2) + m2 * (T)0.25) * inv;
  }
  return d + Cc[(size_t)x * ld + m];
}

// Linear term op(src) for the point (n, m): 0 value, 1 d/dx, 2 d/dz.
__device__ __forceinline__ zd lin_term(const GridC& g, zd s, int op, int n, int m) {
  if (op == 1) {
    const double b = g.dfx * (double)n;
    return mk(-(b * s.y), b * s.x);
  }
  if (op == 2) {
    const double b = g.dfz * (double)m;
    return mk(-(b * s.y), b * s.x);
  }
  return s;
}

// Weighted Adams-Bashforth sum 3 f0 - f1 (AB2) or
// 55 f0 - 59 f1 + 37 f2 - 9 f3 (AB4) (melvin/Integrator.py:5-18); the dt/2
// or dt/24 factor is part of the update coefficients.
__device__ __forceinline__ zd ab_sum(const zd* h, size_t slot, int order, int curr, zd f0) {
  if (order == 2) {
    const zd f1 = h[(size_t)((curr + 1) & 1) * slot];
    return mk(3 * f0.x - f1.x, 3 * f0.y - f1.y);
  }
  const zd f1 = h[(size_t)((curr + 3) & 3) * slot];
  const zd f2 = h[(size_t)((curr + 2) & 3) * slot];
  const zd f3 = h[(size_t)((curr + 1) & 3) * slot];
  return mk(((55 * f0.x - 59 * f1.x) + 37 * f2.x) - 9 * f3.x, ((55 * f0.y - 59 * f1.y) + 37 * f2.y) - 9 * f3.y);
}

template <typename T, int N, int F>
__global__ void __launch_bounds__(NT, MinCTAs<T>::value) k_xf_step(const XfArgs a) {
  constexpr int C = XTile<T, N>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const int m0 = blockIdx.x * C;
  const int sdo = g.sdo;
  const size_t moff = (size_t)blockIdx.y * a.b.inter_stride;
  const int mslot = batch_slot(a.b, blockIdx.y);
#pragma unroll
  for (int f = 0; f < F; ++f) {
    const cx<T>* A = (const cx<T>*)((const char*)a.ain[f] + moff);
    const cx<T>* Cc = (const cx<T>*)((const char*)a.cin[f] + moff);
    cx<T>* bf = buf + f * sbuf_elems<C>(N);
    for (int e = threadIdx.x; e < N * C; e += NT) {
      const int x = e / C, c = e - x * C, m = m0 + c;
      bf[sx<C>(x, c)] = (m < g.cols) ? jac_x<T, N>(A, Cc, x, m, a.ld, sdo, (T)a.fdx) : mk<T>(0, 0);
    }
  }
  __syncthreads();
#pragma unroll
  for (int f = 0; f < F; ++f) block_fft<T, N, C, C, NT, -1>(buf + f * sbuf_elems<C>(N), (const cx<T>*)a.tw);

  // -1/(nx*nz) is a power of two for the grids built, so scaling in T is exact
  const T neg_norm = (T)(-a.inv_norm);
  const size_t slot = (size_t)g.rows * g.cols;
  zd* qf[F];
  zd* hf[F];
#pragma unroll
  for (int f = 0; f < F; ++f) {
    qf[f] = a.q[f] + (size_t)mslot * a.b.q_stride;
    hf[f] = a.hist[f] + (size_t)mslot * a.b.h_stride;
  }
  const double* tco = a.b.tcoef ? a.b.tcoef + (size_t)mslot * 12 : nullptr;
  for (int e = threadIdx.x; e < g.rows * C; e += NT) {
    const int r = e / C, c = e - r * C, m = m0 + c;
    if (m >= g.cols) continue;
    const int n = row_mode(r, g.nn), k = row_bin(r, g.nn, N);
    const size_t idx = (size_t)r * g.cols + m;
    zd qo[F];
#pragma unroll
    for (int f = 0; f < F; ++f) qo[f] = qf[f][idx];
    zd psi = mk(0.0, 0.0);
    if (a.need_psi) {
      const double rl = a.rlap[idx];
      psi = mk(-(qo[0].x * rl), -(qo[0].y * rl));
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
      const XfField& eq = a.eq[f];
      // dq[:] = -q.vec_dot_nabla(...) + linear terms
      const cx<T> J = buf[f * sbuf_elems<C>(N) + sx<C>(k, c)] * neg_norm;
      zd fv = cvt<double>(J);
      for (int t = 0; t < eq.nterms; ++t) {
        const int sidx = eq.tsrc[t];
        zd s = psi;
#pragma unroll
        for (int q2 = 0; q2 < F; ++q2)
          if (sidx == q2) s = qo[q2];
        const zd v = lin_term(g, s, eq.top[t], n, m);
        const double cc = tco ? tco[f * 4 + t] : eq.tcoef[t];
        fv = mk(fv.x + cc * v.x, fv.y + cc * v.y);
      }
      const zd cf = a.coef[f][idx];
      zd qn;
      if (a.integrator == MGB_INT_SEMI_IMPLICIT) {
        // q' = ((1 + (1-a) dt L) q + AB) / (1 - a dt L) = cf.x q + cf.y * sum
        hf[f][(size_t)a.curr * slot + idx] = fv;
        const zd sm = ab_sum(hf[f] + idx, slot, a.order, a.curr, fv);
        qn = mk(cf.x * qo[f].x + cf.y * sm.x, cf.x * qo[f].y + cf.y * sm.y);
      } else {
        // explicit: the history keeps N + D, D = kappa * snabla2(q) = cf.x q
        fv = mk(fv.x + cf.x * qo[f].x, fv.y + cf.x * qo[f].y);
        hf[f][(size_t)a.curr * slot + idx] = fv;
        const zd sm = ab_sum(hf[f] + idx, slot, a.order, a.curr, fv);
        qn = mk(qo[f].x + cf.y * sm.x, qo[f].y + cf.y * sm.y);
      }
      if ((eq.bc & MGB_BC_ZERO_M0) && m == 0) qn = mk(0.0, 0.0);
      qf[f][idx] = qn;
    }
  }
}

// ---------------------------------------------------------------------------
// Per-verb kernels (FP64): z passes to / from physical rows and an x pass to
// a spectral output.
// ---------------------------------------------------------------------------

struct ZinvArgs {
  GridC g;
  int ld;
  const void* in[2];
  double* out[2];
  const void* tw;
};

template <typename T, int N, int NF>
__global__ void __launch_bounds__(NT) k_zinv_phys(const ZinvArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const int x0 = 2 * blockIdx.x;
  const size_t r0 = (size_t)x0 * a.ld, r1 = r0 + a.ld;
  for (int e = threadIdx.x; e < sbuf_elems<NF>(N); e += NT) buf[e] = mk<T>(0, 0);
  __syncthreads();
  for (int m = threadIdx.x; m < a.g.cols; m += NT) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const cx<T>* q = (const cx<T>*)a.in[f];
      put_pair<T, N, NF>(buf, f, m, q[r0 + m], q[r1 + m]);
    }
  }
  __syncthreads();
  block_fft<T, N, NF, NF, NT, +1>(buf, (const cx<T>*)a.tw);
  for (int z = threadIdx.x; z < N; z += NT) {
#pragma unroll
    for (int f = 0; f < NF; ++f) {
      const cx<T> w = buf[sx<NF>(z, f)];
      a.out[f][(size_t)x0 * N + z] = (double)w.x;
      a.out[f][(size_t)(x0 + 1) * N + z] = (double)w.y;
    }
  }
}

struct ZfwdArgs {
  GridC g;
  int ld;
  const double* in;
  void* out;
  const void* tw;
};

template <typename T, int N>
__global__ void __launch_bounds__(NT) k_zfwd_phys(const ZfwdArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const int x0 = 2 * blockIdx.x;
  for (int z = threadIdx.x; z < N; z += NT)
    buf[sx<1>(z, 0)] = mk((T)a.in[(size_t)x0 * N + z], (T)a.in[(size_t)(x0 + 1) * N + z]);
  __syncthreads();
  block_fft<T, N, 1, 1, NT, -1>(buf, (const cx<T>*)a.tw);
  cx<T>* out = (cx<T>*)a.out;
  for (int m = threadIdx.x; m < a.g.cols; m += NT) {
    cx<T> A, B;
    get_pair<T, N, 1>(buf, 0, m, A, B);
    out[(size_t)x0 * a.ld + m] = A;
    out[(size_t)(x0 + 1) * a.ld + m] = B;
  }
}

struct ZvdnArgs {
  GridC g;
  int ld;
  const void* qin;
  double* qphys;
  const double* ux;
  const double* uz;
  void* aout;  // may alias qin
  void* cout;
  double fdz;
  const void* tw;
};

// z pass of vec_dot_nabla: q to physical (written out), a = ux*q,
// c = d/dz(uz*q), forward r2c of a + i c.
template <typename T, int N>
__global__ void __launch_bounds__(NT) k_zz_vdn(const ZvdnArgs a) {
  constexpr int CS = 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const int x0 = 2 * blockIdx.x;
  const size_t r0 = (size_t)x0 * a.ld, r1 = r0 + a.ld;
  for (int e = threadIdx.x; e < sbuf_elems<CS>(N); e += NT) buf[e] = mk<T>(0, 0);
  __syncthreads();
  const cx<T>* q = (const cx<T>*)a.qin;
  for (int m = threadIdx.x; m < a.g.cols; m += NT) put_pair<T, N, CS>(buf, 0, m, q[r0 + m], q[r1 + m]);
  __syncthreads();
  block_fft<T, N, 1, CS, NT, +1>(buf, (const cx<T>*)a.tw);
  const size_t p0 = (size_t)x0 * N, p1 = p0 + N;
  for (int z = threadIdx.x; z < N; z += NT) {
    const cx<T> w = buf[sx<CS>(z, 0)];
    const double q0 = (double)w.x, q1 = (double)w.y;
    a.qphys[p0 + z] = q0;
    a.qphys[p1 + z] = q1;
    buf[sx<CS>(z, 0)] = mk((T)(a.ux[p0 + z] * q0), (T)(a.uz[p0 + z] * q0));
    buf[sx<CS>(z, 1)] = mk((T)(a.ux[p1 + z] * q1), (T)(a.uz[p1 + z] * q1));
  }
  __syncthreads();
  fd_imag_columns<T, N, CS, 2>(buf, a.g.sdo, (T)a.fdz);
  block_fft<T, N, 2, CS, NT, -1>(buf, (const cx<T>*)a.tw);
  cx<T>* ao = (cx<T>*)a.aout;
  cx<T>* co = (cx<T>*)a.cout;
  for (int m = threadIdx.x; m < a.g.cols; m += NT) {
    cx<T> A, Cc;
    get_pair<T, N, CS>(buf, 0, m, A, Cc);
    ao[r0 + m] = A;
    co[r0 + m] = Cc;
    get_pair<T, N, CS>(buf, 1, m, A, Cc);
    ao[r1 + m] = A;
    co[r1 + m] = Cc;
  }
}

struct XfOutArgs {
  GridC g;
  int ld;
  const void* ain;
  const void* cin;  // null: J = A; otherwise J = d/dx A + C
  zd* out;
  double scale;
  double fdx;
  const void* tw;
};

template <typename T, int N>
__global__ void __launch_bounds__(NT) k_xf_out(const XfOutArgs a) {
  constexpr int C = XTile<T, N>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* buf = reinterpret_cast<cx<T>*>(smem_raw);
  const GridC& g = a.g;
  const int m0 = blockIdx.x * C;
  const cx<T>* A = (const cx<T>*)a.ain;
  const cx<T>* Cc = (const cx<T>*)a.cin;
  for (int e = threadIdx.x; e < N * C; e += NT) {
    const int x = e / C, c = e - x * C, m = m0 + c;
    cx<T> v = mk<T>(0, 0);
    if (m < g.cols) v = Cc ? jac_x<T, N>(A, Cc, x, m, a.ld, g.sdo, (T)a.fdx) : A[(size_t)x * a.ld + m];
    buf[sx<C>(x, c)] = v;
  }
  __syncthreads();
  block_fft<T, N, C, C, NT, -1>(buf, (const cx<T>*)a.tw);
  for (int e = threadIdx.x; e < g.rows * C; e += NT) {
    const int r = e / C, c = e - r * C, m = m0 + c;
    if (m >= g.cols) continue;
    const cx<T> v = buf[sx<C>(row_bin(r, g.nn, N), c)];
    a.out[(size_t)r * g.cols + m] = mk((double)v.x * a.scale, (double)v.y * a.scale);
  }
}

// ---------------------------------------------------------------------------
// Launchers (one instantiation set per transform length N).
// ---------------------------------------------------------------------------

// Opt in to more than the default 48 KB of shared memory per CTA, once per
// kernel and device (the first launch sets the attribute, so later launches,
// including those inside a stream capture, make no attribute call).  Kernels
// here use at most 1 KB of static shared memory, so any dynamic request above
// 47 KB opts in; the attribute is set to the largest size any launch needs.
bool smem_optin_done(const void* kernel, int device, size_t smem);
void smem_optin_record(const void* kernel, int device, size_t smem);

template <typename K>
inline cudaError_t prep_smem(K kernel, size_t smem) {
  if (smem <= 47 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (smem_optin_done((const void*)kernel, dev, smem)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) smem_optin_record((const void*)kernel, dev, smem);
  return e;
}

template <typename T, int N>
cudaError_t launch_xinv(const XinvArgs& a, int njobs, int nb, cudaStream_t s) {
  constexpr int C = XTile<T, N>::C;
  const size_t smem = (size_t)sbuf_elems<C>(N) * sizeof(cx<T>);
  cudaError_t e = prep_smem(k_xinv<T, N>, smem);
  if (e != cudaSuccess) return e;
  dim3 grid((a.g.cols + C - 1) / C, njobs, nb);
  k_xinv<T, N><<<grid, NT, smem, s>>>(a);
  return cudaGetLastError();
}

// Largest dynamic shared memory a CTA may request (227 KB minus the static
// reduction scratch).
constexpr size_t kMaxDynSmem = 232448 - 1024;

template <typename T, int N, int F>
cudaError_t launch_zz_step(const ZzArgs& a, int nb, cudaStream_t s) {
  constexpr int CS = (2 + F) > (2 * F) ? (2 + F) : (2 * F);
  constexpr size_t smem = (size_t)sbuf_elems<CS>(N) * sizeof(cx<T>);
  if constexpr (smem > kMaxDynSmem) {
    return cudaErrorInvalidConfiguration;
  } else {
    cudaError_t e = prep_smem(k_zz_step<T, N, F>, smem);
    if (e != cudaSuccess) return e;
    k_zz_step<T, N, F><<<dim3(a.g.nx / 2, nb), NT, smem, s>>>(a);
    return cudaGetLastError();
  }
}

template <typename T, int N, int F>
cudaError_t launch_xf_step(const XfArgs& a, int nb, cudaStream_t s) {
  constexpr int C = XTile<T, N>::C;
  constexpr size_t smem = (size_t)F * sbuf_elems<C>(N) * sizeof(cx<T>);
  if constexpr (smem > kMaxDynSmem) {
    return cudaErrorInvalidConfiguration;
  } else {
    cudaError_t e = prep_smem(k_xf_step<T, N, F>, smem);
    if (e != cudaSuccess) return e;
    k_xf_step<T, N, F><<<dim3((a.g.cols + C - 1) / C, nb), NT, smem, s>>>(a);
    return cudaGetLastError();
  }
}

template <int N, int NF>
cudaError_t launch_zinv_phys(const ZinvArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)sbuf_elems<NF>(N) * sizeof(zd);
  cudaError_t e = prep_smem(k_zinv_phys<double, N, NF>, smem);
  if (e != cudaSuccess) return e;
  k_zinv_phys<double, N, NF><<<a.g.nx / 2, NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_zfwd_phys(const ZfwdArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)sbuf_elems<1>(N) * sizeof(zd);
  cudaError_t e = prep_smem(k_zfwd_phys<double, N>, smem);
  if (e != cudaSuccess) return e;
  k_zfwd_phys<double, N><<<a.g.nx / 2, NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_zz_vdn(const ZvdnArgs& a, cudaStream_t s) {
  const size_t smem = (size_t)sbuf_elems<2>(N) * sizeof(zd);
  cudaError_t e = prep_smem(k_zz_vdn<double, N>, smem);
  if (e != cudaSuccess) return e;
  k_zz_vdn<double, N><<<a.g.nx / 2, NT, smem, s>>>(a);
  return cudaGetLastError();
}

template <int N>
cudaError_t launch_xf_out(const XfOutArgs& a, cudaStream_t s) {
  constexpr int C = XTile<double, N>::C;
  const size_t smem = (size_t)sbuf_elems<C>(N) * sizeof(zd);
  cudaError_t e = prep_smem(k_xf_out<double, N>, smem);
  if (e != cudaSuccess) return e;
  k_xf_out<double, N><<<(a.g.cols + C - 1) / C, NT, smem, s>>>(a);
  return cudaGetLastError();
}

// Table of launchers for one length N, filled by the per-N translation units.
struct FsLaunchers {
  cudaError_t (*xinv[3])(const XinvArgs&, int, int, cudaStream_t);  // [precision](args, jobs, members)
  cudaError_t (*zz_step[3][3])(const ZzArgs&, int, cudaStream_t);    // [precision][F-1](args, members)
  cudaError_t (*xf_step[3][3])(const XfArgs&, int, cudaStream_t);
  cudaError_t (*zinv_phys[2])(const ZinvArgs&, cudaStream_t);        // [NF-1]
  cudaError_t (*zfwd_phys)(const ZfwdArgs&, cudaStream_t);
  cudaError_t (*zz_vdn)(const ZvdnArgs&, cudaStream_t);
  cudaError_t (*xf_out)(const XfOutArgs&, cudaStream_t);
};

template <int N>
FsLaunchers make_fs_launchers() {
  FsLaunchers L;
  L.xinv[0] = launch_xinv<double, N>;
  L.xinv[1] = launch_xinv<float, N>;
  L.xinv[2] = launch_xinv<df64, N>;
  L.zz_step[0][0] = launch_zz_step<double, N, 1>;
  L.zz_step[0][1] = launch_zz_step<double, N, 2>;
  L.zz_step[0][2] = launch_zz_step<double, N, 3>;
  L.zz_step[1][0] = launch_zz_step<float, N, 1>;
  L.zz_step[1][1] = launch_zz_step<float, N, 2>;
  L.zz_step[1][2] = launch_zz_step<float, N, 3>;
  L.zz_step[2][0] = launch_zz_step<df64, N, 1>;
  L.zz_step[2][1] = launch_zz_step<df64, N, 2>;
  L.zz_step[2][2] = launch_zz_step<df64, N, 3>;
  L.xf_step[0][0] = launch_xf_step<double, N, 1>;
  L.xf_step[0][1] = launch_xf_step<double, N, 2>;
  L.xf_step[0][2] = launch_xf_step<double, N, 3>;
  L.xf_step[1][0] = launch_xf_step<float, N, 1>;
  L.xf_step[1][1] = launch_xf_step<float, N, 2>;
  L.xf_step[1][2] = launch_xf_step<float, N, 3>;
  L.xf_step[2][0] = launch_xf_step<df64, N, 1>;
  L.xf_step[2][1] = launch_xf_step<df64, N, 2>;
  L.xf_step[2][2] = launch_xf_step<df64, N, 3>;
  L.zinv_phys[0] = launch_zinv_phys<N, 1>;
  L.zinv_phys[1] = launch_zinv_phys<N, 2>;
  L.zfwd_phys = launch_zfwd_phys<N>;
  L.zz_vdn = launch_zz_vdn<N>;
  L.xf_out = launch_xf_out<N>;
  return L;
}

// Defined by fs_n<N>.cu; returns nullptr for lengths that are not built.
const FsLaunchers* fs_launchers(int N);

}  // namespace mgb
