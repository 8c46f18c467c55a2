// Fully spectral transforms with cosine and sine bases
// (melvin/SpectralTransformer.py:90-199 with BasisFunctions.COSINE / SINE).
//
// The reference treats a cosine or sine axis of n points as a periodic
// signal of L = 2(n-1) points: to_spectral mirrors the physical data
// (even for cosine, odd for sine: x[j] for j < n-1, s*x[L-j] for j >= n-1)
// and takes rfft2 / (x_factor * z_factor); to_physical takes irfft2 of the
// kept modes times x_factor * z_factor and keeps the first n points.  The
// factors are n (complex exponential), n-1 (cosine) and -i(n-1) (sine); a
// cosine axis also doubles (to_physical) or halves (to_spectral) its zeroth
// mode.  With the unnormalised transforms here, to_physical multiplies by
// x_factor * z_factor / (Lx * Lz): 1, 1/2 or -i/2 per axis, exact; to_spectral
// multiplies by the rounded reciprocal of x_factor * z_factor.
//
// The kernels reuse the block FFT: a length-L transform for each axis when
// L is a power of two (n = 2^k + 1 on a mirrored axis); other lengths in
// [16, 4096] take the Bluestein twins of these kernels (bluestein.cu).
// FP64 only (per-verb transforms).
#include "mirror.cuh"

namespace mgb {

namespace {

// to_physical, x pass: spectral column m -> length-Lx inverse transform ->
// first nxp rows of the intermediate.
template <int L>
__global__ void __launch_bounds__(NT) k_mx_inv(const MirrorArgs a) {
  constexpr int C = MTile<L>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* buf = reinterpret_cast<zd*>(smem_raw);
  const GridC& g = a.g;
  const int m0 = blockIdx.x * C;
  for (int e = threadIdx.x; e < sbuf_elems<double, C>(L); e += NT) buf[e] = mk(0.0, 0.0);
  __syncthreads();
  for (int e = threadIdx.x; e < g.rows * C; e += NT) {
    const int r = e / C, c = e - r * C, m = m0 + c;
    zd v = mk(0.0, 0.0);
    if (m < g.cols) {
      v = cmuld(a.spec_in[(size_t)r * g.cols + m], a.scale);
      // a cosine axis doubles its zeroth mode (melvin/SpectralTransformer.py:122-125)
      if (a.bx == 1 && r == 0) v = mk(2 * v.x, 2 * v.y);
      if (a.bz == 1 && m == 0) v = mk(2 * v.x, 2 * v.y);
    }
    buf[sx<double, C>(mbin(r, g.nn, L), c)] = v;
  }
  __syncthreads();
  block_fft<double, L, C, C, NT, +1>(buf, (const zd*)a.twx);
  for (int e = threadIdx.x; e < a.nxp * C; e += NT) {
    const int x = e / C, c = e - x * C, m = m0 + c;
    if (m < g.cols) a.inter[(size_t)x * g.cols + m] = buf[sx<double, C>(x, c)];
  }
}

// to_physical, z pass: two intermediate rows -> length-Lz c2r -> first nzp
// points (the second row of an odd last pair is zero and not written).
template <int L>
__global__ void __launch_bounds__(NT) k_mz_inv(const MirrorArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* buf = reinterpret_cast<zd*>(smem_raw);
  const GridC& g = a.g;
  const int x0 = 2 * blockIdx.x;
  const bool two = x0 + 1 < a.nxp;
  for (int e = threadIdx.x; e < sbuf_elems<double, 1>(L); e += NT) buf[e] = mk(0.0, 0.0);
  __syncthreads();
  for (int m = threadIdx.x; m < g.cols; m += NT) {
    const zd A = a.inter[(size_t)x0 * g.cols + m];
    const zd B = two ? a.inter[(size_t)(x0 + 1) * g.cols + m] : mk(0.0, 0.0);
    put_pair<double, L, 1>(buf, 0, m, A, B);
  }
  __syncthreads();
  block_fft<double, L, 1, 1, NT, +1>(buf, (const zd*)a.twz);
  for (int z = threadIdx.x; z < a.nzp; z += NT) {
    const zd w = buf[sx<double, 1>(z, 0)];
    a.phys_out[(size_t)x0 * a.nzp + z] = w.x;
    if (two) a.phys_out[(size_t)(x0 + 1) * a.nzp + z] = w.y;
  }
}

// to_spectral, z pass: two physical rows -> extension -> length-Lz r2c ->
// the nm kept modes of each row into the intermediate.
template <int L>
__global__ void __launch_bounds__(NT) k_mz_fwd(const MirrorArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* buf = reinterpret_cast<zd*>(smem_raw);
  const GridC& g = a.g;
  const int x0 = 2 * blockIdx.x;
  const bool two = x0 + 1 < a.nxp;
  for (int j = threadIdx.x; j < L; j += NT) {
    double s;
    const int z = mirror_src(j, a.nzp, L, a.bz, s);
    const double u = a.phys_in[(size_t)x0 * a.nzp + z];
    const double v = two ? a.phys_in[(size_t)(x0 + 1) * a.nzp + z] : 0.0;
    buf[sx<double, 1>(j, 0)] = mk(s * u, s * v);
  }
  __syncthreads();
  block_fft<double, L, 1, 1, NT, -1>(buf, (const zd*)a.twz);
  for (int m = threadIdx.x; m < g.cols; m += NT) {
    zd A, B;
    get_pair<double, L, 1>(buf, 0, m, A, B);
    a.inter[(size_t)x0 * g.cols + m] = A;
    if (two) a.inter[(size_t)(x0 + 1) * g.cols + m] = B;
  }
}

// to_spectral, x pass: intermediate column m (nxp rows) -> extension ->
// length-Lx forward transform -> the 2nn+1 kept rows, scaled.
template <int L>
__global__ void __launch_bounds__(NT) k_mx_fwd(const MirrorArgs a) {
  constexpr int C = MTile<L>::C;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  zd* buf = reinterpret_cast<zd*>(smem_raw);
  const GridC& g = a.g;
  const int m0 = blockIdx.x * C;
  for (int e = threadIdx.x; e < L * C; e += NT) {
    const int j = e / C, c = e - j * C, m = m0 + c;
    zd v = mk(0.0, 0.0);
    if (m < g.cols) {
      double s;
      const int x = mirror_src(j, a.nxp, L, a.bx, s);
      const zd w = a.inter[(size_t)x * g.cols + m];
      v = mk(s * w.x, s * w.y);
    }
    buf[sx<double, C>(j, c)] = v;
  }
  __syncthreads();
  block_fft<double, L, C, C, NT, -1>(buf, (const zd*)a.twx);
  for (int e = threadIdx.x; e < g.rows * C; e += NT) {
    const int r = e / C, c = e - r * C, m = m0 + c;
    if (m >= g.cols) continue;
    zd v = cmuld(buf[sx<double, C>(mbin(r, g.nn, L), c)], a.scale);
    if (a.bx == 1 && r == 0) v = mk(0.5 * v.x, 0.5 * v.y);
    if (a.bz == 1 && m == 0) v = mk(0.5 * v.x, 0.5 * v.y);
    a.spec_out[(size_t)r * g.cols + m] = v;
  }
}

template <int L>
cudaError_t launch_m(int which, const MirrorArgs& a, cudaStream_t s) {
  constexpr int C = MTile<L>::C;
  const size_t sx_smem = (size_t)sbuf_elems<double, C>(L) * sizeof(zd);
  const size_t sz_smem = (size_t)sbuf_elems<double, 1>(L) * sizeof(zd);
  cudaError_t e = cudaSuccess;
  switch (which) {
    case 0:
      e = prep_smem(k_mx_inv<L>, sx_smem);
      if (e == cudaSuccess) k_mx_inv<L><<<(a.g.cols + C - 1) / C, NT, sx_smem, s>>>(a);
      break;
    case 1:
      e = prep_smem(k_mz_inv<L>, sz_smem);
      if (e == cudaSuccess) k_mz_inv<L><<<(a.nxp + 1) / 2, NT, sz_smem, s>>>(a);
      break;
    case 2:
      e = prep_smem(k_mz_fwd<L>, sz_smem);
      if (e == cudaSuccess) k_mz_fwd<L><<<(a.nxp + 1) / 2, NT, sz_smem, s>>>(a);
      break;
    default:
      e = prep_smem(k_mx_fwd<L>, sx_smem);
      if (e == cudaSuccess) k_mx_fwd<L><<<(a.g.cols + C - 1) / C, NT, sx_smem, s>>>(a);
      break;
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t launch_mirror(int L, int which, const MirrorArgs& a, cudaStream_t s) {
  switch (L) {
    case 16: return launch_m<16>(which, a, s);
    case 32: return launch_m<32>(which, a, s);
    case 64: return launch_m<64>(which, a, s);
    case 128: return launch_m<128>(which, a, s);
    case 256: return launch_m<256>(which, a, s);
    case 512: return launch_m<512>(which, a, s);
    case 1024: return launch_m<1024>(which, a, s);
    case 2048: return launch_m<2048>(which, a, s);
    case 4096: return launch_m<4096>(which, a, s);
    default: return cudaErrorInvalidValue;
  }
}

// x_factor * z_factor of the reference: n, n-1 or -i(n-1) per axis.
zd axis_factor(int basis, int n) {
  if (basis == 0) return mk((double)n, 0.0);
  if (basis == 1) return mk((double)(n - 1), 0.0);
  return mk(0.0, -(double)(n - 1));
}

zd cmul_host(zd a, zd b) { return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

int launched(cudaError_t e, const char* what) { return e == cudaSuccess ? MGB_OK : cuda_check(e, what); }

}  // namespace

int basis_length(int basis, int n) { return basis == 0 ? n : 2 * (n - 1); }

static bool pow2_len(int n) { return n >= 16 && n <= 4096 && (n & (n - 1)) == 0; }
static bool any_len(int n) { return n >= 16 && n <= 4096; }

// One pass of a basis transform: the power-of-two kernel, or its Bluestein
// twin for another length.
static int mirror_pass(const mgb_plan* p, int L, int which, const MirrorArgs& a, cudaStream_t s, const char* what) {
  if (pow2_len(L)) return launched(launch_mirror(L, which, a, s), what);
  BlueTables b;
  if (int st = bluestein_tables(p, L, b)) return st;
  return launched(launch_bluestein(which, a, b, s), what);
}

static int mirror_args(const mgb_plan* p, int bx, int bz, MirrorArgs& a, const char* fn) {
  const GridC& g = p->g;
  if (g.fdm) return fail(MGB_ERR_UNSUPPORTED, "%s: cosine and sine bases need a fully spectral grid", fn);
  if (bx < 0 || bx > 2 || bz < 0 || bz > 2) return fail(MGB_ERR_INVALID, "%s: basis (%d, %d)", fn, bx, bz);
  a = MirrorArgs{};
  a.g = g;
  a.nxp = g.nx;
  a.nzp = g.nz;
  a.lx = basis_length(bx, g.nx);
  a.lz = basis_length(bz, g.nz);
  a.bx = bx;
  a.bz = bz;
  if (!any_len(a.lx) || !any_len(a.lz))
    return fail(MGB_ERR_UNSUPPORTED,
                "%s: transform lengths %d x %d (the basis needs 2(n-1) for cosine/sine and n for complex "
                "exponentials in [16, 4096])", fn, a.lx, a.lz);
  a.twx = pow2_len(a.lx) ? mirror_twiddles(p, a.lx) : nullptr;
  a.twz = pow2_len(a.lz) ? mirror_twiddles(p, a.lz) : nullptr;
  if ((pow2_len(a.lx) && !a.twx) || (pow2_len(a.lz) && !a.twz))
    return fail(MGB_ERR_CUDA, "%s: twiddle tables for lengths %d, %d", fn, a.lx, a.lz);
  return MGB_OK;
}

int mirror_to_physical(const mgb_plan* p, int bx, int bz, const zd* spec, double* phys, void* work, cudaStream_t s) {
  MirrorArgs a;
  if (int st = mirror_args(p, bx, bz, a, "mgb_to_physical_basis")) return st;
  // x_factor * z_factor / (Lx * Lz): 1, 1/2 or -i/2 per axis (exact)
  const zd fx = bx == 0 ? mk(1.0, 0.0) : (bx == 1 ? mk(0.5, 0.0) : mk(0.0, -0.5));
  const zd fz = bz == 0 ? mk(1.0, 0.0) : (bz == 1 ? mk(0.5, 0.0) : mk(0.0, -0.5));
  a.scale = cmul_host(fx, fz);
  a.spec_in = spec;
  a.phys_out = phys;
  a.inter = (zd*)work;
  int st = mirror_pass(p, a.lx, 0, a, s, "basis to_physical x pass");
  if (st) return st;
  return mirror_pass(p, a.lz, 1, a, s, "basis to_physical z pass");
}

int mirror_to_spectral(const mgb_plan* p, int bx, int bz, const double* phys, zd* spec, void* work, cudaStream_t s) {
  MirrorArgs a;
  if (int st = mirror_args(p, bx, bz, a, "mgb_to_spectral_basis")) return st;
  const zd f = cmul_host(axis_factor(bx, p->g.nx), axis_factor(bz, p->g.nz));
  // 1 / f for f = r or f = -i r or f = -r (products of n, n-1 and -i(n-1))
  const double r = f.x != 0.0 ? f.x : f.y;
  const double inv = 1.0 / r;
  a.scale = f.x != 0.0 ? mk(inv, 0.0) : mk(0.0, -inv);
  a.phys_in = phys;
  a.spec_out = spec;
  a.inter = (zd*)work;
  int st = mirror_pass(p, a.lz, 2, a, s, "basis to_spectral z pass");
  if (st) return st;
  return mirror_pass(p, a.lx, 3, a, s, "basis to_spectral x pass");
}

}  // namespace mgb
