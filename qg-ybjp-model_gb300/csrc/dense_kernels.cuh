// Kernels behind the routine-level drop-ins (fft_r2c, fft_c2r, convol_waqg,
// refraction_waqg, compute_qw): unpruned 2D transforms on the reference's
// dense half-spectrum layout, so arbitrary (also unmasked) inputs give what
// the Fortran routines give.
#pragma once
#include "step_kernels.cuh"

namespace qg {

// dense spectral: double2 [nz][n][iktx]; W: cplx<T> [nz][n(y)][iktxP]; phys: T [nz][n][n]

template <typename T, int N>
__global__ void __launch_bounds__(kThreads)
k_dcol_inv(int iktxP, const double2* __restrict__ in, cplx<T>* __restrict__ W, const cplx<T>* __restrict__ twg) {
  constexpr int CT = Tile<T>::CT, LD = N + 1, IKTX = N / 2 + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bufA = tw + N;
  cplx<T>* bufB = bufA + CT * LD;
  const int z = blockIdx.y, kx0 = blockIdx.x * CT;
  load_twiddles<T, N>(tw, twg);
  for (int idx = threadIdx.x; idx < CT * N; idx += blockDim.x) {
    const int c = idx % CT, j = idx / CT, kx = kx0 + c;
    cplx<T> v = mk<T>(0, 0);
    if (kx < IKTX) { const double2 d = in[((long long)z * N + j) * IKTX + kx]; v = mk<T>((T)d.x, (T)d.y); }
    bufA[c * LD + j] = v;
  }
  __syncthreads();
  if (kx0 == 0) realit_col<T>(bufA, N);
  __syncthreads();
  cplx<T>* res = block_fft<T, N, false>(bufA, bufB, LD, CT, tw);
  for (int idx = threadIdx.x; idx < CT * N; idx += blockDim.x) {
    const int c = idx % CT, y = idx / CT;
    W[((long long)z * N + y) * iktxP + kx0 + c] = res[c * LD + y];
  }
}

// Hermitian extension of two half spectra with kx in [0, n/2] (the Nyquist
// entry, like kx=0, contributes its real part only, as FFTW's c2r does).
template <typename T>
__device__ __forceinline__ cplx<T> pack_full(const cplx<T>* X, const cplx<T>* Y, int k, int n) {
  if (k == 0 || k == n / 2) return mk<T>(X[k].x, Y[k].x);
  if (k < n / 2) { cplx<T> a = X[k], b = Y[k]; return mk<T>(a.x - b.y, a.y + b.x); }
  const int kk = n - k; cplx<T> a = X[kk], b = Y[kk]; return mk<T>(a.x + b.y, b.x - a.y);
}

template <typename T, int N>
__global__ void __launch_bounds__(kThreads)
k_drow_c2r(int iktxP, const cplx<T>* __restrict__ W, T* __restrict__ phys, const cplx<T>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bA = tw + N;
  cplx<T>* bB = bA + N;
  const int z = blockIdx.y, y0 = 2 * blockIdx.x;
  load_twiddles<T, N>(tw, twg);
  const cplx<T>* X = W + ((long long)z * N + y0) * iktxP;
  const cplx<T>* Y = X + iktxP;
  for (int k = threadIdx.x; k < N; k += blockDim.x) bA[k] = pack_full<T>(X, Y, k, N);
  __syncthreads();
  cplx<T>* res = block_fft<T, N, false>(bA, bB, N, 1, tw);
  for (int x = threadIdx.x; x < N; x += blockDim.x) {
    phys[((long long)z * N + y0) * N + x] = res[x].x;
    phys[((long long)z * N + y0 + 1) * N + x] = res[x].y;
  }
}

// Same transform as k_drow_c2r, written straight into the reference's padded
// physical layout double[nz][N][N+2] (the two padding values of a row are 0).
template <typename T, int N>
__global__ void __launch_bounds__(kThreads)
k_drow_c2r_pad(int iktxP, const cplx<T>* __restrict__ W, double* __restrict__ out, const cplx<T>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bA = tw + N;
  cplx<T>* bB = bA + N;
  const int z = blockIdx.y, y0 = 2 * blockIdx.x;
  load_twiddles<T, N>(tw, twg);
  const cplx<T>* X = W + ((long long)z * N + y0) * iktxP;
  const cplx<T>* Y = X + iktxP;
  for (int k = threadIdx.x; k < N; k += blockDim.x) bA[k] = pack_full<T>(X, Y, k, N);
  __syncthreads();
  cplx<T>* res = block_fft<T, N, false>(bA, bB, N, 1, tw);
  double* r0 = out + ((long long)z * N + y0) * (N + 2);
  double* r1 = r0 + (N + 2);
  for (int x = threadIdx.x; x < N + 2; x += blockDim.x) {
    r0[x] = x < N ? (double)res[x].x : 0.0;
    r1[x] = x < N ? (double)res[x].y : 0.0;
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(kThreads)
k_drow_r2c(int iktxP, const T* __restrict__ phys, cplx<T>* __restrict__ W, const cplx<T>* __restrict__ twg) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bA = tw + N;
  cplx<T>* bB = bA + N;
  const int z = blockIdx.y, y0 = 2 * blockIdx.x;
  load_twiddles<T, N>(tw, twg);
  for (int x = threadIdx.x; x < N; x += blockDim.x)
    bA[x] = mk<T>(phys[((long long)z * N + y0) * N + x], phys[((long long)z * N + y0 + 1) * N + x]);
  __syncthreads();
  cplx<T>* F = block_fft<T, N, true>(bA, bB, N, 1, tw);
  for (int k = threadIdx.x; k <= N / 2; k += blockDim.x) {
    cplx<T> a, b;
    unpack_spec<T>(F, k, N, a, b);
    W[((long long)z * N + y0) * iktxP + k] = a;
    W[((long long)z * N + y0 + 1) * iktxP + k] = b;
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(kThreads)
k_dcol_fwd(int iktxP, const cplx<T>* __restrict__ W, double2* __restrict__ out, const cplx<T>* __restrict__ twg) {
  constexpr int CT = Tile<T>::CT, LD = N + 1, IKTX = N / 2 + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bufA = tw + N;
  cplx<T>* bufB = bufA + CT * LD;
  const int z = blockIdx.y, kx0 = blockIdx.x * CT;
  load_twiddles<T, N>(tw, twg);
  for (int idx = threadIdx.x; idx < CT * N; idx += blockDim.x) {
    const int c = idx % CT, y = idx / CT;
    bufA[c * LD + y] = W[((long long)z * N + y) * iktxP + kx0 + c];
  }
  __syncthreads();
  cplx<T>* res = block_fft<T, N, true>(bufA, bufB, LD, CT, tw);
  const double s = 1.0 / ((double)N * (double)N);
  for (int idx = threadIdx.x; idx < CT * N; idx += blockDim.x) {
    const int c = idx % CT, j = idx / CT, kx = kx0 + c;
    if (kx < IKTX) {
      const cplx<T> v = res[c * LD + j];
      out[((long long)z * N + j) * IKTX + kx] = make_double2((double)v.x * s, (double)v.y * s);
    }
  }
}

// ---- elementwise helpers on the dense layouts ----------------------------
__device__ __forceinline__ void dense_mode(long long m, int n, int& kx, int& ky, int& iky) {
  const int iktx = n / 2 + 1;
  iky = (int)((m / iktx) % n);
  kx = (int)(m % iktx);
  ky = iky < n / 2 ? iky : (iky == n / 2 ? 0 : iky - n);
}
__device__ __forceinline__ bool dense_L(int kx, int ky, int iky, int n, int kmax2) {
  return iky != n / 2 && kx * kx + ky * ky <= kmax2 && !(kx == 0 && ky < 0);
}

// op: 0 = -kh^2 a ; 1 = i kx a ; 2 = i ky a ; 3 = -i ky a ; 4 = a    (masked by L)
static __global__ void k_dense_op(int n, int kmax2, long long tot, int op, const double2* __restrict__ a, double2* __restrict__ o) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    int kx, ky, iky; dense_mode(m, n, kx, ky, iky);
    double2 v = make_double2(0.0, 0.0);
    if (dense_L(kx, ky, iky, n, kmax2)) {
      const double2 s = a[m];
      switch (op) {
        case 0: { const double k2 = -(double)(kx * kx + ky * ky); v = make_double2(k2 * s.x, k2 * s.y); break; }
        case 1: v = make_double2(-kx * s.y, kx * s.x); break;
        case 2: v = make_double2(-ky * s.y, ky * s.x); break;
        case 3: v = make_double2(ky * s.y, -ky * s.x); break;
        default: v = s;
      }
    }
    o[m] = v;
  }
}

// out = L ? i kx ut + i ky vt : 0
static __global__ void k_dense_ik(int n, int kmax2, long long tot, const double2* __restrict__ ut, const double2* __restrict__ vt,
                           double2* __restrict__ o) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    int kx, ky, iky; dense_mode(m, n, kx, ky, iky);
    double2 v = make_double2(0.0, 0.0);
    if (dense_L(kx, ky, iky, n, kmax2)) {
      const double2 a = ut[m], b = vt[m];
      v = make_double2(-kx * a.y - ky * b.y, kx * a.x + ky * b.x);
    }
    o[m] = v;
  }
}

// out = L ? (a - 0.25 kh^2 b) * s : 0  (compute_qw, derivatives.f90:1010-1027)
static __global__ void k_dense_qw(int n, int kmax2, long long tot, const double2* __restrict__ a, const double2* __restrict__ b,
                           double s1, double s2, double2* __restrict__ o) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    int kx, ky, iky; dense_mode(m, n, kx, ky, iky);
    double2 v = make_double2(0.0, 0.0);
    if (dense_L(kx, ky, iky, n, kmax2)) {
      const double k4 = 0.25 * (double)(kx * kx + ky * ky);
      const double2 x = a[m], y = b[m];
      v = make_double2((x.x - k4 * y.x) * s1 * s2, (x.y - k4 * y.y) * s1 * s2);
    }
    o[m] = v;
  }
}

// out = L ? a : 0
static __global__ void k_dense_mask(int n, int kmax2, long long tot, const double2* __restrict__ a, double2* __restrict__ o) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    int kx, ky, iky; dense_mode(m, n, kx, ky, iky);
    o[m] = dense_L(kx, ky, iky, n, kmax2) ? a[m] : make_double2(0.0, 0.0);
  }
}

// physical products: mode 0: o = a*b ; 1: o = a*a + b*b ; 2: o = a*b - c*d
template <typename T>
__global__ void k_phys(long long tot, int mode, const T* __restrict__ a, const T* __restrict__ b, const T* __restrict__ c,
                       const T* __restrict__ d, T* __restrict__ o) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    if (mode == 0) o[i] = a[i] * b[i];
    else if (mode == 1) o[i] = a[i] * a[i] + b[i] * b[i];
    else o[i] = a[i] * b[i] - c[i] * d[i];
  }
}

// padded host layout [nz][n][n+2] <-> compact physical [nz][n][n]
template <typename T>
__global__ void k_phys_unpad(int n, long long tot, const double* __restrict__ in, T* __restrict__ o) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long row = i / n; const int x = (int)(i % n);
    o[i] = (T)in[row * (n + 2) + x];
  }
}
template <typename T>
__global__ void k_phys_pad(int n, long long tot, const T* __restrict__ in, double* __restrict__ o) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long row = i / (n + 2); const int x = (int)(i % (n + 2));
    o[i] = x < n ? (double)in[row * n + x] : 0.0;
  }
}

// Output path (netCDF dumps).  YBJ+ B -> LA on the retained modes
// (diagnostics.f90:1698-1727): LA = B + 0.25*kh2*A/Bu, left to right; 0 elsewhere.
static __global__ void k_dense_la(int n, int kmax2, long long tot, const double2* __restrict__ B,
                                  const double2* __restrict__ A, double Bu, double2* __restrict__ out) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    int kx, ky, iky; dense_mode(m, n, kx, ky, iky);
    double2 v = make_double2(0.0, 0.0);
    if (dense_L(kx, ky, iky, n, kmax2)) {
      const double c = 0.25 * (double)(kx * kx + ky * ky);
      const double2 b = B[m], a = A[m];
      v = make_double2(b.x + (c * a.x) / Bu, b.y + (c * a.y) / Bu);
    }
    out[m] = v;
  }
}

// dimensional FP32 copy of a physical field: out = float((x * s1) * s2)
// (IO_ncf.f90:47-52, 139-146: real(field*scale))
template <typename T>
__global__ void k_phys_f32(long long tot, const T* __restrict__ in, double s1, double s2, float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)(((double)in[i] * s1) * s2);
}

// Omega equation right-hand side, spectral part (derivatives.f90:1489-1560):
// psi_z at the unstaggered level between z and z+1 (0 at the top level),
// bx = i kx psi_z, by = i ky psi_z, xx = -i kx kh2 psi_avg, xy = -i ky kh2
// psi_avg with psi_avg = (psi(z+1) + psi(z))/2, psi at the top level itself.
static __global__ void k_omega_spec(int n, int n3, int kmax2, double dz, const double2* __restrict__ psi,
                                    double2* __restrict__ bx, double2* __restrict__ by, double2* __restrict__ xx,
                                    double2* __restrict__ xy) {
  const long long per = (long long)n * (n / 2 + 1), tot = per * n3;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    int kx, ky, iky; dense_mode(m, n, kx, ky, iky);
    const bool top = m / per == n3 - 1;
    double2 vbx = make_double2(0.0, 0.0), vby = vbx, vxx = vbx, vxy = vbx;
    if (dense_L(kx, ky, iky, n, kmax2)) {
      const double2 p0 = psi[m];
      const double fkx = (double)kx, fky = (double)ky, kh2 = (double)(kx * kx + ky * ky);
      if (!top) {
        const double2 p1 = psi[m + per];
        const double2 rz = make_double2((p1.x - p0.x) / dz, (p1.y - p0.y) / dz);
        vbx = make_double2(-fkx * rz.y, fkx * rz.x);        // i kx psi_z
        vby = make_double2(-fky * rz.y, fky * rz.x);        // i ky psi_z
        const double2 sm = make_double2(p1.x + p0.x, p1.y + p0.y);
        const double cx = fkx * kh2 * 0.5, cy = fky * kh2 * 0.5;   // -i kx kh2 0.5 (psi1 + psi0)
        vxx = make_double2(cx * sm.y, -cx * sm.x);
        vxy = make_double2(cy * sm.y, -cy * sm.x);
      } else {
        const double cx = fkx * kh2, cy = fky * kh2;
        vxx = make_double2(cx * p0.y, -cx * p0.x);
        vxy = make_double2(cy * p0.y, -cy * p0.x);
      }
    }
    bx[m] = vbx; by[m] = vby; xx[m] = vxx; xy[m] = vxy;
  }
}

// physical part: rhsr = 2 (bx xy - by xx)  (derivatives.f90:1569-1577)
template <typename T>
__global__ void k_omega_phys(long long tot, const T* __restrict__ bx, const T* __restrict__ by, const T* __restrict__ xx,
                             const T* __restrict__ xy, T* __restrict__ o) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x)
    o[i] = (T)2 * (bx[i] * xy[i] - by[i] * xx[i]);
}

// omega_equation (elliptic.f90:463-567): one thread per dense column with
// kh2 != 0 and L = 1; n3-1 unstaggered levels; DGTSV's elimination order
// (no interchange: |d| >= 2 >= |dl|) in correctly rounded FP64 operations,
// the same factorisation for the real and imaginary right-hand sides
// (dz^2 * rhs).  w at the top level and in every other column is 0.
// scr: 3 * (n3-1) * per doubles (modified diagonal, two right-hand sides).
static __global__ void k_omega_solve(int n, int n3, int kmax2, double dz, const double* __restrict__ t1,
                                     const double* __restrict__ du, const double* __restrict__ dl,
                                     const double* __restrict__ a, const double2* __restrict__ rhs,
                                     double* __restrict__ scr, double2* __restrict__ w) {
  const long long per = (long long)n * (n / 2 + 1);
  const long long col = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (col >= per) return;
  int kx, ky, iky; dense_mode(col, n, kx, ky, iky);
  const int kh2i = kx * kx + ky * ky;
  if (kh2i == 0 || !dense_L(kx, ky, iky, n, kmax2) || n3 < 2) {
    for (int z = 0; z < n3; ++z) w[z * per + col] = make_double2(0.0, 0.0);
    return;
  }
  const int m = n3 - 1;
  const double dz2 = __dmul_rn(dz, dz), kh2 = (double)kh2i, dzk = __dmul_rn(dz2, kh2);
  double* dd = scr;
  double* br = scr + (long long)m * per;
  double* bi = scr + 2LL * m * per;
  auto diag = [&](int i) { return -__dadd_rn(t1[i], __ddiv_rn(dzk, a[i])); };
  double dprev = diag(0);
  double rprev = __dmul_rn(dz2, rhs[col].x), iprev = __dmul_rn(dz2, rhs[col].y);
  dd[col] = dprev; br[col] = rprev; bi[col] = iprev;
  for (int i = 0; i + 1 < m; ++i) {
    const double fact = __ddiv_rn(dl[i], dprev);
    const double dn = __dsub_rn(diag(i + 1), __dmul_rn(fact, du[i]));
    const double2 q = rhs[(long long)(i + 1) * per + col];
    rprev = __dsub_rn(__dmul_rn(dz2, q.x), __dmul_rn(fact, rprev));
    iprev = __dsub_rn(__dmul_rn(dz2, q.y), __dmul_rn(fact, iprev));
    dprev = dn;
    const long long o = (long long)(i + 1) * per + col;
    dd[o] = dn; br[o] = rprev; bi[o] = iprev;
  }
  // back substitution
  double xr = __ddiv_rn(rprev, dprev), xi = __ddiv_rn(iprev, dprev);
  w[(long long)(m - 1) * per + col] = make_double2(xr, xi);
  for (int i = m - 2; i >= 0; --i) {
    const long long o = (long long)i * per + col;
    xr = __ddiv_rn(__dsub_rn(br[o], __dmul_rn(du[i], xr)), dd[o]);
    xi = __ddiv_rn(__dsub_rn(bi[o], __dmul_rn(du[i], xi)), dd[o]);
    w[o] = make_double2(xr, xi);
  }
  w[(long long)m * per + col] = make_double2(0.0, 0.0);
}

}  // namespace qg
