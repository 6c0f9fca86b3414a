// Shared types for the QG-YBJ+ step kernels: complex helpers, the compact
// spectral geometry and the step parameters.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace qg {

template <typename T> struct CT;
template <> struct CT<float> { using type = float2; };
template <> struct CT<double> { using type = double2; };
template <typename T> using cplx = typename CT<T>::type;

template <typename T> __host__ __device__ __forceinline__ cplx<T> mk(T x, T y) { cplx<T> r; r.x = x; r.y = y; return r; }
template <typename C> __host__ __device__ __forceinline__ C cadd(C a, C b) { a.x += b.x; a.y += b.y; return a; }
template <typename C> __host__ __device__ __forceinline__ C csub(C a, C b) { a.x -= b.x; a.y -= b.y; return a; }
template <typename C> __host__ __device__ __forceinline__ C cmul(C a, C b) {
  C r; r.x = a.x * b.x - a.y * b.y; r.y = a.x * b.y + a.y * b.x; return r;
}
template <typename C> __host__ __device__ __forceinline__ C cconj(C a) { a.y = -a.y; return a; }
template <typename C, typename S> __host__ __device__ __forceinline__ C cscale(C a, S s) { a.x *= s; a.y *= s; return a; }
// multiply by +i and by -i
template <typename C> __host__ __device__ __forceinline__ C cmul_i(C a) { C r; r.x = -a.y; r.y = a.x; return r; }
template <typename C> __host__ __device__ __forceinline__ C cmul_mi(C a) { C r; r.x = a.y; r.y = -a.x; return r; }

// Compact spectral layout.  A field holds the retained rectangle
// kx in [0,K], ky in [-K,K] of every level:
//   index = (z*KY + r)*KXP + kx,  r in [0,KY): ky = r for r<=K, r-KY otherwise.
// Modes of the rectangle outside the 2/3 disk (L=0, init.f90:51-74) are
// stored as exact zeros; kx in (K, KXP) is padding.
struct Geom {
  int n;       // n1 == n2
  int n3;      // levels
  int K;       // largest retained |kx|, |ky|
  int KX;      // K+1
  int KY;      // 2K+1
  int KXP;     // padded row length
  int kmax2;   // L=1 iff kx^2+ky^2 <= kmax2 and not (kx==0 && ky<0)
  long long plane;  // KY*KXP
  // levels per vertical segment: n3 for one run; for a stack of ensemble
  // members of one shape, n3 = members * nseg and each member is a segment
  // with its own top and bottom (no vertical coupling across segments)
  int nseg;
  __host__ __device__ __forceinline__ int ky_of_row(int r) const { return r <= K ? r : r - KY; }
  __host__ __device__ __forceinline__ int row_of_ky(int ky) const { return ky >= 0 ? ky : ky + KY; }
  __host__ __device__ __forceinline__ bool mask(int kx, int ky) const {
    return kx <= K && (kx * kx + ky * ky) <= kmax2 && !(kx == 0 && ky < 0);
  }
  // FFT index j in [0,n) of a compact row (ky) and back (-1: not in rectangle)
  __host__ __device__ __forceinline__ int fft_index_of_row(int r) const { return r <= K ? r : r - KY + n; }
  __host__ __device__ __forceinline__ int row_of_fft_index(int j) const {
    return j <= K ? j : (j >= n - K ? j - n + KY : -1);
  }
};

struct StepParams {
  double delt, gamma, Bu, Ro, W2F, dz, nuz;
  double cdisp;       // 0.5/(Bu*Ro)
  int adv;            // 0 when linear == 1
  int refr;           // 0 when passive_scalar == 1
  int disp;           // 0 when no_dispersion == 1 or passive_scalar == 1
  int use_dq;         // inviscid == 0 && nuz != 0
  int euler;          // forward Euler first step
  int ybj;            // 1: YBJ+ (A from A_solver_ybj_plus); 0: regular YBJ (A from the vertical integral of B)
  // a stack of ensemble members (Geom::nseg levels each): per member
  // {delt, 0.5/(Bu Ro), Ro, W2F} at mpar[4 m .. 4 m + 3], and the integrating
  // factor tables of member m at + m * plane; nullptr for one run
  const double* mpar;
};

}  // namespace qg
