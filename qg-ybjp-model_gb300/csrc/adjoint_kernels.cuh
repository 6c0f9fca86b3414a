// Elementwise kernels of the adjoint (FP64, the reference's dense spectral
// layout double2 [nz][n][n/2+1] and physical layout double [nz][n][n]).
#pragma once
#include "dense_kernels.cuh"

namespace qg {

// One term s * mult(k) * in of a spectral linear combination; s complex,
// mult: 0 -> 1, 1 -> kx, 2 -> ky, 3 -> kh^2, 4 -> per-mode table (dense [n][n/2+1]).
struct SpecTerm {
  const double2* in;
  double sr, si;
  int mult;
  const double* tab;
};

// out = mask( (acc ? out : 0) + sum_t s_t mult_t in_t )
static __global__ void k_spec_lin(int n, int kmax2, long long tot, int nt, SpecTerm t0, SpecTerm t1, SpecTerm t2,
                                  int acc, double2* out) {
  const long long plane = (long long)n * (n / 2 + 1);
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    int kx, ky, iky;
    dense_mode(m, n, kx, ky, iky);
    double2 o = make_double2(0.0, 0.0);
    if (dense_L(kx, ky, iky, n, kmax2)) {
      if (acc) o = out[m];
      const SpecTerm* ts[3] = {&t0, &t1, &t2};
#pragma unroll
      for (int t = 0; t < 3; ++t) {
        if (t >= nt) break;
        const SpecTerm& T = *ts[t];
        double f = 1.0;
        if (T.mult == 1) f = (double)kx;
        else if (T.mult == 2) f = (double)ky;
        else if (T.mult == 3) f = (double)(kx * kx + ky * ky);
        else if (T.mult == 4) f = T.tab[m % plane];
        const double cr = T.sr * f, ci = T.si * f;
        const double2 v = T.in[m];
        o.x += cr * v.x - ci * v.y;
        o.y += cr * v.y + ci * v.x;
      }
    }
    out[m] = o;
  }
}

// out = (acc ? out : 0) + s * x * (y ? y : 1)
static __global__ void k_phys_acc(long long tot, const double* __restrict__ x, const double* __restrict__ y, double s,
                                  int acc, double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const double v = s * x[i] * (y ? y[i] : 1.0);
    out[i] = acc ? out[i] + v : v;
  }
}

// transpose of c2r on the retained modes: out (+)= mask(2 N^2 Y), (0,0): N^2 Re Y
static __global__ void k_ct_weights(int n, int kmax2, long long tot, double N2, const double2* __restrict__ Y, int acc,
                                    double2* __restrict__ out) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    int kx, ky, iky;
    dense_mode(m, n, kx, ky, iky);
    double2 v = make_double2(0.0, 0.0);
    if (dense_L(kx, ky, iky, n, kmax2)) {
      const double2 y = Y[m];
      v = (kx == 0 && ky == 0) ? make_double2(N2 * y.x, 0.0) : make_double2(2.0 * N2 * y.x, 2.0 * N2 * y.y);
      if (acc) { const double2 o = out[m]; v.x += o.x; v.y += o.y; }
    }
    out[m] = v;
  }
}

// spectrum whose c2r is the transpose of (r2c then mask): mask(Y)/(2 N^2), (0,0) entry 2 Re Y00/(2 N^2)
static __global__ void k_rt_prep(int n, int kmax2, long long tot, double inv2N2, const double2* __restrict__ Y,
                                 double2* __restrict__ out) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    int kx, ky, iky;
    dense_mode(m, n, kx, ky, iky);
    double2 v = make_double2(0.0, 0.0);
    if (dense_L(kx, ky, iky, n, kmax2)) {
      const double2 y = Y[m];
      v = (kx == 0 && ky == 0) ? make_double2(2.0 * y.x * inv2N2, 0.0) : make_double2(y.x * inv2N2, y.y * inv2N2);
    }
    out[m] = v;
  }
}

// per-block partial sums of W (x^2 + y^2) over the objective's subvolume
// (x, y in [n/4, 3n/4), levels iz >= z0); fixed-order reduction
static __global__ void k_obj_partial(int n, int n3, int z0, const double* __restrict__ a, const double* __restrict__ b,
                                     double* __restrict__ part) {
  __shared__ double red[256];
  const long long tot = (long long)n3 * n * n;
  double acc = 0.0;
  for (long long i = blockIdx.x * 256LL + threadIdx.x; i < tot; i += (long long)gridDim.x * 256) {
    const int x = (int)(i % n), y = (int)((i / n) % n), z = (int)(i / ((long long)n * n));
    if (z >= z0 && x >= n / 4 && x < 3 * n / 4 && y >= n / 4 && y < 3 * n / 4) acc += a[i] * a[i] + b[i] * b[i];
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// x *= W (the subvolume indicator)
static __global__ void k_obj_window(int n, int n3, int z0, double* __restrict__ x) {
  const long long tot = (long long)n3 * n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int xx = (int)(i % n), y = (int)((i / n) % n), z = (int)(i / ((long long)n * n));
    if (!(z >= z0 && xx >= n / 4 && xx < 3 * n / 4 && y >= n / 4 && y < 3 * n / 4)) x[i] = 0.0;
  }
}

// compact per-mode table (plane layout) -> dense per-plane table [n][n/2+1]
template <typename T>
static __global__ void k_table_to_dense(Geom g, const T* __restrict__ t, double* __restrict__ out) {
  const int iktx = g.n / 2 + 1;
  const long long tot = (long long)g.n * iktx;
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < tot; m += (long long)gridDim.x * blockDim.x) {
    const int iky = (int)(m / iktx), kx = (int)(m % iktx);
    const int ky = iky < g.n / 2 ? iky : (iky == g.n / 2 ? 0 : iky - g.n);
    double v = 0.0;
    if (iky != g.n / 2 && kx <= g.K && ky >= -g.K && ky <= g.K) v = (double)t[(long long)g.row_of_ky(ky) * g.KXP + kx];
    out[m] = v;
  }
}

}  // namespace qg
