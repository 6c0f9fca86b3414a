// Elementwise kernels of the adjoint (FP64, the reference's dense spectral
// layout double2 [nz][n][n/2+1] and physical layout double [nz][n][n]).
#pragma once
#include "dense_kernels.cuh"
#include "step_kernels.cuh"

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


// ===========================================================================
// Fused adjoint of one step on the compact layout (FP64).
//
// Phase A' (batches of levels, scratch planes SF and SA, [zb][6][n][KXP]):
//   k_col_inv          y-inverse FFTs of u, v, zeta, q, BR, BI (the forward
//                      kernel, into SF)
//   k_adj_col_inv      adjoint tendencies lNq, lTR, lTI from the incoming
//                      adjoint state; y-inverse FFTs of l and -i ky l (SA)
//   k_adj_row          x-c2r of 14 physical fields, the transposed products,
//                      x-r2c of the 6 results (SA)
//   k_adj_col_fwd      y-forward FFTs; transposed filter / leapfrog / Euler
//                      update; right-hand sides of the symmetric solves
// Phase B: the FP64 tridiagonal solves (psi_solver, A_solver_ybj_plus) of
//   the forward step applied to (lpsi, lAR, lAI).
// Phase C' (q^w transpose):
//   k_adj_qw_col_inv   y-inverse FFTs of BR, i ky BR, BI, i ky BI, w, ky^2 w (SF)
//   k_adj_qw_row       x-c2r, transposed q^w products, x-r2c (SF)
//   k_adj_qw_col_fwd   y-forward FFTs; lq += w, lB += A-solve + q^w terms
//
// Transposes (N = n): C = c2r of the retained modes (realit included) has
// C^T y = w_k F(y) with F the unnormalised r2c, w_k = 2 and 1 at (0,0) (real
// part); (mask R)^T Y = C(Y')/(2 N^2), Y'_00 = 2 Re Y_00.
// ===========================================================================
struct AdjP {
  double dt, gam;
  double cdisp;   // disp * 0.5/(Bu Ro)
  double adv;     // 0 when linear
  double refr;    // 0 when passive_scalar
  double s;       // Ro W2F (q^w coefficient)
  int first;      // transposing the forward Euler first step
};
struct AdjIn { const double2* l[6]; };                   // (lq, lr, lBR, lBI, lcR, lcI) after the step
struct AdjOut { double2* l[6]; double2* lpsi; double2* lAR; double2* lAI; };

// transposed time update of one mode: outputs before the solves and the
// product terms, and the adjoint tendencies of q, BR, BI
__device__ __forceinline__ void adj_update(const AdjP& p, const AdjIn& L, long long m, double e1, double e2,
                                           double e1w, double e2w, double2 o[6], double2& lNq, double2& lTR,
                                           double2& lTI) {
  const double2 lq1 = L.l[0][m], lBR1 = L.l[2][m], lBI1 = L.l[3][m];
  if (p.first) {
    const double2 lr1 = L.l[1][m], lcR1 = L.l[4][m], lcI1 = L.l[5][m];
    o[0] = cadd(lr1, cscale(lq1, e1));
    o[2] = cadd(lcR1, cscale(lBR1, e1w));
    o[3] = cadd(lcI1, cscale(lBI1, e1w));
    o[1] = o[4] = o[5] = make_double2(0.0, 0.0);
    lNq = cscale(lq1, -p.dt * e1);
    lTR = cscale(lBR1, -p.dt * e1w);
    lTI = cscale(lBI1, -p.dt * e1w);
  } else {
    const double2 lr1 = L.l[1][m], lcR1 = L.l[4][m], lcI1 = L.l[5][m];
    const double g = p.gam, d2 = 2.0 * p.dt;
    const double2 lqp = cadd(lq1, cscale(lr1, g));
    const double2 lRp = cadd(lBR1, cscale(lcR1, g));
    const double2 lIp = cadd(lBI1, cscale(lcI1, g));
    o[0] = cscale(lr1, 1.0 - 2.0 * g);
    o[2] = cscale(lcR1, 1.0 - 2.0 * g);
    o[3] = cscale(lcI1, 1.0 - 2.0 * g);
    o[1] = cadd(cscale(lr1, g), cscale(lqp, e2));
    o[4] = cadd(cscale(lcR1, g), cscale(lRp, e2w));
    o[5] = cadd(cscale(lcI1, g), cscale(lIp, e2w));
    lNq = cscale(lqp, -d2 * e1);
    lTR = cscale(lRp, -d2 * e1w);
    lTI = cscale(lIp, -d2 * e1w);
  }
}

// spectrum entering a c2r that applies (mask R)^T: Y/(2N^2), (0,0): Re Y/N^2
__device__ __forceinline__ double2 rt_scale(double2 v, int kx, int ky, double inv2n2) {
  return (kx == 0 && ky == 0) ? make_double2(2.0 * v.x * inv2n2, 0.0) : cscale(v, inv2n2);
}

// packed spectrum X + iY of two real rows from half-spectrum values given at
// kk = k (k <= K) or kk = n - k (k >= n - K); imaginary parts at kx = 0 ignored
__device__ __forceinline__ double2 pack_xy(double2 X, double2 Y, int k, int K, int n) {
  if (k == 0) return make_double2(X.x, Y.x);
  if (k <= K) return make_double2(X.x - Y.y, X.y + Y.x);
  if (k >= n - K) return make_double2(X.x + Y.y, Y.x - X.y);
  return make_double2(0.0, 0.0);
}

template <int N>
__global__ void __launch_bounds__(kColThreads, Tiles<double, N>::MINB)
k_adj_col_inv(Geom g, AdjP p, int zbase, AdjIn L, const double* __restrict__ e1t, const double* __restrict__ e2t,
              const double* __restrict__ e1wt, const double* __restrict__ e2wt, double2* __restrict__ SA,
              const double2* __restrict__ twg) {
  using T = double;
  constexpr int CT = Tiles<T, N>::CT, LD = Tiles<T, N>::LD, NT = kColThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* tw = reinterpret_cast<double2*>(smem_raw);
  double2* buf = tw + N;                       // [6][CT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  load_tw<T, N>(tw, twg, NT);
  const long long zoff = (long long)z * g.plane;
  const double inv2n2 = 0.5 / ((double)N * (double)N);
  for (int e = tid; e < CT * N; e += NT) {
    const int c = e % CT, j = e / CT;
    const int kx = kx0 + c;
    const int r = g.row_of_fft_index(j);
    double2 v[6];
#pragma unroll
    for (int f = 0; f < 6; ++f) v[f] = make_double2(0.0, 0.0);
    if (kx <= g.K && r >= 0) {
      const int ky = g.ky_of_row(r);
      if (g.mask(kx, ky)) {
        const long long m = zoff + (long long)r * g.KXP + kx, mt = (long long)r * g.KXP + kx;
        double2 o[6], lN, lR, lI;
        adj_update(p, L, m, e1t[mt], e2t[mt], e1wt[mt], e2wt[mt], o, lN, lR, lI);
        lN = rt_scale(lN, kx, ky, inv2n2);
        lR = rt_scale(lR, kx, ky, inv2n2);
        lI = rt_scale(lI, kx, ky, inv2n2);
        v[0] = lN; v[1] = cscale(cmul_mi(lN), (double)ky);
        v[2] = lR; v[3] = cscale(cmul_mi(lR), (double)ky);
        v[4] = lI; v[5] = cscale(cmul_mi(lI), (double)ky);
      }
    }
#pragma unroll
    for (int f = 0; f < 6; ++f) buf[(f * CT + c) * LD + pad_idx(j)] = v[f];
  }
  __syncthreads();
  if (kx0 == 0) {
    for (int e = tid; e < 6 * (N / 2 - 1); e += NT) {
      const int f = e / (N / 2 - 1), j = 1 + e % (N / 2 - 1);
      double2* col = buf + f * CT * LD;
      col[pad_idx(N - j)] = cconj(col[pad_idx(j)]);
    }
    __syncthreads();
  }
  fft_ip<T, N, false, 3 * CT, NT, LD>(buf, tw);
  fft_ip<T, N, false, 3 * CT, NT, LD>(buf + 3 * CT * LD, tw);
#pragma unroll 4
  for (int e = tid; e < 6 * CT * N; e += NT) {
    const int c = e % CT, y = (e / CT) % N, f = e / (CT * N);
    SA[scr_off(zb, f, y, N, g.KXP) + kx0 + c] = buf[(f * CT + c) * LD + pad_idx(y)];
  }
}

// rows: SF holds (u, v, zeta, q, BR, BI), SA the adjoint planes
// (lNq, -i ky lNq, lTR, -i ky lTR, lTI, -i ky lTI) after the y-inverse FFT;
// writes SA = (F_x lu, -i kx F_x lv - kx^2 F_x lZ, F_x lZ, F_x lQ, F_x lBR, F_x lBI)
template <int N>
__global__ void __launch_bounds__(kThreadsB)
k_adj_row(Geom g, AdjP p, const double2* __restrict__ SF, double2* __restrict__ SA, const double2* __restrict__ twg) {
  using T = double;
  constexpr int RT = Tiles<T, N>::RT, LD = Tiles<T, N>::LD, NT = kThreadsB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* tw = reinterpret_cast<double2*>(smem_raw);
  double2* bA = tw + N;                 // [7][RT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y;
  const int y0 = blockIdx.x * RT;
  const int K = g.K;
  load_tw<T, N>(tw, twg, NT);
  const double adv = p.adv, hr = 0.5 * p.refr;
  for (int e = tid; e < 7 * RT * N; e += NT) {
    const int k = e % N, rr = (e / N) % RT, q = e / (RT * N);
    const int y = y0 + rr;
    const int kk = k <= K ? k : N - k;
    double2 v = make_double2(0.0, 0.0);
    if (k <= K || k >= N - K) {
      double2 X, Y;
      if (q < 3) {
        X = SF[scr_off(zb, 2 * q, y, N, g.KXP) + kk];
        Y = SF[scr_off(zb, 2 * q + 1, y, N, g.KXP) + kk];
      } else if (q < 6) {
        const int f = q - 3;
        X = cscale(cmul_mi(SA[scr_off(zb, 2 * f, y, N, g.KXP) + kk]), adv * (double)kk);
        Y = cscale(SA[scr_off(zb, 2 * f + 1, y, N, g.KXP) + kk], adv);
      } else {
        X = cscale(SA[scr_off(zb, 4, y, N, g.KXP) + kk], hr);
        Y = cscale(SA[scr_off(zb, 2, y, N, g.KXP) + kk], -hr);
      }
      v = pack_xy(X, Y, k, K, N);
    }
    bA[(q * RT + rr) * LD + pad_idx(k)] = v;
  }
  __syncthreads();
  fft_ip<T, N, false, 7 * RT, NT, LD>(bA, tw);
  for (int e = tid; e < RT * N; e += NT) {
    const int x = e % N, rr = e / N;
    const int px = pad_idx(x);
    const double2 uv = bA[(0 * RT + rr) * LD + px], zq = bA[(1 * RT + rr) * LD + px];
    const double2 bb = bA[(2 * RT + rr) * LD + px];
    const double2 aq = bA[(3 * RT + rr) * LD + px], aR = bA[(4 * RT + rr) * LD + px];
    const double2 aI = bA[(5 * RT + rr) * LD + px], zz = bA[(6 * RT + rr) * LD + px];
    const double u = uv.x, v = uv.y, Z = zq.x, Q = zq.y, br = bb.x, bi = bb.y;
    const double lu = aq.x * Q + aR.x * br + aI.x * bi;
    const double lv = aq.y * Q + aR.y * br + aI.y * bi;
    const double lZ = zz.x * br + zz.y * bi;
    const double lQ = aq.x * u + aq.y * v;
    const double lBR = aR.x * u + aR.y * v + zz.x * Z;
    const double lBI = aI.x * u + aI.y * v + zz.y * Z;
    bA[(0 * RT + rr) * LD + px] = make_double2(lu, lv);
    bA[(1 * RT + rr) * LD + px] = make_double2(lZ, lQ);
    bA[(2 * RT + rr) * LD + px] = make_double2(lBR, lBI);
  }
  __syncthreads();
  fft_ip<T, N, true, 3 * RT, NT, LD>(bA, tw);
  for (int e = tid; e < RT * (K + 1); e += NT) {
    const int k = e % (K + 1), rr = e / (K + 1);
    const int y = y0 + rr;
    double2 lu, lv, lZ, lQ, lBR, lBI;
    unpack_pad<T>(bA + (0 * RT + rr) * LD, k, N, lu, lv);
    unpack_pad<T>(bA + (1 * RT + rr) * LD, k, N, lZ, lQ);
    unpack_pad<T>(bA + (2 * RT + rr) * LD, k, N, lBR, lBI);
    const double kx = (double)k;
    SA[scr_off(zb, 0, y, N, g.KXP) + k] = lu;
    SA[scr_off(zb, 1, y, N, g.KXP) + k] = csub(cscale(cmul_mi(lv), kx), cscale(lZ, kx * kx));
    SA[scr_off(zb, 2, y, N, g.KXP) + k] = lZ;
    SA[scr_off(zb, 3, y, N, g.KXP) + k] = lQ;
    SA[scr_off(zb, 4, y, N, g.KXP) + k] = lBR;
    SA[scr_off(zb, 5, y, N, g.KXP) + k] = lBI;
  }
}

template <int N>
__global__ void __launch_bounds__(kColThreads, Tiles<double, N>::MINB)
k_adj_col_fwd(Geom g, AdjP p, int zbase, AdjIn L, AdjOut O, const double* __restrict__ e1t,
              const double* __restrict__ e2t, const double* __restrict__ e1wt, const double* __restrict__ e2wt,
              const double2* __restrict__ SA, const double2* __restrict__ twg) {
  using T = double;
  constexpr int CT = Tiles<T, N>::CT, LD = Tiles<T, N>::LD, NT = kColThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* tw = reinterpret_cast<double2*>(smem_raw);
  double2* buf = tw + N;                 // [6][CT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  load_tw<T, N>(tw, twg, NT);
#pragma unroll 4
  for (int e = tid; e < 6 * CT * N; e += NT) {
    const int c = e % CT, y = (e / CT) % N, h = e / (CT * N);
    const int kx = kx0 + c;
    cp_async_c<T>(buf + (h * CT + c) * LD + pad_idx(y), SA + scr_off(zb, h, y, N, g.KXP) + kx, kx <= g.K);
  }
  cp_async_wait_all();
  __syncthreads();
  fft_ip<T, N, true, 3 * CT, NT, LD>(buf, tw);
  fft_ip<T, N, true, 3 * CT, NT, LD>(buf + 3 * CT * LD, tw);
  const long long zoff = (long long)z * g.plane;
  for (int e = tid; e < CT * g.KY; e += NT) {
    const int c = e % CT, r = e / CT;
    const int kx = kx0 + c;
    if (kx > g.K) continue;
    const int ky = g.ky_of_row(r);
    const long long m = zoff + (long long)r * g.KXP + kx, mt = (long long)r * g.KXP + kx;
    double2 o[6], lpsi = make_double2(0.0, 0.0), lAR = lpsi, lAI = lpsi;
#pragma unroll
    for (int f = 0; f < 6; ++f) o[f] = lpsi;
    if (g.mask(kx, ky)) {
      const int j = pad_idx(g.fft_index_of_row(r));
      const bool dc = kx == 0 && ky == 0;
      const double wt = dc ? 1.0 : 2.0, fky = (double)ky, kh2 = (double)(kx * kx + ky * ky);
      double2 hv[6];
#pragma unroll
      for (int f = 0; f < 6; ++f) {
        hv[f] = cscale(buf[(f * CT + c) * LD + j], wt);
        if (dc) hv[f].y = 0.0;
      }
      double2 lN, lR, lI;
      adj_update(p, L, m, e1t[mt], e2t[mt], e1wt[mt], e2wt[mt], o, lN, lR, lI);
      // psi -> (u, v, zeta) = (-i ky, i kx, -kh^2) psi: transposes i ky, -i kx, -kh^2
      lpsi = csub(cadd(cscale(cmul_i(hv[0]), fky), hv[1]), cscale(hv[2], fky * fky));
      o[0] = cadd(o[0], hv[3]);
      o[2] = cadd(o[2], hv[4]);
      o[3] = cadd(o[3], hv[5]);
      // T_R = N_BR + c kh^2 A_I - r_BI/2, T_I = N_BI - c kh^2 A_R + r_BR/2
      lAI = cscale(lR, p.cdisp * kh2);
      lAR = cscale(lI, -p.cdisp * kh2);
    }
#pragma unroll
    for (int f = 0; f < 6; ++f) O.l[f][m] = o[f];
    O.lpsi[m] = lpsi;
    O.lAR[m] = lAR;
    O.lAI[m] = lAI;
  }
}

// y-inverse FFTs for the q^w transpose: BR, i ky BR, BI, i ky BI, w', ky^2 w'
// with w' = w/(2N^2) ((0,0): Re w/N^2), into SF
template <int N>
__global__ void __launch_bounds__(kColThreads, Tiles<double, N>::MINB)
k_adj_qw_col_inv(Geom g, int zbase, const double2* __restrict__ BR, const double2* __restrict__ BI,
                 const double2* __restrict__ w, double2* __restrict__ SF, const double2* __restrict__ twg) {
  using T = double;
  constexpr int CT = Tiles<T, N>::CT, LD = Tiles<T, N>::LD, NT = kColThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* tw = reinterpret_cast<double2*>(smem_raw);
  double2* buf = tw + N;                 // [6][CT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  load_tw<T, N>(tw, twg, NT);
  const long long zoff = (long long)z * g.plane;
#pragma unroll
  for (int src = 0; src < 3; ++src) {
    const double2* F = src == 0 ? BR : (src == 1 ? BI : w);
    double2* slot = buf + 2 * src * CT * LD;
#pragma unroll 4
    for (int e = tid; e < CT * N; e += NT) {
      const int c = e % CT, j = e / CT;
      const int kx = kx0 + c;
      const int r = g.row_of_fft_index(j);
      const bool in = kx <= g.K && r >= 0;
      cp_async_c<T>(slot + c * LD + pad_idx(j), in ? F + zoff + (long long)r * g.KXP + kx : F, in);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  const double inv2n2 = 0.5 / ((double)N * (double)N);
  for (int e = tid; e < CT * N; e += NT) {
    const int c = e % CT, j = e / CT;
    const int kx = kx0 + c;
    const int r = g.row_of_fft_index(j);
    const int ky = r >= 0 ? g.ky_of_row(r) : 0;
    const int o = c * LD + pad_idx(j);
    const double fky = (double)ky;
    buf[1 * CT * LD + o] = cscale(cmul_i(buf[0 * CT * LD + o]), fky);
    buf[3 * CT * LD + o] = cscale(cmul_i(buf[2 * CT * LD + o]), fky);
    const double2 wv = rt_scale(buf[4 * CT * LD + o], kx, ky, inv2n2);
    buf[4 * CT * LD + o] = wv;
    buf[5 * CT * LD + o] = cscale(wv, fky * fky);
  }
  __syncthreads();
  if (kx0 == 0) {
    for (int e = tid; e < 6 * (N / 2 - 1); e += NT) {
      const int f = e / (N / 2 - 1), j = 1 + e % (N / 2 - 1);
      double2* col = buf + f * CT * LD;
      col[pad_idx(N - j)] = cconj(col[pad_idx(j)]);
    }
    __syncthreads();
  }
  fft_ip<T, N, false, 3 * CT, NT, LD>(buf, tw);
  fft_ip<T, N, false, 3 * CT, NT, LD>(buf + 3 * CT * LD, tw);
#pragma unroll 4
  for (int e = tid; e < 6 * CT * N; e += NT) {
    const int c = e % CT, y = (e / CT) % N, f = e / (CT * N);
    SF[scr_off(zb, f, y, N, g.KXP) + kx0 + c] = buf[(f * CT + c) * LD + pad_idx(y)];
  }
}

// rows of the q^w transpose: P1 = BRy BIx - BRx BIy, P2 = BR^2 + BI^2 with
// q^w = s R(P1) - s kh^2/4 R(P2); writes (G_R, H_R, G_I, H_I) with
// lB = w_k [F_y(G) - i ky F_y(H)], G = -i kx F_x(a) + F_x(c), H = F_x(b)
template <int N>
__global__ void __launch_bounds__(kThreadsB)
k_adj_qw_row(Geom g, AdjP p, double2* __restrict__ SF, const double2* __restrict__ twg) {
  using T = double;
  constexpr int RT = Tiles<T, N>::RT, LD = Tiles<T, N>::LD, NT = kThreadsB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* tw = reinterpret_cast<double2*>(smem_raw);
  double2* bA = tw + N;                 // [4][RT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y;
  const int y0 = blockIdx.x * RT;
  const int K = g.K;
  load_tw<T, N>(tw, twg, NT);
  const double s = p.s;
  for (int e = tid; e < 4 * RT * N; e += NT) {
    const int k = e % N, rr = (e / N) % RT, q = e / (RT * N);
    const int y = y0 + rr;
    const int kk = k <= K ? k : N - k;
    double2 v = make_double2(0.0, 0.0);
    if (k <= K || k >= N - K) {
      const double fk = (double)kk;
      double2 X, Y;
      if (q == 0) {
        X = SF[scr_off(zb, 0, y, N, g.KXP) + kk]; Y = SF[scr_off(zb, 2, y, N, g.KXP) + kk];
      } else if (q == 1) {
        X = cscale(cmul_i(SF[scr_off(zb, 0, y, N, g.KXP) + kk]), fk);
        Y = cscale(cmul_i(SF[scr_off(zb, 2, y, N, g.KXP) + kk]), fk);
      } else if (q == 2) {
        X = SF[scr_off(zb, 1, y, N, g.KXP) + kk]; Y = SF[scr_off(zb, 3, y, N, g.KXP) + kk];
      } else {
        const double2 w1 = SF[scr_off(zb, 4, y, N, g.KXP) + kk], w2 = SF[scr_off(zb, 5, y, N, g.KXP) + kk];
        X = cscale(w1, -s);
        Y = cscale(cadd(cscale(w1, fk * fk), w2), 0.25 * s);
      }
      v = pack_xy(X, Y, k, K, N);
    }
    bA[(q * RT + rr) * LD + pad_idx(k)] = v;
  }
  __syncthreads();
  fft_ip<T, N, false, 4 * RT, NT, LD>(bA, tw);
  for (int e = tid; e < RT * N; e += NT) {
    const int x = e % N, rr = e / N;
    const int px = pad_idx(x);
    const double2 b = bA[(0 * RT + rr) * LD + px], bx = bA[(1 * RT + rr) * LD + px];
    const double2 by = bA[(2 * RT + rr) * LD + px], lp = bA[(3 * RT + rr) * LD + px];
    const double l1 = lp.x, l2 = lp.y;
    bA[(0 * RT + rr) * LD + px] = make_double2(-l1 * by.y, l1 * by.x);          // a_R, a_I
    bA[(1 * RT + rr) * LD + px] = make_double2(l1 * bx.y, -l1 * bx.x);          // b_R, b_I
    bA[(2 * RT + rr) * LD + px] = make_double2(2.0 * b.x * l2, 2.0 * b.y * l2); // c_R, c_I
  }
  __syncthreads();
  fft_ip<T, N, true, 3 * RT, NT, LD>(bA, tw);
  for (int e = tid; e < RT * (K + 1); e += NT) {
    const int k = e % (K + 1), rr = e / (K + 1);
    const int y = y0 + rr;
    double2 aR, aI, bR, bI, cR, cI;
    unpack_pad<T>(bA + (0 * RT + rr) * LD, k, N, aR, aI);
    unpack_pad<T>(bA + (1 * RT + rr) * LD, k, N, bR, bI);
    unpack_pad<T>(bA + (2 * RT + rr) * LD, k, N, cR, cI);
    const double kx = (double)k;
    SF[scr_off(zb, 0, y, N, g.KXP) + k] = cadd(cscale(cmul_mi(aR), kx), cR);
    SF[scr_off(zb, 1, y, N, g.KXP) + k] = bR;
    SF[scr_off(zb, 2, y, N, g.KXP) + k] = cadd(cscale(cmul_mi(aI), kx), cI);
    SF[scr_off(zb, 3, y, N, g.KXP) + k] = bI;
  }
}

// final adds: lq += w, lB += A_solver(lA) (+ q^w transpose when with_qw)
template <int N>
__global__ void __launch_bounds__(kColThreads, Tiles<double, N>::MINB)
k_adj_qw_col_fwd(Geom g, int zbase, int with_qw, double2* __restrict__ lq, double2* __restrict__ lBR,
                 double2* __restrict__ lBI, const double2* __restrict__ w, const double2* __restrict__ lBRa,
                 const double2* __restrict__ lBIa, const double2* __restrict__ SF, const double2* __restrict__ twg) {
  using T = double;
  constexpr int CT = Tiles<T, N>::CT, LD = Tiles<T, N>::LD, NT = kColThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2* tw = reinterpret_cast<double2*>(smem_raw);
  double2* buf = tw + N;                 // [4][CT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  if (with_qw) {
    load_tw<T, N>(tw, twg, NT);
#pragma unroll 4
    for (int e = tid; e < 4 * CT * N; e += NT) {
      const int c = e % CT, y = (e / CT) % N, h = e / (CT * N);
      const int kx = kx0 + c;
      cp_async_c<T>(buf + (h * CT + c) * LD + pad_idx(y), SF + scr_off(zb, h, y, N, g.KXP) + kx, kx <= g.K);
    }
    cp_async_wait_all();
    __syncthreads();
    fft_ip<T, N, true, 4 * CT, NT, LD>(buf, tw);
  }
  const long long zoff = (long long)z * g.plane;
  for (int e = tid; e < CT * g.KY; e += NT) {
    const int c = e % CT, r = e / CT;
    const int kx = kx0 + c;
    if (kx > g.K) continue;
    const int ky = g.ky_of_row(r);
    const long long m = zoff + (long long)r * g.KXP + kx;
    double2 oq = make_double2(0.0, 0.0), oR = oq, oI = oq;
    if (g.mask(kx, ky)) {
      oq = cadd(lq[m], w[m]);
      oR = cadd(lBR[m], lBRa[m]);
      oI = cadd(lBI[m], lBIa[m]);
      if (with_qw) {
        const int j = pad_idx(g.fft_index_of_row(r));
        const bool dc = kx == 0 && ky == 0;
        const double wt = dc ? 1.0 : 2.0, fky = (double)ky;
        double2 dR = csub(buf[(0 * CT + c) * LD + j], cscale(cmul_i(buf[(1 * CT + c) * LD + j]), fky));
        double2 dI = csub(buf[(2 * CT + c) * LD + j], cscale(cmul_i(buf[(3 * CT + c) * LD + j]), fky));
        dR = cscale(dR, wt); dI = cscale(dI, wt);
        if (dc) { dR.y = 0.0; dI.y = 0.0; }
        oR = cadd(oR, dR);
        oI = cadd(oI, dI);
      }
    }
    lq[m] = oq; lBR[m] = oR; lBI[m] = oI;
  }
}

// out = mask(a + s b) on the compact layout
static __global__ void k_adj_sum(Geom g, long long tot, const double2* __restrict__ a, const double2* __restrict__ b,
                                 double s, double2* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const long long mm = i % g.plane;
    const int r = (int)(mm / g.KXP), kx = (int)(mm % g.KXP);
    out[i] = g.mask(kx, g.ky_of_row(r)) ? cadd(a[i], cscale(b[i], s)) : make_double2(0.0, 0.0);
  }
}

}  // namespace qg
