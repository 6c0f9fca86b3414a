// Kernels of one QG-YBJ+ step on the compact spectral layout (common.cuh).
//
// Phase A (z-local, batches of Zb levels, scratch S[zb][6][n][KXP]):
//   col_inv    : y-inverse FFTs of u,v,zeta (from psi), q, BR, BI
//   row_main   : x-c2r, 8 physical products, x-r2c, ik-combination
//   col_update : y-forward FFTs -> J(psi,q), J(psi,B) +- refraction; leapfrog /
//                Euler update, Robert-Asselin filter, integrating factor;
//                y-inverse FFTs of the new BR, BI and their y-derivatives
//   row_qw     : x-c2r of B, B_x, B_y; q^w products; x-r2c
//   col_qw     : y-forward FFTs -> q^w, q* = q - q^w
// Phase B (column-local): FP64 tridiagonal solves q*->psi, B->A.
#pragma once
#include "common.cuh"
#include "fft_block.cuh"

namespace qg {

constexpr int kThreads = 256;
constexpr int kNScr = 6;  // scratch (kx,y) planes per level

template <typename T> struct Tile;
template <> struct Tile<float> { static constexpr int CT = 8; static constexpr int RT = 2; };
template <> struct Tile<double> { static constexpr int CT = 4; static constexpr int RT = 1; };

__host__ __device__ __forceinline__ long long scr_off(int zb, int f, int y, int n, int KXP) {
  return (((long long)zb * kNScr + f) * n + y) * KXP;
}

// ---------------------------------------------------------------------------
// column helpers
// ---------------------------------------------------------------------------
// realit (fft.f90:88-107) on the kx=0 column held in buf[0..n): entries of
// negative ky become the conjugates of the positive ones.
template <typename T>
__device__ __forceinline__ void realit_col(cplx<T>* col, int n) {
  for (int j = 1 + threadIdx.x; j < n / 2; j += blockDim.x) col[n - j] = cconj(col[j]);
}

// Tile shapes: CT columns per column-kernel CTA (6*CT transforms ~100 KB of
// shared memory), RT rows per row-kernel CTA.
template <typename T, int N> struct Tiles {
  static constexpr int CB = (int)sizeof(cplx<T>);
  static constexpr int ct0 = (16384 / CB) / N;
  static constexpr int CT = ct0 >= 8 ? 8 : (ct0 >= 1 ? ct0 : 1);
  static constexpr int rt0 = (8192 / CB) / N;
  static constexpr int RT = rt0 >= 2 ? 2 : 1;
  static constexpr int LD = PadLD<N>::value;
};
constexpr int kColThreads = 256;   // k_col_inv, k_col_update
constexpr int kThreadsB = 256;     // row kernels, k_col_qw

template <typename T, int N>
__device__ __forceinline__ void load_tw(cplx<T>* tw_s, const cplx<T>* __restrict__ tw_g, int nt) {
  for (int i = threadIdx.x; i < N; i += nt) tw_s[i] = tw_g[i];
}

// ===========================================================================
// Phase A, kernel 1: y-inverse FFTs of the six fields needed in physical space
// ===========================================================================
template <typename T, int N>
__global__ void __launch_bounds__(kColThreads, 2)
k_col_inv(Geom g, int zbase, const cplx<T>* __restrict__ psi, const cplx<T>* __restrict__ q,
          const cplx<T>* __restrict__ BR, const cplx<T>* __restrict__ BI, cplx<T>* __restrict__ S,
          const cplx<T>* __restrict__ twg) {
  constexpr int CT = Tiles<T, N>::CT, LD = Tiles<T, N>::LD, NT = kColThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + N;                       // [6][CT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  load_tw<T, N>(tw, twg, NT);
  const long long zoff = (long long)z * g.plane;
#pragma unroll
  for (int src = 0; src < 4; ++src) {
    const cplx<T>* F = src == 0 ? psi : (src == 1 ? q : (src == 2 ? BR : BI));
#pragma unroll 4
    for (int e = tid; e < CT * N; e += NT) {
      const int c = e % CT, j = e / CT;
      const int kx = kx0 + c;
      const int r = g.row_of_fft_index(j);
      const bool in = kx <= g.K && r >= 0;
      const cplx<T> sv = in ? F[zoff + (long long)r * g.KXP + kx] : mk<T>(0, 0);
      const int o = c * LD + pad_idx(j);
      if (src == 0) {
        const T ky = in ? (T)g.ky_of_row(r) : (T)0;
        buf[0 * CT * LD + o] = cscale(cmul_mi(sv), ky);                          // u = -i ky psi (derivatives.f90:1309)
        buf[1 * CT * LD + o] = cscale(cmul_i(sv), (T)kx);                        // v = i kx psi  (derivatives.f90:1310)
        buf[2 * CT * LD + o] = cscale(sv, -((T)(kx * kx) + ky * ky));            // zeta = -kh^2 psi (derivatives.f90:842)
      } else {
        buf[(src + 2) * CT * LD + o] = sv;
      }
    }
  }
  __syncthreads();
  if (kx0 == 0) {    // realit (fft.f90:88-107) on the kx=0 column of each field
    for (int e = tid; e < 6 * (N / 2 - 1); e += NT) {
      const int f = e / (N / 2 - 1), j = 1 + e % (N / 2 - 1);
      cplx<T>* col = buf + f * CT * LD;
      col[pad_idx(N - j)] = cconj(col[pad_idx(j)]);
    }
    __syncthreads();
  }
  // two groups of three fields keep a thread's butterflies in registers
  fft_ip<T, N, false, 3 * CT, NT>(buf, tw);
  fft_ip<T, N, false, 3 * CT, NT>(buf + 3 * CT * LD, tw);
#pragma unroll 4
  for (int e = tid; e < 6 * CT * N; e += NT) {
    const int c = e % CT, y = (e / CT) % N, f = e / (CT * N);
    S[scr_off(zb, f, y, N, g.KXP) + kx0 + c] = buf[(f * CT + c) * LD + pad_idx(y)];
  }
}

// Hermitian-extended packed spectrum X + iY of two real rows from their
// half spectra (kx in [0,K]); the imaginary parts of the kx=0 entries are
// ignored, as a c2r transform does.
template <typename T>
__device__ __forceinline__ cplx<T> pack_spec(const cplx<T>* __restrict__ X, const cplx<T>* __restrict__ Y,
                                             int k, int n, int K) {
  if (k == 0) return mk<T>(X[0].x, Y[0].x);
  if (k <= K) { cplx<T> a = X[k], b = Y[k]; return mk<T>(a.x - b.y, a.y + b.x); }
  if (k >= n - K) { const int kk = n - k; cplx<T> a = X[kk], b = Y[kk]; return mk<T>(a.x + b.y, b.x - a.y); }
  return mk<T>(0, 0);
}

// Split FFT(x + i y) into the half spectra of x and y at index k (F has n entries).
template <typename T>
__device__ __forceinline__ void unpack_spec(const cplx<T>* F, int k, int n, cplx<T>& X, cplx<T>& Y) {
  const cplx<T> a = F[k], b = F[k == 0 ? 0 : n - k];
  X = mk<T>((a.x + b.x) * (T)0.5, (a.y - b.y) * (T)0.5);
  Y = mk<T>((a.y + b.y) * (T)0.5, (b.x - a.x) * (T)0.5);
}
// the same on a padded shared-memory transform
template <typename T>
__device__ __forceinline__ void unpack_pad(const cplx<T>* F, int k, int n, cplx<T>& X, cplx<T>& Y) {
  const cplx<T> a = F[pad_idx(k)], b = F[pad_idx(k == 0 ? 0 : n - k)];
  X = mk<T>((a.x + b.x) * (T)0.5, (a.y - b.y) * (T)0.5);
  Y = mk<T>((a.y + b.y) * (T)0.5, (b.x - a.x) * (T)0.5);
}

// ===========================================================================
// Phase A, kernel 2: rows — physical products of convol_waqg / refraction_waqg
// ===========================================================================
template <typename T, int N>
__global__ void __launch_bounds__(kThreadsB)
k_row_main(Geom g, StepParams sp, cplx<T>* __restrict__ S, const cplx<T>* __restrict__ twg) {
  constexpr int RT = Tiles<T, N>::RT, LD = Tiles<T, N>::LD, NT = kThreadsB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bA = tw + N;                 // [RT][3][LD]: (u,v), (zeta,q), (br,bi)
  cplx<T>* bC = bA + 3 * RT * LD;       // [RT][4][LD]: products
  const int tid = threadIdx.x;
  const int zb = blockIdx.y;
  const int y0 = blockIdx.x * RT;
  const int K = g.K;
  load_tw<T, N>(tw, twg, NT);
#pragma unroll 4
  for (int e = tid; e < 3 * RT * N; e += NT) {
    const int k = e % N, p = (e / N) % 3, rr = e / (3 * N);
    const int y = y0 + rr;
    const cplx<T>* X = S + scr_off(zb, 2 * p, y, N, g.KXP);
    const cplx<T>* Y = S + scr_off(zb, 2 * p + 1, y, N, g.KXP);
    bA[(rr * 3 + p) * LD + pad_idx(k)] = pack_spec<T>(X, Y, k, N, K);
  }
  __syncthreads();
  fft_ip<T, N, false, 3 * RT, NT>(bA, tw);
  // products: (u q, v q), (u br, v br), (u bi, v bi), (zeta br, zeta bi)
#pragma unroll 4
  for (int e = tid; e < RT * N; e += NT) {
    const int x = e % N, rr = e / N;
    const int px = pad_idx(x);
    const cplx<T> uv = bA[(rr * 3 + 0) * LD + px];
    const cplx<T> zq = bA[(rr * 3 + 1) * LD + px];
    const cplx<T> bb = bA[(rr * 3 + 2) * LD + px];
    bC[(rr * 4 + 0) * LD + px] = mk<T>(uv.x * zq.y, uv.y * zq.y);
    bC[(rr * 4 + 1) * LD + px] = mk<T>(uv.x * bb.x, uv.y * bb.x);
    bC[(rr * 4 + 2) * LD + px] = mk<T>(uv.x * bb.y, uv.y * bb.y);
    bC[(rr * 4 + 3) * LD + px] = mk<T>(zq.x * bb.x, zq.x * bb.y);
  }
  __syncthreads();
  fft_ip<T, N, true, 4 * RT, NT>(bC, tw);
  const T adv = sp.adv ? (T)1 : (T)0;
  const T half = sp.refr ? (T)0.5 : (T)0;
  for (int e = tid; e < RT * (K + 1); e += NT) {
    const int k = e % (K + 1), rr = e / (K + 1);
    const int y = y0 + rr;
    cplx<T> uq, vq, ubr, vbr, ubi, vbi, zbr, zbi;
    unpack_pad<T>(bC + (rr * 4 + 0) * LD, k, N, uq, vq);
    unpack_pad<T>(bC + (rr * 4 + 1) * LD, k, N, ubr, vbr);
    unpack_pad<T>(bC + (rr * 4 + 2) * LD, k, N, ubi, vbi);
    unpack_pad<T>(bC + (rr * 4 + 3) * LD, k, N, zbr, zbi);
    const T kx = (T)k;
    // G = i kx F(uX) (+- refraction), H = F(vX); tendency = F_y(G) + i ky F_y(H)
    S[scr_off(zb, 0, y, N, g.KXP) + k] = cscale(cmul_i(uq), kx * adv);
    S[scr_off(zb, 1, y, N, g.KXP) + k] = cscale(vq, adv);
    S[scr_off(zb, 2, y, N, g.KXP) + k] = csub(cscale(cmul_i(ubr), kx * adv), cscale(zbi, half));
    S[scr_off(zb, 3, y, N, g.KXP) + k] = cscale(vbr, adv);
    S[scr_off(zb, 4, y, N, g.KXP) + k] = cadd(cscale(cmul_i(ubi), kx * adv), cscale(zbr, half));
    S[scr_off(zb, 5, y, N, g.KXP) + k] = cscale(vbi, adv);
  }
}

// Pointers of the state fields used by the update
template <typename T> struct StateP {
  cplx<T>* q; cplx<T>* qo; cplx<T>* BR; cplx<T>* BI; cplx<T>* BRo; cplx<T>* BIo;
  cplx<T>* psi; cplx<T>* AR; cplx<T>* AI; cplx<T>* qstar; const cplx<T>* dq;
};

// ===========================================================================
// Phase A, kernel 3: y-forward FFTs, time update, y-inverse FFTs for q^w
// ===========================================================================
template <typename T, int N>
__global__ void __launch_bounds__(kColThreads, 2)
k_col_update(Geom g, StepParams sp, int zbase, StateP<T> st, const T* __restrict__ e1t, const T* __restrict__ e2t,
             const T* __restrict__ e1wt, const T* __restrict__ e2wt, cplx<T>* __restrict__ S,
             const cplx<T>* __restrict__ twg, int qw_prep) {
  constexpr int CT = Tiles<T, N>::CT, LD = Tiles<T, N>::LD, NT = kColThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + N;                 // [6][CT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  const int KY = g.KY;
  load_tw<T, N>(tw, twg, NT);
#pragma unroll 4
  for (int e = tid; e < 6 * CT * N; e += NT) {
    const int c = e % CT, y = (e / CT) % N, h = e / (CT * N);
    const int kx = kx0 + c;
    buf[(h * CT + c) * LD + pad_idx(y)] = kx <= g.K ? S[scr_off(zb, h, y, N, g.KXP) + kx] : mk<T>(0, 0);
  }
  __syncthreads();
  fft_ip<T, N, true, 3 * CT, NT>(buf, tw);
  fft_ip<T, N, true, 3 * CT, NT>(buf + 3 * CT * LD, tw);
  // tendencies and time update (main_waqg.f90:237-264, 362-415)
  const T inv_n2 = (T)1 / ((T)N * (T)N);
  const long long zoff = (long long)z * g.plane;
  const T dt = (T)sp.delt;
  const T gam = (T)sp.gamma;
  const T cdisp = sp.disp ? (T)sp.cdisp : (T)0;
  for (int e = tid; e < 3 * CT * KY; e += NT) {
    const int c = e % CT, r = (e / CT) % KY, X = e / (CT * KY);
    const int kx = kx0 + c;
    if (kx > g.K) continue;
    const int ky = g.ky_of_row(r);
    const int j = pad_idx(g.fft_index_of_row(r));
    const cplx<T> G = buf[((2 * X) * CT + c) * LD + j];
    const cplx<T> H = buf[((2 * X + 1) * CT + c) * LD + j];
    const cplx<T> tend = cscale(mk<T>(G.x - (T)ky * H.y, G.y + (T)ky * H.x), inv_n2);   // G + i ky H
    const long long m = zoff + (long long)r * g.KXP + kx;
    const long long mt = (long long)r * g.KXP + kx;
    const bool L = g.mask(kx, ky);
    const T kh2 = (T)(kx * kx + ky * ky);
    cplx<T>* cur = X == 0 ? st.q : (X == 1 ? st.BR : st.BI);
    cplx<T>* old = X == 0 ? st.qo : (X == 1 ? st.BRo : st.BIo);
    const cplx<T> xc = cur[m];
    const cplx<T> xo = sp.euler ? xc : old[m];
    cplx<T> xn = mk<T>(0, 0), xf = mk<T>(0, 0);
    if (L) {
      if (X == 0) {
        const T e1 = e1t[mt], e2 = e2t[mt];
        const cplx<T> dqv = sp.use_dq ? st.dq[m] : mk<T>(0, 0);
        if (sp.euler) {
          xn = cscale(cadd(csub(xo, cscale(tend, dt)), cscale(dqv, dt)), e1);
        } else {
          xn = cadd(csub(cscale(xo, e2), cscale(cscale(tend, (T)2 * dt), e1)), cscale(cscale(dqv, (T)2 * dt), e2));
        }
      } else {
        const T e1 = e1wt[mt], e2 = e2wt[mt];
        // BR: tend_BR + c kh2 AI ; BI: tend_BI - c kh2 AR
        const cplx<T> Av = X == 1 ? st.AI[m] : st.AR[m];
        const T sgn = X == 1 ? (T)1 : (T)-1;
        const cplx<T> full = cadd(tend, cscale(Av, sgn * cdisp * kh2));
        if (sp.euler) {
          xn = cscale(csub(xo, cscale(full, dt)), e1);
        } else {
          xn = csub(cscale(xo, e2), cscale(cscale(full, (T)2 * dt), e1));
        }
      }
      if (sp.euler) {
        xf = xo;      // old level <- current (main_waqg.f90:232-234)
      } else {        // Robert-Asselin filter (main_waqg.f90:395-410)
        xf = cadd(xc, cscale(cadd(csub(xo, cscale(xc, (T)2)), xn), gam));
      }
    } else if (sp.euler) {
      xf = xo;
    }
    cur[m] = xn;
    old[m] = xf;
  }
  if (!qw_prep) return;
  __syncthreads();   // this CTA's writes of BR, BI are visible to it after the barrier
  // y-inverse FFTs of BR, i ky BR, BI, i ky BI at n+1 (compute_qw, derivatives.f90:929-957)
#pragma unroll 4
  for (int e = tid; e < 4 * CT * N; e += NT) {
    const int c = e % CT, j = (e / CT) % N, f = e / (CT * N);
    const int kx = kx0 + c;
    const int r = g.row_of_fft_index(j);
    cplx<T> v = mk<T>(0, 0);
    if (kx <= g.K && r >= 0) {
      const cplx<T> s = (f < 2 ? st.BR : st.BI)[zoff + (long long)r * g.KXP + kx];
      v = (f & 1) ? cscale(cmul_i(s), (T)g.ky_of_row(r)) : s;
    }
    buf[(f * CT + c) * LD + pad_idx(j)] = v;
  }
  __syncthreads();
  if (kx0 == 0) {
    for (int e = tid; e < 4 * (N / 2 - 1); e += NT) {
      const int f = e / (N / 2 - 1), j = 1 + e % (N / 2 - 1);
      cplx<T>* col = buf + f * CT * LD;
      col[pad_idx(N - j)] = cconj(col[pad_idx(j)]);
    }
    __syncthreads();
  }
  fft_ip<T, N, false, 2 * CT, NT>(buf, tw);
  fft_ip<T, N, false, 2 * CT, NT>(buf + 2 * CT * LD, tw);
#pragma unroll 4
  for (int e = tid; e < 4 * CT * N; e += NT) {
    const int c = e % CT, y = (e / CT) % N, f = e / (CT * N);
    S[scr_off(zb, f, y, N, g.KXP) + kx0 + c] = buf[(f * CT + c) * LD + pad_idx(y)];
  }
}

// ===========================================================================
// Phase A, kernel 4: rows — products of compute_qw
// ===========================================================================
template <typename T, int N>
__global__ void __launch_bounds__(kThreadsB)
k_row_qw(Geom g, cplx<T>* __restrict__ S, const cplx<T>* __restrict__ twg) {
  constexpr int RT = Tiles<T, N>::RT, LD = Tiles<T, N>::LD, NT = kThreadsB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bA = tw + N;               // [RT][3][LD]
  cplx<T>* bC = bA + 3 * RT * LD;     // [RT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y;
  const int y0 = blockIdx.x * RT;
  const int K = g.K;
  load_tw<T, N>(tw, twg, NT);
  // packed: (BR, BI), (BRx, BIx), (BRy, BIy)
#pragma unroll 4
  for (int e = tid; e < 3 * RT * N; e += NT) {
    const int k = e % N, p = (e / N) % 3, rr = e / (3 * N);
    const int y = y0 + rr;
    const cplx<T>* sBR = S + scr_off(zb, 0, y, N, g.KXP);
    const cplx<T>* sBRy = S + scr_off(zb, 1, y, N, g.KXP);
    const cplx<T>* sBI = S + scr_off(zb, 2, y, N, g.KXP);
    const cplx<T>* sBIy = S + scr_off(zb, 3, y, N, g.KXP);
    cplx<T> v;
    if (p == 0) {
      v = pack_spec<T>(sBR, sBI, k, N, K);
    } else if (p == 2) {
      v = pack_spec<T>(sBRy, sBIy, k, N, K);
    } else if (k == 0 || (k > K && k < N - K)) {
      v = mk<T>(0, 0);      // x-derivatives vanish at kx = 0
    } else {
      const int kk = k <= K ? k : N - k;
      const cplx<T> a = cscale(cmul_i(sBR[kk]), (T)kk), b = cscale(cmul_i(sBI[kk]), (T)kk);
      v = k <= K ? mk<T>(a.x - b.y, a.y + b.x) : mk<T>(a.x + b.y, b.x - a.y);
    }
    bA[(rr * 3 + p) * LD + pad_idx(k)] = v;
  }
  __syncthreads();
  fft_ip<T, N, false, 3 * RT, NT>(bA, tw);
#pragma unroll 4
  for (int e = tid; e < RT * N; e += NT) {
    const int x = e % N, rr = e / N;
    const int px = pad_idx(x);
    const cplx<T> b = bA[(rr * 3 + 0) * LD + px];    // (br, bi)
    const cplx<T> bx = bA[(rr * 3 + 1) * LD + px];   // (brx, bix)
    const cplx<T> by = bA[(rr * 3 + 2) * LD + px];   // (bry, biy)
    const T p1 = by.x * bx.y - bx.x * by.y;           // BRy BIx - BRx BIy (derivatives.f90:973)
    const T p2 = b.x * b.x + b.y * b.y;               // BR^2 + BI^2     (derivatives.f90:996)
    bC[rr * LD + px] = mk<T>(p1, p2);
  }
  __syncthreads();
  fft_ip<T, N, true, RT, NT>(bC, tw);
  for (int e = tid; e < RT * (K + 1); e += NT) {
    const int k = e % (K + 1), rr = e / (K + 1);
    const int y = y0 + rr;
    cplx<T> P1, P2;
    unpack_pad<T>(bC + rr * LD, k, N, P1, P2);
    const T qk = (T)0.25 * (T)(k * k);
    S[scr_off(zb, 0, y, N, g.KXP) + k] = csub(P1, cscale(P2, qk));
    S[scr_off(zb, 1, y, N, g.KXP) + k] = P2;
  }
}

// ===========================================================================
// Phase A, kernel 5: y-forward FFTs of the q^w planes, q* = q - q^w
// ===========================================================================
template <typename T, int N>
__global__ void __launch_bounds__(kThreadsB)
k_col_qw(Geom g, StepParams sp, int zbase, const cplx<T>* __restrict__ q, cplx<T>* __restrict__ qstar,
         const cplx<T>* __restrict__ S, const cplx<T>* __restrict__ twg) {
  constexpr int CT = Tiles<T, N>::CT, LD = Tiles<T, N>::LD, NT = kThreadsB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* buf = tw + N;                 // [2][CT][LD]
  const int tid = threadIdx.x;
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  const int KY = g.KY;
  load_tw<T, N>(tw, twg, NT);
#pragma unroll 4
  for (int e = tid; e < 2 * CT * N; e += NT) {
    const int c = e % CT, y = (e / CT) % N, h = e / (CT * N);
    const int kx = kx0 + c;
    buf[(h * CT + c) * LD + pad_idx(y)] = kx <= g.K ? S[scr_off(zb, h, y, N, g.KXP) + kx] : mk<T>(0, 0);
  }
  __syncthreads();
  fft_ip<T, N, true, 2 * CT, NT>(buf, tw);
  const T inv_n2 = (T)1 / ((T)N * (T)N);
  const T s = (T)sp.Ro * (T)sp.W2F;
  const long long zoff = (long long)z * g.plane;
  for (int e = tid; e < CT * KY; e += NT) {
    const int c = e % CT, r = e / CT;
    const int kx = kx0 + c;
    if (kx > g.K) continue;
    const int ky = g.ky_of_row(r);
    const int j = pad_idx(g.fft_index_of_row(r));
    const long long m = zoff + (long long)r * g.KXP + kx;
    cplx<T> out = mk<T>(0, 0);
    if (g.mask(kx, ky)) {
      const cplx<T> R = csub(buf[c * LD + j], cscale(buf[(CT + c) * LD + j], (T)0.25 * (T)ky * (T)ky));
      const cplx<T> qw = cscale(cscale(R, inv_n2), s);
      out = csub(q[m], qw);       // q* = q - q^w (main_waqg.f90:430-439)
    }
    qstar[m] = out;
  }
}

// q* = q where the feedback is off (no_feedback == 1)
template <typename T>
__global__ void k_copy_field(const cplx<T>* __restrict__ a, cplx<T>* __restrict__ b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = a[i];
}

// dissipation_q_nv (derivatives.f90:1877-1926): nuz * d2q/dz2 of the old level
template <typename T>
__global__ void k_dissipation(Geom g, double nuz, double dz, const cplx<T>* __restrict__ qo, cplx<T>* __restrict__ dq) {
  const long long tot = (long long)g.n3 * g.plane;
  const T c = (T)(nuz / (dz * dz));
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / g.plane);
    const long long m = i - (long long)z * g.plane;
    const int r = (int)(m / g.KXP), kx = (int)(m % g.KXP);
    cplx<T> v = mk<T>(0, 0);
    if (g.mask(kx, g.ky_of_row(r))) {
      const cplx<T> q0 = qo[i];
      if (z == 0) {
        v = cscale(csub(qo[i + g.plane], q0), c);
      } else if (z == g.n3 - 1) {
        v = cscale(csub(qo[i - g.plane], q0), c);
      } else {
        v = cscale(cadd(csub(qo[i + g.plane], cscale(q0, (T)2)), qo[i - g.plane]), c);
      }
    }
    dq[i] = v;
  }
}

// ===========================================================================
// Phase B: FP64 tridiagonal solves per (kx,ky) column (elliptic.f90:145-460)
// ===========================================================================
// fac[idx*n3 + i] = {f_i = dl_i/d'_i, p_i} of DGTSV's elimination for the
// distinct kh^2 row idx; du[i] = rho_ut(i)*a(i)/rho_st(i).
//   EXACT (FP64 path): p_i = d'_i, and every operation is the correctly
//     rounded IEEE operation of DGTSV (no contraction, true division), so
//     the solve reproduces LAPACK's reference DGTSV bit for bit.
//   fast (mixed path): p_i = 1/d'_i, fused multiply-adds.
template <bool EXACT>
struct Tri {
  static __device__ __forceinline__ double fwd(double b, double f, double bp) {
    return EXACT ? __dsub_rn(b, __dmul_rn(f, bp)) : fma(-f, bp, b);
  }
  static __device__ __forceinline__ double back(double b, double u, double x, double p) {
    return EXACT ? __ddiv_rn(__dsub_rn(b, __dmul_rn(u, x)), p) : fma(-u, x, b) * p;
  }
  static __device__ __forceinline__ double last(double b, double p) { return EXACT ? __ddiv_rn(b, p) : b * p; }
};

template <typename T>
__global__ void __launch_bounds__(128)
k_solve(Geom g, double dz, double Bu, const int* __restrict__ tab_idx,
        const double2* __restrict__ fac_psi, const double2* __restrict__ fac_A, const double* __restrict__ du,
        const cplx<T>* __restrict__ qs, const cplx<T>* __restrict__ BR, const cplx<T>* __restrict__ BI,
        cplx<T>* __restrict__ psi, cplx<T>* __restrict__ AR, cplx<T>* __restrict__ AI,
        double2* __restrict__ bscr, int do_psi, int do_A) {
  using Op = Tri<sizeof(T) == 8>;
  const long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (m >= g.plane) return;
  const int kx = (int)(m % g.KXP);
  if (kx > g.K) return;
  const int n3 = g.n3;
  const long long P = g.plane;
  const int idx = tab_idx[m];
  if (idx < 0) {
    for (int i = 0; i < n3; ++i) {
      if (do_psi) psi[i * P + m] = mk<T>(0, 0);
      if (do_A) { AR[i * P + m] = mk<T>(0, 0); AI[i * P + m] = mk<T>(0, 0); }
    }
    return;
  }
  if (do_psi) {
    const double2* F = fac_psi + (long long)idx * n3;
    const double s = __dmul_rn(dz, dz);
    cplx<T> v = qs[m];
    double br = __dmul_rn(s, (double)v.x), bi = __dmul_rn(s, (double)v.y);
    bscr[m] = make_double2(br, bi);
    for (int i = 1; i < n3; ++i) {
      const double f = F[i - 1].x;
      v = qs[i * P + m];
      br = Op::fwd(__dmul_rn(s, (double)v.x), f, br);
      bi = Op::fwd(__dmul_rn(s, (double)v.y), f, bi);
      bscr[i * P + m] = make_double2(br, bi);
    }
    double xr = Op::last(br, F[n3 - 1].y), xi = Op::last(bi, F[n3 - 1].y);
    psi[(n3 - 1) * P + m] = mk<T>((T)xr, (T)xi);
    for (int i = n3 - 2; i >= 0; --i) {
      const double2 b = bscr[i * P + m];
      const double p = F[i].y, u = du[i];
      xr = Op::back(b.x, u, xr, p);
      xi = Op::back(b.y, u, xi, p);
      psi[i * P + m] = mk<T>((T)xr, (T)xi);
    }
  }
  if (do_A) {
    const double2* F = fac_A + (long long)idx * n3;
    const double s = __dmul_rn(__dmul_rn(dz, dz), Bu);
    cplx<T> vr = BR[m], vi = BI[m];
    double a0 = __dmul_rn(s, (double)vr.x), a1 = __dmul_rn(s, (double)vr.y);
    double b0 = __dmul_rn(s, (double)vi.x), b1 = __dmul_rn(s, (double)vi.y);
    bscr[m] = make_double2(a0, a1);
    bscr[n3 * P + m] = make_double2(b0, b1);
    for (int i = 1; i < n3; ++i) {
      const double f = F[i - 1].x;
      vr = BR[i * P + m]; vi = BI[i * P + m];
      a0 = Op::fwd(__dmul_rn(s, (double)vr.x), f, a0); a1 = Op::fwd(__dmul_rn(s, (double)vr.y), f, a1);
      b0 = Op::fwd(__dmul_rn(s, (double)vi.x), f, b0); b1 = Op::fwd(__dmul_rn(s, (double)vi.y), f, b1);
      bscr[i * P + m] = make_double2(a0, a1);
      bscr[(n3 + i) * P + m] = make_double2(b0, b1);
    }
    const double pn = F[n3 - 1].y;
    a0 = Op::last(a0, pn); a1 = Op::last(a1, pn); b0 = Op::last(b0, pn); b1 = Op::last(b1, pn);
    AR[(n3 - 1) * P + m] = mk<T>((T)a0, (T)a1);
    AI[(n3 - 1) * P + m] = mk<T>((T)b0, (T)b1);
    for (int i = n3 - 2; i >= 0; --i) {
      const double2 x = bscr[i * P + m], y = bscr[(n3 + i) * P + m];
      const double p = F[i].y, u = du[i];
      a0 = Op::back(x.x, u, a0, p); a1 = Op::back(x.y, u, a1, p);
      b0 = Op::back(y.x, u, b0, p); b1 = Op::back(y.y, u, b1, p);
      AR[i * P + m] = mk<T>((T)a0, (T)a1);
      AI[i * P + m] = mk<T>((T)b0, (T)b1);
    }
  }
}

// ===========================================================================
// Conversions between the reference layout and the compact layout
// ===========================================================================
// dense: double2 [nlev][ikty][iktx]
template <typename T>
static __global__ void k_dense_to_compact(Geom g, int level0, int nlev, const double2* __restrict__ dense, cplx<T>* __restrict__ f) {
  const int iktx = g.n / 2 + 1;
  const long long tot = (long long)nlev * g.plane;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(i / g.plane);
    const long long m = i - (long long)l * g.plane;
    const int r = (int)(m / g.KXP), kx = (int)(m % g.KXP);
    const int ky = g.ky_of_row(r);
    cplx<T> v = mk<T>(0, 0);
    if (g.mask(kx, ky)) {
      const int iky = ky >= 0 ? ky : g.n + ky;
      const double2 d = dense[((long long)l * g.n + iky) * iktx + kx];
      v = mk<T>((T)d.x, (T)d.y);
    }
    f[(long long)(level0 + l) * g.plane + m] = v;
  }
}

// mode: 0 plain copy, 1 vertical difference (A_z, elliptic.f90:437-450)
template <typename T>
__global__ void k_compact_to_dense(Geom g, int level0, int nlev, const cplx<T>* __restrict__ f, double2* __restrict__ dense,
                                   int mode, double dz) {
  const int iktx = g.n / 2 + 1;
  const long long per = (long long)g.n * iktx;
  const long long tot = (long long)nlev * per;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(i / per);
    const long long m = i - (long long)l * per;
    const int iky = (int)(m / iktx), kx = (int)(m % iktx);
    const int ky = iky < g.n / 2 ? iky : (iky == g.n / 2 ? 0 : iky - g.n);
    double2 v = make_double2(0.0, 0.0);
    if (iky != g.n / 2 && kx <= g.K && ky >= -g.K && ky <= g.K) {
      const int z = level0 + l;
      const long long c = (long long)g.row_of_ky(ky) * g.KXP + kx;
      if (mode == 0) {
        const cplx<T> a = f[(long long)z * g.plane + c];
        v = make_double2((double)a.x, (double)a.y);
      } else if (z < g.n3 - 1) {
        const cplx<T> a = f[(long long)z * g.plane + c], b = f[(long long)(z + 1) * g.plane + c];
        v = make_double2(((double)b.x - (double)a.x) / dz, ((double)b.y - (double)a.y) / dz);
      }
    }
    dense[i] = v;
  }
}

// ===========================================================================
// Initialisation helpers (once per run)
// ===========================================================================
// sumB (derivatives.f90:1073-1118): remove the vertical mean of B where kh>0.
template <typename T>
__global__ void k_sumB(Geom g, cplx<T>* __restrict__ BR, cplx<T>* __restrict__ BI) {
  const long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (m >= g.plane) return;
  const int r = (int)(m / g.KXP), kx = (int)(m % g.KXP);
  const int ky = g.ky_of_row(r);
  if (!g.mask(kx, ky) || kx * kx + ky * ky == 0) return;
  double sr0 = 0, sr1 = 0, si0 = 0, si1 = 0;
  for (int z = 0; z < g.n3; ++z) {
    const cplx<T> a = BR[z * g.plane + m], b = BI[z * g.plane + m];
    sr0 += a.x; sr1 += a.y; si0 += b.x; si1 += b.y;
  }
  sr0 /= g.n3; sr1 /= g.n3; si0 /= g.n3; si1 /= g.n3;
  for (int z = 0; z < g.n3; ++z) {
    cplx<T> a = BR[z * g.plane + m], b = BI[z * g.plane + m];
    a.x = (T)((double)a.x - sr0); a.y = (T)((double)a.y - sr1);
    b.x = (T)((double)b.x - si0); b.y = (T)((double)b.y - si1);
    BR[z * g.plane + m] = a; BI[z * g.plane + m] = b;
  }
}

// init_q (init.f90:591-652): q = [d/dz(a dpsi/dz) - kh^2 psi] with Neumann
// ends, evaluated in FP64 in the reference's order with correctly rounded
// operations and no contraction: the terms a*psi (a up to ~e^10 under
// strong stratification) cancel, so the rounding sequence matters.
template <typename T, typename TI>
__global__ void k_init_q(Geom g, double dz, const double* __restrict__ cu, const double* __restrict__ cl,
                         const cplx<TI>* __restrict__ psi, cplx<T>* __restrict__ q) {
  const long long tot = (long long)g.n3 * g.plane;
  const double dz2 = __dmul_rn(dz, dz);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / g.plane);
    const long long m = i - (long long)z * g.plane;
    const int r = (int)(m / g.KXP), kx = (int)(m % g.KXP);
    const int ky = g.ky_of_row(r);
    cplx<T> out = mk<T>(0, 0);
    if (g.mask(kx, ky)) {
      const double kdz = __dmul_rn(__dmul_rn((double)(kx * kx + ky * ky), dz), dz);
      const cplx<TI> p0 = psi[i];
      double vr, vi;
      if (z == 0) {
        const cplx<TI> pp = psi[i + g.plane];
        const double d = __dadd_rn(cu[0], kdz);
        vr = __dsub_rn(__dmul_rn(cu[0], (double)pp.x), __dmul_rn(d, (double)p0.x));
        vi = __dsub_rn(__dmul_rn(cu[0], (double)pp.y), __dmul_rn(d, (double)p0.y));
      } else if (z == g.n3 - 1) {
        const cplx<TI> pm = psi[i - g.plane];
        const double d = __dadd_rn(cl[z], kdz);
        vr = __dadd_rn(-__dmul_rn(d, (double)p0.x), __dmul_rn(cl[z], (double)pm.x));
        vi = __dadd_rn(-__dmul_rn(d, (double)p0.y), __dmul_rn(cl[z], (double)pm.y));
      } else {
        const cplx<TI> pp = psi[i + g.plane], pm = psi[i - g.plane];
        const double d = __dadd_rn(__dadd_rn(cu[z], cl[z]), kdz);
        vr = __dadd_rn(__dsub_rn(__dmul_rn(cu[z], (double)pp.x), __dmul_rn(d, (double)p0.x)),
                       __dmul_rn(cl[z], (double)pm.x));
        vi = __dadd_rn(__dsub_rn(__dmul_rn(cu[z], (double)pp.y), __dmul_rn(d, (double)p0.y)),
                       __dmul_rn(cl[z], (double)pm.y));
      }
      out = mk<T>((T)__ddiv_rn(vr, dz2), (T)__ddiv_rn(vi, dz2));
    }
    q[i] = out;
  }
}

// ===========================================================================
// FP64 diagnostics: per-level partial sums, then a fixed-order vertical sum
// ===========================================================================
constexpr int kNDiag = 7;
template <typename T>
__global__ void __launch_bounds__(256)
k_diag_level(Geom g, double dz, double Bu, const double* __restrict__ r2, const cplx<T>* __restrict__ BR,
             const cplx<T>* __restrict__ BI, const cplx<T>* __restrict__ AR, const cplx<T>* __restrict__ AI,
             const cplx<T>* __restrict__ psi, double* __restrict__ part) {
  __shared__ double red[kNDiag][256];
  const int z = blockIdx.x;
  const long long zo = (long long)z * g.plane;
  const bool top = (z == g.n3 - 1);
  const double rz = r2[z];
  double acc[kNDiag] = {0, 0, 0, 0, 0, 0, 0};
  for (long long m = threadIdx.x; m < g.plane; m += blockDim.x) {
    const int r = (int)(m / g.KXP), kx = (int)(m % g.KXP);
    const int ky = g.ky_of_row(r);
    if (!g.mask(kx, ky)) continue;
    const double kh2 = (double)(kx * kx + ky * ky);
    const double w00 = (kx == 0 && ky == 0) ? 0.5 : 1.0;
    const cplx<T> br = BR[zo + m], bi = BI[zo + m], ar = AR[zo + m], ai = AI[zo + m], p = psi[zo + m];
    const double b2 = (double)br.x * br.x + (double)br.y * br.y + (double)bi.x * bi.x + (double)bi.y * bi.y;
    acc[0] += w00 * b2;
    double c2 = 0.0, pz2 = 0.0;
    if (!top) {
      const cplx<T> ar1 = AR[zo + g.plane + m], ai1 = AI[zo + g.plane + m], p1 = psi[zo + g.plane + m];
      const double crx = ((double)ar1.x - ar.x) / dz, cry = ((double)ar1.y - ar.y) / dz;
      const double cix = ((double)ai1.x - ai.x) / dz, ciy = ((double)ai1.y - ai.y) / dz;
      c2 = crx * crx + cry * cry + cix * cix + ciy * ciy;
      const double bx = ((double)p1.x - p.x) / dz, by = ((double)p1.y - p.y) / dz;
      pz2 = bx * bx + by * by;
    }
    acc[1] += (0.5 / (rz * Bu)) * kh2 * c2;
    const double a2 = (double)ar.x * ar.x + (double)ar.y * ar.y + (double)ai.x * ai.x + (double)ai.y * ai.y;
    acc[2] += (1.0 / 8.0) * (1.0 / (Bu * Bu)) * kh2 * kh2 * a2;
    const double ps2 = (double)p.x * p.x + (double)p.y * p.y;
    acc[3] += kh2 * ps2;
    acc[4] += w00 * (Bu / rz) * pz2;
    acc[5] += 2.0 * kh2 * kh2 * ps2;
    acc[6] += 2.0 * kh2 * pz2;
  }
  for (int k = 0; k < kNDiag; ++k) red[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int k = 0; k < kNDiag; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < kNDiag) part[z * kNDiag + threadIdx.x] = red[threadIdx.x][0];
}

static __global__ void k_diag_sum(int n3, const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x < kNDiag) {
    double s = 0.0;
    for (int z = 0; z < n3; ++z) s += part[z * kNDiag + threadIdx.x];
    out[threadIdx.x] = s / n3;
  }
}

}  // namespace qg
