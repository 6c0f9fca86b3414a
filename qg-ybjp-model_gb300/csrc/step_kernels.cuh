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
#include <type_traits>
#include "common.cuh"
#include "fft_block.cuh"
#include "colfft.cuh"
#include "bulk_copy.cuh"

namespace qg {

constexpr int kThreads = 256;
constexpr int kNScr = 6;  // scratch (kx,y) planes per level

template <typename T> struct Tile;
template <> struct Tile<float> { static constexpr int CT = 8; static constexpr int RT = 2; };
template <> struct Tile<double> { static constexpr int CT = 4; static constexpr int RT = 1; };

__host__ __device__ __forceinline__ long long scr_off(int zb, int f, int y, int n, int KXP) {
  return (((long long)zb * kNScr + f) * n + y) * KXP;
}
// The y-inverse transforms of B^{n+1} that k_col_update computes for q^w are
// those of the next step's B^n: with kReuseB they are kept for every level in
// Q[z][2][n][KXP] (BR, BI), read by the next step's k_row_main and by
// k_row_qw, and k_col_inv transforms only u, v, zeta and q.
constexpr int kNQ = 2;
__host__ __device__ __forceinline__ long long q_off(int zb, int f, int y, int n, int KXP) {
  return (((long long)zb * kNQ + f) * n + y) * KXP;
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
// CTAs per SM the register budgets of the FP32 kernels target (FP64
// kernels: at most 2); shared memory caps them further per shape
constexpr int kRowMinB = 4;        // k_row_main, k_row_qw
constexpr int kRowThreads = 256;   // threads of k_row_main, k_row_qw
constexpr int kRowRT = 0;          // rows per CTA of k_row_main, k_row_qw (0: Tiles RT)
constexpr int kRowQwThreads = 128; // k_row_qw: half the threads of k_row_main, twice the CTAs
constexpr int kRowQwMinB = 5;
#ifndef QG_COLINV_NF2
#define QG_COLINV_NF2 1
#endif
// k_col_inv (FP32): the six transforms as three passes of two instead of two
// of three (80 registers instead of 128: 3 CTAs per SM; 0.536 -> 0.496 ms at
// 512^2 x 256)
constexpr bool kColInvNF2 = QG_COLINV_NF2 != 0;
#ifndef QG_COLINV_MINB
#define QG_COLINV_MINB 3
#endif
constexpr int kColInvMinB = QG_COLINV_MINB;     // k_col_inv
#ifndef QG_COLQW_MINB
#define QG_COLQW_MINB 4
#endif
constexpr int kColQwMinB = QG_COLQW_MINB;      // k_col_qw
constexpr bool kRowPass0 = true;   // row kernels: first inverse pass fed from registers
constexpr bool kRowFuse = true;    // k_row_main: inverse last pass, products, forward first pass in registers
constexpr int kRowMainMinB = 2;    // k_row_main CTAs per SM when fused
constexpr bool kRowPrefetch = true; // fused row kernels: persistent, next item's rows bulk-copied ahead
constexpr bool kRowSwizzle = true;  // k_row_qw (N = 512): conflict-free XOR placement (lay_idx<1>)
#ifndef QG_ROWMAIN_SWZ
#define QG_ROWMAIN_SWZ 0
#endif
constexpr bool kRowMainSwizzle = QG_ROWMAIN_SWZ != 0;  // k_row_main: the same (its index arithmetic spills at 128 registers)
#ifndef QG_ROWMAIN_MIDSWZ
#define QG_ROWMAIN_MIDSWZ 1
#endif
constexpr bool kRowMainMidSwz = QG_ROWMAIN_MIDSWZ != 0;   // k_row_main forward transforms: XOR placement between the last two passes (0.965 -> 0.921 ms at 512^2 x 256 with the last pass in registers)
#ifndef QG_ROWMAIN_MIDSWZI
#define QG_ROWMAIN_MIDSWZI 1
#endif
constexpr bool kRowMainMidSwzInv = QG_ROWMAIN_MIDSWZI != 0;
#ifndef QG_ROWQW_MIDSWZ
#define QG_ROWQW_MIDSWZ 1
#endif
constexpr bool kRowQwMidSwz = QG_ROWQW_MIDSWZ != 0;   // k_row_qw (N = 256, 128): the mid-pass hand-off in layout 2, 3  // the same for its inverse transforms (0.921 -> 0.907 ms)
#ifndef QG_ROW_SHFL_LAST
#define QG_ROW_SHFL_LAST 1
#endif
// fused row kernels (N = 512): last forward pass and spectrum split in registers (warp shuffles)
constexpr bool kRowShflLast = QG_ROW_SHFL_LAST != 0;
#ifndef QG_UPD_TABLES_SMEM
#define QG_UPD_TABLES_SMEM 1
#endif
constexpr bool kUpdTablesSmem = QG_UPD_TABLES_SMEM != 0;   // k_col_update (FP32 lean): IF tables staged in shared memory
constexpr bool kUpdLean = true;    // k_col_update (FP32): smaller shared footprint ...
constexpr bool kUpdStage16 = true; // k_col_update (FP32): state staged by 16-byte copies
#ifndef QG_UPD_MINB
#define QG_UPD_MINB 2
#endif
constexpr int kUpdMinB = QG_UPD_MINB;        // ... for this many CTAs per SM (3, with the tables read from global memory, measured slower)
__host__ __device__ constexpr int smem_ctas(int bytes) {
  return 233472 / (bytes + 1024) >= 8 ? 8 : (233472 / (bytes + 1024) >= 1 ? 233472 / (bytes + 1024) : 1);
}
__host__ __device__ constexpr int imin(int a, int b) { return a < b ? a : b; }
__host__ __device__ constexpr int imax(int a, int b) { return a > b ? a : b; }
// CTAs of `bytes` shared memory that fit on an SM, at most cap (<= 32)
__host__ __device__ constexpr int smem_ctas_cap(int bytes, int cap) {
  return 233472 / (bytes + 1024) >= cap ? cap : (233472 / (bytes + 1024) >= 1 ? 233472 / (bytes + 1024) : 1);
}

template <typename T, int N> struct Tiles {
  static constexpr int CB = (int)sizeof(cplx<T>);
  static constexpr int ct0 = (16384 / CB) / N;
  static constexpr int CT = ct0 >= 8 ? 8 : (ct0 >= 1 ? ct0 : 1);
  static constexpr int rt0 = (8192 / CB) / N;
  static constexpr int RT = rt0 >= 2 ? 2 : 1;
  // transform stride.  A warp filling or draining a column tile touches CT
  // columns x (32/CT) consecutive rows; with LD = 32/CT modulo the elements
  // of one 128-byte shared-memory wavefront (SLOTS), the columns' row runs
  // interleave and every bank slot is hit equally often (no replays beyond
  // the access width)
  static constexpr int SLOTS = 128 / CB;
  static constexpr int RW = 32 / CT;
  static constexpr int P0 = PadLD<N>::value;
  static constexpr int LD = P0 + ((RW % SLOTS) - (P0 % SLOTS) + SLOTS) % SLOTS;
  // CTAs per SM that the shared memory of a six-field column tile allows
  // (228 KB per SM, 1 KB reserved per CTA), the column kernels' occupancy target
  static constexpr int SM6 = (N + 6 * CT * LD) * CB;
  static constexpr int mb0 = 233472 / (SM6 + 1024);
  static constexpr int MINB = mb0 >= 4 ? 4 : (mb0 >= 1 ? mb0 : 1);
  static constexpr int FSC = ColLay<N, CT>::FS;      // interleaved column tile (colfft.cuh)
  // column layouts of the three column kernels (colfft.cuh col_idx: 16 or 8
  // = one pad every 16 or 8 elements, 0 = XOR placement), chosen by timing
  // the 512^2 x 256 step and the C3 ensemble: k_col_inv pad 8 (0.325 ->
  // 0.300 ms; XOR spills), k_col_update XOR (1.063 -> 1.048 ms; with pad 8,
  // whose extra shared memory likely crosses a carve-out step: 1.10 ms),
  // k_col_qw pad 16 (XOR and pad 8 no faster); below N = 512 pad 16 (the
  // ensemble 0.5-1 % slower with the others)
  static constexpr int CIP = N >= 512 ? 8 : 16;
  static constexpr int CUP = N >= 512 ? 0 : 16;
  static constexpr int CQP = 16;
  static constexpr int FSCI = ColLay<N, CT, CIP>::FS;
  static constexpr int FSCQ = ColLay<N, CT, CQP>::FS;
  static constexpr int RRT = kRowRT > 0 ? kRowRT : RT;   // rows per CTA of the forward row kernels
  static constexpr int RMINB = imin(CB == 8 ? kRowMinB : 2, smem_ctas((N + 4 * RRT * LD) * CB));
  // rows per k_row_qw CTA: one (row, butterfly) task per thread where its
  // transforms can be fused in registers (below), else RRT
  static constexpr bool QFUSABLE = kRowFuse && CB == 8 && kRowPass0 && N >= 64 && N <= 512 &&
                                   LastNS<N>::value == N / radix_of(N) &&
                                   (CB == 8 ? kRowQwThreads : kRowThreads) % (N / radix_of(N)) == 0;
  static constexpr int QRT = QFUSABLE ? (CB == 8 ? kRowQwThreads : kRowThreads) / (N / radix_of(N)) : RRT;
  static constexpr int QMINB = imin(CB == 8 ? kRowQwMinB : 2, smem_ctas((N + 3 * QRT * LD) * CB));
  // FP32: the first inverse row pass fed from registers, k_row_qw on 128
  // threads; FP64 keeps the shared-memory fill and 256 threads (the
  // register-fed pass doubles its registers and halves its occupancy)
  static constexpr bool RPASS0 = kRowPass0 && CB == 8;
  static constexpr int QTHREADS = CB == 8 ? kRowQwThreads : kRowThreads;
  // k_row_main with the inverse last pass, the products and the forward first
  // pass in registers: needs the inverse's last radix to equal the forward's
  // first (N = 512: 8 x 8 x 8) and one (row, butterfly) task per thread
  static constexpr bool RFUSE = kRowFuse && RPASS0 && N >= 64 && N <= 512 && LastNS<N>::value == N / radix_of(N) &&
                                kRowThreads % (N / radix_of(N)) == 0;
  static constexpr int RTM = RFUSE ? kRowThreads / (N / radix_of(N)) : RRT;   // rows per k_row_main CTA
  static constexpr int MMINB = imin(CB == 8 ? (RFUSE ? kRowMainMinB : kRowMinB) : 2, smem_ctas((N + 4 * RTM * LD) * CB));
  // the same for k_row_qw (rows QRT, QTHREADS threads)
  static constexpr bool QFUSE = kRowFuse && RPASS0 && N >= 64 && N <= 512 && LastNS<N>::value == N / radix_of(N) &&
                                QRT * (N / radix_of(N)) == QTHREADS;
  // persistent row kernels that bulk-copy the next item's scratch rows into
  // shared memory during the current item (the fused FP32 row kernels)
  static constexpr bool RPRE = kRowPrefetch && RFUSE;
  static constexpr bool QPRE = kRowPrefetch && QFUSE;
  // element placement of the fused row kernels' transforms (lay_idx)
  static constexpr int RLAY = kRowMainSwizzle && RFUSE && N == 512 ? 1 : 0;
  // (the mid-pass hand-off layouts: 1 at N = 512, 2 at N = 256, 3 at N = 128)
  static constexpr int MIDL = N == 512 ? 1
                            : (N == 256 && LastNS<N>::value == 32 && radix_of(N) == 8) ? 2
                            : (N == 128 && LastNS<N>::value == 16 && radix_of(N) == 8) ? 3 : 0;
  static constexpr int RMID = !kRowMainSwizzle && kRowMainMidSwz && RFUSE ? MIDL : 0;
  static constexpr int RMIDI = !kRowMainSwizzle && kRowMainMidSwzInv && RFUSE ? MIDL : 0;
  static constexpr int QLAY = kRowSwizzle && QFUSE && N == 512 ? 1 : 0;
  static constexpr int QMID = kRowQwMidSwz && QFUSE && N < 512 ? MIDL : 0;   // k_row_qw at N = 256, 128
  // the forward transforms' last pass and the split of the packed spectra in
  // registers (colfft.cuh:row_last_fwd512): one row per 64 threads
  static constexpr bool RSHL = kRowShflLast && RFUSE && N == 512 && RTM * 64 == kRowThreads;
  static constexpr bool QSHL = kRowShflLast && QFUSE && N == 512 && QRT * 64 == QTHREADS;
  // threads of the column kernels: one per (column, butterfly) task of the
  // first pass (256 at N >= 256 in FP32; fewer for small N and in FP64,
  // where a 256-thread CTA left threads idle in every pass), with the CTAs
  // per SM scaled up by CSCALE so that the threads per SM stay the same
  static constexpr int CNT = imin(256, imax(32, CT * (N / radix_of(N))));
  static constexpr int CSCALE = 256 / CNT;
  // transforms in flight in k_col_inv: two per pass in FP32 (kColInvNF2), three in FP64
  static constexpr int CINF = (kColInvNF2 && CB == 8) ? 2 : 3;
  static constexpr int CIMINB = imin((CB == 8 ? kColInvMinB : 2) * CSCALE, smem_ctas_cap((N + CINF * FSCI) * CB, 32));
  static constexpr int CQMINB = imin((CB == 8 ? kColQwMinB : 2) * CSCALE, smem_ctas_cap((N + 2 * FSCQ) * CB, 32));
};
constexpr int kColThreads = 256;   // the adjoint's column kernels
constexpr int kThreadsB = 256;     // row kernels

// per-pass twiddle table of fft_ip (at most N entries)
template <typename T, int N>
__device__ __forceinline__ void load_tw(cplx<T>* tw_s, const cplx<T>* __restrict__ tw_g, int nt) {
  load_tw_passes<T, N, 1>(tw_s, tw_g, nt);
}

// Asynchronous global->shared copies of one complex value (8 or 16 bytes);
// src_bytes = 0 writes zeros (modes outside the retained set).
template <typename T>
__device__ __forceinline__ void cp_async_c(cplx<T>* dst, const cplx<T>* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(cplx<T>) == 8) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 8 : 0));
  } else {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 16 : 0));
  }
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// ===========================================================================
// Phase A, kernel 1: y-inverse FFTs of the six fields needed in physical space
// ===========================================================================
// one column entry of a field at FFT index idx, realit (fft.f90:88-107)
// applied: at kx = 0 the entries of negative ky are the conjugates of the
// positive ones.  `row` is the compact row the value comes from (-1: zero),
// `cj` whether it is conjugated.
__device__ __forceinline__ void col_src(const Geom& g, int kx, int idx, int& row, bool& cj) {
  cj = kx == 0 && idx > g.n / 2;
  row = kx <= g.K ? g.row_of_fft_index(cj ? g.n - idx : idx) : -1;
}

template <typename T, int N>
__global__ void __launch_bounds__(Tiles<T, N>::CNT, Tiles<T, N>::CIMINB)
k_col_inv(Geom g, int zbase, const cplx<T>* __restrict__ psi, const cplx<T>* __restrict__ q,
          const cplx<T>* __restrict__ BR, const cplx<T>* __restrict__ BI, cplx<T>* __restrict__ S,
          const cplx<T>* __restrict__ twg, cplx<T>* __restrict__ Qb, int bmode) {
  // bmode 0: all six transforms into S; 1: u, v, zeta, q into S (BR, BI are
  // kept in Qb); 2: BR, BI into Qb only (before a step whose Qb is stale)
  constexpr int CT = Tiles<T, N>::CT, NT = Tiles<T, N>::CNT;
  constexpr int R0 = radix_of(N), NB0 = N / R0, NSL = LastNS<N>::value, RL = N / NSL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* sm = tw + N;                        // [CINF][FS] (column layout Tiles::CIP)
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  load_tw<T, N>(tw, twg, NT);
  __syncthreads();
  const long long zoff = (long long)z * g.plane;
  // u = -i ky psi (derivatives.f90:1309), v = i kx psi (1310), zeta = -kh^2 psi (842)
  auto pro_psi = [&](int c, int j, cplx<T> (&v)[3][R0]) {
    const int kx = kx0 + c;
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      int row; bool cj;
      col_src(g, kx, j + r * NB0, row, cj);
      const cplx<T> sv = row >= 0 ? psi[zoff + (long long)row * g.KXP + kx] : mk<T>(0, 0);
      const T ky = row >= 0 ? (T)g.ky_of_row(row) : (T)0;
      const T fkx = (T)kx;
      cplx<T> a = cscale(cmul_mi(sv), ky), b = cscale(cmul_i(sv), fkx), d = cscale(sv, -(fkx * fkx + ky * ky));
      if (cj) { a = cconj(a); b = cconj(b); d = cconj(d); }
      v[0][r] = a; v[1][r] = b; v[2][r] = d;
    }
  };
  auto pro_raw = [&](int c, int j, cplx<T> (&v)[3][R0]) {
    const int kx = kx0 + c;
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      int row; bool cj;
      col_src(g, kx, j + r * NB0, row, cj);
      const long long m = zoff + (long long)row * g.KXP + kx;
      cplx<T> a = row >= 0 ? q[m] : mk<T>(0, 0), b = row >= 0 ? BR[m] : mk<T>(0, 0), d = row >= 0 ? BI[m] : mk<T>(0, 0);
      if (cj) { a = cconj(a); b = cconj(b); d = cconj(d); }
      v[0][r] = a; v[1][r] = b; v[2][r] = d;
    }
  };
  auto epi = [&](int f0) {
    return [&, f0](int c, int j, cplx<T> (&v)[3][RL]) {
#pragma unroll
      for (int f = 0; f < 3; ++f)
#pragma unroll
        for (int r = 0; r < RL; ++r) S[scr_off(zb, f0 + f, j + r * NSL, N, g.KXP) + kx0 + c] = v[f][r];
    };
  };
  if constexpr (kColInvNF2 && sizeof(T) == 4) {
    // three passes of two transforms: (u, v), (zeta, q), (BR, BI)
    auto pro2 = [&](int which) {
      return [&, which](int c, int j, cplx<T> (&v)[2][R0]) {
        const int kx = kx0 + c;
#pragma unroll
        for (int r = 0; r < R0; ++r) {
          int row; bool cj;
          col_src(g, kx, j + r * NB0, row, cj);
          const long long m = zoff + (long long)row * g.KXP + kx;
          const T ky = row >= 0 ? (T)g.ky_of_row(row) : (T)0;
          const T fkx = (T)kx;
          cplx<T> a, b;
          if (which == 0) {
            const cplx<T> sv = row >= 0 ? psi[m] : mk<T>(0, 0);
            a = cscale(cmul_mi(sv), ky);
            b = cscale(cmul_i(sv), fkx);
          } else if (which == 1) {
            const cplx<T> sv = row >= 0 ? psi[m] : mk<T>(0, 0);
            a = cscale(sv, -(fkx * fkx + ky * ky));
            b = row >= 0 ? q[m] : mk<T>(0, 0);
          } else {
            a = row >= 0 ? BR[m] : mk<T>(0, 0);
            b = row >= 0 ? BI[m] : mk<T>(0, 0);
          }
          if (cj) { a = cconj(a); b = cconj(b); }
          v[0][r] = a; v[1][r] = b;
        }
      };
    };
    auto epi2 = [&](int f0) {
      return [&, f0](int c, int j, cplx<T> (&v)[2][RL]) {
#pragma unroll
        for (int f = 0; f < 2; ++f)
#pragma unroll
          for (int r = 0; r < RL; ++r) S[scr_off(zb, f0 + f, j + r * NSL, N, g.KXP) + kx0 + c] = v[f][r];
      };
    };
    auto epiq = [&](int c, int j, cplx<T> (&v)[2][RL]) {
#pragma unroll
      for (int f = 0; f < 2; ++f)
#pragma unroll
        for (int r = 0; r < RL; ++r) Qb[q_off(zb, f, j + r * NSL, N, g.KXP) + kx0 + c] = v[f][r];
    };
    if (bmode != 2) {
      col_fft<T, N, false, 2, CT, NT, Tiles<T, N>::CIP>(sm, tw, pro2(0), epi2(0));
      __syncthreads();
      col_fft<T, N, false, 2, CT, NT, Tiles<T, N>::CIP>(sm, tw, pro2(1), epi2(2));
    }
    if (bmode == 0) {
      __syncthreads();
      col_fft<T, N, false, 2, CT, NT, Tiles<T, N>::CIP>(sm, tw, pro2(2), epi2(4));
    } else if (bmode == 2) {
      col_fft<T, N, false, 2, CT, NT, Tiles<T, N>::CIP>(sm, tw, pro2(2), epiq);
    }
  } else {
    col_fft<T, N, false, 3, CT, NT, Tiles<T, N>::CIP>(sm, tw, pro_psi, epi(0));
    __syncthreads();
    col_fft<T, N, false, 3, CT, NT, Tiles<T, N>::CIP>(sm, tw, pro_raw, epi(3));
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
// the same on a shared-memory transform laid out by lay_idx<LAY>
template <typename T, int LAY = 0>
__device__ __forceinline__ void unpack_pad(const cplx<T>* F, int k, int n, cplx<T>& X, cplx<T>& Y) {
  const cplx<T> a = F[lay_idx<LAY>(k)], b = F[lay_idx<LAY>(k == 0 ? 0 : n - k)];
  X = mk<T>((a.x + b.x) * (T)0.5, (a.y - b.y) * (T)0.5);
  Y = mk<T>((a.y + b.y) * (T)0.5, (b.x - a.x) * (T)0.5);
}

// ===========================================================================
// Phase A, kernel 2: rows — physical products of convol_waqg / refraction_waqg
// ===========================================================================
// One CTA item: rows y0..y0+RT-1 of level zb of the batch.  src(f, rr)
// points at row rr of scratch plane f (global memory, or the item's copy
// in shared memory); after_pass0() runs once the first pass has read them
// all (after a CTA barrier).  bA: [4][RT][LD].
template <typename T, int N, class Src, class After>
__device__ __forceinline__ void row_main_item(const Geom& g, const StepParams& sp, cplx<T>* __restrict__ S,
                                              const cplx<T>* __restrict__ tw, cplx<T>* __restrict__ bA, int zb,
                                              int y0, Src src, After after_pass0) {
  constexpr int RT = Tiles<T, N>::RTM, LD = Tiles<T, N>::LD, NT = kRowThreads, LAY = Tiles<T, N>::RLAY;
  // MID / MIDI: forward / inverse hand-off before the last pass in layout 1;
  // LL: layout the inverse's last pass reads
  constexpr int MID = Tiles<T, N>::RMID, MIDI = Tiles<T, N>::RMIDI, LL = MIDI ? MIDI : LAY;
  const int tid = threadIdx.x;
  const int K = g.K;
  constexpr int R0 = radix_of(N), NB0 = N / R0;
  if constexpr (Tiles<T, N>::RPASS0) {
    row_pass0<T, N, false, 3, RT, NT, LD, LAY>(bA, [&](int rr, int j, cplx<T> (&v)[3][R0]) {
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        const cplx<T>* X = src(2 * p, rr);
        const cplx<T>* Y = src(2 * p + 1, rr);
#pragma unroll
        for (int r = 0; r < R0; ++r) v[p][r] = pack_spec<T>(X, Y, j + r * NB0, N, K);
      }
    });
    __syncthreads();
    after_pass0();
    if constexpr (Tiles<T, N>::RFUSE) {
      constexpr int NS = LastNS<N>::value, R = N / NS;     // == R0, NS == NB0
      ip_passes_but_last<T, N, false, 3 * RT, NT, LD, R0, LAY, MIDI>(bA, tw);
      // last inverse pass into registers: task (row, j) holds the physical
      // values at x = j + r*NS of the three packed pairs
      const int j = tid % NS, rr = tid / NS;
      cplx<T> v[3][R];
      constexpr int off = tw_off<N>(NS);
#pragma unroll
      for (int f = 0; f < 3; ++f) {
#pragma unroll
        for (int r = 0; r < R; ++r) v[f][r] = bA[(f * RT + rr) * LD + lay_idx<LL>(j + r * NS)];
#pragma unroll
        for (int r = 1; r < R; ++r) {
          cplx<T> w = tw[off + (r - 1) * NS + j];
          w.y = -w.y;
          v[f][r] = cmul(v[f][r], w);
        }
        dftR<T, R, false>(v[f]);
      }
      __syncthreads();
      // products (u q, v q), (u br, v br), (u bi, v bi), (zeta br, zeta bi)
      // at the same x are the first forward pass's inputs
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        cplx<T> w[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const cplx<T> uv = v[0][r], zq = v[1][r], bb = v[2][r];
          w[r] = f == 0 ? mk<T>(uv.x * zq.y, uv.y * zq.y)
               : f == 1 ? mk<T>(uv.x * bb.x, uv.y * bb.x)
               : f == 2 ? mk<T>(uv.x * bb.y, uv.y * bb.y)
                        : mk<T>(zq.x * bb.x, zq.x * bb.y);
        }
        dftR<T, R, true>(w);
#pragma unroll
        for (int r = 0; r < R; ++r) bA[(f * RT + rr) * LD + lay_idx<LAY>(j * R + r)] = w[r];
      }
      __syncthreads();
      if constexpr (Tiles<T, N>::RSHL) {
        ip_passes_but_last<T, N, true, 4 * RT, NT, LD, R0, LAY, MID>(bA, tw);
      } else {
        ip_passes<T, N, true, 4 * RT, NT, LD, R0, LAY, MID>(bA, tw);
      }
    } else {
      ip_passes<T, N, false, 3 * RT, NT, LD, R0, LAY>(bA, tw);
    }
  } else {
#pragma unroll 4
    for (int e = tid; e < 3 * RT * N; e += NT) {
      const int k = e % N, p = (e / N) % 3, rr = e / (3 * N);
      bA[(p * RT + rr) * LD + pad_idx(k)] = pack_spec<T>(src(2 * p, rr), src(2 * p + 1, rr), k, N, K);
    }
    __syncthreads();
    after_pass0();
    fft_ip<T, N, false, 3 * RT, NT, LD>(bA, tw);
  }
  if constexpr (!Tiles<T, N>::RFUSE) {
    // products: (u q, v q), (u br, v br), (u bi, v bi), (zeta br, zeta bi)
#pragma unroll 4
    for (int e = tid; e < RT * N; e += NT) {
      const int x = e % N, rr = e / N;
      const int px = pad_idx(x);
      const cplx<T> uv = bA[(0 * RT + rr) * LD + px];
      const cplx<T> zq = bA[(1 * RT + rr) * LD + px];
      const cplx<T> bb = bA[(2 * RT + rr) * LD + px];
      bA[(0 * RT + rr) * LD + px] = mk<T>(uv.x * zq.y, uv.y * zq.y);
      bA[(1 * RT + rr) * LD + px] = mk<T>(uv.x * bb.x, uv.y * bb.x);
      bA[(2 * RT + rr) * LD + px] = mk<T>(uv.x * bb.y, uv.y * bb.y);
      bA[(3 * RT + rr) * LD + px] = mk<T>(zq.x * bb.x, zq.x * bb.y);
    }
    __syncthreads();
    fft_ip<T, N, true, 4 * RT, NT, LD>(bA, tw);
  }
  const T adv = sp.adv ? (T)1 : (T)0;
  const T half = sp.refr ? (T)0.5 : (T)0;
  if constexpr (Tiles<T, N>::RSHL) {
    // last forward pass per task (row, j), spectra split by shuffles; the
    // (zeta br, zeta bi) transform first: its halves enter planes 2 and 4
    const RowLastTask tk = row_last_task(tid);
    const int rr = tid / 64, y = y0 + rr;
    constexpr int LL2 = MID ? MID : LAY;
    cplx<T> w[8], b[3], zr[3], zi[3];
    row_last_fwd512<T, LL2>(bA + (3 * RT + rr) * LD, tw, tk, w, b);
#pragma unroll
    for (int q = 0; q < 3; ++q) split_pair<T>(w[q], b[q], zr[q], zi[q]);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      row_last_fwd512<T, LL2>(bA + (f * RT + rr) * LD, tw, tk, w, b);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int k = tk.j + 64 * q;
        if (k > K) continue;
        cplx<T> X, Y;
        split_pair<T>(w[q], b[q], X, Y);
        const cplx<T> G = cscale(cmul_i(X), (T)k * adv);
        // G = i kx F(uX) (+- refraction), H = F(vX), as below
        S[scr_off(zb, 2 * f, y, N, g.KXP) + k] = f == 0 ? G : (f == 1 ? csub(G, cscale(zi[q], half))
                                                                        : cadd(G, cscale(zr[q], half)));
        S[scr_off(zb, 2 * f + 1, y, N, g.KXP) + k] = cscale(Y, adv);
      }
    }
    return;
  }
  for (int e = tid; e < RT * (K + 1); e += NT) {
    const int k = e % (K + 1), rr = e / (K + 1);
    const int y = y0 + rr;
    cplx<T> uq, vq, ubr, vbr, ubi, vbi, zbr, zbi;
    unpack_pad<T, LAY>(bA + (0 * RT + rr) * LD, k, N, uq, vq);
    unpack_pad<T, LAY>(bA + (1 * RT + rr) * LD, k, N, ubr, vbr);
    unpack_pad<T, LAY>(bA + (2 * RT + rr) * LD, k, N, ubi, vbi);
    unpack_pad<T, LAY>(bA + (3 * RT + rr) * LD, k, N, zbr, zbi);
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

// Rows of the batch: grid (N/RT, levels) with one item per CTA, or, with
// the prefetch (Tiles::RPRE), a persistent grid whose CTAs walk the items
// it = blockIdx.x, += gridDim.x (item it: level it / (N/RT), rows
// (it % (N/RT))*RT...), each CTA bulk-copying the six scratch rows of its
// next item into shared memory while it transforms the current one.
// A copy that does not land within the bounded wait sets *wflag and ends the
// CTA.
template <typename T, int N>
__global__ void __launch_bounds__(kRowThreads, Tiles<T, N>::MMINB)
k_row_main(Geom g, StepParams sp, cplx<T>* __restrict__ S, const cplx<T>* __restrict__ twg, int nitems,
           int* __restrict__ wflag, const cplx<T>* __restrict__ Qb) {
  // planes 4, 5 (BR, BI) from the kept-B planes Qb when given
  auto plane = [&](int zb, int f, int y) -> const cplx<T>* {
    return (Qb && f >= 4) ? Qb + q_off(zb, f - 4, y, N, g.KXP) : S + scr_off(zb, f, y, N, g.KXP);
  };
  constexpr int RT = Tiles<T, N>::RTM, LD = Tiles<T, N>::LD, NT = kRowThreads;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  // [4][RT][LD]: (u,v), (zeta,q), (br,bi); then, in place, the 4 products
  cplx<T>* bA = tw + N;
  load_tw<T, N>(tw, twg, NT);
  if constexpr (Tiles<T, N>::RPRE) {
    constexpr int NGY = N / RT;
    cplx<T>* stg = bA + 4 * RT * LD;                 // [6][RT][KXP]: the item's scratch rows
    const unsigned bar = smem_u32(stg + 6 * RT * g.KXP);
    const unsigned fb = (unsigned)(RT * g.KXP * sizeof(cplx<T>));
    auto issue = [&](int it) {
      const int zb = it / NGY, y0 = (it % NGY) * RT;
      mbar_expect_tx(bar, 6u * fb);
#pragma unroll
      for (int f = 0; f < 6; ++f) bulk_g2s(stg + f * RT * g.KXP, plane(zb, f, y0), fb, bar);
    };
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      if ((int)blockIdx.x < nitems) issue(blockIdx.x);
    }
    __syncthreads();
    unsigned ph = 0;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x, ph ^= 1u) {
      // also orders the previous item's last reads of bA before this one's writes
      const bool ok = mbar_wait(bar, ph);
      if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) { raise_wait_flag(wflag); (void)mbar_wait(bar, ph); }
        return;
      }
      const int nxt = it + (int)gridDim.x;
      row_main_item<T, N>(g, sp, S, tw, bA, it / NGY, (it % NGY) * RT,
                          [&](int f, int rr) -> const cplx<T>* { return stg + (f * RT + rr) * g.KXP; },
                          [&]() {
                            if (threadIdx.x == 0 && nxt < nitems) { fence_proxy_async(); issue(nxt); }
                          });
    }
  } else {
    const int zb = blockIdx.y, y0 = blockIdx.x * RT;
    row_main_item<T, N>(g, sp, S, tw, bA, zb, y0,
                        [&](int f, int rr) -> const cplx<T>* { return plane(zb, f, y0 + rr); },
                        []() {});
  }
}

// Pointers of the state fields used by the update
template <typename T> struct StateP {
  cplx<T>* q; cplx<T>* qo; cplx<T>* BR; cplx<T>* BI; cplx<T>* BRo; cplx<T>* BIo;
  cplx<T>* psi; cplx<T>* AR; cplx<T>* AI; cplx<T>* qstar; const cplx<T>* dq;
  cplx<T>* sig1; cplx<T>* sig2;   // regular YBJ: per-level terms of sigma (compute_sigma)
};

// ===========================================================================
// Phase A, kernel 3: y-forward FFTs, time update, y-inverse FFTs for q^w
// ===========================================================================
// Shared memory: twiddles | two interleaved transforms | the tile's state of
// the variable being updated (3 complex fields, staged by cp.async while its
// tendencies are transformed) | B^{n+1} (2 complex fields) | 2 IF tables.
template <typename T, int N> struct UpdLay {
  static constexpr int CT = Tiles<T, N>::CT;
  static constexpr int KYM = 2 * ((N + 2) / 3) + 1;     // >= KY for this n
  static constexpr int FE = CT * KYM;                   // entries per staged field
  // the four q^w inverse transforms reuse the transform and staging regions
  static constexpr int PAD = 4 * ColLay<N, CT, Tiles<T, N>::CUP>::FS > 2 * ColLay<N, CT, Tiles<T, N>::CUP>::FS + 3 * FE
                                 ? 4 * ColLay<N, CT, Tiles<T, N>::CUP>::FS - 2 * ColLay<N, CT, Tiles<T, N>::CUP>::FS - 3 * FE : 0;
  // lean (FP32): B^{n+1} re-read from global memory for the q^w transforms
  // (two passes of two) instead of kept in shared memory
  static constexpr bool LEAN = kUpdLean && sizeof(T) == 4;
  static constexpr int MINB0 = LEAN ? kUpdMinB : Tiles<T, N>::MINB;
  // lean with the IF tables of the variable staged after the state
  // (kUpdTablesSmem) or read from global memory in the epilogue
  static constexpr bool GTAB = LEAN && !kUpdTablesSmem;
  static constexpr size_t bytes() {
    return LEAN ? (size_t)(N + 2 * ColLay<N, CT, Tiles<T, N>::CUP>::FS + 3 * FE) * sizeof(cplx<T>) + (GTAB ? 0 : (size_t)2 * FE * sizeof(T))
                : (size_t)(N + 2 * ColLay<N, CT, Tiles<T, N>::CUP>::FS + 5 * FE + PAD) * sizeof(cplx<T>) + (size_t)2 * FE * sizeof(T);
  }
  // CTAs per SM: scaled with the column CTAs' size (Tiles::CSCALE)
  static constexpr int MINB = imin(MINB0 * Tiles<T, N>::CSCALE, smem_ctas_cap((int)bytes(), 32));
};

// 16-byte asynchronous copy of nbytes (0, 8 or 16) and zeros for the rest
__device__ __forceinline__ void cp_async_16(void* dst, const void* src, int nbytes) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(nbytes));
}

template <typename T>
__device__ __forceinline__ void cp_async_s(T* dst, const T* src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(T) == 4) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 4 : 0));
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 8 : 0));
  }
}

template <typename T, int N>
__global__ void __launch_bounds__(Tiles<T, N>::CNT, UpdLay<T, N>::MINB)
k_col_update(Geom g, StepParams sp, int zbase, StateP<T> st, const T* __restrict__ e1t, const T* __restrict__ e2t,
             const T* __restrict__ e1wt, const T* __restrict__ e2wt, cplx<T>* __restrict__ S,
             const cplx<T>* __restrict__ twg, int qw_prep, cplx<T>* __restrict__ Qb) {
  using L = UpdLay<T, N>;
  constexpr int CT = Tiles<T, N>::CT, NT = Tiles<T, N>::CNT, FE = L::FE;
  constexpr int R0 = radix_of(N), NB0 = N / R0, NSL = LastNS<N>::value, RL = N / NSL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* sm = tw + N;                          // [2][FS]
  cplx<T>* stg = sm + 2 * ColLay<N, CT, Tiles<T, N>::CUP>::FS;   // [3][FE]: x, x_old, third (dq / AI / AR)
  cplx<T>* bnew = stg + 3 * FE + L::PAD;         // [2][FE]: BR, BI at n+1 (not LEAN)
  // [2][FE]: e1, e2 or e1w, e2w (not GTAB)
  T* tab = reinterpret_cast<T*>(L::LEAN ? stg + 3 * FE : bnew + 2 * FE);
  const int tid = threadIdx.x;
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  const int KY = g.KY;
  load_tw<T, N>(tw, twg, NT);
  const T inv_n2 = (T)1 / ((T)N * (T)N);
  const long long zoff = (long long)z * g.plane;
  const int mem = sp.mpar ? z / g.nseg : 0;          // ensemble member of this level (stacks)
  if (sp.mpar) {
    const long long to = (long long)mem * g.plane;
    e1t += to; e2t += to; e1wt += to; e2wt += to;
  }
  const T dt = (T)(sp.mpar ? sp.mpar[4 * mem] : sp.delt);
  const T dt2 = (T)2 * dt;
  const T gam = (T)sp.gamma;
  const T cdisp = sp.disp ? (T)(sp.mpar ? sp.mpar[4 * mem + 1] : sp.cdisp) : (T)0;
  const bool eul = sp.euler != 0;
  // staged entry (c, row) at row*CT + c
  auto stage = [&](int which) {
    const cplx<T>* X = which == 0 ? st.q : (which == 1 ? st.BR : st.BI);
    const cplx<T>* Xo = which == 0 ? st.qo : (which == 1 ? st.BRo : st.BIo);
    const cplx<T>* X3 = which == 0 ? st.dq : (which == 1 ? st.AI : st.AR);
    const bool need3 = which != 0 || sp.use_dq;
    if constexpr (kUpdStage16 && sizeof(T) == 4 && CT % 2 == 0) {
      // FP32: 16-byte copies of column pairs (zero-filled past kx = K)
      for (int e2 = tid; e2 < (CT / 2) * KY; e2 += NT) {
        const int c = (e2 % (CT / 2)) * 2, row = e2 / (CT / 2);
        const int kx = kx0 + c;
        const int nb = kx + 1 <= g.K ? 16 : (kx <= g.K ? 8 : 0);
        const long long m = zoff + (long long)row * g.KXP + kx;
        const int e = row * CT + c;
        cp_async_16(stg + e, nb ? X + m : X, nb);
        if (!eul) cp_async_16(stg + FE + e, nb ? Xo + m : Xo, nb);
        if (need3) cp_async_16(stg + 2 * FE + e, nb ? X3 + m : X3, nb);
      }
    } else {
      for (int e = tid; e < CT * KY; e += NT) {
        const int c = e % CT, row = e / CT;
        const int kx = kx0 + c;
        const bool in = kx <= g.K;
        const long long m = zoff + (long long)row * g.KXP + kx;
        cp_async_c<T>(stg + e, in ? X + m : X, in);
        if (!eul) cp_async_c<T>(stg + FE + e, in ? Xo + m : Xo, in);
        if (need3) cp_async_c<T>(stg + 2 * FE + e, in ? X3 + m : X3, in);
      }
    }
    if constexpr (!L::GTAB) {
      if (which < 2 && sizeof(T) == 4 && CT * sizeof(T) == 16) {
        // FP32: one 16-byte copy per row of the tile (the tables' rows hold KXP entries)
        const T* t1 = which == 0 ? e1t : e1wt;
        const T* t2 = which == 0 ? e2t : e2wt;
        for (int e = tid; e < 2 * KY; e += NT) {
          const int row = e >> 1;
          const long long mt = (long long)row * g.KXP + kx0;
          cp_async_16(tab + (e & 1) * FE + row * CT, ((e & 1) ? t2 : t1) + mt, 16);
        }
      } else if (which < 2) {
        for (int e = tid; e < CT * KY; e += NT) {
          const int c = e % CT, row = e / CT;
          const int kx = kx0 + c;
          const bool in = kx <= g.K;
          const long long mt = (long long)row * g.KXP + kx;
          const T* t1 = which == 0 ? e1t : e1wt;
          const T* t2 = which == 0 ? e2t : e2wt;
          cp_async_s<T>(tab + e, in ? t1 + mt : t1, in);
          cp_async_s<T>(tab + FE + e, in ? t2 + mt : t2, in);
        }
      }
    }
  };
  // tendencies G + i ky H of (q, BR, BI) from the (G, H) plane pairs 0-1, 2-3, 4-5
  auto pro_planes = [&](int h0) {
    return [&, h0](int c, int j, cplx<T> (&v)[2][R0]) {
      const int kx = kx0 + c;
#pragma unroll
      for (int r = 0; r < R0; ++r) {
        const int y = j + r * NB0;
        const bool in = kx <= g.K;
        v[0][r] = in ? S[scr_off(zb, h0, y, N, g.KXP) + kx] : mk<T>(0, 0);
        v[1][r] = in ? S[scr_off(zb, h0 + 1, y, N, g.KXP) + kx] : mk<T>(0, 0);
      }
    };
  };
  // time update (main_waqg.f90:237-264, 362-415) of one variable
  // (which = 0 q, 1 BR, 2 BI), one mode per output index
  auto epi_update = [&](int which) {
    return [&, which](int c, int j, cplx<T> (&v)[2][RL]) {
      const int kx = kx0 + c;
      if (kx > g.K) return;
      cplx<T>* X = which == 0 ? st.q : (which == 1 ? st.BR : st.BI);
      cplx<T>* Xo = which == 0 ? st.qo : (which == 1 ? st.BRo : st.BIo);
#pragma unroll
      for (int r = 0; r < RL; ++r) {
        const int row = g.row_of_fft_index(j + r * NSL);
        if (row < 0) continue;
        const int ky = g.ky_of_row(row);
        const int e = row * CT + c;
        const long long m = zoff + (long long)row * g.KXP + kx;
        const T fky = (T)ky;
        const cplx<T> G = v[0][r], H = v[1][r];
        const cplx<T> tnd = cscale(mk<T>(G.x - fky * H.y, G.y + fky * H.x), inv_n2);   // G + i ky H
        const cplx<T> x0 = stg[e];
        const cplx<T> xo = eul ? x0 : stg[FE + e];
        cplx<T> xn = mk<T>(0, 0), xf = eul ? xo : mk<T>(0, 0);
        if (g.mask(kx, ky)) {
          if (which == 0) {
            const cplx<T> dqv = sp.use_dq ? stg[2 * FE + e] : mk<T>(0, 0);
            const long long mt = (long long)row * g.KXP + kx;
            const T e1 = L::GTAB ? e1t[mt] : tab[e], e2 = L::GTAB ? e2t[mt] : tab[FE + e];
            if (eul) {
              xn = cscale(cadd(csub(xo, cscale(tnd, dt)), cscale(dqv, dt)), e1);
            } else {
              xn = cadd(csub(cscale(xo, e2), cscale(cscale(tnd, dt2), e1)), cscale(cscale(dqv, dt2), e2));
            }
          } else {
            const long long mt = (long long)row * g.KXP + kx;
            const T e1w = L::GTAB ? e1wt[mt] : tab[e], e2w = L::GTAB ? e2wt[mt] : tab[FE + e];
            const T ck = cdisp * (T)(kx * kx + ky * ky);
            // nBR - 0.5 rBI + c kh2 AI ; nBI + 0.5 rBR - c kh2 AR
            const cplx<T> a3 = stg[2 * FE + e];
            const cplx<T> fr = which == 1 ? cadd(tnd, cscale(a3, ck)) : csub(tnd, cscale(a3, ck));
            if (eul) {
              xn = cscale(csub(xo, cscale(fr, dt)), e1w);
            } else {
              xn = csub(cscale(xo, e2w), cscale(cscale(fr, dt2), e1w));
            }
          }
          // Robert-Asselin filter (main_waqg.f90:395-410)
          if (!eul) xf = cadd(x0, cscale(cadd(csub(xo, cscale(x0, (T)2)), xn), gam));
        }
        X[m] = xn;
        Xo[m] = xf;
        if (!L::LEAN && which > 0) bnew[(which - 1) * FE + e] = xn;
        if (!sp.ybj && which > 0) {
          // compute_sigma (derivatives.f90:1037-1068) with the tendencies
          // T_R = nBR - rBI/2, T_I = nBI + rBR/2: (rBR + 2 nBI) = 2 T_I,
          // (rBI - 2 nBR) = -2 T_R, divided by kh2 where kh2 > 0 and L = 1
          const int kh2 = kx * kx + ky * ky;
          cplx<T> sv = mk<T>(0, 0);
          if (kh2 > 0 && g.mask(kx, ky)) sv = cscale(tnd, (which == 2 ? (T)2 : (T)-2) / (T)kh2);
          (which == 2 ? st.sig1 : st.sig2)[m] = sv;
        }
      }
    };
  };
  stage(0);
  col_fft<T, N, true, 2, CT, NT, Tiles<T, N>::CUP>(sm, tw, pro_planes(0), epi_update(0));
  __syncthreads();
  stage(1);
  col_fft<T, N, true, 2, CT, NT, Tiles<T, N>::CUP>(sm, tw, pro_planes(2), epi_update(1));
  __syncthreads();
  stage(2);
  col_fft<T, N, true, 2, CT, NT, Tiles<T, N>::CUP>(sm, tw, pro_planes(4), epi_update(2));
  if (!qw_prep) return;
  __syncthreads();
  // y-inverse FFTs of B and i ky B at n+1 (compute_qw, derivatives.f90:929-957)
  // BR, i ky BR, BI, i ky BI: one pass over the four transforms in FP32 (the
  // transform and staging regions are free now), two passes of two in FP64
  // (four FP64 transforms per task would spill)
  auto pro_B = [&](int b0i, auto nf) {
    constexpr int NFQ = decltype(nf)::value;
    return [&, b0i](int c, int j, cplx<T> (&v)[NFQ][R0]) {
      const int kx = kx0 + c;
#pragma unroll
      for (int r = 0; r < R0; ++r) {
        int row; bool cj;
        col_src(g, kx, j + r * NB0, row, cj);
        const T ky = row >= 0 ? (T)g.ky_of_row(row) : (T)0;
#pragma unroll
        for (int b = 0; b < NFQ / 2; ++b) {
          // B^{n+1}: this CTA's own writes, visible after the barrier
          const cplx<T>* Xg = (b0i + b) == 0 ? st.BR : st.BI;
          const cplx<T> x = row < 0 ? mk<T>(0, 0)
                          : L::LEAN ? Xg[zoff + (long long)row * g.KXP + kx] : bnew[(b0i + b) * FE + row * CT + c];
          cplx<T> u0 = x, u1 = cscale(cmul_i(x), ky);
          if (cj) { u0 = cconj(u0); u1 = cconj(u1); }
          v[2 * b][r] = u0; v[2 * b + 1][r] = u1;
        }
      }
    };
  };
  // planes (BR, i ky BR, BI, i ky BI) = 0..3; with Qb, BR and BI go to the
  // kept-B planes (Q 0 and 1) instead of S 0 and 2
  auto epi_store = [&](int f0, auto nf) {
    constexpr int NFQ = decltype(nf)::value;
    return [&, f0](int c, int j, cplx<T> (&v)[NFQ][RL]) {
#pragma unroll
      for (int f = 0; f < NFQ; ++f)
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          const int p = f0 + f, y = j + r * NSL;
          cplx<T>* dst = (Qb && (p & 1) == 0) ? Qb + q_off(zb, p >> 1, y, N, g.KXP) : S + scr_off(zb, p, y, N, g.KXP);
          dst[kx0 + c] = v[f][r];
        }
    };
  };
  if constexpr (sizeof(T) == 4 && !L::LEAN) {
    using NF4 = std::integral_constant<int, 4>;
    col_fft<T, N, false, 4, CT, NT, Tiles<T, N>::CUP>(sm, tw, pro_B(0, NF4{}), epi_store(0, NF4{}));
  } else {
    using NF2 = std::integral_constant<int, 2>;
    col_fft<T, N, false, 2, CT, NT, Tiles<T, N>::CUP>(sm, tw, pro_B(0, NF2{}), epi_store(0, NF2{}));
    __syncthreads();
    col_fft<T, N, false, 2, CT, NT, Tiles<T, N>::CUP>(sm, tw, pro_B(1, NF2{}), epi_store(2, NF2{}));
  }
}

// ===========================================================================
// Phase A, kernel 4: rows — products of compute_qw
// ===========================================================================
// One CTA item of k_row_qw: rows y0..y0+RT-1 of level zb; src(f, rr) and
// after_pass0 as in row_main_item.  bA: [3][RT][LD].
template <typename T, int N, class Src, class After>
__device__ __forceinline__ void row_qw_item(const Geom& g, cplx<T>* __restrict__ S, const cplx<T>* __restrict__ tw,
                                            cplx<T>* __restrict__ bA, int zb, int y0, Src src, After after_pass0) {
  constexpr int RT = Tiles<T, N>::QRT, LD = Tiles<T, N>::LD, NT = Tiles<T, N>::QTHREADS, LAY = Tiles<T, N>::QLAY;
  const int tid = threadIdx.x;
  const int K = g.K;
  // packed: (BR, BI), (BRx, BIx), (BRy, BIy)
  auto packed = [&](int p, int rr, int k) -> cplx<T> {
    const cplx<T>* sBR = src(0, rr);
    const cplx<T>* sBRy = src(1, rr);
    const cplx<T>* sBI = src(2, rr);
    const cplx<T>* sBIy = src(3, rr);
    if (p == 0) return pack_spec<T>(sBR, sBI, k, N, K);
    if (p == 2) return pack_spec<T>(sBRy, sBIy, k, N, K);
    if (k == 0 || (k > K && k < N - K)) return mk<T>(0, 0);      // x-derivatives vanish at kx = 0
    const int kk = k <= K ? k : N - k;
    const cplx<T> a = cscale(cmul_i(sBR[kk]), (T)kk), b = cscale(cmul_i(sBI[kk]), (T)kk);
    return k <= K ? mk<T>(a.x - b.y, a.y + b.x) : mk<T>(a.x + b.y, b.x - a.y);
  };
  if constexpr (Tiles<T, N>::RPASS0) {
    constexpr int R0 = radix_of(N), NB0 = N / R0;
    row_pass0<T, N, false, 3, RT, NT, LD, LAY>(bA, [&](int rr, int j, cplx<T> (&v)[3][R0]) {
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
        for (int r = 0; r < R0; ++r) v[p][r] = packed(p, rr, j + r * NB0);
    });
    __syncthreads();
    after_pass0();
    if constexpr (Tiles<T, N>::QFUSE) {
      // inverse last pass, the q^w products and the forward first pass in
      // registers (the same (row, butterfly) task holds both ends)
      constexpr int R0 = radix_of(N), NS = LastNS<N>::value, R = N / NS;
      constexpr int QM = Tiles<T, N>::QMID, QL = QM ? QM : LAY;
      ip_passes_but_last<T, N, false, 3 * RT, NT, LD, R0, LAY, QM>(bA, tw);
      const int j = tid % NS, rr = tid / NS;
      cplx<T> v[3][R];
      constexpr int off = tw_off<N>(NS);
#pragma unroll
      for (int f = 0; f < 3; ++f) {
#pragma unroll
        for (int r = 0; r < R; ++r) v[f][r] = bA[(f * RT + rr) * LD + lay_idx<QL>(j + r * NS)];
#pragma unroll
        for (int r = 1; r < R; ++r) {
          cplx<T> w = tw[off + (r - 1) * NS + j];
          w.y = -w.y;
          v[f][r] = cmul(v[f][r], w);
        }
        dftR<T, R, false>(v[f]);
      }
      __syncthreads();
      cplx<T> w[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const cplx<T> b = v[0][r], bx = v[1][r], by = v[2][r];
        w[r] = mk<T>(by.x * bx.y - bx.x * by.y, b.x * b.x + b.y * b.y);
      }
      dftR<T, R, true>(w);
#pragma unroll
      for (int r = 0; r < R; ++r) bA[rr * LD + lay_idx<LAY>(j * R + r)] = w[r];
      __syncthreads();
      if constexpr (Tiles<T, N>::QSHL) {
        ip_passes_but_last<T, N, true, RT, NT, LD, R0, LAY>(bA, tw);
      } else {
        ip_passes<T, N, true, RT, NT, LD, R0, LAY, QM>(bA, tw);
      }
    } else {
      ip_passes<T, N, false, 3 * RT, NT, LD, radix_of(N), LAY>(bA, tw);
    }
  } else {
#pragma unroll 4
    for (int e = tid; e < 3 * RT * N; e += NT) {
      const int k = e % N, p = (e / N) % 3, rr = e / (3 * N);
      bA[(p * RT + rr) * LD + pad_idx(k)] = packed(p, rr, k);
    }
    __syncthreads();
    after_pass0();
    fft_ip<T, N, false, 3 * RT, NT, LD>(bA, tw);
  }
  if constexpr (!Tiles<T, N>::QFUSE) {
#pragma unroll 4
    for (int e = tid; e < RT * N; e += NT) {
      const int x = e % N, rr = e / N;
      const int px = pad_idx(x);
      const cplx<T> b = bA[(0 * RT + rr) * LD + px];    // (br, bi)
      const cplx<T> bx = bA[(1 * RT + rr) * LD + px];   // (brx, bix)
      const cplx<T> by = bA[(2 * RT + rr) * LD + px];   // (bry, biy)
      const T p1 = by.x * bx.y - bx.x * by.y;           // BRy BIx - BRx BIy (derivatives.f90:973)
      const T p2 = b.x * b.x + b.y * b.y;               // BR^2 + BI^2     (derivatives.f90:996)
      bA[rr * LD + px] = mk<T>(p1, p2);
    }
    __syncthreads();
    fft_ip<T, N, true, RT, NT, LD>(bA, tw);
  }
  if constexpr (Tiles<T, N>::QSHL) {
    // last forward pass per task (row, j), spectrum split by shuffles
    const RowLastTask tk = row_last_task(tid);
    const int rr = tid / 64, y = y0 + rr;
    cplx<T> w[8], b[3];
    row_last_fwd512<T, LAY>(bA + rr * LD, tw, tk, w, b);
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int k = tk.j + 64 * q;
      if (k > K) continue;
      cplx<T> P1, P2;
      split_pair<T>(w[q], b[q], P1, P2);
      const T qk = (T)0.25 * (T)(k * k);
      S[scr_off(zb, 0, y, N, g.KXP) + k] = csub(P1, cscale(P2, qk));
      S[scr_off(zb, 1, y, N, g.KXP) + k] = P2;
    }
    return;
  }
  for (int e = tid; e < RT * (K + 1); e += NT) {
    const int k = e % (K + 1), rr = e / (K + 1);
    const int y = y0 + rr;
    cplx<T> P1, P2;
    unpack_pad<T, LAY>(bA + rr * LD, k, N, P1, P2);
    const T qk = (T)0.25 * (T)(k * k);
    S[scr_off(zb, 0, y, N, g.KXP) + k] = csub(P1, cscale(P2, qk));
    S[scr_off(zb, 1, y, N, g.KXP) + k] = P2;
  }
}

// Rows of the batch for compute_qw: one item per CTA on a grid (N/RT,
// levels), or persistent with the next item's four scratch rows
// bulk-copied into shared memory during the current one (Tiles::QPRE), as
// k_row_main.
template <typename T, int N>
__global__ void __launch_bounds__(Tiles<T, N>::QTHREADS, Tiles<T, N>::QMINB)
k_row_qw(Geom g, cplx<T>* __restrict__ S, const cplx<T>* __restrict__ twg, int nitems, int* __restrict__ wflag,
         const cplx<T>* __restrict__ Qb) {
  // planes 0, 2 (BR, BI) from the kept-B planes Qb when given
  auto plane = [&](int zb, int f, int y) -> const cplx<T>* {
    return (Qb && (f & 1) == 0) ? Qb + q_off(zb, f >> 1, y, N, g.KXP) : S + scr_off(zb, f, y, N, g.KXP);
  };
  constexpr int RT = Tiles<T, N>::QRT, LD = Tiles<T, N>::LD, NT = Tiles<T, N>::QTHREADS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* bA = tw + N;               // [3][RT][LD]; then, in place, (P1, P2) in the first RT
  load_tw<T, N>(tw, twg, NT);
  if constexpr (Tiles<T, N>::QPRE) {
    constexpr int NGY = N / RT;
    cplx<T>* stg = bA + 3 * RT * LD;                 // [4][RT][KXP]: the item's scratch rows
    const unsigned bar = smem_u32(stg + 4 * RT * g.KXP);
    const unsigned fb = (unsigned)(RT * g.KXP * sizeof(cplx<T>));
    auto issue = [&](int it) {
      const int zb = it / NGY, y0 = (it % NGY) * RT;
      mbar_expect_tx(bar, 4u * fb);
#pragma unroll
      for (int f = 0; f < 4; ++f) bulk_g2s(stg + f * RT * g.KXP, plane(zb, f, y0), fb, bar);
    };
    if (threadIdx.x == 0) {
      mbar_init(bar, 1);
      if ((int)blockIdx.x < nitems) issue(blockIdx.x);
    }
    __syncthreads();
    unsigned ph = 0;
    for (int it = blockIdx.x; it < nitems; it += gridDim.x, ph ^= 1u) {
      const bool ok = mbar_wait(bar, ph);
      if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) { raise_wait_flag(wflag); (void)mbar_wait(bar, ph); }
        return;
      }
      const int nxt = it + (int)gridDim.x;
      row_qw_item<T, N>(g, S, tw, bA, it / NGY, (it % NGY) * RT,
                        [&](int f, int rr) -> const cplx<T>* { return stg + (f * RT + rr) * g.KXP; },
                        [&]() {
                          if (threadIdx.x == 0 && nxt < nitems) { fence_proxy_async(); issue(nxt); }
                        });
    }
  } else {
    const int zb = blockIdx.y, y0 = blockIdx.x * RT;
    row_qw_item<T, N>(g, S, tw, bA, zb, y0,
                      [&](int f, int rr) -> const cplx<T>* { return plane(zb, f, y0 + rr); },
                      []() {});
  }
}

// ===========================================================================
// Phase A, kernel 5: y-forward FFTs of the q^w planes, q* = q - q^w
// ===========================================================================
template <typename T, int N>
__global__ void __launch_bounds__(Tiles<T, N>::CNT, Tiles<T, N>::CQMINB)
k_col_qw(Geom g, StepParams sp, int zbase, const cplx<T>* __restrict__ q, cplx<T>* __restrict__ qstar,
         const cplx<T>* __restrict__ S, const cplx<T>* __restrict__ twg, int* __restrict__ nflag) {
  constexpr int CT = Tiles<T, N>::CT, NT = Tiles<T, N>::CNT;
  constexpr int R0 = radix_of(N), NB0 = N / R0, NSL = LastNS<N>::value, RL = N / NSL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tw = reinterpret_cast<cplx<T>*>(smem_raw);
  cplx<T>* sm = tw + N;                 // [2][FS]
  __shared__ int s_bad;   // a non-finite q* in this tile (the state has blown up)
  const int zb = blockIdx.y, z = zbase + zb;
  const int kx0 = blockIdx.x * CT;
  if (threadIdx.x == 0) s_bad = 0;
  load_tw<T, N>(tw, twg, NT);
  __syncthreads();
  const T inv_n2 = (T)1 / ((T)N * (T)N);
  const int mem = sp.mpar ? z / g.nseg : 0;          // ensemble member of this level (stacks)
  const T s = sp.mpar ? (T)sp.mpar[4 * mem + 2] * (T)sp.mpar[4 * mem + 3] : (T)sp.Ro * (T)sp.W2F;
  const long long zoff = (long long)z * g.plane;
  auto pro = [&](int c, int j, cplx<T> (&v)[2][R0]) {
    const int kx = kx0 + c;
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      const int y = j + r * NB0;
      const bool in = kx <= g.K;
      v[0][r] = in ? S[scr_off(zb, 0, y, N, g.KXP) + kx] : mk<T>(0, 0);
      v[1][r] = in ? S[scr_off(zb, 1, y, N, g.KXP) + kx] : mk<T>(0, 0);
    }
  };
  auto epi = [&](int c, int j, cplx<T> (&v)[2][RL]) {
    const int kx = kx0 + c;
    if (kx > g.K) return;
#pragma unroll
    for (int r = 0; r < RL; ++r) {
      const int row = g.row_of_fft_index(j + r * NSL);
      if (row < 0) continue;
      const int ky = g.ky_of_row(row);
      const long long m = zoff + (long long)row * g.KXP + kx;
      cplx<T> out = mk<T>(0, 0);
      if (g.mask(kx, ky)) {
        const cplx<T> R = csub(v[0][r], cscale(v[1][r], (T)0.25 * (T)ky * (T)ky));
        const cplx<T> qw = cscale(cscale(R, inv_n2), s);
        out = csub(q[m], qw);       // q* = q - q^w (main_waqg.f90:430-439)
        if (!isfinite(out.x) || !isfinite(out.y)) s_bad = 1;
      }
      qstar[m] = out;
    }
  };
  col_fft<T, N, true, 2, CT, NT, Tiles<T, N>::CQP>(sm, tw, pro, epi);
  __syncthreads();
  if (threadIdx.x == 0 && s_bad) raise_wait_flag(nflag);
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
    const int zl = z % g.nseg;
    if (g.mask(kx, g.ky_of_row(r))) {
      const cplx<T> q0 = qo[i];
      if (zl == 0) {
        v = cscale(csub(qo[i + g.plane], q0), c);
      } else if (zl == g.nseg - 1) {
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
// Elimination factors of DGTSV for the distinct kh^2 row idx, one double4
// per level i:
//   EXACT (FP64 path): {f_i = dl_i/d'_i, d'_i, -, -}; every operation is the
//     correctly rounded IEEE operation of DGTSV (no contraction, true
//     division), so the solve reproduces LAPACK's reference DGTSV bit for bit.
//   fast (mixed path): {f_i, s/d'_i, u_i/d'_i, -} with s the RHS scaling
//     (dz^2 or dz^2 Bu) and u_i = rho_ut(i) a(i)/rho_st(i): the forward sweep
//     runs on the unscaled RHS, c_i = b_i - f_{i-1} c_{i-1}, and the back
//     substitution is one fused multiply-add on the recurrence,
//     x_i = fma(-(u_i/d'_i), x_{i+1}, (s/d'_i) c_i).
// The FP32 <-> FP64 conversions of the mixed path are done with integer
// operations only (exact, round-to-nearest-even like the hardware
// conversions, every class of input included), which keeps them off the
// FP64 pipe that bounds this kernel: a fallback to the hardware conversion
// for the rare classes would be predicated into every conversion and still
// take an FP64-pipe issue slot.  qg_selftest_conversions compares both with
// the hardware conversions bit for bit.
__device__ __forceinline__ double f32_to_f64(float v) {
  const unsigned b = __float_as_uint(v);
  const unsigned s = b & 0x80000000u, e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
  unsigned hi, lo;
  if (e - 1u < 0xfeu) {                       // normal: rebias 127 -> 1023
    hi = s | ((e + 896u) << 20) | (m >> 3);
    lo = m << 29;
  } else if (e == 0xffu) {                    // inf; nan made quiet
    hi = s | 0x7ff00000u | (m >> 3) | (m ? 0x80000u : 0u);
    lo = m << 29;
  } else if (m == 0u) {                       // signed zero
    hi = s;
    lo = 0u;
  } else {                                    // subnormal m * 2^-149: normalise
    const int p = 31 - __clz((int)m);         // leading one, 0..22
    const unsigned long long f = (unsigned long long)(m ^ (1u << p)) << (52 - p);
    hi = s | ((unsigned)(p + 874) << 20) | (unsigned)(f >> 32);
    lo = (unsigned)f;
  }
  return __hiloint2double((int)hi, (int)lo);
}
__device__ __forceinline__ float f64_to_f32(double v) {
  const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
  const unsigned s = hi & 0x80000000u;
  const int E = (int)((hi >> 20) & 0x7ffu);
  const int e = E - 896;                      // float exponent field if normal
  unsigned r;
  if (E == 0x7ff) {                           // inf; nan made quiet
    const unsigned mh = hi & 0xfffffu;
    r = (mh | lo) ? (s | 0x7fc00000u | (mh << 3) | (lo >> 29)) : (s | 0x7f800000u);
  } else if (e >= 255) {                      // overflow
    r = s | 0x7f800000u;
  } else if (e > 0) {                         // normal: keep 23 bits, round to nearest even
    r = s | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rest = lo & 0x1fffffffu;   // the 29 dropped mantissa bits
    if (rest > 0x10000000u || (rest == 0x10000000u && (r & 1u))) r += 1u;   // may carry into inf
  } else {                                    // float subnormal or zero: round(M * 2^(E-926))
    const int sh = 926 - E;                   // >= 30
    if (sh > 54 || E == 0) {
      r = s;                                  // below half the smallest subnormal
    } else {
      const unsigned long long M = (1ull << 52) | ((unsigned long long)(hi & 0xfffffu) << 32) | lo;
      const unsigned long long q = M >> sh, rem = M & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
      r = s | (unsigned)(q + ((rem > half || (rem == half && (q & 1ull))) ? 1ull : 0ull));
    }
  }
  return __uint_as_float(r);
}
template <typename T> __device__ __forceinline__ double to64(T v) { return (double)v; }
template <> __device__ __forceinline__ double to64<float>(float v) { return f32_to_f64(v); }
template <typename T> __device__ __forceinline__ T from64(double v) { return (T)v; }
template <> __device__ __forceinline__ float from64<float>(double v) { return f64_to_f32(v); }

// Thread (chain, c) of a CTA runs one real recurrence (chain = 2*rhs +
// {re, im}; rhs = q*->psi, BR->AR, BI->AI) of column c of TC consecutive
// columns.  The forward sweep keeps only a checkpoint every kSeg levels (in
// shared memory); the back substitution recomputes each kSeg-level segment
// from its checkpoint in registers and then substitutes through it.  One
// extra FMA per level buys a kernel with no scratch memory: the engine uses
// it when the scratch of k_solve_st (below) cannot be allocated.
constexpr int kSeg = 8;
constexpr int kMaxN3 = 1024;      // checkpoints + upper diagonal fit in shared memory up to here
constexpr int kSolveTC = 32;
constexpr int kSolveThreads = 6 * kSolveTC;

__host__ __device__ constexpr size_t solve_smem(int n3) {
  return (size_t)n3 * 8 + (size_t)((n3 + kSeg - 1) / kSeg) * kSolveThreads * 8;
}

template <typename T>
__global__ void __launch_bounds__(kSolveThreads, 3)
k_solve(Geom g, double dz, double Bu, const int* __restrict__ tab_idx,
        const double4* __restrict__ fac_psi, const double4* __restrict__ fac_A, const double* __restrict__ du,
        const cplx<T>* __restrict__ qs, const cplx<T>* __restrict__ BR, const cplx<T>* __restrict__ BI,
        cplx<T>* __restrict__ psi, cplx<T>* __restrict__ AR, cplx<T>* __restrict__ AI,
        int do_psi, int do_A, int seg0) {
  constexpr bool EXACT = sizeof(T) == 8;
  constexpr int TC = kSolveTC, NTH = kSolveThreads, S = kSeg;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n3 = g.nseg;                          // levels of one column (blockIdx.y: its segment)
  double* du_s = reinterpret_cast<double*>(smem_raw);
  double* ck = du_s + n3 + threadIdx.x;           // checkpoint of segment j at ck[j*NTH]
  for (int i = threadIdx.x; i < n3; i += NTH) du_s[i] = du[i];
  __syncthreads();
  const int chain = threadIdx.x / TC, c = threadIdx.x % TC;
  const int rhs_id = chain >> 1, part = chain & 1;
  if (rhs_id == 0 ? !do_psi : !do_A) return;
  const long long m = (long long)blockIdx.x * TC + c;
  if (m >= g.plane) return;
  const int kx = (int)(m % g.KXP);
  if (kx > g.K) return;
  const long long P = g.plane;
  const long long moff = 2 * (long long)(seg0 + blockIdx.y) * n3 * P;     // this segment's levels
  const T* rhs = reinterpret_cast<const T*>(rhs_id == 0 ? qs : (rhs_id == 1 ? BR : BI)) + part + moff;
  T* out = reinterpret_cast<T*>(rhs_id == 0 ? psi : (rhs_id == 1 ? AR : AI)) + part + moff;
  const int idx = tab_idx[m];
  if (idx < 0) {
    for (int i = 0; i < n3; ++i) out[2 * (i * P + m)] = (T)0;
    return;
  }
  const double4* F = (rhs_id == 0 ? fac_psi : fac_A) + (long long)idx * n3;
  const double s = rhs_id == 0 ? __dmul_rn(dz, dz) : __dmul_rn(__dmul_rn(dz, dz), Bu);
  const int nseg = (n3 + S - 1) / S;
  // one forward step: EXACT reproduces DGTSV (scaled RHS), fast runs unscaled
  auto fwd = [&](double x, double f, T r) -> double {
    return EXACT ? __dsub_rn(__dmul_rn(s, to64<T>(r)), __dmul_rn(f, x)) : fma(-f, x, to64<T>(r));
  };
  // forward sweep, checkpoints only
  double x = 0.0;
  for (int j = 0; j < nseg; ++j) {
    ck[(size_t)j * NTH] = x;
    T r[S];
    double f[S];
#pragma unroll
    for (int k = 0; k < S; ++k) {
      const int i = j * S + k;
      r[k] = i < n3 ? rhs[2 * (i * P + m)] : (T)0;
      f[k] = (i > 0 && i < n3) ? F[i - 1].x : 0.0;
    }
#pragma unroll
    for (int k = 0; k < S; ++k)
      if (j * S + k < n3) x = fwd(x, f[k], r[k]);
  }
  // back substitution, segment by segment from the top
  double xn = 0.0;      // x_{i+1}
  for (int j = nseg - 1; j >= 0; --j) {
    T r[S];
    double4 fl[S];
    double fprev[S];
#pragma unroll
    for (int k = 0; k < S; ++k) {
      const int i = j * S + k;
      r[k] = i < n3 ? rhs[2 * (i * P + m)] : (T)0;
      fprev[k] = (i > 0 && i < n3) ? F[i - 1].x : 0.0;
      fl[k] = i < n3 ? F[i] : make_double4(0, 1, 0, 0);
    }
    double v[S];
    double xc = ck[(size_t)j * NTH];
#pragma unroll
    for (int k = 0; k < S; ++k) {
      if (j * S + k < n3) xc = fwd(xc, fprev[k], r[k]);
      v[k] = xc;
    }
#pragma unroll
    for (int k = S - 1; k >= 0; --k) {
      const int i = j * S + k;
      if (i < n3) {
        if (i == n3 - 1) xn = EXACT ? __ddiv_rn(v[k], fl[k].y) : fl[k].y * v[k];
        else if (EXACT) xn = __ddiv_rn(__dsub_rn(v[k], __dmul_rn(du_s[i], xn)), fl[k].y);
        else xn = fma(-fl[k].z, xn, fl[k].y * v[k]);
        out[2 * (i * P + m)] = from64<T>(xn);
      }
    }
  }
}

// The same recurrences with every forward value kept in global scratch
// (vbuf: 6 chains x n3 x plane doubles) instead of checkpoints plus
// recomputation: one FMA per level less on the FP64 pipe, the values
// round-trip through memory (coalesced: a warp covers 32 consecutive
// columns of one chain).  Same arithmetic, bitwise the same results.
// TC columns per CTA (16, 32 or 64: the block shape the autotuner picks),
// 6*TC threads, the register budget of 4 CTAs of 192 threads.
constexpr bool kSolveStore = true;
constexpr bool kSolvePerColumn = true;  // mixed solves read per-column factor copies (k_expand_fac)
constexpr int kSegSt = 8;          // k_solve_st: levels per register segment of the sweeps
constexpr int kSolveStBlocks = 128;  // k_solve_st: register target of 128/TC CTAs of 6*TC threads per SM
// The A solves (B^{n+1} -> A, 4 of the 6 recurrences per column) depend only
// on k_col_update's B^{n+1}: with kSolveOverlap they run on a second,
// lower-priority stream beside k_row_qw / k_col_qw / the psi solve, and the
// persistent k_row_qw takes kQwReserve fewer CTAs per SM than fit, leaving
// registers for solve CTAs.  Off by default: at 512^2 x 256 the step is
// 0.07-0.10 ms slower with it (the solves stream ~2 GB per step through DRAM
// - q*, B, the per-column factors, their forward values - and contend with
// the q^w kernels for bandwidth rather than only filling the idle FP64 pipe).
#ifndef QG_SOLVE_OVERLAP
#define QG_SOLVE_OVERLAP 0
#endif
#ifndef QG_QW_RESERVE
#define QG_QW_RESERVE 1
#endif
constexpr bool kSolveOverlap = QG_SOLVE_OVERLAP != 0;
#ifndef QG_REUSE_B
#define QG_REUSE_B 1
#endif
constexpr bool kReuseB = QG_REUSE_B != 0;   // kept y-inverse planes of B (q_off)
// Phase-A batches are independent (z-local): with several batches per step,
// up to kBatchLanes of them run at once on their own streams and scratch
// slots, so that different kernels of different batches share the GPU and
// each batch's (kx,y) planes can stay in L2 between its kernels.
#ifndef QG_BATCH_LANES
#define QG_BATCH_LANES 1
#endif
constexpr int kBatchLanes = QG_BATCH_LANES;
constexpr int kQwReserve = QG_QW_RESERVE;
// Per-column copies of the mixed path's elimination factors, expanded from
// the per-kh^2 tables so that the consecutive columns of a warp read
// consecutive words (the per-kh^2 rows of neighbouring columns are scattered:
// one 32-byte sector per column and level).  pc[(o*3 + q)*L + i*P + m],
// L = n3*P, operator o (0 psi, 1 A), q = 0: f_{i-1} (0 at i = 0),
// 1: s/d'_i, 2: u_i/d'_i; zeros where the column holds no retained mode.
static __global__ void k_expand_fac(Geom g, const int* __restrict__ tab_idx, const double4* __restrict__ fac_psi,
                                    const double4* __restrict__ fac_A, double* __restrict__ pc,
                                    const int* __restrict__ cols, int ncols) {
  const long long P = ncols, L = (long long)g.nseg * P;     // one segment's levels, listed columns
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < L; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / P);
    const long long m = e - (long long)i * P;
    const int idx = tab_idx[cols[m]];
#pragma unroll
    for (int o = 0; o < 2; ++o) {
      double f = 0.0, y = 0.0, z = 0.0;
      if (idx >= 0) {
        const double4* Fc = (o == 0 ? fac_psi : fac_A) + (long long)idx * g.nseg;
        f = i > 0 ? Fc[i - 1].x : 0.0;
        y = Fc[i].y;
        z = Fc[i].z;
      }
      pc[(o * 3 + 0) * L + e] = f;
      pc[(o * 3 + 1) * L + e] = y;
      pc[(o * 3 + 2) * L + e] = z;
    }
  }
}

// PC (mixed path): factors from the per-column copies pc (k_expand_fac)
// instead of the per-kh^2 tables; the same values, so the same results.
template <typename T, int TC, bool PC>
__global__ void __launch_bounds__(6 * TC, kSolveStBlocks / TC)
k_solve_st(Geom g, double dz, double Bu, const int* __restrict__ tab_idx,
           const double4* __restrict__ fac_psi, const double4* __restrict__ fac_A, const double* __restrict__ du,
           const cplx<T>* __restrict__ qs, const cplx<T>* __restrict__ BR, const cplx<T>* __restrict__ BI,
           cplx<T>* __restrict__ psi, cplx<T>* __restrict__ AR, cplx<T>* __restrict__ AI,
           int do_psi, int do_A, double* __restrict__ vbuf, const double* __restrict__ pc, int seg0,
           const int* __restrict__ cols, int ncols) {
  constexpr bool EXACT = sizeof(T) == 8;
  constexpr bool USEPC = PC && !EXACT;
  constexpr int S = kSegSt;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n3 = g.nseg;          // levels of one column (blockIdx.y: its segment)
  double* du_s = reinterpret_cast<double*>(smem_raw);
  for (int i = threadIdx.x; i < n3; i += blockDim.x) du_s[i] = du[i];
  __syncthreads();
  // the CTA runs the recurrences asked for: 2*TC threads per right-hand
  // side, psi's first (chains 0, 1: psi; 2, 3: AR; 4, 5: AI)
  const int chain = (do_psi ? 0 : 2) + threadIdx.x / TC, c = threadIdx.x % TC;
  const int rhs_id = chain >> 1, part = chain & 1;
  if (rhs_id == 0 ? !do_psi : !do_A) return;
  // thread column: entry li of the list of retained columns (cols), whose
  // forward values and per-column factors are stored at li with a stride of
  // ncols per level; the state fields at m with a stride of the plane
  const long long li = (long long)blockIdx.x * TC + c;
  if (li >= ncols) return;
  const long long m = cols[li];
  const long long P = g.plane;
  const long long moff = (long long)(seg0 + blockIdx.y) * n3 * P;     // this segment's first level
  const T* rhs = reinterpret_cast<const T*>(rhs_id == 0 ? qs : (rhs_id == 1 ? BR : BI)) + part + 2 * moff;
  T* out = reinterpret_cast<T*>(rhs_id == 0 ? psi : (rhs_id == 1 ? AR : AI)) + part + 2 * moff;
  const int idx = tab_idx[m];
  if (idx < 0) {
    for (int i = 0; i < n3; ++i) out[2 * (i * P + m)] = (T)0;
    return;
  }
  const double4* F = (rhs_id == 0 ? fac_psi : fac_A) + (long long)idx * n3;
  const double s = rhs_id == 0 ? __dmul_rn(dz, dz) : __dmul_rn(__dmul_rn(dz, dz), Bu);
  const long long NL = ncols;
  double* vb = vbuf + (long long)chain * g.n3 * NL + (long long)(seg0 + blockIdx.y) * n3 * NL + li;
  const long long L = (long long)n3 * NL;         // per-column factors: one segment's levels
  // (USEPC) f_{i-1}, s/d'_i, u_i/d'_i of this column at + q*L + i*NL
  const double* pcf = USEPC ? pc + (rhs_id == 0 ? 0 : 3) * L + li : nullptr;
  auto fwd = [&](double x, double f, T r) -> double {
    return EXACT ? __dsub_rn(__dmul_rn(s, to64<T>(r)), __dmul_rn(f, x)) : fma(-f, x, to64<T>(r));
  };
  const int nseg = (n3 + S - 1) / S;
  double x = 0.0;
  auto load_seg = [&](int j, T (&r)[S], double (&f)[S]) {
#pragma unroll
    for (int k = 0; k < S; ++k) {
      const int i = j * S + k;
      r[k] = i < n3 ? rhs[2 * (i * P + m)] : (T)0;
      if constexpr (USEPC) f[k] = i < n3 ? pcf[(long long)i * NL] : 0.0;
      else f[k] = (i > 0 && i < n3) ? F[i - 1].x : 0.0;
    }
  };
  auto run_seg = [&](int j, const T (&r)[S], const double (&f)[S]) {
#pragma unroll
    for (int k = 0; k < S; ++k) {
      const int i = j * S + k;
      if (i < n3) { x = fwd(x, f[k], r[k]); vb[(long long)i * NL] = x; }
    }
  };
  for (int j = 0; j < nseg; ++j) {
    T r[S];
    double f[S];
    load_seg(j, r, f);
    run_seg(j, r, f);
  }
  double xn = 0.0;
  for (int j = nseg - 1; j >= 0; --j) {
    double v[S], yk[S], zk[S];
#pragma unroll
    for (int k = 0; k < S; ++k) {
      const int i = j * S + k;
      v[k] = i < n3 ? vb[(long long)i * NL] : 0.0;
      if constexpr (USEPC) {
        yk[k] = i < n3 ? pcf[L + (long long)i * NL] : 1.0;
        zk[k] = i < n3 ? pcf[2 * L + (long long)i * NL] : 0.0;
      } else {
        const double4 fl = i < n3 ? F[i] : make_double4(0, 1, 0, 0);
        yk[k] = fl.y;
        zk[k] = fl.z;
      }
    }
#pragma unroll
    for (int k = S - 1; k >= 0; --k) {
      const int i = j * S + k;
      if (i < n3) {
        if (i == n3 - 1) xn = EXACT ? __ddiv_rn(v[k], yk[k]) : yk[k] * v[k];
        else if (EXACT) xn = __ddiv_rn(__dsub_rn(v[k], __dmul_rn(du_s[i], xn)), yk[k]);
        else xn = fma(-zk[k], xn, yk[k] * v[k]);
        out[2 * (i * P + m)] = from64<T>(xn);
      }
    }
  }
}

// ===========================================================================
// Conversions between the reference layout and the compact layout
// ===========================================================================
// dense: double2 [nlev][ikty][iktx]
// nflag (optional, mapped page-locked word): set to 1 when a retained mode
// of the input is NaN or infinite (modes with L=0 are discarded unread).
template <typename T>
static __global__ void k_dense_to_compact(Geom g, int level0, int nlev, const double2* __restrict__ dense,
                                          cplx<T>* __restrict__ f, int* __restrict__ nflag = nullptr) {
  const int iktx = g.n / 2 + 1;
  const long long tot = (long long)nlev * g.plane;
  bool bad = false;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot; i += (long long)gridDim.x * blockDim.x) {
    const int l = (int)(i / g.plane);
    const long long m = i - (long long)l * g.plane;
    const int r = (int)(m / g.KXP), kx = (int)(m % g.KXP);
    const int ky = g.ky_of_row(r);
    cplx<T> v = mk<T>(0, 0);
    if (g.mask(kx, ky)) {
      const int iky = ky >= 0 ? ky : g.n + ky;
      const double2 d = dense[((long long)l * g.n + iky) * iktx + kx];
      bad |= !isfinite(d.x) || !isfinite(d.y);
      v = mk<T>((T)d.x, (T)d.y);
    }
    f[(long long)(level0 + l) * g.plane + m] = v;
  }
  if (nflag && __syncthreads_or(bad) && threadIdx.x == 0) raise_wait_flag(nflag);
}

// compact FP64 values rounded to T (the same rounding as k_dense_to_compact)
template <typename T>
__global__ void k_round_compact(long long n, const cplx<double>* __restrict__ src, cplx<T>* __restrict__ dst) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const cplx<double> v = src[i];
    dst[i] = mk<T>((T)v.x, (T)v.y);
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
      } else if (z % g.nseg < g.nseg - 1) {   // A_z = 0 on each segment's top level
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
__global__ void k_sumB(Geom g, cplx<T>* __restrict__ BR, cplx<T>* __restrict__ BI, int zbeg, int zend) {
  const long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (m >= g.plane) return;
  const int r = (int)(m / g.KXP), kx = (int)(m % g.KXP);
  const int ky = g.ky_of_row(r);
  if (!g.mask(kx, ky) || kx * kx + ky * ky == 0) return;
  for (int z0 = zbeg; z0 < zend; z0 += g.nseg) {   // each vertical segment of [zbeg, zend) on its own
    double sr0 = 0, sr1 = 0, si0 = 0, si1 = 0;
    for (int z = z0; z < z0 + g.nseg; ++z) {
      const cplx<T> a = BR[z * g.plane + m], b = BI[z * g.plane + m];
      sr0 += a.x; sr1 += a.y; si0 += b.x; si1 += b.y;
    }
    sr0 /= g.nseg; sr1 /= g.nseg; si0 /= g.nseg; si1 /= g.nseg;
    for (int z = z0; z < z0 + g.nseg; ++z) {
      cplx<T> a = BR[z * g.plane + m], b = BI[z * g.plane + m];
      a.x = (T)((double)a.x - sr0); a.y = (T)((double)a.y - sr1);
      b.x = (T)((double)b.x - si0); b.y = (T)((double)b.y - si1);
      BR[z * g.plane + m] = a; BI[z * g.plane + m] = b;
    }
  }
}

// init_q (init.f90:591-652): q = [d/dz(a dpsi/dz) - kh^2 psi] with Neumann
// ends, evaluated in FP64 in the reference's order with correctly rounded
// operations and no contraction: the terms a*psi (a up to ~e^10 under
// strong stratification) cancel, so the rounding sequence matters.
template <typename T, typename TI>
__global__ void k_init_q(Geom g, double dz, const double* __restrict__ cu, const double* __restrict__ cl,
                         const cplx<TI>* __restrict__ psi, cplx<T>* __restrict__ q, int zbeg, int zend) {
  const long long tot = (long long)zend * g.plane;
  const double dz2 = __dmul_rn(dz, dz);
  for (long long i = (long long)zbeg * g.plane + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < tot;
       i += (long long)gridDim.x * blockDim.x) {
    const int z = (int)(i / g.plane), zl = z % g.nseg;   // zl: level within its segment
    const long long m = i - (long long)z * g.plane;
    const int r = (int)(m / g.KXP), kx = (int)(m % g.KXP);
    const int ky = g.ky_of_row(r);
    cplx<T> out = mk<T>(0, 0);
    if (g.mask(kx, ky)) {
      const double kdz = __dmul_rn(__dmul_rn((double)(kx * kx + ky * ky), dz), dz);
      const cplx<TI> p0 = psi[i];
      double vr, vi;
      if (zl == 0) {
        const cplx<TI> pp = psi[i + g.plane];
        const double d = __dadd_rn(cu[0], kdz);
        vr = __dsub_rn(__dmul_rn(cu[0], (double)pp.x), __dmul_rn(d, (double)p0.x));
        vi = __dsub_rn(__dmul_rn(cu[0], (double)pp.y), __dmul_rn(d, (double)p0.y));
      } else if (zl == g.nseg - 1) {
        const cplx<TI> pm = psi[i - g.plane];
        const double d = __dadd_rn(cl[zl], kdz);
        vr = __dadd_rn(-__dmul_rn(d, (double)p0.x), __dmul_rn(cl[zl], (double)pm.x));
        vi = __dadd_rn(-__dmul_rn(d, (double)p0.y), __dmul_rn(cl[zl], (double)pm.y));
      } else {
        const cplx<TI> pp = psi[i + g.plane], pm = psi[i - g.plane];
        const double d = __dadd_rn(__dadd_rn(cu[zl], cl[zl]), kdz);
        vr = __dadd_rn(__dsub_rn(__dmul_rn(cu[zl], (double)pp.x), __dmul_rn(d, (double)p0.x)),
                       __dmul_rn(cl[zl], (double)pm.x));
        vi = __dadd_rn(__dsub_rn(__dmul_rn(cu[zl], (double)pp.y), __dmul_rn(d, (double)p0.y)),
                       __dmul_rn(cl[zl], (double)pm.y));
      }
      out = mk<T>((T)__ddiv_rn(vr, dz2), (T)__ddiv_rn(vi, dz2));
    }
    q[i] = out;
  }
}

// ===========================================================================
// Regular YBJ (ybj_plus = 0): sumB and compute_A after the update, one thread
// per retained column, FP64 (derivatives.f90:1073-1118, 1141-1264)
// ===========================================================================
template <typename T>
__global__ void k_ybj_A(Geom g, double dz, double Bu, double Ro, const double* __restrict__ r2, cplx<T>* __restrict__ BR,
                        cplx<T>* __restrict__ BI, const cplx<T>* __restrict__ sig1, const cplx<T>* __restrict__ sig2,
                        cplx<T>* __restrict__ AR, cplx<T>* __restrict__ AI) {
  const long long mcol = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (mcol >= g.plane) return;
  const int r = (int)(mcol / g.KXP), kx = (int)(mcol % g.KXP);
  const int ky = g.ky_of_row(r);
  const int n3 = g.n3;
  if (kx > g.K) return;
  if (!(g.mask(kx, ky) && kx * kx + ky * ky > 0)) {
    for (int z = 0; z < n3; ++z) { AR[z * g.plane + mcol] = mk<T>(0, 0); AI[z * g.plane + mcol] = mk<T>(0, 0); }
    return;
  }
  // sumB: remove the vertical mean of B
  double sR[2] = {0, 0}, sI[2] = {0, 0}, g1[2] = {0, 0}, g2[2] = {0, 0};
  for (int z = 0; z < n3; ++z) {
    const long long m = z * g.plane + mcol;
    const cplx<T> br = BR[m], bi = BI[m], a = sig1[m], b = sig2[m];
    sR[0] += to64<T>(br.x); sR[1] += to64<T>(br.y);
    sI[0] += to64<T>(bi.x); sI[1] += to64<T>(bi.y);
    g1[0] += to64<T>(a.x); g1[1] += to64<T>(a.y);
    g2[0] += to64<T>(b.x); g2[1] += to64<T>(b.y);
  }
  const double mR[2] = {sR[0] / n3, sR[1] / n3}, mI[2] = {sI[0] / n3, sI[1] / n3};
  // sigma = sigma * Bu * Ro (derivatives.f90:1066)
  const double s1[2] = {g1[0] * Bu * Ro, g1[1] * Bu * Ro}, s2[2] = {g2[0] * Bu * Ro, g2[1] * Bu * Ro};
  // A~(0) = 0, A~(z) = A~(z-1) + sumB r_2ut(z-1) dz dz, sumB the running sum of B
  double aR[2] = {0, 0}, aI[2] = {0, 0}, bR[2], bI[2], tR[2] = {0, 0}, tI[2] = {0, 0};
  {
    const cplx<T> br = BR[mcol], bi = BI[mcol];
    bR[0] = to64<T>(br.x) - mR[0]; bR[1] = to64<T>(br.y) - mR[1];
    bI[0] = to64<T>(bi.x) - mI[0]; bI[1] = to64<T>(bi.y) - mI[1];
    BR[mcol] = mk<T>(from64<T>(bR[0]), from64<T>(bR[1]));
    BI[mcol] = mk<T>(from64<T>(bI[0]), from64<T>(bI[1]));
    AR[mcol] = mk<T>(0, 0); AI[mcol] = mk<T>(0, 0);
  }
  for (int z = 1; z < n3; ++z) {
    const long long m = z * g.plane + mcol;
    const double c = r2[z - 1];
    for (int k = 0; k < 2; ++k) {
      aR[k] = aR[k] + bR[k] * c * dz * dz;
      aI[k] = aI[k] + bI[k] * c * dz * dz;
      tR[k] += aR[k];
      tI[k] += aI[k];
    }
    AR[m] = mk<T>(from64<T>(aR[0]), from64<T>(aR[1]));
    AI[m] = mk<T>(from64<T>(aI[0]), from64<T>(aI[1]));
    const cplx<T> br = BR[m], bi = BI[m];
    const double nbR[2] = {to64<T>(br.x) - mR[0], to64<T>(br.y) - mR[1]};
    const double nbI[2] = {to64<T>(bi.x) - mI[0], to64<T>(bi.y) - mI[1]};
    BR[m] = mk<T>(from64<T>(nbR[0]), from64<T>(nbR[1]));
    BI[m] = mk<T>(from64<T>(nbI[0]), from64<T>(nbI[1]));
    for (int k = 0; k < 2; ++k) { bR[k] += nbR[k]; bI[k] += nbI[k]; }
  }
  // A = A~ + (sigma - sum A~)/n3
  const double cR[2] = {(s1[0] - tR[0]) / n3, (s1[1] - tR[1]) / n3};
  const double cI[2] = {(s2[0] - tI[0]) / n3, (s2[1] - tI[1]) / n3};
  for (int z = 0; z < n3; ++z) {
    const long long m = z * g.plane + mcol;
    const cplx<T> a = AR[m], b = AI[m];
    AR[m] = mk<T>(from64<T>(to64<T>(a.x) + cR[0]), from64<T>(to64<T>(a.y) + cR[1]));
    AI[m] = mk<T>(from64<T>(to64<T>(b.x) + cI[0]), from64<T>(to64<T>(b.y) + cI[1]));
  }
}

// ===========================================================================
// FP64 diagnostics (diagnostics.f90: wave_energy 647-743, the rotational part
// of diag_zentrum 16-211, enstrophy 1262-1363): column partial sums, then a
// fixed-order sum of the partials
// ===========================================================================
// A thread owns one retained column (kx, ky) and walks a chunk of levels of
// one vertical segment, loading each level's B, A and psi
// once (the level above is the next iteration's level) and accumulating six
// column sums: |B|^2, w1_z |A(z+1)-A(z)|^2, |A|^2, |psi|^2,
// w4_z |psi(z+1)-psi(z)|^2 and |psi(z+1)-psi(z)|^2, with the per-level
// weights w1_z = 0.5/(r2_z Bu dz^2), w4_z = Bu/(r2_z dz^2) (the difference
// terms vanish on a segment's top level).  The column's factors (kh^2,
// kh^4, the half weight of the (0,0) mode) multiply the sums once, in FP64,
// giving the seven integrals:
//   wke = w00 S_b, wpe = kh^2 S_w1c, wce = kh^4 S_a / (8 Bu^2), ke = kh^2 S_p,
//   pe = w00 S_w4b, zeta2 = 2 kh^4 S_p, omegah2 = 2 kh^2 S_b' / dz^2.
constexpr int kNDiag = 7;
constexpr int kDiagSums = 6;
#ifndef QG_DIAG_MINB
#define QG_DIAG_MINB 10
#endif
constexpr int kDiagMinB = QG_DIAG_MINB;   // register target: CTAs per SM
#ifndef QG_DIAG_UNROLL
#define QG_DIAG_UNROLL 2
#endif
constexpr int kDiagUnroll = QG_DIAG_UNROLL;   // levels per iteration of the FP32-pair loop
constexpr int kDiagThreads = 128;  // columns per CTA

// --- FP32-pair ("double-float") arithmetic for the FP32 state --------------
// A pair (h, l) stands for the real number h + l.  GB300 issues FP32 at many
// times its FP64 rate, and every FP32 product x*y is exactly p + e with
// p = fl(x*y), e = fma(x, y, -p); two FP32 numbers add exactly into s + t
// (Knuth's TwoSum, 6 additions).  With these error-free transformations the
// sums of squares of FP32 values below are FP64-grade (about 2^-44 relative
// per sum) on the FP32 pipes.
struct f2 { float h, l; };
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& t) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  t = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// x0^2 + x1^2: every square exact as p + e, the p's added with TwoSum, the
// e's and the TwoSum remainder in the low word
__device__ __forceinline__ f2 f2_sq2(float a, float b) {
  const float pa = __fmul_rn(a, a), ea = __fmaf_rn(a, a, -pa);
  const float pb = __fmul_rn(b, b), eb = __fmaf_rn(b, b, -pb);
  f2 r;
  float t;
  two_sum(pa, pb, r.h, t);
  r.l = __fadd_rn(__fadd_rn(ea, eb), t);
  return r;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  f2 r;
  float t;
  two_sum(a.h, b.h, r.h, t);
  r.l = __fadd_rn(__fadd_rn(a.l, b.l), t);
  return r;
}
// (a1 - a0)^2 + (b1 - b0)^2: each difference exact as d + err (TwoSum), its
// square as p + e + 2 d err (err^2 <= 2^-48 d^2 is dropped)
__device__ __forceinline__ f2 f2_dsq2(float a1, float a0, float b1, float b0) {
  float da, ra, db, rb;
  two_sum(a1, -a0, da, ra);
  two_sum(b1, -b0, db, rb);
  const float pa = __fmul_rn(da, da), ea = __fmaf_rn(__fmul_rn(2.0f, da), ra, __fmaf_rn(da, da, -pa));
  const float pb = __fmul_rn(db, db), eb = __fmaf_rn(__fmul_rn(2.0f, db), rb, __fmaf_rn(db, db, -pb));
  f2 r;
  float t;
  two_sum(pa, pb, r.h, t);
  r.l = __fadd_rn(__fadd_rn(ea, eb), t);
  return r;
}
// (wh + wl) * (h + l): wh*h exact as q + r, the cross terms rounded
__device__ __forceinline__ f2 f2_mul(float wh, float wl, f2 a) {
  f2 r;
  r.h = __fmul_rn(wh, a.h);
  r.l = __fmaf_rn(wl, a.h, __fmaf_rn(wh, a.l, __fmaf_rn(wh, a.h, -r.h)));
  return r;
}
// accumulator += a, renormalised so that |l| <= ulp(h)/2 (Fast2Sum)
__device__ __forceinline__ void f2_acc(f2& s, f2 a) {
  float h, t;
  two_sum(s.h, a.h, h, t);
  const float l = __fadd_rn(__fadd_rn(s.l, a.l), t);
  s.h = __fadd_rn(h, l);
  s.l = __fsub_rn(l, __fsub_rn(s.h, h));
}
__device__ __forceinline__ bool f2_finite(f2 a) { return fabsf(a.h) <= 3.0e38f && fabsf(a.l) <= 3.0e38f; }

// The six column sums of levels [zlo, zhi) of the segment whose top level is
// ztop, in FP64 arithmetic; wz: w1 at [0, nseg), w4 at [nseg, 2 nseg).
template <typename T>
__device__ __forceinline__ void diag_column_fp64(const Geom& g, long long m, int zlo, int zhi, int ztop,
                                                 const double* __restrict__ wz, const cplx<T>* __restrict__ BR,
                                                 const cplx<T>* __restrict__ BI, const cplx<T>* __restrict__ AR,
                                                 const cplx<T>* __restrict__ AI, const cplx<T>* __restrict__ psi,
                                                 double S[kDiagSums]) {
  for (int k = 0; k < kDiagSums; ++k) S[k] = 0.0;
  const long long P = g.plane;
  cplx<T> ar = AR[zlo * P + m], ai = AI[zlo * P + m], ps = psi[zlo * P + m];
  for (int z = zlo; z < zhi; ++z) {
    const cplx<T> br = BR[z * P + m], bi = BI[z * P + m];
    const double brx = to64<T>(br.x), bry = to64<T>(br.y), bix = to64<T>(bi.x), biy = to64<T>(bi.y);
    const double arx = to64<T>(ar.x), ary = to64<T>(ar.y), aix = to64<T>(ai.x), aiy = to64<T>(ai.y);
    const double px = to64<T>(ps.x), py = to64<T>(ps.y);
    S[0] += brx * brx + bry * bry + bix * bix + biy * biy;
    S[2] += arx * arx + ary * ary + aix * aix + aiy * aiy;
    S[3] += px * px + py * py;
    if (z < ztop) {
      const cplx<T> ar1 = AR[(z + 1) * P + m], ai1 = AI[(z + 1) * P + m], p1 = psi[(z + 1) * P + m];
      const double crx = to64<T>(ar1.x) - arx, cry = to64<T>(ar1.y) - ary;
      const double cix = to64<T>(ai1.x) - aix, ciy = to64<T>(ai1.y) - aiy;
      const double bx = to64<T>(p1.x) - px, by = to64<T>(p1.y) - py;
      const double pz2 = bx * bx + by * by;
      const int zl = z - (ztop + 1 - g.nseg);      // level within the segment
      S[1] += wz[zl] * (crx * crx + cry * cry + cix * cix + ciy * ciy);
      S[4] += wz[g.nseg + zl] * pz2;
      S[5] += pz2;
      ar = ar1; ai = ai1; ps = p1;
    }
  }
}

// The same sums of the FP32 state in FP32-pair arithmetic; wzf holds the
// weights as pairs.  Error per sum: about 2^-44 of the sum (the TwoSum
// accumulation, the rounded cross terms, the dropped err^2), plus at most
// 2^-100 absolute per mode for values below 2^-50, whose square's low word
// underflows.  Returns false when a pair is not finite (values beyond ~2^60
// overflow FP32 squares); the caller then recomputes the column in FP64.
__device__ __forceinline__ bool diag_column_f2(const Geom& g, long long m, int zlo, int zhi, int ztop,
                                               const float2* __restrict__ wzf, const cplx<float>* __restrict__ BR,
                                               const cplx<float>* __restrict__ BI,
                                               const cplx<float>* __restrict__ AR,
                                               const cplx<float>* __restrict__ AI,
                                               const cplx<float>* __restrict__ psi, double S[kDiagSums]) {
  f2 s[kDiagSums];
  for (int k = 0; k < kDiagSums; ++k) s[k] = f2{0.0f, 0.0f};
  const long long P = g.plane;
  cplx<float> ar = AR[zlo * P + m], ai = AI[zlo * P + m], ps = psi[zlo * P + m];
#pragma unroll kDiagUnroll
  for (int z = zlo; z < zhi; ++z) {
    const cplx<float> br = BR[z * P + m], bi = BI[z * P + m];
    f2_acc(s[0], f2_add(f2_sq2(br.x, br.y), f2_sq2(bi.x, bi.y)));
    f2_acc(s[2], f2_add(f2_sq2(ar.x, ar.y), f2_sq2(ai.x, ai.y)));
    f2_acc(s[3], f2_sq2(ps.x, ps.y));
    if (z < ztop) {
      const cplx<float> ar1 = AR[(z + 1) * P + m], ai1 = AI[(z + 1) * P + m], p1 = psi[(z + 1) * P + m];
      const int zl = z - (ztop + 1 - g.nseg);      // level within the segment
      const float2 w1 = wzf[zl], w4 = wzf[g.nseg + zl];
      const f2 c2 = f2_add(f2_dsq2(ar1.x, ar.x, ar1.y, ar.y), f2_dsq2(ai1.x, ai.x, ai1.y, ai.y));
      const f2 pz2 = f2_dsq2(p1.x, ps.x, p1.y, ps.y);
      f2_acc(s[1], f2_mul(w1.x, w1.y, c2));
      f2_acc(s[4], f2_mul(w4.x, w4.y, pz2));
      f2_acc(s[5], pz2);
      ar = ar1; ai = ai1; ps = p1;
    }
  }
  bool ok = true;
  for (int k = 0; k < kDiagSums; ++k) {
    ok = ok && f2_finite(s[k]);
    S[k] = f32_to_f64(s[k].h) + f32_to_f64(s[k].l);
  }
  return ok;
}

// grid: (columns / kDiagThreads, chunks of zc levels per segment, segments
// seg0 ...), sized by the host to one wave of resident CTAs; part: kNDiag
// partials per CTA, at ((blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x +
// blockIdx.x) * kNDiag.  c2 = 1/(8 Bu^2), c6 = 2/dz^2.
template <typename T>
__global__ void __launch_bounds__(kDiagThreads, kDiagMinB)
k_diag_cols(Geom g, int seg0, int zc, const double* __restrict__ wz, const float2* __restrict__ wzf, double c2, double c6,
            const cplx<T>* __restrict__ BR, const cplx<T>* __restrict__ BI, const cplx<T>* __restrict__ AR,
            const cplx<T>* __restrict__ AI, const cplx<T>* __restrict__ psi, const int* __restrict__ cols,
            int ncols, double* __restrict__ part) {
  __shared__ double red[kNDiag][kDiagThreads / 32];
  const int li = blockIdx.x * kDiagThreads + threadIdx.x;
  double acc[kNDiag] = {0, 0, 0, 0, 0, 0, 0};
  if (li < ncols) {
    const long long m = cols[li];
    const int r = (int)(m / g.KXP), kx = (int)(m - (long long)r * g.KXP);
    const int ky = g.ky_of_row(r);
    const int zs = (seg0 + blockIdx.z) * g.nseg, ztop = zs + g.nseg - 1;
    const int zlo = zs + blockIdx.y * zc, zhi = zlo + zc < zs + g.nseg ? zlo + zc : zs + g.nseg;
    double S[kDiagSums];
    if constexpr (std::is_same<T, float>::value) {
      if (!diag_column_f2(g, m, zlo, zhi, ztop, wzf, BR, BI, AR, AI, psi, S))
        diag_column_fp64<T>(g, m, zlo, zhi, ztop, wz, BR, BI, AR, AI, psi, S);
    } else {
      diag_column_fp64<T>(g, m, zlo, zhi, ztop, wz, BR, BI, AR, AI, psi, S);
    }
    // exact int -> double without a conversion instruction: (2^52 + k) - 2^52
    const double kh2 = __hiloint2double(0x43300000, kx * kx + ky * ky) - 4503599627370496.0;
    const double kh4 = kh2 * kh2;                      // exact: < 2^53
    const double w00 = (kx == 0 && ky == 0) ? 0.5 : 1.0;
    acc[0] = w00 * S[0];
    acc[1] = kh2 * S[1];
    acc[2] = (kh4 * S[2]) * c2;
    acc[3] = kh2 * S[3];
    acc[4] = w00 * S[4];
    acc[5] = 2.0 * (kh4 * S[3]);
    acc[6] = (kh2 * S[5]) * c6;
  }
  // fixed-order reduction: a butterfly in each warp, then the warps in order
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kNDiag; ++k) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[k][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < kNDiag) {
    double v = 0.0;
    for (int i = 0; i < kDiagThreads / 32; ++i) v += red[threadIdx.x][i];
    part[(((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x) * kNDiag + threadIdx.x] = v;
  }
}

// one warp per quantity: lane l sums partials l, l+32, ... in order, then a
// fixed butterfly over the lanes; the mean over the nlev levels
static __global__ void k_diag_sum(long long nparts, int nlev, const double* __restrict__ part, double* __restrict__ out) {
  const int k = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (k >= kNDiag) return;
  double s = 0.0;
  for (long long p = lane; p < nparts; p += 32) s += part[p * kNDiag + k];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[k] = s / nlev;
}

}  // namespace qg
