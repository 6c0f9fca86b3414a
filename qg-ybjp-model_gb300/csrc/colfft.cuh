// Column (y-direction) FFTs of a tile of CT spectral columns, interleaved in
// shared memory, with the first pass fed from registers and the last pass
// handed back in registers.
//
// Shared layout: element j of column c of field f at f*FS + col_idx(j)*CT + c
// (FS = ColPad<N>*CT), col_idx(j) = pad_idx(j) = j + j/16 or, with CP = 8,
// j + j/8.  Threads take tasks (c, j) with
// c fastest, so a warp touches CT consecutive columns of 32/CT consecutive
// rows: global loads and stores of the prologue / epilogue are coalesced row
// segments.  A half-warp's 8-byte accesses (or a quarter-warp's 16-byte
// ones) cover CT columns of 16/CT (8/CT) consecutive tasks j; with one pad
// slot every 8 elements the first pass's writes (index 8j + r), the middle
// passes' writes and every read fall on distinct bank slots for N >= 64
// (checked at compile time below); one pad every 16 (pad_idx) leaves the
// first pass's writes two-way conflicted but needs 6 % less shared memory:
// with CP = 8, k_col_update and k_col_qw ran 4-6 % slower (likely because
// their CTAs' shared memory then crosses the 164 KB L1/shared carve-out
// step, leaving less L1).
//
// The passes are the Stockham radix-8/4/2 passes of fft_block.cuh (same
// order of operations and twiddles, so results are bitwise those of fft_ip):
//   pass 0 (NS = 1):   v = pro(c, j) -> DFT -> shared
//   middle passes:     shared -> twiddle, DFT -> shared (in place)
//   last pass:         shared -> twiddle, DFT -> epi(c, j, v)
// pro fills v[f][r] with the input at index j + r*N/R0 of field f; epi gets
// v[f][r] = output at index j + r*NS_last.  Every thread's cp.async copies
// issued before the call have landed and are visible to the whole CTA when
// epi runs.  Callers synchronise before reusing the shared buffer after
// col_fft returns.
#pragma once
#include "fft_block.cuh"

namespace qg {

// CP: one pad slot every CP elements (8 or 16), or CP = 0: no padding, the
// XOR placement i ^ ((i / 8) mod Q) with Q = (128 / element bytes) / CT,
// which makes the same accesses conflict free (checked below)
template <int CP = 16, int Q = 1> __host__ __device__ __forceinline__ constexpr int col_idx(int i) {
  return CP == 0 ? (i ^ ((i >> 3) & (Q - 1))) : (CP == 8 ? i + (i >> 3) : pad_idx(i));
}
template <int N, int CP = 16> struct ColPad {
  static constexpr int value = CP == 0 ? N : (CP == 8 ? N + (N >> 3) : PadLD<N>::value);
};
template <typename T, int CT> struct ColQ {
  static constexpr int v = (128 / (int)sizeof(cplx<T>)) / CT;
  static constexpr int value = v >= 1 ? v : 1;
};
template <int N, int CT, int CP = 16> struct ColLay {
  static constexpr int FS = ColPad<N, CP>::value * CT;
};

// Compile-time check of the column layout: for every pass of the radix plan
// of N (radix_of), the reads (index j + r N/R) and writes (index 8j + r in
// the first pass, base + r NS in the others) of each group of 128/CB
// consecutive tasks (c = t % CT, j = t / CT: one 128-byte wavefront of
// CB-byte elements) hit distinct bank slots, slot = (col_idx<8> * CT + c)
// mod (128/CB).  The first pass's reads and the last pass's writes are the
// prologue's and epilogue's registers.
namespace col_check {
constexpr int cidx(int cp, int q, int i) { return cp == 0 ? (i ^ ((i >> 3) & (q - 1))) : (cp == 8 ? i + (i >> 3) : pad_idx(i)); }
constexpr bool group_ok(int N, int CT, int CB, int R, int NS, bool write, int cp) {
  const int lanes = 128 / CB, NB = N / R, TASKS = CT * NB;
  for (int t0 = 0; t0 + lanes <= TASKS; t0 += lanes)
    for (int r = 0; r < R; ++r) {
      bool hit[16] = {};
      for (int t = t0; t < t0 + lanes; ++t) {
        const int c = t % CT, j = t / CT, k = j & (NS - 1);
        const int i = write ? (NS == 1 ? j * R + r : (j - k) * R + k + r * NS) : j + r * NB;
        const int q = lanes / CT >= 1 ? lanes / CT : 1;
        const int slot = (cidx(cp, q, i) * CT + c) % lanes;
        if (hit[slot]) return false;
        hit[slot] = true;
      }
    }
  return true;
}
constexpr bool conflict_free(int N, int CT, int CB, int cp) {
  for (int ns = 1; ns < N; ns *= radix_of(N / ns)) {
    const int R = radix_of(N / ns);
    const bool first = ns == 1, last = ns * R == N;
    if (!first && !group_ok(N, CT, CB, R, ns, false, cp)) return false;
    if (!last && !group_ok(N, CT, CB, R, ns, true, cp)) return false;
  }
  return true;
}
constexpr bool permutes(int N, int CT, int CB) {
  bool seen[1024] = {};
  const int q = (128 / CB) / CT >= 1 ? (128 / CB) / CT : 1;
  for (int i = 0; i < N; ++i) {
    const int p = cidx(0, q, i);
    if (p < 0 || p >= N || seen[p]) return false;
    seen[p] = true;
  }
  return true;
}
// the tiles of Tiles<T, N>::CT: FP32 (CB 8) 2048/N capped at 8, FP64 (CB 16)
// 1024/N capped at 8, at least 1
constexpr int ct_of(int N, int CB) {
  const int c = (16384 / CB) / N;
  return c >= 8 ? 8 : (c >= 1 ? c : 1);
}
// (N = 16 and 32, whose first passes are radix 2 and 4, keep a two-way
// conflict in their first pass's writes under either padding)
constexpr bool all_ok() {
  for (int N = 64; N <= 1024; N *= 2)
    for (int CB = 8; CB <= 16; CB *= 2)
      if (!conflict_free(N, ct_of(N, CB), CB, 8) || !conflict_free(N, ct_of(N, CB), CB, 0) ||
          !permutes(N, ct_of(N, CB), CB))
        return false;
  return true;
}
static_assert(all_ok(), "a pad-8 or XOR column layout leaves a bank conflict");
}  // namespace col_check

// number of passes and the stride NS of the last one
template <int N> struct LastNS {
  static constexpr int calc() {
    int ns = 1;
    while (ns * radix_of(N / ns) < N) ns *= radix_of(N / ns);
    return ns;
  }
  static constexpr int value = calc();
};

// completes this thread's outstanding cp.async copies (staging that a
// caller issued before col_fft; the barrier after the call publishes them)
__device__ __forceinline__ void col_cp_wait() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

template <typename T, int N, int R, int NS, bool FWD, int NF, int CT, int NT, bool LASTMID, int CP>
__device__ __forceinline__ void col_mid_pass(cplx<T>* __restrict__ sm, const cplx<T>* __restrict__ tw) {
  constexpr int FS = ColLay<N, CT, CP>::FS;
  constexpr int NB = N / R;
  constexpr int TASKS = CT * NB;
  constexpr int PER = (TASKS + NT - 1) / NT;
  cplx<T> v[PER][NF][R];
  const int tid = threadIdx.x;
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = tid + p * NT;
    if ((TASKS % NT) == 0 || t < TASKS) {
      const int c = t % CT, j = t / CT;
#pragma unroll
      for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int r = 0; r < R; ++r) v[p][f][r] = sm[f * FS + col_idx<CP, ColQ<T, CT>::value>(j + r * NB) * CT + c];
    }
  }
  __syncthreads();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = tid + p * NT;
    if ((TASKS % NT) == 0 || t < TASKS) {
      const int c = t % CT, j = t / CT;
      const int k = j & (NS - 1);
      constexpr int off = tw_off<N>(NS);
#pragma unroll
      for (int f = 0; f < NF; ++f) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          cplx<T> w = tw[off + (r - 1) * NS + k];
          if (!FWD) w.y = -w.y;
          v[p][f][r] = cmul(v[p][f][r], w);
        }
        dftR<T, R, FWD>(v[p][f]);
      }
      const int base = (j - k) * R + k;
#pragma unroll
      for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int r = 0; r < R; ++r) sm[f * FS + col_idx<CP, ColQ<T, CT>::value>(base + r * NS) * CT + c] = v[p][f][r];
    }
  }
  if constexpr (LASTMID) col_cp_wait();
  __syncthreads();
}

template <typename T, int N, int NS, bool FWD, int NF, int CT, int NT, int CP>
__device__ __forceinline__ void col_mid_passes(cplx<T>* sm, const cplx<T>* tw) {
  constexpr int R = radix_of(N / NS);
  if constexpr (NS < LastNS<N>::value) {
    col_mid_pass<T, N, R, NS, FWD, NF, CT, NT, (NS * R >= LastNS<N>::value), CP>(sm, tw);
    col_mid_passes<T, N, NS * R, FWD, NF, CT, NT, CP>(sm, tw);
  }
}

template <typename T, int N, bool FWD, int NF, int CT, int NT, int CP = 16, class Pro, class Epi>
__device__ __forceinline__ void col_fft(cplx<T>* __restrict__ sm, const cplx<T>* __restrict__ tw, Pro pro, Epi epi) {
  constexpr int FS = ColLay<N, CT, CP>::FS;
  const int tid = threadIdx.x;
  // pass 0 (NS = 1): inputs from the prologue
  {
    constexpr int R = radix_of(N);
    constexpr int NB = N / R;
    constexpr int TASKS = CT * NB;
    constexpr int PER = (TASKS + NT - 1) / NT;
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int t = tid + p * NT;
      if ((TASKS % NT) == 0 || t < TASKS) {
        const int c = t % CT, j = t / CT;
        cplx<T> v[NF][R];
        pro(c, j, v);
#pragma unroll
        for (int f = 0; f < NF; ++f) {
          dftR<T, R, FWD>(v[f]);
#pragma unroll
          for (int r = 0; r < R; ++r) sm[f * FS + col_idx<CP, ColQ<T, CT>::value>(j * R + r) * CT + c] = v[f][r];
        }
      }
    }
  }
  if constexpr (radix_of(N) >= LastNS<N>::value) col_cp_wait();   // no middle pass
  __syncthreads();
  col_mid_passes<T, N, radix_of(N), FWD, NF, CT, NT, CP>(sm, tw);
  // last pass: outputs to the epilogue
  {
    constexpr int NS = LastNS<N>::value;
    constexpr int R = N / NS;
    constexpr int NB = N / R;     // == NS
    constexpr int TASKS = CT * NB;
    constexpr int PER = (TASKS + NT - 1) / NT;
    constexpr int off = tw_off<N>(NS);
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int t = tid + p * NT;
      if ((TASKS % NT) == 0 || t < TASKS) {
        const int c = t % CT, j = t / CT;
        cplx<T> v[NF][R];
#pragma unroll
        for (int f = 0; f < NF; ++f) {
#pragma unroll
          for (int r = 0; r < R; ++r) v[f][r] = sm[f * FS + col_idx<CP, ColQ<T, CT>::value>(j + r * NB) * CT + c];
#pragma unroll
          for (int r = 1; r < R; ++r) {
            cplx<T> w = tw[off + (r - 1) * NS + j];
            if (!FWD) w.y = -w.y;
            v[f][r] = cmul(v[f][r], w);
          }
          dftR<T, R, FWD>(v[f]);
        }
        epi(c, j, v);
      }
    }
  }
}

// First Stockham pass (NS = 1) of NF*RT row transforms stored [f][rr][LD]
// with element i at pad_idx(i), inputs from registers: pro(rr, j, v) fills
// v[f][r] with the input at index j + r*N/R0.  Threads take tasks (rr, j)
// with j fastest (coalesced row reads).  The remaining passes are
// ip_passes<..., radix_of(N)> after a barrier.
template <typename T, int N, bool FWD, int NF, int RT, int NT, int LD, int LAY = 0, class Pro>
__device__ __forceinline__ void row_pass0(cplx<T>* __restrict__ sm, Pro pro) {
  constexpr int R = radix_of(N);
  constexpr int NB = N / R;
  constexpr int TASKS = RT * NB;
  constexpr int PER = (TASKS + NT - 1) / NT;
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * NT;
    if ((TASKS % NT) == 0 || t < TASKS) {
      const int j = t % NB, rr = t / NB;
      cplx<T> v[NF][R];
      pro(rr, j, v);
#pragma unroll
      for (int f = 0; f < NF; ++f) {
        dftR<T, R, FWD>(v[f]);
#pragma unroll
        for (int r = 0; r < R; ++r) sm[(f * RT + rr) * LD + lay_idx<LAY>(j * R + r)] = v[f][r];
      }
    }
  }
}

// In-place Stockham passes (ip_pass) from stride NS up to, not including,
// the last pass; MID (a layout number, 0 for none): the second-to-last pass
// writes layout MID (for a last pass that reads layout MID).
template <typename T, int N, bool FWD, int BATCH, int NT, int LD, int NS, int LAY = 0, int MID = 0>
__device__ __forceinline__ void ip_passes_but_last(cplx<T>* buf, const cplx<T>* tw) {
  if constexpr (NS < LastNS<N>::value) {
    constexpr int R = radix_of(N / NS);
    ip_pass<T, N, R, NS, FWD, BATCH, NT, LD, LAY, (MID && NS * R == LastNS<N>::value) ? MID : LAY>(buf, tw);
    ip_passes_but_last<T, N, FWD, BATCH, NT, LD, NS * R, LAY, MID>(buf, tw);
  }
}

// ---------------------------------------------------------------------------
// Forward row transforms of N = 512 (radices 8 x 8 x 8) ending in registers.
//
// A packed transform F = FFT(x + i y) of two real rows is split into the half
// spectra X[k] = (F[k] + conj F[N-k])/2, Y[k] = (F[k] - conj F[N-k])/(2i),
// k <= K.  The last Stockham pass (NS = 64) leaves task j holding F at
// k = j + 64 r, r = 0..7, and F[N-k] at task 64 - j, r' = 7 - r (task 0 and
// task 32 hold both).  Tasks are placed so that j and 64 - j sit in lanes l
// and l ^ 16 of one warp: warp half h = 0 takes j = 0..15, 32, 63..49 and
// h = 1 takes j = 16..31, 48..33.  The partner values then come by three
// shuffles per transform instead of a round trip through shared memory.
// ---------------------------------------------------------------------------
struct RowLastTask {
  int j;      // butterfly index of the last pass
  bool self;  // j == 0 or j == 32: F[N-k] is this task's own value
};
__device__ __forceinline__ RowLastTask row_last_task(int t) {
  const int l = t & 31, h = (t >> 5) & 1;
  RowLastTask r;
  r.j = h == 0 ? (l < 16 ? l : (l == 16 ? 32 : 80 - l)) : (l < 16 ? 16 + l : 64 - l);
  r.self = r.j == 0 || r.j == 32;
  return r;
}

// Last forward pass of one transform stored at tr (layout LAY) for task j:
// w[r] = F[j + 64 r]; then b[r] = F[N - (j + 64 r)] for r = 0, 1, 2.  Every
// lane of the warp must call (the shuffles are warp-wide).
template <typename T, int LAY>
__device__ __forceinline__ void row_last_fwd512(const cplx<T>* __restrict__ tr, const cplx<T>* __restrict__ tw,
                                                RowLastTask tk, cplx<T> (&w)[8], cplx<T> (&b)[3]) {
  constexpr int N = 512, NS = 64, R = 8;
  constexpr int off = tw_off<N>(NS);
  const int j = tk.j;
#pragma unroll
  for (int r = 0; r < R; ++r) w[r] = tr[lay_idx<LAY>(j + r * NS)];
#pragma unroll
  for (int r = 1; r < R; ++r) w[r] = cmul(w[r], tw[off + (r - 1) * NS + j]);
  dftR<T, R, true>(w);
  cplx<T> t[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    t[q].x = __shfl_xor_sync(0xffffffffu, w[7 - q].x, 16);
    t[q].y = __shfl_xor_sync(0xffffffffu, w[7 - q].y, 16);
  }
  if (j == 0) { b[0] = w[0]; b[1] = w[7]; b[2] = w[6]; }
  else if (j == 32) { b[0] = w[7]; b[1] = w[6]; b[2] = w[5]; }
  else { b[0] = t[0]; b[1] = t[1]; b[2] = t[2]; }
}

// the half spectra at k from a = F[k], b = F[N-k] (unpack_spec's arithmetic)
template <typename T>
__device__ __forceinline__ void split_pair(cplx<T> a, cplx<T> b, cplx<T>& X, cplx<T>& Y) {
  X = mk<T>((a.x + b.x) * (T)0.5, (a.y - b.y) * (T)0.5);
  Y = mk<T>((a.y + b.y) * (T)0.5, (b.x - a.x) * (T)0.5);
}

}  // namespace qg
