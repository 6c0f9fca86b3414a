// Batched power-of-two FFTs held in shared memory, executed by a whole CTA.
//
// Stockham autosort, decimation in time, radices 8/4/2: pass p with radix R
// reads x[j + r*N/R], twiddles by W_{Ns*R}^{(j mod Ns) r}, does a length-R DFT
// in registers and writes y[(j - j mod Ns)*R + j mod Ns + r*Ns]; Ns is the
// product of the radices of the earlier passes.  Forward uses
// W_M = exp(-2 pi i/M) (FFTW_FORWARD); backward uses the conjugate and is
// unnormalised (FFTW_BACKWARD), so backward(forward(x)) = N x.
#pragma once
#include "common.cuh"

namespace qg {

template <typename T, bool FWD> struct Dft;

// forward: multiply by W8^1 = (1-i)/sqrt2, W8^3 = (-1-i)/sqrt2 ; backward: conjugates
template <typename T, bool FWD>
__device__ __forceinline__ void dft2(cplx<T>& a, cplx<T>& b) {
  cplx<T> t = a; a = cadd(t, b); b = csub(t, b);
}

template <typename T, bool FWD>
__device__ __forceinline__ cplx<T> mul_w4(cplx<T> a) {  // * W4^1 (fwd -i, bwd +i)
  return FWD ? cmul_mi(a) : cmul_i(a);
}

template <typename T, bool FWD>
__device__ __forceinline__ void dft4(cplx<T>* v) {
  cplx<T> s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
  cplx<T> s13 = cadd(v[1], v[3]), d13 = mul_w4<T, FWD>(csub(v[1], v[3]));
  v[0] = cadd(s02, s13);
  v[2] = csub(s02, s13);
  v[1] = cadd(d02, d13);
  v[3] = csub(d02, d13);
}

template <typename T, bool FWD>
__device__ __forceinline__ void dft8(cplx<T>* v) {
  const T h = (T)0.70710678118654752440084436210485;
  cplx<T> a[4], b[4];
#pragma unroll
  for (int n = 0; n < 4; ++n) { a[n] = cadd(v[n], v[n + 4]); b[n] = csub(v[n], v[n + 4]); }
  // b[n] *= W8^n
  {
    cplx<T> t = b[1];
    if (FWD) { b[1].x = (t.x + t.y) * h; b[1].y = (t.y - t.x) * h; }
    else     { b[1].x = (t.x - t.y) * h; b[1].y = (t.y + t.x) * h; }
    b[2] = mul_w4<T, FWD>(b[2]);
    t = b[3];
    if (FWD) { b[3].x = (t.y - t.x) * h; b[3].y = -(t.x + t.y) * h; }
    else     { b[3].x = -(t.x + t.y) * h; b[3].y = (t.x - t.y) * h; }
  }
  dft4<T, FWD>(a);
  dft4<T, FWD>(b);
  v[0] = a[0]; v[2] = a[1]; v[4] = a[2]; v[6] = a[3];
  v[1] = b[0]; v[3] = b[1]; v[5] = b[2]; v[7] = b[3];
}

template <typename T, int R, bool FWD>
__device__ __forceinline__ void dftR(cplx<T>* v) {
  if constexpr (R == 8) dft8<T, FWD>(v);
  else if constexpr (R == 4) dft4<T, FWD>(v);
  else dft2<T, FWD>(v[0], v[1]);
}

// Radix of the pass that leaves a remaining length REM = 2^m (the pass with
// stride NS of a length-N transform has REM = N/NS).  Radix 8 wherever it
// fits; a leftover factor 4 or 2 goes to a middle pass (N = 256: 8 x 4 x 8,
// N = 128: 8 x 2 x 8, N = 1024: 8 x 8 x 2 x 8), so that every transform of
// 64 points or more starts and ends with a radix-8 pass: the row kernels
// hand the inverse transform's last pass to the forward transform's first
// pass in registers, which needs the two radices equal.  Below 64 points
// the leftover factor comes first (32: 4 x 8, 16: 2 x 8).
__host__ __device__ constexpr int radix_of(int rem) {
  int m = 0;
  while ((1 << m) < rem) ++m;
  return (m % 3 == 0 || m >= 7) ? 8 : (m % 3 == 2 ? 4 : 2);
}
template <int REM> struct PassRadix { static constexpr int value = radix_of(REM); };

// One Stockham pass over `batch` transforms of length N stored with leading
// dimension ld; tw[m] = W_N^m (forward sign).
template <typename T, int N, int R, int NS, bool FWD>
__device__ __forceinline__ void stockham_pass(const cplx<T>* __restrict__ src, cplx<T>* __restrict__ dst,
                                              int ld, int batch, const cplx<T>* __restrict__ tw) {
  constexpr int NB = N / R;
  const int total = batch * NB;
  for (int t = threadIdx.x; t < total; t += blockDim.x) {
    const int b = t / NB;
    const int j = t - b * NB;
    const cplx<T>* s = src + (long)b * ld;
    cplx<T>* d = dst + (long)b * ld;
    cplx<T> v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[j + r * NB];
    const int k = j & (NS - 1);
    if constexpr (NS > 1) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        cplx<T> w = tw[k * r * (N / (NS * R))];
        if (!FWD) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    dftR<T, R, FWD>(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) d[base + r * NS] = v[r];
  }
}

template <typename T, int N, bool FWD, int NS>
__device__ __forceinline__ cplx<T>* fft_passes(cplx<T>* a, cplx<T>* b, int ld, int batch, const cplx<T>* tw) {
  if constexpr (NS >= N) {
    return a;
  } else {
    constexpr int R = PassRadix<N / NS>::value;
    stockham_pass<T, N, R, NS, FWD>(a, b, ld, batch, tw);
    __syncthreads();
    return fft_passes<T, N, FWD, NS * R>(b, a, ld, batch, tw);
  }
}

// All threads of the CTA must call.  Input in `a`, `b` is scratch of the same
// size; returns the buffer that holds the result.  Ends with __syncthreads().
template <typename T, int N, bool FWD>
__device__ __forceinline__ cplx<T>* block_fft(cplx<T>* a, cplx<T>* b, int ld, int batch, const cplx<T>* tw) {
  return fft_passes<T, N, FWD, 1>(a, b, ld, batch, tw);
}

template <typename T, int N>
__device__ __forceinline__ void load_twiddles(cplx<T>* tw_s, const cplx<T>* __restrict__ tw_g) {
  for (int i = threadIdx.x; i < N; i += blockDim.x) tw_s[i] = tw_g[i];
}

}  // namespace qg

namespace qg {

// ---------------------------------------------------------------------------
// In-place batched FFTs with compile-time shape, used by the step kernels.
//
// BATCH transforms of length N live in one shared buffer, transform b at
// b*PadLD<N> with element i at pad_idx(i) = i + i/16: one padding slot every
// 16 elements makes the radix-8 Stockham reads (stride N/8) and writes
// (stride 1, 8, 64, ...) bank-conflict free for 8- and 16-byte elements.
// Each pass reads all of a thread's butterflies into registers, synchronises,
// then writes them back (so one buffer suffices); NT threads of the CTA take
// part (compile-time, so every loop unrolls).
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ constexpr int pad_idx(int i) { return i + (i >> 4); }
template <int N> struct PadLD { static constexpr int value = N + (N >> 4); };

// Element placement of a transform: LAY 0 is pad_idx; LAY 1 (radix-8
// transforms of N = 512, one task per butterfly) permutes each aligned group
// of 16 elements, i ^ h(i/16) with h(m) = (m & 7) | ((m & 4) << 1): the
// first pass's writes (index 8j + r), the middle pass's writes (index
// 64(j/8) + j%8 + 8r) and all reads (index j + 64r) of 16 consecutive tasks
// then fall on 16 distinct 8-byte bank pairs, where pad_idx leaves the middle
// pass's writes two-way conflicted.  No padding: N entries per transform.
//
// LAY 2 (N = 256 with the radix plan 8 x 4 x 8, used only for the hand-off
// between the middle radix-4 pass and the last radix-8 pass): i ^ 8*bit5(i).
// The middle pass writes index 32(j/8) + j%8 + 8r; a half-warp's 16 tasks
// span two runs of 8 whose low four bits coincide under pad_idx (a two-way
// conflict) and differ in bit 3 here; the last pass reads j + 32r, whose
// bit 5 is the same for the 16 tasks.
//
// LAY 3 (N = 128, plan 8 x 2 x 8, the same hand-off): i ^ 8*bit4(i).  The
// middle radix-2 pass writes 16(j/8) + j%8 + 8r: the two runs of 8 of a
// half-warp differ in bit 4, and under pad_idx overlap in seven bank pairs.
template <int LAY> __host__ __device__ __forceinline__ constexpr int lay_idx(int i) {
  if constexpr (LAY == 0) {
    return pad_idx(i);
  } else if constexpr (LAY == 1) {
    const int m = i >> 4;
    return i ^ ((m & 7) | ((m & 4) << 1));
  } else if constexpr (LAY == 2) {
    return i ^ (((i >> 5) & 1) << 3);
  } else {
    return i ^ (((i >> 4) & 1) << 3);
  }
}

// Compile-time proof of the claims for N = 512: lay_idx<1> permutes
// [0, 512), and each group of 16 consecutive tasks j (one half-warp's 8-byte
// accesses, r fixed) of the three access patterns hits 16 distinct bank pairs
// (slot = index mod 16).
namespace lay_check {
constexpr bool permutes512() {
  bool seen[512] = {};
  for (int i = 0; i < 512; ++i) {
    const int p = lay_idx<1>(i);
    if (p < 0 || p >= 512 || seen[p]) return false;
    seen[p] = true;
  }
  return true;
}
constexpr bool conflict_free512() {
  for (int pat = 0; pat < 3; ++pat)
    for (int r = 0; r < 8; ++r)
      for (int j0 = 0; j0 < 64; j0 += 16) {
        bool hit[16] = {};
        for (int j = j0; j < j0 + 16; ++j) {
          const int i = pat == 0 ? 8 * j + r                            // first pass writes
                      : pat == 1 ? 64 * (j >> 3) + (j & 7) + 8 * r      // middle pass writes
                                 : j + 64 * r;                          // every read, last writes
          const int slot = lay_idx<1>(i) & 15;
          if (hit[slot]) return false;
          hit[slot] = true;
        }
      }
  return true;
}
// lay_idx<2> on N = 256: a permutation of [0, 256), conflict free for the
// middle radix-4 pass's writes and the last pass's reads
constexpr bool permutes256() {
  bool seen[256] = {};
  for (int i = 0; i < 256; ++i) {
    const int p = lay_idx<2>(i);
    if (p < 0 || p >= 256 || seen[p]) return false;
    seen[p] = true;
  }
  return true;
}
constexpr bool conflict_free256() {
  for (int pat = 0; pat < 2; ++pat)
    for (int r = 0; r < (pat == 0 ? 4 : 8); ++r)
      for (int j0 = 0; j0 < (pat == 0 ? 64 : 32); j0 += 16) {
        bool hit[16] = {};
        for (int j = j0; j < j0 + 16; ++j) {
          const int i = pat == 0 ? 32 * (j >> 3) + (j & 7) + 8 * r    // middle (radix-4) pass writes
                                 : j + 32 * r;                        // last pass reads
          const int slot = lay_idx<2>(i) & 15;
          if (hit[slot]) return false;
          hit[slot] = true;
        }
      }
  return true;
}
// lay_idx<3> on N = 128: the middle radix-2 pass's writes and the last
// pass's reads
constexpr bool permutes128() {
  bool seen[128] = {};
  for (int i = 0; i < 128; ++i) {
    const int p = lay_idx<3>(i);
    if (p < 0 || p >= 128 || seen[p]) return false;
    seen[p] = true;
  }
  return true;
}
constexpr bool conflict_free128() {
  for (int pat = 0; pat < 2; ++pat)
    for (int r = 0; r < (pat == 0 ? 2 : 8); ++r)
      for (int j0 = 0; j0 < (pat == 0 ? 64 : 16); j0 += 16) {
        bool hit[16] = {};
        for (int j = j0; j < j0 + 16; ++j) {
          const int i = pat == 0 ? 16 * (j >> 3) + (j & 7) + 8 * r    // middle (radix-2) pass writes
                                 : j + 16 * r;                        // last pass reads
          const int slot = lay_idx<3>(i) & 15;
          if (hit[slot]) return false;
          hit[slot] = true;
        }
      }
  return true;
}
static_assert(permutes512(), "lay_idx<1> is not a permutation of [0, 512)");
static_assert(conflict_free512(), "lay_idx<1> leaves a bank conflict");
static_assert(permutes256(), "lay_idx<2> is not a permutation of [0, 256)");
static_assert(conflict_free256(), "lay_idx<2> leaves a bank conflict");
static_assert(permutes128(), "lay_idx<3> is not a permutation of [0, 128)");
static_assert(conflict_free128(), "lay_idx<3> leaves a bank conflict");
}  // namespace lay_check

// Twiddles laid out per pass: the pass with stride NS and radix R reads
// W_N^{k r N/(NS R)} at tw[off(NS) + (r-1)*NS + k], so the threads of a warp
// (consecutive k) read consecutive words.  Fewer than N entries in total.
template <int N> __host__ __device__ constexpr int tw_off(int ns) {
  int off = 0;
  for (int s = 1; s < ns; s *= radix_of(N / s)) if (s > 1) off += s * (radix_of(N / s) - 1);
  return off;
}

template <typename T, int N, int NS>
__device__ __forceinline__ void load_tw_passes(cplx<T>* tw_s, const cplx<T>* __restrict__ tw_g, int nt) {
  if constexpr (NS < N) {
    constexpr int R = radix_of(N / NS);
    if constexpr (NS > 1) {
      constexpr int off = tw_off<N>(NS);
      for (int i = threadIdx.x; i < NS * (R - 1); i += nt) {
        const int r = 1 + i / NS, k = i % NS;
        tw_s[off + i] = tw_g[k * r * (N / (NS * R))];
      }
    }
    load_tw_passes<T, N, NS * R>(tw_s, tw_g, nt);
  }
}

// reads in layout LAY, writes in layout LAYW (lay_idx)
template <typename T, int N, int R, int NS, bool FWD, int BATCH, int NT, int LD, int LAY = 0, int LAYW = LAY>
__device__ __forceinline__ void ip_pass(cplx<T>* __restrict__ buf, const cplx<T>* __restrict__ tw) {
  constexpr int NB = N / R;
  constexpr int TASKS = BATCH * NB;
  constexpr int PER = (TASKS + NT - 1) / NT;
  cplx<T> v[PER][R];
  const int tid = threadIdx.x;
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = tid + p * NT;
    if ((TASKS % NT) == 0 || t < TASKS) {
      const int b = t / NB, j = t % NB;
      const cplx<T>* s = buf + b * LD;
#pragma unroll
      for (int r = 0; r < R; ++r) v[p][r] = s[lay_idx<LAY>(j + r * NB)];
    }
  }
  __syncthreads();
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = tid + p * NT;
    if ((TASKS % NT) == 0 || t < TASKS) {
      const int b = t / NB, j = t % NB;
      const int k = j & (NS - 1);
      if constexpr (NS > 1) {
        constexpr int off = tw_off<N>(NS);
#pragma unroll
        for (int r = 1; r < R; ++r) {
          cplx<T> w = tw[off + (r - 1) * NS + k];
          if (!FWD) w.y = -w.y;
          v[p][r] = cmul(v[p][r], w);
        }
      }
      dftR<T, R, FWD>(v[p]);
      cplx<T>* d = buf + b * LD;
      const int base = (j - k) * R + k;
#pragma unroll
      for (int r = 0; r < R; ++r) d[lay_idx<LAYW>(base + r * NS)] = v[p][r];
    }
  }
  __syncthreads();
}

// MID (a layout number, 0 for none): the second-to-last pass writes, and
// the last pass reads, layout MID (the other hand-offs stay in LAY)
template <typename T, int N, bool FWD, int BATCH, int NT, int LD, int NS, int LAY = 0, int MID = 0>
__device__ __forceinline__ void ip_passes(cplx<T>* buf, const cplx<T>* tw) {
  if constexpr (NS < N) {
    constexpr int R = PassRadix<N / NS>::value;
    constexpr bool last = NS * R == N;
    constexpr bool pen = !last && NS * R * PassRadix<(last ? 1 : N / (NS * R))>::value == N;
    ip_pass<T, N, R, NS, FWD, BATCH, NT, LD, (MID && last) ? MID : LAY, (MID && pen) ? MID : LAY>(buf, tw);
    ip_passes<T, N, FWD, BATCH, NT, LD, NS * R, LAY, MID>(buf, tw);
  }
}

// All NT threads must call; the data must be visible to all of them (call
// after a __syncthreads()).  Transform b starts at buf + b*LD (LD >= the
// padded length).  Ends with a __syncthreads().
template <typename T, int N, bool FWD, int BATCH, int NT, int LD = PadLD<N>::value>
__device__ __forceinline__ void fft_ip(cplx<T>* buf, const cplx<T>* tw) {
  static_assert(LD >= PadLD<N>::value, "transform stride shorter than the padded transform");
  ip_passes<T, N, FWD, BATCH, NT, LD, 1>(buf, tw);
}

}  // namespace qg
