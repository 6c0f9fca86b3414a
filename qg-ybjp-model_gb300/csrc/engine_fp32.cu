// Mixed-precision instantiation: FP32 transforms, products and update;
// FP64 tridiagonal solves and diagnostics.
#include "engine_impl.cuh"
namespace qg {
EngineBase* make_engine_fp32() { return new Engine<float>(); }

// Low 29 mantissa bits that sit on the FP64 -> FP32 rounding boundaries
// (exact, just above/below/at the tie, the largest remainder).
__device__ __forceinline__ unsigned long long tie_bits(unsigned k) {
  return k == 0 ? 0ull : k == 1 ? 1ull : k == 2 ? 0x0fffffffull : k == 3 ? 0x10000000ull : k == 4 ? 0x10000001ull
                                                                                                  : 0x1fffffffull;
}

// Every FP32 bit pattern through f32_to_f64, and 2^32 FP64 patterns (each
// sign/exponent field with 2^20 hashed mantissas, six of every eight with
// their low 29 bits set to a rounding boundary) through f64_to_f32, each
// compared bit for bit with the hardware conversion (NaN matches NaN).
__global__ void k_conv_selftest(unsigned long long* __restrict__ bad) {
  unsigned long long b32 = 0, b64 = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < (1ull << 32);
       i += stride) {
    const float f = __uint_as_float((unsigned)i);
    const double a = f32_to_f64(f), h = (double)f;
    if (!(__double_as_longlong(a) == __double_as_longlong(h) || (a != a && h != h))) ++b32;
    unsigned long long z = i + 0x9e3779b97f4a7c15ull;       // splitmix64 of the index
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    unsigned long long mant = z & ((1ull << 52) - 1ull);
    const unsigned k = (unsigned)(i & 7u);
    if (k < 6) mant = (mant & ~0x1fffffffull) | tie_bits(k);
    const double d = __longlong_as_double((long long)(((i >> 20) << 52) | mant));
    const float c = f64_to_f32(d), hc = (float)d;
    if (!(__float_as_uint(c) == __float_as_uint(hc) || (c != c && hc != hc))) ++b64;
  }
  if (b32) atomicAdd(&bad[0], b32);
  if (b64) atomicAdd(&bad[1], b64);
}

int selftest_conversions(int device, long long* bad32, long long* bad64, std::string& err) {
  cudaError_t e = cudaSetDevice(device);
  unsigned long long* d = nullptr;
  unsigned long long h[2] = {0, 0};
  if (e == cudaSuccess) e = cudaMalloc(&d, sizeof(h));
  if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(h));
  if (e == cudaSuccess) {
    k_conv_selftest<<<152 * 8, 256>>>(d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (e != cudaSuccess) {
    err = std::string("qg_selftest_conversions: ") + cudaGetErrorString(e);
    return QG_ERR_CUDA;
  }
  *bad32 = (long long)h[0];
  *bad64 = (long long)h[1];
  return QG_OK;
}
}  // namespace qg
