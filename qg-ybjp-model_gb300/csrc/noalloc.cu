// qg_fft_c2r_noalloc: the per-level 2D c2r transform of fft.f90:71-83 (realit,
// then an unnormalised c2r) for callers that cannot allocate device memory.
//
// Who needs it: a host whose device memory is fixed at start-up and shared
// under a hard cap (for example several model instances or an I/O process
// co-located on one GPU, each given a fixed budget), or a host loop that
// cannot afford cudaMalloc/cudaFree — cudaFree synchronises the whole device,
// which would stall the step kernels running on other streams.  Such a
// caller owns its input and output buffers; this entry point adds no
// allocation of its own.  Its intermediate (kx, y) plane lives in the
// file-scope array below, which every GPU that loads the library holds
// until the process exits.
#include <cmath>
#include <mutex>
#include <string>
#include <vector>
#include "dense_kernels.cuh"
#include "engine.h"
#include "noalloc_check.h"

namespace {

// Scratch for the (kx, y) intermediate of one chunk of levels: 8 MiB holds at
// least one level for every n <= 512 (n * (n/2+1 rounded up to 4) * 16 bytes).
constexpr size_t kScratchBytes = size_t(8) << 20;
__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];
// Twiddles W_n^m = exp(-2 pi i m / n) of every supported n, packed: n = 16, 32, ..., 512.
constexpr int kTwEntries = 16 + 32 + 64 + 128 + 256 + 512;
__device__ __align__(256) double2 g_noalloc_tw[kTwEntries];

constexpr int kMaxDevices = 64;
struct DeviceSetup {
  bool ready = false;
  double2* scratch = nullptr;   // device address of g_noalloc_scratch on this device
  double2* tw = nullptr;        // device address of g_noalloc_tw on this device
};
DeviceSetup g_setup[kMaxDevices];
std::mutex g_setup_mu;

int tw_offset(int n) {
  int off = 0;
  for (int m = 16; m < n; m *= 2) off += m;
  return off;
}

int iktxp(int n) {
  constexpr int ct = qg::Tile<double>::CT;
  return ((n / 2 + 1 + ct - 1) / ct) * ct;
}

int fail(int code, const std::string& msg) {
  qg::set_handleless_error(msg);
  return code;
}

#define NA_CK(call)                                                                           \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(QG_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

// Once per device, with that device current: device addresses of the static
// arrays, the twiddle tables and the kernels' shared-memory limits.
int setup_device(int dev, DeviceSetup** out) {
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup& s = g_setup[dev];
  if (!s.ready) {
    void* p = nullptr;
    NA_CK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    s.scratch = static_cast<double2*>(p);
    NA_CK(cudaGetSymbolAddress(&p, g_noalloc_tw));
    s.tw = static_cast<double2*>(p);
    std::vector<double2> tw(kTwEntries);
    const double twopi = 4.0 * std::asin(1.0);
    for (int n = 16, off = 0; n <= 512; off += n, n *= 2) {
      for (int m = 0; m < n; ++m) {
        double cs, sn;
        if ((4 * m) % n == 0) {
          const double C4[4] = {1, 0, -1, 0}, S4[4] = {0, 1, 0, -1};
          cs = C4[(4 * m) / n]; sn = S4[(4 * m) / n];
        } else {
          const double th = twopi * (double)m / (double)n;
          cs = std::cos(th); sn = std::sin(th);
        }
        tw[off + m] = make_double2(cs, -sn);
      }
    }
    NA_CK(cudaMemcpyToSymbol(g_noalloc_tw, tw.data(), sizeof(double2) * kTwEntries));
    const int mx = cudaFuncAttributeMaxDynamicSharedMemorySize;
    const int ct = qg::Tile<double>::CT;
#define NA_ATTR(NN)                                                                                        \
    NA_CK(cudaFuncSetAttribute(qg::k_dcol_inv<double, NN>, (cudaFuncAttribute)mx,                          \
                               (int)((NN + 2 * ct * (NN + 1)) * sizeof(double2))));                        \
    NA_CK(cudaFuncSetAttribute(qg::k_drow_c2r_pad<double, NN>, (cudaFuncAttribute)mx, (int)(3 * NN * sizeof(double2))));
    NA_ATTR(16) NA_ATTR(32) NA_ATTR(64) NA_ATTR(128) NA_ATTR(256) NA_ATTR(512)
#undef NA_ATTR
    s.ready = true;
  }
  *out = &s;
  return QG_OK;
}

// QG_OK when p is memory a kernel on device `dev` can read or write at
// `align`-byte alignment; otherwise QG_ERR_ARG with the reason.
int check_device_pointer(const void* p, int dev, uintptr_t align, const char* name) {
  cudaPointerAttributes a;
  int type = 0, owner = -1;
  if (cudaPointerGetAttributes(&a, p) == cudaSuccess) {
    type = (int)a.type;
    owner = a.device;
  } else {
    cudaGetLastError();   // the query's own error (an unregistered host pointer)
  }
  switch (qgna::check_pointer(type, owner, dev, p, align)) {
    case qgna::kPointerOk: return QG_OK;
    case qgna::kPointerNotDevice:
      return fail(QG_ERR_ARG, std::string("qg_fft_c2r_noalloc: ") + name + " must be device memory");
    case qgna::kPointerOtherDevice:
      return fail(QG_ERR_ARG, std::string("qg_fft_c2r_noalloc: ") + name +
                                  " belongs to another device than the current one");
    default:
      return fail(QG_ERR_ARG, std::string("qg_fft_c2r_noalloc: ") + name + " must be " +
                                  std::to_string((unsigned long long)align) + "-byte aligned");
  }
}

// the launch just made: its configuration error, if any (no earlier error
// was pending when the call began, so whatever is pending now is this call's)
#define NA_LAUNCH_CK()                                                                          \
  do {                                                                                          \
    cudaError_t e_ = cudaPeekAtLastError();                                                     \
    if (e_ != cudaSuccess) {                                                                    \
      cudaGetLastError();                                                                       \
      return fail(QG_ERR_CUDA, std::string("qg_fft_c2r_noalloc launch: ") + cudaGetErrorString(e_)); \
    }                                                                                           \
  } while (0)

template <int N>
int launch_chunks(const double2* in, double* out, int nz, cudaStream_t st, const DeviceSetup& s) {
  const int ip = iktxp(N);
  const size_t per_level = (size_t)N * ip * sizeof(double2);
  const int chunk = (int)(kScratchBytes / per_level);
  const int ct = qg::Tile<double>::CT;
  const size_t sm_col = (size_t)(N + 2 * ct * (N + 1)) * sizeof(double2);
  const size_t sm_row = (size_t)(3 * N) * sizeof(double2);
  const double2* tw = s.tw + tw_offset(N);
  for (int z0 = 0; z0 < nz; z0 += chunk) {
    const int zc = nz - z0 < chunk ? nz - z0 : chunk;
    qg::k_dcol_inv<double, N><<<dim3(ip / ct, zc), qg::kThreads, sm_col, st>>>(
        ip, in + (size_t)z0 * N * (N / 2 + 1), s.scratch, tw);
    NA_LAUNCH_CK();
    qg::k_drow_c2r_pad<double, N><<<dim3(N / 2, zc), qg::kThreads, sm_row, st>>>(
        ip, s.scratch, out + (size_t)z0 * N * (N + 2), tw);
    NA_LAUNCH_CK();
  }
  return QG_OK;
}

}  // namespace

extern "C" int qg_fft_c2r_noalloc(const double* kvar, double* rvar, int n, int nz, void* stream) {
  if (!kvar || !rvar) return fail(QG_ERR_ARG, "qg_fft_c2r_noalloc: null pointer");
  if (nz <= 0) return fail(QG_ERR_ARG, "qg_fft_c2r_noalloc: nz must be positive");
  if (n < 16 || n > 512 || (n & (n - 1)))
    return fail(QG_ERR_UNSUPPORTED, "qg_fft_c2r_noalloc: n must be a power of two in [16, 512] (one level's "
                                    "(kx,y) plane must fit the 8 MiB static scratch)");
  int dev = 0;
  NA_CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(QG_ERR_UNSUPPORTED, "qg_fft_c2r_noalloc: device ordinal too large");
  // an error left pending by the caller's earlier work stays the caller's:
  // refuse without consuming it
  {
    const cudaError_t pend = cudaPeekAtLastError();
    if (pend != cudaSuccess)
      return fail(QG_ERR_CUDA, std::string("qg_fft_c2r_noalloc: a CUDA error from earlier work is pending "
                                           "(left for its owner to read): ") + cudaGetErrorString(pend));
  }
  // kvar is read as 16-byte complex values, rvar written as doubles
  int rc = check_device_pointer(kvar, dev, 16, "kvar");
  if (rc) return rc;
  rc = check_device_pointer(rvar, dev, 8, "rvar");
  if (rc) return rc;
  DeviceSetup* s = nullptr;
  rc = setup_device(dev, &s);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const double2* in = reinterpret_cast<const double2*>(kvar);
  switch (n) {
    case 16: return launch_chunks<16>(in, rvar, nz, st, *s);
    case 32: return launch_chunks<32>(in, rvar, nz, st, *s);
    case 64: return launch_chunks<64>(in, rvar, nz, st, *s);
    case 128: return launch_chunks<128>(in, rvar, nz, st, *s);
    case 256: return launch_chunks<256>(in, rvar, nz, st, *s);
    default: return launch_chunks<512>(in, rvar, nz, st, *s);
  }
}
