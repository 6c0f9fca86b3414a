// Engine<T>: device buffers, launch sequence and CUDA-graph replay of the
// step, state conversions, routine-level drop-ins.  T = float (mixed
// precision: FP64 only in the tridiagonal solves and the diagnostics) or
// T = double (FP64 everywhere).
#pragma once
#include <cstdio>
#include <cstring>
#include <cmath>
#include <algorithm>
#include "engine.h"
#include "dense_kernels.cuh"

namespace qg {

#define QG_CK(call)                                                                          \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) {                                                                 \
      char b_[512];                                                                          \
      snprintf(b_, sizeof b_, "%s:%d: %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      err = b_;                                                                              \
      return e_ == cudaErrorMemoryAllocation ? QG_ERR_NOMEM : QG_ERR_CUDA;                   \
    }                                                                                        \
  } while (0)

#define QG_LAUNCHED() QG_CK(cudaGetLastError())

#define QG_SWITCH_N(n, ...)                      \
  switch (n) {                                    \
    case 16: { constexpr int NN = 16; __VA_ARGS__; break; }    \
    case 32: { constexpr int NN = 32; __VA_ARGS__; break; }    \
    case 64: { constexpr int NN = 64; __VA_ARGS__; break; }    \
    case 128: { constexpr int NN = 128; __VA_ARGS__; break; }  \
    case 256: { constexpr int NN = 256; __VA_ARGS__; break; }  \
    case 512: { constexpr int NN = 512; __VA_ARGS__; break; }  \
    case 1024: { constexpr int NN = 1024; __VA_ARGS__; break; }\
    default: err = "unsupported n"; return QG_ERR_UNSUPPORTED; \
  }

enum { F_Q = 0, F_QO, F_BR, F_BI, F_BRO, F_BIO, F_PSI, F_AR, F_AI, F_QSTAR, F_DQ, F_NINT };

template <typename T>
class Engine : public EngineBase {
  using C = cplx<T>;

 public:
  ~Engine() override { release(); }

  int init(const qg_config& c, const HostTables& t) override {
    cfg = c;
    g.n = t.n; g.n3 = t.n3; g.K = t.K; g.KX = t.KX; g.KY = t.KY; g.KXP = t.KXP; g.kmax2 = t.kmax2;
    g.nseg = t.nseg > 0 ? t.nseg : t.n3;
    members = g.n3 / g.nseg;
    g.plane = t.plane;
    QG_CK(cudaSetDevice(cfg.device));
    // the step's stream at the highest priority, the overlapped A solves on
    // a second stream at the lowest: pending CTAs of the FP32 kernels are
    // placed first and the solves fill the room they leave
    int prio_low = 0, prio_high = 0;
    QG_CK(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
    QG_CK(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio_high));
    QG_CK(cudaStreamCreateWithPriority(&st2, cudaStreamNonBlocking, prio_low));
    QG_CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    QG_CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    QG_CK(cudaEventCreateWithFlags(&ev_diag, cudaEventDisableTiming));
    const size_t fbytes = (size_t)g.n3 * g.plane * sizeof(C);
    for (int f = 0; f < F_NINT; ++f) {
      if (f == F_DQ && !(cfg.inviscid == 0 && cfg.nuz != 0.0)) continue;
      QG_CK(cudaMalloc(&F[f], fbytes));
      QG_CK(cudaMemsetAsync(F[f], 0, fbytes, st));
    }
    if (!cfg.ybj_plus && !cfg.passive_scalar) {
      for (auto& p : sig) { QG_CK(cudaMalloc(&p, fbytes)); QG_CK(cudaMemsetAsync(p, 0, fbytes, st)); }
    }
    // tables
    // integrating factors: [members][plane]
    std::vector<T> tmp((size_t)members * g.plane);
    auto up = [&](T** d, const std::vector<double>& h) -> int {
      for (size_t i = 0; i < tmp.size(); ++i) tmp[i] = (T)h[i];
      QG_CK(cudaMalloc(d, tmp.size() * sizeof(T)));
      QG_CK(cudaMemcpy(*d, tmp.data(), tmp.size() * sizeof(T), cudaMemcpyHostToDevice));
      return QG_OK;
    };
    if (members > 1) {
      QG_CK(cudaMalloc(&mpar, t.mpar.size() * sizeof(double)));
      QG_CK(cudaMemcpy(mpar, t.mpar.data(), t.mpar.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    int rc;
    if ((rc = up(&e1, t.e1)) || (rc = up(&e2, t.e2)) || (rc = up(&e1w, t.e1w)) || (rc = up(&e2w, t.e2w))) return rc;
    {
      const std::vector<double>* om[4] = {&t.om_t1, &t.om_du, &t.om_dl, &t.om_a};
      double** dst[4] = {&om_t1, &om_du, &om_dl, &om_a};
      for (int k = 0; k < 4; ++k) {
        QG_CK(cudaMalloc(dst[k], (size_t)g.n3 * sizeof(double)));
        QG_CK(cudaMemcpy(*dst[k], om[k]->data(), (size_t)g.n3 * sizeof(double), cudaMemcpyHostToDevice));
      }
    }
    std::vector<C> twh(g.n);
    for (int m = 0; m < g.n; ++m) twh[m] = mk<T>((T)t.tw[2 * m], (T)t.tw[2 * m + 1]);
    QG_CK(cudaMalloc(&tw, g.n * sizeof(C)));
    QG_CK(cudaMemcpy(tw, twh.data(), g.n * sizeof(C), cudaMemcpyHostToDevice));
    QG_CK(cudaMalloc(&tab_idx, g.plane * sizeof(int)));
    QG_CK(cudaMemcpy(tab_idx, t.tab_idx.data(), g.plane * sizeof(int), cudaMemcpyHostToDevice));
    // columns of the solves: every column of the rectangle (any output
    // array), and the retained ones only (the resident fields, whose other
    // entries are zeros the solves need not rewrite)
    {
      std::vector<int> all(g.plane), ret;
      for (long long m = 0; m < g.plane; ++m) {
        all[m] = (int)m;
        const int r = (int)(m / g.KXP), kx = (int)(m % g.KXP);
        if (g.mask(kx, g.ky_of_row(r))) ret.push_back((int)m);
      }
      nret = (int)ret.size();
      QG_CK(cudaMalloc(&cols_all, all.size() * sizeof(int)));
      QG_CK(cudaMemcpy(cols_all, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice));
      QG_CK(cudaMalloc(&cols_ret, ret.size() * sizeof(int)));
      QG_CK(cudaMemcpy(cols_ret, ret.data(), ret.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    const size_t fb = std::max<size_t>(1, (size_t)t.ndistinct * g.nseg) * sizeof(double4);
    QG_CK(cudaMalloc(&fac_psi, fb));
    QG_CK(cudaMalloc(&fac_A, fb));
    if (t.ndistinct > 0) {
      QG_CK(cudaMemcpy(fac_psi, t.fac_psi.data(), (size_t)t.ndistinct * g.nseg * sizeof(double4), cudaMemcpyHostToDevice));
      QG_CK(cudaMemcpy(fac_A, t.fac_A.data(), (size_t)t.ndistinct * g.nseg * sizeof(double4), cudaMemcpyHostToDevice));
    }
    auto upd = [&](double** d, const std::vector<double>& h) -> int {
      QG_CK(cudaMalloc(d, h.size() * sizeof(double)));
      QG_CK(cudaMemcpy(*d, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
      return QG_OK;
    };
    if ((rc = upd(&du, t.du)) || (rc = upd(&cu, t.cu)) || (rc = upd(&cl, t.cl)) || (rc = upd(&r2, t.r2))) return rc;
    {
      // per-level weights of the diagnostics' vertical-difference sums:
      // w1 = 0.5/(r2 Bu dz^2) (wpe), w4 = Bu/(r2 dz^2) (pe), in FP64 and as
      // FP32 pairs (h, l) with h + l = w to ~2^-48
      std::vector<double> wv(2 * (size_t)g.nseg);
      std::vector<float2> wf(2 * (size_t)g.nseg);
      const double inv_dz2 = 1.0 / (cfg.dz * cfg.dz);
      for (int i = 0; i < g.nseg; ++i) {
        wv[i] = (0.5 / (t.r2[i] * cfg.Bu)) * inv_dz2;
        wv[g.nseg + i] = (cfg.Bu / t.r2[i]) * inv_dz2;
      }
      for (size_t i = 0; i < wv.size(); ++i) {
        const float h = (float)wv[i];
        wf[i] = make_float2(h, (float)(wv[i] - (double)h));
      }
      if ((rc = upd(&dwz, wv))) return rc;
      QG_CK(cudaMalloc(&fwz, wf.size() * sizeof(float2)));
      QG_CK(cudaMemcpy(fwz, wf.data(), wf.size() * sizeof(float2), cudaMemcpyHostToDevice));
    }
    {
      int occ = 0;
      QG_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, cfg.device));
      QG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_diag_cols<T>, kDiagThreads, 0));
      diag_slots = std::max(1, occ) * nsm;
      // partials of the largest launch (any number of whole segments)
      size_t mx = 0;
      for (int ns = 1; ns <= g.n3 / g.nseg; ++ns) mx = std::max(mx, diag_parts(ns));
      diag_part_n = mx;
    }
    QG_CK(cudaMalloc(&diag_part, diag_part_n * kNDiag * sizeof(double)));
    QG_CK(cudaMalloc(&diag_out, kNDiag * sizeof(double)));
    QG_CK(cudaMallocHost(&diag_host, kNDiag * sizeof(double)));
    QG_CK(cudaHostAlloc(&wflag_h, 3 * sizeof(int), cudaHostAllocMapped));
    wflag_h[0] = wflag_h[1] = wflag_h[2] = 0;
    QG_CK(cudaHostGetDevicePointer(&wflag, wflag_h, 0));
    nflag = wflag + 1;
    iflag = wflag + 2;
    QG_CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, cfg.device));
    // phase-A batching: by default as many levels per batch as 1.25 GB of
    // scratch planes hold (deep batches run fewer, fuller waves and longer
    // persistent row kernels; on GB300 the 512^2x256 step is fastest with
    // all 256 levels in one batch although its scratch outgrows L2)
    const size_t per_level = (size_t)kNScr * g.n * g.KXP * sizeof(C);
    int zb = cfg.levels_per_batch;
    if (zb <= 0) zb = (int)std::max<size_t>(1, (size_t)(1280u << 20) / per_level);
    zb = std::min(zb, g.n3);
    const int nb = (g.n3 + zb - 1) / zb;
    Zb = (g.n3 + nb - 1) / nb;
    lanes = std::max(1, std::min(kBatchLanes, nb));
    QG_CK(cudaMalloc(&S, (size_t)lanes * Zb * per_level));
    s_levels = lanes * Zb;
    for (int i = 1; i < kMaxLanes; ++i) {
      QG_CK(cudaStreamCreateWithPriority(&lst[i], cudaStreamNonBlocking, prio_high));
      QG_CK(cudaEventCreateWithFlags(&lev[i], cudaEventDisableTiming));
    }
    QG_CK(cudaEventCreateWithFlags(&ev_start, cudaEventDisableTiming));
    sp.delt = cfg.delt; sp.gamma = cfg.gamma; sp.Bu = cfg.Bu; sp.Ro = cfg.Ro; sp.W2F = cfg.W2F;
    sp.dz = cfg.dz; sp.nuz = cfg.nuz; sp.cdisp = 0.5 / (cfg.Bu * cfg.Ro);
    sp.adv = cfg.linear ? 0 : 1;
    sp.refr = cfg.passive_scalar ? 0 : 1;
    sp.disp = (cfg.no_dispersion || cfg.passive_scalar) ? 0 : 1;
    sp.use_dq = (cfg.inviscid == 0 && cfg.nuz != 0.0) ? 1 : 0;
    sp.euler = 0;
    sp.ybj = cfg.ybj_plus ? 1 : 0;
    sp.mpar = mpar;
    need_qw = (!cfg.fixed_flow && !cfg.no_feedback);
    // kept y-inverse planes of B (FP32 YBJ+ runs whose update transforms B^{n+1} for q^w)
    if (kReuseB && sizeof(T) == 4 && need_qw && cfg.ybj_plus && kColInvNF2) {
      QG_CK(cudaMalloc(&Qp, (size_t)g.n3 * kNQ * g.n * g.KXP * sizeof(C)));
    }
    int r0 = set_smem_attrs();
    if (r0) return r0;
    if (cfg.solve_columns != 0 && cfg.solve_columns != 16 && cfg.solve_columns != 32 && cfg.solve_columns != 64) {
      err = "solve_columns must be 0, 16, 32 or 64";
      return QG_ERR_ARG;
    }
    solve_tc = cfg.solve_columns ? cfg.solve_columns : 32;
    // forward values of the column solves; without this scratch the solves
    // checkpoint and recompute instead (k_solve)
    if (kSolveStore && cudaMalloc(&vbuf, (size_t)6 * g.n3 * g.plane * sizeof(double)) != cudaSuccess) {
      vbuf = nullptr;
      (void)cudaGetLastError();
    }
    // mixed path: per-column copies of the solve factors (coalesced reads);
    // without them the solves read the per-kh^2 tables
    if (kSolvePerColumn && sizeof(T) == 4 && vbuf) {
      if (cudaMalloc(&pcfac, (size_t)6 * g.nseg * nret * sizeof(double)) != cudaSuccess) {
        pcfac = nullptr;
        (void)cudaGetLastError();
      } else {
        k_expand_fac<<<grid_for((long long)g.nseg * nret), 256, 0, st>>>(g, tab_idx, fac_psi, fac_A, pcfac,
                                                                         cols_ret, nret);
        QG_LAUNCHED();
      }
    }
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

  void* stream() override { return (void*)st; }

  int enqueue(int euler) override { return enqueue_step(euler ? 1 : 0); }

  int batch_levels() const override { return Zb; }
  int levels_per_member() const override { return g.nseg; }
  int member_count() const override { return members; }

  int set_batch_levels(int zb) override {
    QG_CK(cudaStreamSynchronize(st));
    for (auto& x : gexec) if (x) { cudaGraphExecDestroy(x); x = nullptr; }
    const size_t per_level = (size_t)kNScr * g.n * g.KXP * sizeof(C);
    zb = std::max(1, std::min(zb, g.n3));
    const int nb = (g.n3 + zb - 1) / zb;
    const int nz = (g.n3 + nb - 1) / nb;
    const int nl = std::max(1, std::min(want_lanes, nb));
    if (nl * nz > s_levels) {
      cudaFree(S);
      S = nullptr;
      QG_CK(cudaMalloc(&S, (size_t)nl * nz * per_level));
      s_levels = nl * nz;
    }
    Zb = nz;
    lanes = nl;
    return QG_OK;
  }

  // phase-A batches in flight at once (each on its own stream and scratch)
  int batch_lanes() const override { return lanes; }
  int set_batch_lanes(int nl) override {
    if (nl < 1 || nl > kMaxLanes) { err = "batch lanes must be in [1, 8]"; return QG_ERR_ARG; }
    want_lanes = nl;
    return set_batch_levels(Zb);
  }

  int solve_columns() const override { return solve_tc; }
  int set_solve_columns(int tc) override {
    if (tc == 0) tc = 32;
    if (tc != 16 && tc != 32 && tc != 64) { err = "solve_columns must be 16, 32 or 64"; return QG_ERR_ARG; }
    QG_CK(cudaStreamSynchronize(st));
    for (auto& x : gexec) if (x) { cudaGraphExecDestroy(x); x = nullptr; }
    solve_tc = tc;
    return QG_OK;
  }

  int synchronize() override {
    QG_CK(cudaStreamSynchronize(st));
    return check_waits();
  }

  int selftest_wait() override {
    k_wait_expire<<<1, 32, 0, st>>>(wflag);
    QG_LAUNCHED();
    return synchronize();
  }

  // QG_ERR_TIMEOUT when a kernel's bounded wait expired since the last check,
  // QG_ERR_NONFINITE when a step produced a NaN or infinite q* (call after
  // the stream has drained)
  int check_waits() override {
    if (wflag_h && *(volatile int*)wflag_h) {
      *(volatile int*)wflag_h = 0;
      err = "a bounded device-side wait expired (bulk copy of the row kernels)";
      return QG_ERR_TIMEOUT;
    }
    if (wflag_h && *(volatile int*)(wflag_h + 1)) {
      *(volatile int*)(wflag_h + 1) = 0;
      err = "non-finite q* after a step: the state has blown up (time step too large?)";
      return QG_ERR_NONFINITE;
    }
    return QG_OK;
  }

  // ---- state --------------------------------------------------------------
  int set_state(int field, const double* kvar, int level0, int nlev) override {
    const int f = map_field(field);
    if (f < 0 || field == QG_CR || field == QG_CI || field == QG_QSTAR) { err = "field is read-only or unknown"; return QG_ERR_ARG; }
    if (!kvar || level0 < 0 || nlev <= 0 || level0 + nlev > g.n3) { err = "bad level range or null pointer"; return QG_ERR_ARG; }
    const size_t bytes = (size_t)nlev * g.n * (g.n / 2 + 1) * sizeof(double2);
    // pinned host or device arrays are read in place (only the retained
    // modes cross the link); others go through a device staging copy
    const double2* src = static_cast<const double2*>(device_view(kvar));
    if (!src) {
      int rc = ensure(&stage, &stage_bytes, bytes);
      if (rc) return rc;
      QG_CK(cudaMemcpyAsync(stage, kvar, bytes, cudaMemcpyDefault, st));
      src = (const double2*)stage;
    }
    *(volatile int*)(wflag_h + 2) = 0;
    if (f == F_BR || f == F_BI) q_valid = false;
    if (f == F_PSI && sizeof(T) == 4) {
      // mixed path: keep psi in FP64 until qg_init_state has built q from it
      // (init_q's vertical second difference would amplify FP32 rounding);
      // the FP32 field is rounded from that copy on the device, so the input
      // crosses the host link once
      if (!psi64) QG_CK(cudaMalloc(&psi64, (size_t)g.n3 * g.plane * sizeof(double2)));
      k_dense_to_compact<double><<<grid_for((long long)nlev * g.plane), 256, 0, st>>>(g, level0, nlev, src, psi64,
                                                                                        iflag);
      QG_LAUNCHED();
      k_round_compact<T><<<grid_for((long long)nlev * g.plane), 256, 0, st>>>(
          (long long)nlev * g.plane, reinterpret_cast<const cplx<double>*>(psi64) + (size_t)level0 * g.plane,
          F[f] + (size_t)level0 * g.plane);
      QG_LAUNCHED();
    } else {
      k_dense_to_compact<T><<<grid_for((long long)nlev * g.plane), 256, 0, st>>>(g, level0, nlev, src, F[f], iflag);
      QG_LAUNCHED();
    }
    QG_CK(cudaStreamSynchronize(st));
    if (*(volatile int*)(wflag_h + 2)) {
      *(volatile int*)(wflag_h + 2) = 0;
      err = "non-finite value (NaN or Inf) on a retained mode of the input array";
      return QG_ERR_NONFINITE;
    }
    return QG_OK;
  }

  int get_state(int field, double* kvar, int level0, int nlev) override {
    int f = map_field(field);
    if (f < 0) { err = "unknown field"; return QG_ERR_ARG; }
    if (!kvar || level0 < 0 || nlev <= 0 || level0 + nlev > g.n3) { err = "bad level range or null pointer"; return QG_ERR_ARG; }
    if (field == QG_QSTAR && !need_qw) f = F_Q;
    const int mode = (field == QG_CR || field == QG_CI) ? 1 : 0;
    const size_t bytes = (size_t)nlev * g.n * (g.n / 2 + 1) * sizeof(double2);
    double2* dst = static_cast<double2*>(const_cast<void*>(device_view(kvar)));
    if (!dst) {
      int rc = ensure(&stage, &stage_bytes, bytes);
      if (rc) return rc;
    }
    k_compact_to_dense<T><<<grid_for((long long)nlev * g.n * (g.n / 2 + 1)), 256, 0, st>>>(
        g, level0, nlev, F[f], dst ? dst : (double2*)stage, mode, cfg.dz);
    QG_LAUNCHED();
    if (!dst) QG_CK(cudaMemcpyAsync(kvar, stage, bytes, cudaMemcpyDefault, st));
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

  // Device address through which kernels may access p: device memory as is,
  // page-locked host memory through its mapping; nullptr for anything else
  // (pageable or managed memory is staged through a copy instead).
  static const void* device_view(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) { (void)cudaGetLastError(); return nullptr; }
    if (at.type == cudaMemoryTypeDevice) return p;
    if (at.type == cudaMemoryTypeHost && at.devicePointer) return at.devicePointer;
    return nullptr;
  }

  int init_state(int apply_sumB, int q_from_psi) override {
    int rc = init_state_range(0, g.n3, apply_sumB, q_from_psi);
    if (rc) return rc;
    release_init_buffers();
    return QG_OK;
  }

  // The initialisation sequence on levels [z0, z0 + nz) (whole segments):
  // one run, or one member of a stack (whose FP64 psi copy stays until
  // release_init_buffers, so that every member's q is built from it)
  int init_state_range(int z0, int nz, int apply_sumB, int q_from_psi) override {
    if (z0 < 0 || nz <= 0 || z0 + nz > g.n3 || z0 % g.nseg || nz % g.nseg) {
      err = "initialisation range must cover whole members";
      return QG_ERR_ARG;
    }
    q_valid = false;
    if (apply_sumB) {
      k_sumB<T><<<(unsigned)((g.plane + 127) / 128), 128, 0, st>>>(g, F[F_BR], F[F_BI], z0, z0 + nz);
      QG_LAUNCHED();
    }
    const size_t lb = (size_t)g.plane * sizeof(C), off = (size_t)z0 * g.plane;
    if (cfg.fixed_flow) {
      // fixed flow: q = 0 for all times (main_waqg.f90:141-146)
      QG_CK(cudaMemsetAsync(F[F_Q] + off, 0, (size_t)nz * lb, st));
    } else if (q_from_psi) {
      if (psi64) {
        k_init_q<T, double><<<grid_for((long long)nz * g.plane), 256, 0, st>>>(g, cfg.dz, cu, cl, psi64, F[F_Q], z0,
                                                                               z0 + nz);
      } else {
        k_init_q<T, T><<<grid_for((long long)nz * g.plane), 256, 0, st>>>(g, cfg.dz, cu, cl, F[F_PSI], F[F_Q], z0,
                                                                          z0 + nz);
      }
      QG_LAUNCHED();
    }
    QG_CK(cudaMemcpyAsync(F[F_QO] + off, F[F_Q] + off, (size_t)nz * lb, cudaMemcpyDeviceToDevice, st));
    QG_CK(cudaMemcpyAsync(F[F_BRO] + off, F[F_BR] + off, (size_t)nz * lb, cudaMemcpyDeviceToDevice, st));
    QG_CK(cudaMemcpyAsync(F[F_BIO] + off, F[F_BI] + off, (size_t)nz * lb, cudaMemcpyDeviceToDevice, st));
    if (!cfg.passive_scalar && cfg.ybj_plus) {   // regular YBJ keeps the A the host set
      int rc = solve_generic(nullptr, F[F_BR], F[F_BI], nullptr, F[F_AR], F[F_AI], 0, 1, st, z0 / g.nseg,
                             nz / g.nseg, true);
      if (rc) return rc;
    }
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

  // the FP64 copy of psi that qg_set_state keeps for init_q (mixed path)
  void release_init_buffers() override {
    if (psi64) { cudaStreamSynchronize(st); cudaFree(psi64); psi64 = nullptr; }
  }

  // ---- the step -------------------------------------------------------------
  int step(int euler) override {
    int rc = run_step(euler ? 1 : 0);
    if (rc) return rc;
    QG_CK(cudaStreamSynchronize(st));
    return check_waits();
  }

  int steps_async(int nsteps, int euler) override {
    for (int i = 0; i < nsteps; ++i) {
      int rc = run_step((euler && i == 0) ? 1 : 0);
      if (rc) return rc;
    }
    return QG_OK;
  }

  int diagnostics(qg_energy* out) override { return diagnostics_range(0, g.n3, out); }

  // k_diag_cols over nsegs whole segments: the levels of each segment in
  // chunks of zc, as many chunks as keep the grid within one wave of
  // resident CTAs (a second, partial wave would run at a fraction of the
  // GPU); returns the grid
  dim3 diag_grid(int nsegs, int* zc) const {
    const int cb = (nret + kDiagThreads - 1) / kDiagThreads;
    const long long per = (long long)cb * nsegs;
    const int nch0 = (int)std::max<long long>(1, std::min<long long>(g.nseg, (long long)diag_slots / per));
    *zc = (g.nseg + nch0 - 1) / nch0;
    return dim3(cb, (g.nseg + *zc - 1) / *zc, nsegs);
  }
  size_t diag_parts(int nsegs) const {
    int zc;
    const dim3 gr = diag_grid(nsegs, &zc);
    return (size_t)gr.x * gr.y * gr.z;
  }
  // the seven integrals of segments [seg0, seg0 + nsegs) into out (device)
  int launch_diag(int seg0, int nsegs, double* part, double* out, cudaStream_t s) {
    int zc;
    const dim3 grid = diag_grid(nsegs, &zc);
    const double c2 = (1.0 / 8.0) * (1.0 / (cfg.Bu * cfg.Bu)), c6 = 2.0 * (1.0 / (cfg.dz * cfg.dz));
    k_diag_cols<T><<<grid, kDiagThreads, 0, s>>>(g, seg0, zc, dwz, fwz, c2, c6, F[F_BR], F[F_BI], F[F_AR],
                                                 F[F_AI], F[F_PSI], cols_ret, nret, part);
    QG_LAUNCHED();
    k_diag_sum<<<1, 32 * kNDiag, 0, s>>>((long long)grid.x * grid.y * grid.z, nsegs * g.nseg, part, out);
    QG_LAUNCHED();
    return QG_OK;
  }

  // The integrals of the state as it stands after the work queued so far, on
  // a stream of their own: the next step's first kernels (which only read
  // the state) run beside them, and its update kernels wait for them in the
  // graph (external event wait before each k_col_update).  diagnostics_wait
  // returns the values.
  int diagnostics_async() override {
    if (!std_) {
      int prio_low = 0, prio_high = 0;
      QG_CK(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
      QG_CK(cudaStreamCreateWithPriority(&std_, cudaStreamNonBlocking, prio_low));
      QG_CK(cudaEventCreateWithFlags(&ev_state, cudaEventDisableTiming));
      QG_CK(cudaMalloc(&diag_part_a, diag_part_n * kNDiag * sizeof(double)));
      QG_CK(cudaMalloc(&diag_out_a, kNDiag * sizeof(double)));
      QG_CK(cudaMallocHost(&diag_host_a, kNDiag * sizeof(double)));
    }
    if (diag_pending) { err = "the previous asynchronous diagnostics were not collected"; return QG_ERR_ARG; }
    QG_CK(cudaEventRecord(ev_state, st));
    QG_CK(cudaStreamWaitEvent(std_, ev_state, 0));
    if (int rc = launch_diag(0, g.n3 / g.nseg, diag_part_a, diag_out_a, std_)) return rc;
    QG_CK(cudaMemcpyAsync(diag_host_a, diag_out_a, kNDiag * sizeof(double), cudaMemcpyDeviceToHost, std_));
    QG_CK(cudaEventRecord(ev_diag, std_));
    diag_pending = true;
    return QG_OK;
  }

  int diagnostics_wait(qg_energy* out) override {
    if (!diag_pending) { err = "no asynchronous diagnostics pending"; return QG_ERR_ARG; }
    QG_CK(cudaEventSynchronize(ev_diag));
    diag_pending = false;
    out->wke = diag_host_a[0]; out->wpe = diag_host_a[1]; out->wce = diag_host_a[2];
    out->ke = diag_host_a[3]; out->pe = diag_host_a[4]; out->zeta2 = diag_host_a[5]; out->omegah2 = diag_host_a[6];
    return QG_OK;
  }

  // the integrals over levels [z0, z0 + nz): one run, or one member of a stack
  int diagnostics_range(int z0, int nz, qg_energy* out) override {
    if (z0 % g.nseg || nz % g.nseg || nz <= 0) { err = "diagnostics range is not a set of whole segments"; return QG_ERR_ARG; }
    if (int rc = launch_diag(z0 / g.nseg, nz / g.nseg, diag_part, diag_out, st)) return rc;
    QG_CK(cudaMemcpyAsync(diag_host, diag_out, kNDiag * sizeof(double), cudaMemcpyDeviceToHost, st));
    QG_CK(cudaStreamSynchronize(st));
    out->wke = diag_host[0]; out->wpe = diag_host[1]; out->wce = diag_host[2];
    out->ke = diag_host[3]; out->pe = diag_host[4]; out->zeta2 = diag_host[5]; out->omegah2 = diag_host[6];
    return QG_OK;
  }

  // ---- output path ----------------------------------------------------------
  int dump_real(int which, float* out0, float* out1, int level0, int nlev, double s1, double s2) override {
    if (level0 < 0 || nlev <= 0 || level0 + nlev > g.n3) { err = "bad level range"; return QG_ERR_ARG; }
    int rc = prep_dense(nlev);
    if (rc) return rc;
    const long long tot = (long long)nlev * g.n * (g.n / 2 + 1), np = (long long)nlev * g.n * g.n;
    float* o32 = reinterpret_cast<float*>(dstage);        // nlev*n*(n+2) doubles hold nlev*n*n floats
    const int nf = which == 0 ? 1 : 2;
    for (int c = 0; c < nf; ++c) {
      const C* src = which == 0 ? F[F_PSI] : (c == 0 ? F[F_BR] : F[F_BI]);
      k_compact_to_dense<T><<<grid_for(tot), 256, 0, st>>>(g, level0, nlev, src, D[0], 0, cfg.dz);
      QG_LAUNCHED();
      const double2* spec = D[0];
      if (which == 2) {
        k_compact_to_dense<T><<<grid_for(tot), 256, 0, st>>>(g, level0, nlev, c == 0 ? F[F_AR] : F[F_AI], D[1], 0,
                                                            cfg.dz);
        QG_LAUNCHED();
        k_dense_la<<<grid_for(tot), 256, 0, st>>>(g.n, g.kmax2, tot, D[0], D[1], cfg.Bu, D[2]);
        QG_LAUNCHED();
        spec = D[2];
      }
      if ((rc = d_c2r(spec, P[0], nlev))) return rc;
      k_phys_f32<T><<<grid_for(np), 256, 0, st>>>(np, P[0], s1, s2, o32);
      QG_LAUNCHED();
      QG_CK(cudaMemcpyAsync(c == 0 ? out0 : out1, o32, (size_t)np * sizeof(float), cudaMemcpyDefault, st));
      QG_CK(cudaStreamSynchronize(st));
    }
    return QG_OK;
  }

  // ---- omega equation (the vertical-velocity diagnostic) ---------------------
  // right-hand side from the dense psi in D[0] into D[5]
  int omega_rhs_dev() {
    const long long tot = (long long)g.n3 * g.n * (g.n / 2 + 1), pt = (long long)g.n3 * g.n * g.n;
    k_omega_spec<<<grid_for(tot), 256, 0, st>>>(g.n, g.n3, g.kmax2, cfg.dz, D[0], D[1], D[2], D[3], D[4]);
    QG_LAUNCHED();
    int rc;
    for (int k = 0; k < 4; ++k)
      if ((rc = d_c2r(D[1 + k], P[k], g.n3))) return rc;
    k_omega_phys<T><<<grid_for(pt), 256, 0, st>>>(pt, P[0], P[1], P[2], P[3], P[4]);
    QG_LAUNCHED();
    return d_r2c(P[4], D[5], g.n3);
  }
  // w from the dense right-hand side in `rhs` into D[1]
  int omega_solve_dev(const double2* rhs) {
    const long long per = (long long)g.n * (g.n / 2 + 1);
    if (!om_scr) QG_CK(cudaMalloc(&om_scr, (size_t)3 * (g.n3 > 1 ? g.n3 - 1 : 1) * per * sizeof(double)));
    k_omega_solve<<<(unsigned)((per + 127) / 128), 128, 0, st>>>(g.n, g.n3, g.kmax2, cfg.dz, om_t1, om_du, om_dl, om_a,
                                                                 rhs, om_scr, D[1]);
    QG_LAUNCHED();
    return QG_OK;
  }
  int omega_eqn_rhs(const double* psik, double* rhs) override {
    int rc = prep_dense(g.n3);
    if (rc) return rc;
    QG_CK(cudaMemcpyAsync(D[0], psik, dense_bytes(g.n3), cudaMemcpyDefault, st));
    if ((rc = omega_rhs_dev())) return rc;
    QG_CK(cudaMemcpyAsync(rhs, D[5], dense_bytes(g.n3), cudaMemcpyDefault, st));
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }
  int omega_equation(const double* rhs, double* wk) override {
    int rc = prep_dense(g.n3);
    if (rc) return rc;
    QG_CK(cudaMemcpyAsync(D[0], rhs, dense_bytes(g.n3), cudaMemcpyDefault, st));
    if ((rc = omega_solve_dev(D[0]))) return rc;
    QG_CK(cudaMemcpyAsync(wk, D[1], dense_bytes(g.n3), cudaMemcpyDefault, st));
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }
  int omega_from_state(double* wk) override {
    int rc = prep_dense(g.n3);
    if (rc) return rc;
    k_compact_to_dense<T><<<grid_for((long long)g.n3 * g.n * (g.n / 2 + 1)), 256, 0, st>>>(g, 0, g.n3, F[F_PSI], D[0], 0,
                                                                                          cfg.dz);
    QG_LAUNCHED();
    if ((rc = omega_rhs_dev()) || (rc = omega_solve_dev(D[5]))) return rc;
    QG_CK(cudaMemcpyAsync(wk, D[1], dense_bytes(g.n3), cudaMemcpyDefault, st));
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

  // ---- routine-level drop-ins ---------------------------------------------
  int fft_r2c(const double* rvar, double* kvar, int nz) override {
    int rc = prep_dense(nz);
    if (rc) return rc;
    const long long np = (long long)nz * g.n * (g.n + 2);
    QG_CK(cudaMemcpyAsync(dstage, rvar, np * sizeof(double), cudaMemcpyDefault, st));
    k_phys_unpad<T><<<grid_for((long long)nz * g.n * g.n), 256, 0, st>>>(g.n, (long long)nz * g.n * g.n, dstage, P[0]);
    QG_LAUNCHED();
    if ((rc = d_r2c(P[0], D[0], nz))) return rc;
    QG_CK(cudaMemcpyAsync(kvar, D[0], dense_bytes(nz), cudaMemcpyDefault, st));
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

  int fft_c2r(const double* kvar, double* rvar, int nz) override {
    int rc = prep_dense(nz);
    if (rc) return rc;
    QG_CK(cudaMemcpyAsync(D[0], kvar, dense_bytes(nz), cudaMemcpyDefault, st));
    if ((rc = d_c2r(D[0], P[0], nz))) return rc;
    const long long np = (long long)nz * g.n * (g.n + 2);
    k_phys_pad<T><<<grid_for(np), 256, 0, st>>>(g.n, np, P[0], dstage);
    QG_LAUNCHED();
    QG_CK(cudaMemcpyAsync(rvar, dstage, np * sizeof(double), cudaMemcpyDefault, st));
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

  int convol_waqg(const double* uk, const double* vk, const double* qk, const double* BRk, const double* BIk,
                  double* nqk, double* nBRk, double* nBIk, int nz) override {
    int rc = prep_dense(nz);
    if (rc) return rc;
    const size_t db = dense_bytes(nz);
    const long long tot = (long long)nz * g.n * (g.n / 2 + 1), pt = (long long)nz * g.n * g.n;
    QG_CK(cudaMemcpyAsync(D[0], uk, db, cudaMemcpyDefault, st));
    QG_CK(cudaMemcpyAsync(D[1], vk, db, cudaMemcpyDefault, st));
    if ((rc = d_c2r(D[0], P[0], nz)) || (rc = d_c2r(D[1], P[1], nz))) return rc;
    const double* ins[3] = {qk, BRk, BIk};
    double* outs[3] = {nqk, nBRk, nBIk};
    for (int k = 0; k < 3; ++k) {
      QG_CK(cudaMemcpyAsync(D[2], ins[k], db, cudaMemcpyDefault, st));
      if ((rc = d_c2r(D[2], P[2], nz))) return rc;
      k_phys<T><<<grid_for(pt), 256, 0, st>>>(pt, 0, P[0], P[2], nullptr, nullptr, P[3]);
      QG_LAUNCHED();
      if ((rc = d_r2c(P[3], D[3], nz))) return rc;
      k_phys<T><<<grid_for(pt), 256, 0, st>>>(pt, 0, P[1], P[2], nullptr, nullptr, P[3]);
      QG_LAUNCHED();
      if ((rc = d_r2c(P[3], D[4], nz))) return rc;
      k_dense_ik<<<grid_for(tot), 256, 0, st>>>(g.n, g.kmax2, tot, D[3], D[4], D[5]);
      QG_LAUNCHED();
      QG_CK(cudaMemcpyAsync(outs[k], D[5], db, cudaMemcpyDefault, st));
      QG_CK(cudaStreamSynchronize(st));
    }
    return QG_OK;
  }

  int refraction_waqg(const double* BRk, const double* BIk, const double* psik, double* rBRk, double* rBIk,
                      int nz) override {
    int rc = prep_dense(nz);
    if (rc) return rc;
    const size_t db = dense_bytes(nz);
    const long long tot = (long long)nz * g.n * (g.n / 2 + 1), pt = (long long)nz * g.n * g.n;
    QG_CK(cudaMemcpyAsync(D[0], psik, db, cudaMemcpyDefault, st));
    k_dense_op<<<grid_for(tot), 256, 0, st>>>(g.n, g.kmax2, tot, 0, D[0], D[1]);
    QG_LAUNCHED();
    if ((rc = d_c2r(D[1], P[0], nz))) return rc;
    const double* ins[2] = {BRk, BIk};
    double* outs[2] = {rBRk, rBIk};
    for (int k = 0; k < 2; ++k) {
      QG_CK(cudaMemcpyAsync(D[2], ins[k], db, cudaMemcpyDefault, st));
      if ((rc = d_c2r(D[2], P[1], nz))) return rc;
      k_phys<T><<<grid_for(pt), 256, 0, st>>>(pt, 0, P[0], P[1], nullptr, nullptr, P[2]);
      QG_LAUNCHED();
      if ((rc = d_r2c(P[2], D[3], nz))) return rc;
      k_dense_mask<<<grid_for(tot), 256, 0, st>>>(g.n, g.kmax2, tot, D[3], D[4]);
      QG_LAUNCHED();
      QG_CK(cudaMemcpyAsync(outs[k], D[4], db, cudaMemcpyDefault, st));
      QG_CK(cudaStreamSynchronize(st));
    }
    return QG_OK;
  }

  int compute_qw(const double* BRk, const double* BIk, double* qwk, int nz) override {
    int rc = prep_dense(nz);
    if (rc) return rc;
    const size_t db = dense_bytes(nz);
    const long long tot = (long long)nz * g.n * (g.n / 2 + 1), pt = (long long)nz * g.n * g.n;
    QG_CK(cudaMemcpyAsync(D[0], BRk, db, cudaMemcpyDefault, st));
    QG_CK(cudaMemcpyAsync(D[1], BIk, db, cudaMemcpyDefault, st));
    // BRx, BRy, BIx, BIy -> P0..P3
    const int ops[4] = {1, 2, 1, 2};
    for (int k = 0; k < 4; ++k) {
      k_dense_op<<<grid_for(tot), 256, 0, st>>>(g.n, g.kmax2, tot, ops[k], D[k < 2 ? 0 : 1], D[2]);
      QG_LAUNCHED();
      if ((rc = d_c2r(D[2], P[k], nz))) return rc;
    }
    // qwr = BRy*BIx - BRx*BIy
    k_phys<T><<<grid_for(pt), 256, 0, st>>>(pt, 2, P[1], P[2], P[0], P[3], P[4]);
    QG_LAUNCHED();
    if ((rc = d_r2c(P[4], D[3], nz))) return rc;
    if ((rc = d_c2r(D[0], P[0], nz)) || (rc = d_c2r(D[1], P[1], nz))) return rc;
    k_phys<T><<<grid_for(pt), 256, 0, st>>>(pt, 1, P[0], P[1], nullptr, nullptr, P[4]);
    QG_LAUNCHED();
    if ((rc = d_r2c(P[4], D[4], nz))) return rc;
    k_dense_qw<<<grid_for(tot), 256, 0, st>>>(g.n, g.kmax2, tot, D[3], D[4], cfg.Ro, cfg.W2F, D[5]);
    QG_LAUNCHED();
    QG_CK(cudaMemcpyAsync(qwk, D[5], db, cudaMemcpyDefault, st));
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

  int psi_solver(const double* qstar, double* psik) override {
    int rc = ensure_tmp();
    if (rc) return rc;
    if ((rc = upload_compact(qstar, tmpF[0]))) return rc;
    if ((rc = solve_generic(tmpF[0], nullptr, nullptr, tmpF[1], nullptr, nullptr, 1, 0))) return rc;
    return download_compact(tmpF[1], psik, 0);
  }

  int A_solver(const double* bk, double* ak, double* ck) override {
    int rc = ensure_tmp();
    if (rc) return rc;
    if ((rc = upload_compact(bk, tmpF[0]))) return rc;
    if ((rc = solve_generic(nullptr, tmpF[0], tmpF[0], nullptr, tmpF[1], tmpF[2], 0, 1))) return rc;
    if ((rc = download_compact(tmpF[1], ak, 0))) return rc;
    if (ck) return download_compact(tmpF[1], ck, 1);
    return QG_OK;
  }

 protected:
  qg_config cfg{};
  Geom g{};
  StepParams sp{};
  cudaStream_t st = nullptr;
  cudaStream_t st2 = nullptr;                          // the overlapped A solves
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;   // B^{n+1} ready / A solves done
  // asynchronous diagnostics: their stream, state-ready and done events,
  // their own buffers
  cudaStream_t std_ = nullptr;
  cudaEvent_t ev_state = nullptr, ev_diag = nullptr;
  double *diag_part_a = nullptr, *diag_out_a = nullptr, *diag_host_a = nullptr;
  bool diag_pending = false;
  C* F[F_NINT] = {};
  T *e1 = nullptr, *e2 = nullptr, *e1w = nullptr, *e2w = nullptr;
  C* tw = nullptr;
  int* tab_idx = nullptr;
  int* cols_all = nullptr;   // 0 .. plane-1
  int* cols_ret = nullptr;   // the retained columns (L = 1), ascending
  int nret = 0;
  double4 *fac_psi = nullptr, *fac_A = nullptr;
  double* pcfac = nullptr;   // per-column solve factors of the mixed path (k_expand_fac), or null
  double* vbuf = nullptr;    // forward values of the column solves (k_solve_st)
  int solve_tc = 32;         // columns per CTA of k_solve_st
  double *du = nullptr, *cu = nullptr, *cl = nullptr, *r2 = nullptr;
  double *diag_part = nullptr, *diag_out = nullptr, *diag_host = nullptr;
  double* dwz = nullptr;     // diagnostics' per-level weights (w1, w4), FP64
  float2* fwz = nullptr;     // the same as FP32 pairs
  int diag_slots = 1;        // resident k_diag_cols CTAs on the GPU
  size_t diag_part_n = 0;    // partials the diagnostics buffers hold
  // set by a kernel whose bounded wait expired (mapped page-locked word)
  // mapped page-locked words raised on the device: [0] a bounded wait
  // expired, [1] a step produced a non-finite q*, [2] qg_set_state's input
  // held a non-finite retained mode (wflag, nflag, iflag: device views)
  int* wflag_h = nullptr;
  int* wflag = nullptr;
  int* nflag = nullptr;
  int* iflag = nullptr;
  int nsm = 1, occ_rm = 1, occ_rq = 1;   // SMs; resident CTAs per SM of the persistent row kernels
  double *om_t1 = nullptr, *om_du = nullptr, *om_dl = nullptr, *om_a = nullptr, *om_scr = nullptr;
  C* sig[2] = {};     // regular YBJ: per-level sigma terms
  C* Qp = nullptr;             // kept y-inverse planes of B, [n3][2][n][KXP], or null
  bool q_valid = false;        // Qp holds the transforms of the current B
  int members = 1;             // ensemble members stacked in z (segments of g.nseg levels)
  double* mpar = nullptr;      // their step parameters (StepParams::mpar)
  C* S = nullptr;              // [lanes][Zb][kNScr][n][KXP] scratch planes
  int s_levels = 0;            // levels of scratch allocated
  double2* psi64 = nullptr;
  int Zb = 1;
  // phase-A batches run on `lanes` streams (lane 0: st), batch b on lane
  // b % lanes with its own scratch slot; they join st before the solves
  static constexpr int kMaxLanes = 8;
  int lanes = 1, want_lanes = kBatchLanes;
  cudaStream_t lst[kMaxLanes] = {};
  cudaEvent_t lev[kMaxLanes] = {};
  cudaEvent_t ev_start = nullptr;
  bool need_qw = true;
  void* stage = nullptr; size_t stage_bytes = 0;
  // dense drop-in buffers
  int dense_nz = 0;
  double2* D[6] = {};
  T* P[5] = {};
  C* W = nullptr;
  double* dstage = nullptr;
  C* tmpF[3] = {};
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};

  void release() {
    if (st) cudaStreamSynchronize(st);
    for (auto& x : gexec) if (x) { cudaGraphExecDestroy(x); x = nullptr; }
    for (auto& p : F) if (p) { cudaFree(p); p = nullptr; }
    void* ps[] = {e1, e2, e1w, e2w, tw, tab_idx, cols_all, cols_ret, fac_psi, fac_A, pcfac, vbuf, du, cu, cl, r2, diag_part, diag_out, dwz, fwz, S, stage,
                  W, dstage, psi64, om_t1, om_du, om_dl, om_a, om_scr, sig[0], sig[1], mpar, Qp};
    for (void* p : ps) if (p) cudaFree(p);
    for (auto& p : D) if (p) cudaFree(p);
    for (auto& p : P) if (p) cudaFree(p);
    for (auto& p : tmpF) if (p) cudaFree(p);
    if (diag_host) cudaFreeHost(diag_host);
    if (wflag_h) cudaFreeHost(wflag_h);
    wflag_h = nullptr;
    wflag = nullptr;
    nflag = nullptr;
    iflag = nullptr;
    for (int i = 1; i < kMaxLanes; ++i) {
      if (lst[i]) { cudaStreamSynchronize(lst[i]); cudaStreamDestroy(lst[i]); lst[i] = nullptr; }
      if (lev[i]) { cudaEventDestroy(lev[i]); lev[i] = nullptr; }
    }
    if (ev_start) { cudaEventDestroy(ev_start); ev_start = nullptr; }
    if (std_) { cudaStreamSynchronize(std_); cudaStreamDestroy(std_); std_ = nullptr; }
    if (ev_state) { cudaEventDestroy(ev_state); ev_state = nullptr; }
    if (ev_diag) { cudaEventDestroy(ev_diag); ev_diag = nullptr; }
    if (diag_part_a) { cudaFree(diag_part_a); diag_part_a = nullptr; }
    if (diag_out_a) { cudaFree(diag_out_a); diag_out_a = nullptr; }
    if (diag_host_a) { cudaFreeHost(diag_host_a); diag_host_a = nullptr; }
    if (st2) cudaStreamSynchronize(st2);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    ev_fork = ev_join = nullptr;
    if (st2) cudaStreamDestroy(st2);
    st2 = nullptr;
    if (st) cudaStreamDestroy(st);
    st = nullptr;
  }

  static unsigned grid_for(long long n) {
    long long b = (n + 255) / 256;
    return (unsigned)std::max<long long>(1, std::min<long long>(b, 152LL * 16));
  }

  int map_field(int field) const {
    switch (field) {
      case QG_Q: return F_Q; case QG_QOLD: return F_QO; case QG_BR: return F_BR; case QG_BI: return F_BI;
      case QG_BROLD: return F_BRO; case QG_BIOLD: return F_BIO; case QG_PSI: return F_PSI;
      case QG_AR: case QG_CR: return F_AR;
      case QG_AI: case QG_CI: return F_AI;
      case QG_QSTAR: return F_QSTAR;
      default: return -1;
    }
  }

  int ensure(void** p, size_t* have, size_t need) {
    if (*have >= need) return QG_OK;
    if (*p) { QG_CK(cudaStreamSynchronize(st)); cudaFree(*p); *p = nullptr; *have = 0; }
    QG_CK(cudaMalloc(p, need));
    *have = need;
    return QG_OK;
  }

  // shared memory of the step kernels (twiddles + padded transforms)
  // column kernels on the interleaved tile (colfft.cuh): NF fields in flight
  template <int NN, int CP = 16> static constexpr size_t sm_ci(int nf) {
    return (size_t)(NN + nf * ColLay<NN, Tiles<T, NN>::CT, CP>::FS) * sizeof(C);
  }
  template <int NN> static constexpr size_t sm_col6() { return (size_t)(NN + 6 * Tiles<T, NN>::CT * Tiles<T, NN>::LD) * sizeof(C); }
  template <int NN> static constexpr size_t sm_row7() { return (size_t)(NN + 7 * Tiles<T, NN>::RT * Tiles<T, NN>::LD) * sizeof(C); }
  template <int NN> static constexpr size_t sm_rr3() { return (size_t)(NN + 3 * Tiles<T, NN>::QRT * Tiles<T, NN>::LD) * sizeof(C); }
  template <int NN> static constexpr size_t sm_rm4() { return (size_t)(NN + 4 * Tiles<T, NN>::RTM * Tiles<T, NN>::LD) * sizeof(C); }
  // the persistent row kernels add a staging copy of an item's scratch rows
  // (nf planes x rows x kxp) and its mbarrier; the attribute is set for the
  // widest rows any mask of this n can have (kxp for K = n/2)
  template <int NN> static constexpr int kxp_max() { return ((NN / 2 + 1 + 7) / 8) * 8; }
  template <int NN> static constexpr size_t sm_rm(int kxp) {
    return sm_rm4<NN>() + (Tiles<T, NN>::RPRE ? (size_t)6 * Tiles<T, NN>::RTM * kxp * sizeof(C) + 16 : 0);
  }
  template <int NN> static constexpr size_t sm_rq(int kxp) {
    return sm_rr3<NN>() + (Tiles<T, NN>::QPRE ? (size_t)4 * Tiles<T, NN>::QRT * kxp * sizeof(C) + 16 : 0);
  }
  template <int NN> static constexpr size_t sm_row4() { return (size_t)(NN + 4 * Tiles<T, NN>::RT * Tiles<T, NN>::LD) * sizeof(C); }
  // shared memory of the dense (routine-level) kernels
  size_t sm_colinv() const { return (size_t)(g.n + 2 * Tile<T>::CT * (g.n + 1)) * sizeof(C); }
  size_t sm_drow() const { return (size_t)(3 * g.n) * sizeof(C); }

  int set_smem_attrs() {
    const int mx = cudaFuncAttributeMaxDynamicSharedMemorySize;
    QG_SWITCH_N(g.n, {
      QG_CK(cudaFuncSetAttribute(k_col_inv<T, NN>, (cudaFuncAttribute)mx, (int)sm_ci<NN, Tiles<T, NN>::CIP>(Tiles<T, NN>::CINF)));
      QG_CK(cudaFuncSetAttribute(k_row_main<T, NN>, (cudaFuncAttribute)mx, (int)sm_rm<NN>(kxp_max<NN>())));
      QG_CK(cudaFuncSetAttribute(k_col_update<T, NN>, (cudaFuncAttribute)mx, (int)UpdLay<T, NN>::bytes()));
      QG_CK(cudaFuncSetAttribute(k_row_qw<T, NN>, (cudaFuncAttribute)mx, (int)sm_rq<NN>(kxp_max<NN>())));
      QG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_rm, k_row_main<T, NN>, kRowThreads, sm_rm<NN>(g.KXP)));
      QG_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_rq, k_row_qw<T, NN>, Tiles<T, NN>::QTHREADS,
                                                          sm_rq<NN>(g.KXP)));
      occ_rm = std::max(occ_rm, 1);
      occ_rq = std::max(occ_rq, 1);
      QG_CK(cudaFuncSetAttribute(k_col_qw<T, NN>, (cudaFuncAttribute)mx, (int)sm_ci<NN, Tiles<T, NN>::CQP>(2)));
      // per-function attribute shared by every handle: set it for the deepest supported column
      QG_CK(cudaFuncSetAttribute(k_solve<T>, (cudaFuncAttribute)mx, (int)solve_smem(kMaxN3)));
      QG_CK(cudaFuncSetAttribute(k_dcol_inv<T, NN>, (cudaFuncAttribute)mx, (int)sm_colinv()));
      QG_CK(cudaFuncSetAttribute(k_dcol_fwd<T, NN>, (cudaFuncAttribute)mx, (int)sm_colinv()));
      QG_CK(cudaFuncSetAttribute(k_drow_c2r<T, NN>, (cudaFuncAttribute)mx, (int)sm_drow()));
      QG_CK(cudaFuncSetAttribute(k_drow_r2c<T, NN>, (cudaFuncAttribute)mx, (int)sm_drow()));
    });
    return QG_OK;
  }

  StateP<T> state_ptrs() {
    StateP<T> p;
    p.q = F[F_Q]; p.qo = F[F_QO]; p.BR = F[F_BR]; p.BI = F[F_BI]; p.BRo = F[F_BRO]; p.BIo = F[F_BIO];
    p.psi = F[F_PSI]; p.AR = F[F_AR]; p.AI = F[F_AI]; p.qstar = F[F_QSTAR]; p.dq = F[F_DQ];
    p.sig1 = sig[0]; p.sig2 = sig[1];
    return p;
  }

  // Profiling: events around each launch when prof_on is set.
  bool prof_on = false;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_ev;
  int pbeg(int kind, cudaStream_t on = nullptr) {
    if (!prof_on) return QG_OK;
    cudaEvent_t a, b;
    QG_CK(cudaEventCreate(&a)); QG_CK(cudaEventCreate(&b));
    QG_CK(cudaEventRecord(a, on ? on : st));
    prof_ev.push_back({kind, {a, b}});
    return QG_OK;
  }
  int pend(cudaStream_t on = nullptr) {
    if (!prof_on) return QG_OK;
    QG_CK(cudaEventRecord(prof_ev.back().second.second, on ? on : st));
    return QG_OK;
  }

 public:
  int profile_step(int euler, double* ms, int* launches, int nclasses) override {
    for (int i = 0; i < nclasses; ++i) { ms[i] = 0.0; launches[i] = 0; }
    if (int rc = prepare()) return rc;
    prof_on = true;
    prof_ev.clear();
    int rc = enqueue_step(euler ? 1 : 0);
    prof_on = false;
    cudaError_t e = cudaStreamSynchronize(st);
    for (auto& pe : prof_ev) {
      float t = 0.f;
      if (rc == QG_OK && e == cudaSuccess && cudaEventElapsedTime(&t, pe.second.first, pe.second.second) == cudaSuccess &&
          pe.first < nclasses) {
        ms[pe.first] += t;
        launches[pe.first] += 1;
      }
      cudaEventDestroy(pe.second.first);
      cudaEventDestroy(pe.second.second);
    }
    prof_ev.clear();
    if (rc) return rc;
    QG_CK(e);
    return QG_OK;
  }

 protected:
  // Enqueue one step on st (no synchronisation; graph-capturable).
  int enqueue_step(int euler) {
    StepParams s = sp;
    s.euler = euler;
    if (s.use_dq) {
      if (int rc0 = pbeg(QG_K_DISSIPATION)) return rc0;
      k_dissipation<T><<<grid_for((long long)g.n3 * g.plane), 256, 0, st>>>(g, cfg.nuz, cfg.dz,
                                                                              euler ? F[F_Q] : F[F_QO], F[F_DQ]);
      QG_LAUNCHED();
      if (int rc0 = pend()) return rc0;
    }
    StateP<T> sptr = state_ptrs();
    const int do_psi = cfg.fixed_flow ? 0 : 1;
    const int do_A = (cfg.passive_scalar || !cfg.ybj_plus) ? 0 : 1;
    // A solves beside the q^w kernels (a second stream; serialised while
    // profiling so that every launch is timed alone)
    const int nbat = (g.n3 + Zb - 1) / Zb;
    const int L = prof_on ? 1 : std::min(lanes, nbat);   // serialised while profiling
    const bool split = kSolveOverlap && need_qw && do_psi && do_A && kSolveStore && vbuf && L == 1;
    const bool overlap = split && !prof_on;
    if (L > 1) {
      QG_CK(cudaEventRecord(ev_start, st));
      for (int i = 1; i < L; ++i) QG_CK(cudaStreamWaitEvent(lst[i], ev_start, 0));
    }
    const size_t slot = (size_t)Zb * kNScr * g.n * g.KXP;
    for (int z0 = 0, b = 0; z0 < g.n3; z0 += Zb, ++b) {
      const int zc = std::min(Zb, g.n3 - z0);
      const bool last = z0 + Zb >= g.n3;
      const int lane = b % L;
      cudaStream_t bs = lane == 0 ? st : lst[lane];
      C* Sb = S + lane * slot;
      QG_SWITCH_N(g.n, {
        // column tiles up to kx = K (the padding columns beyond K are never read)
        const dim3 gc((g.K + Tiles<T, NN>::CT) / Tiles<T, NN>::CT, zc), gr(g.n / Tiles<T, NN>::QRT, zc),
            grm(g.n / Tiles<T, NN>::RTM, zc);
        if (int rc0 = pbeg(QG_K_COL_INV, bs)) return rc0;
        C* Qb = Qp ? Qp + (size_t)z0 * kNQ * g.n * g.KXP : nullptr;
        k_col_inv<T, NN><<<gc, Tiles<T, NN>::CNT, sm_ci<NN, Tiles<T, NN>::CIP>(Tiles<T, NN>::CINF), bs>>>(g, z0, F[F_PSI], F[F_Q], F[F_BR], F[F_BI], Sb, tw,
                                                                Qb, Qb ? 1 : 0);
        QG_LAUNCHED();
        if (int rc0 = pend(bs)) return rc0;
        if (int rc0 = pbeg(QG_K_ROW_MAIN, bs)) return rc0;
        if constexpr (Tiles<T, NN>::RPRE) {
          const int items = zc * (NN / Tiles<T, NN>::RTM);
          k_row_main<T, NN><<<std::min(items, std::max(1, nsm * occ_rm / L)), kRowThreads, sm_rm<NN>(g.KXP), bs>>>(g, s, Sb, tw, items,
                                                                                                 wflag, Qb);
        } else {
          k_row_main<T, NN><<<grm, kRowThreads, sm_rm<NN>(g.KXP), bs>>>(g, s, Sb, tw, 0, wflag, Qb);
        }
        QG_LAUNCHED();
        if (int rc0 = pend(bs)) return rc0;
        {
          // asynchronous diagnostics of the previous state read B, A and psi:
          // the update waits for them (an external event node when captured)
          cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
          QG_CK(cudaStreamIsCapturing(bs, &cs));
          QG_CK(cudaStreamWaitEvent(bs, ev_diag, cs == cudaStreamCaptureStatusActive ? cudaEventWaitExternal : 0));
        }
        if (int rc0 = pbeg(QG_K_COL_UPDATE, bs)) return rc0;
        k_col_update<T, NN><<<gc, Tiles<T, NN>::CNT, UpdLay<T, NN>::bytes(), bs>>>(g, s, z0, sptr, e1, e2, e1w, e2w, Sb, tw,
                                                                need_qw ? 1 : 0, Qb);
        QG_LAUNCHED();
        if (int rc0 = pend(bs)) return rc0;
        if (overlap && last) {
          // B^{n+1} of every level is written: fork the A solves
          QG_CK(cudaEventRecord(ev_fork, bs));
          QG_CK(cudaStreamWaitEvent(st2, ev_fork, 0));
          if (int rc0 = solve_generic(nullptr, F[F_BR], F[F_BI], nullptr, F[F_AR], F[F_AI], 0, 1, st2, 0, -1, true))
            return rc0;
          QG_CK(cudaEventRecord(ev_join, st2));
        }
        if (need_qw) {
          if (int rc0 = pbeg(QG_K_ROW_QW, bs)) return rc0;
          if constexpr (Tiles<T, NN>::QPRE) {
            const int items = zc * (NN / Tiles<T, NN>::QRT);
            const int per_sm = (split && last) ? std::max(1, occ_rq - kQwReserve) : occ_rq;
            k_row_qw<T, NN><<<std::min(items, std::max(1, nsm * per_sm / L)), Tiles<T, NN>::QTHREADS, sm_rq<NN>(g.KXP), bs>>>(
                g, Sb, tw, items, wflag, Qb);
          } else {
            k_row_qw<T, NN><<<gr, Tiles<T, NN>::QTHREADS, sm_rq<NN>(g.KXP), bs>>>(g, Sb, tw, 0, wflag, Qb);
          }
          QG_LAUNCHED();
          if (int rc0 = pend(bs)) return rc0;
          if (int rc0 = pbeg(QG_K_COL_QW, bs)) return rc0;
          k_col_qw<T, NN><<<gc, Tiles<T, NN>::CNT, sm_ci<NN, Tiles<T, NN>::CQP>(2), bs>>>(g, s, z0, F[F_Q], F[F_QSTAR], Sb, tw, nflag);
          QG_LAUNCHED();
          if (int rc0 = pend(bs)) return rc0;
        }
      });
    }
    for (int i = 1; i < L; ++i) {
      QG_CK(cudaEventRecord(lev[i], lst[i]));
      QG_CK(cudaStreamWaitEvent(st, lev[i], 0));
    }
    if (int rc0 = pbeg(QG_K_SOLVE)) return rc0;
    int rc = launch_solve(need_qw ? F[F_QSTAR] : F[F_Q], do_psi, split ? 0 : do_A);
    if (rc) return rc;
    if (overlap) {
      QG_CK(cudaStreamWaitEvent(st, ev_join, 0));
    } else if (split) {
      if (int rc0 = pend()) return rc0;
      if (int rc0 = pbeg(QG_K_SOLVE_A)) return rc0;
      if ((rc = launch_solve(nullptr, 0, 1))) return rc;
    }
    if (!cfg.ybj_plus && !cfg.passive_scalar) {
      // regular YBJ: sumB on B^{n+1}, then A from the vertical integral (main_waqg.f90:449-460)
      k_ybj_A<T><<<(unsigned)((g.plane + 127) / 128), 128, 0, st>>>(g, cfg.dz, cfg.Bu, cfg.Ro, r2, F[F_BR], F[F_BI],
                                                                    sig[0], sig[1], F[F_AR], F[F_AI]);
      QG_LAUNCHED();
    }
    return pend();
  }

  int launch_solve(C* qs, int do_psi, int do_A) {
    return solve_generic(qs, F[F_BR], F[F_BI], F[F_PSI], F[F_AR], F[F_AI], do_psi, do_A, nullptr, 0, -1, true);
  }

  // the column solves of segments [seg0, seg0 + nsegs) (nsegs < 0: all)
  // retained: the outputs are resident fields (zeros off the retained
  // modes already), so only the retained columns are solved
  int solve_generic(const C* qs, const C* br, const C* bi, C* psi, C* ar, C* ai, int do_psi, int do_A,
                    cudaStream_t on = nullptr, int seg0 = 0, int nsegs = -1, bool retained = false) {
    if (!do_psi && !do_A) return QG_OK;
    if (!on) on = st;
    if (nsegs < 0) nsegs = members - seg0;
    const int* cl = retained ? cols_ret : cols_all;
    const int ncl = retained ? nret : (int)g.plane;
    double* const pcf = retained ? pcfac : nullptr;     // the per-column factors follow the retained list
    if (kSolveStore && vbuf) {
      const int nrec = (do_psi ? 2 : 0) + (do_A ? 4 : 0);   // recurrences per column
#define QG_SOLVE_ST(TCV, PCV)                                                                              \
  k_solve_st<T, TCV, PCV><<<dim3((unsigned)((ncl + TCV - 1) / TCV), nsegs), nrec * TCV,                 \
                            (size_t)g.nseg * 8, on>>>(                                                     \
      g, cfg.dz, cfg.Bu, tab_idx, fac_psi, fac_A, du, qs, br, bi, psi, ar, ai, do_psi, do_A, vbuf, pcf, seg0, cl, ncl)
      if (pcf) {
        if (solve_tc == 16) QG_SOLVE_ST(16, true);
        else if (solve_tc == 64) QG_SOLVE_ST(64, true);
        else QG_SOLVE_ST(32, true);
      } else {
        if (solve_tc == 16) QG_SOLVE_ST(16, false);
        else if (solve_tc == 64) QG_SOLVE_ST(64, false);
        else QG_SOLVE_ST(32, false);
      }
#undef QG_SOLVE_ST
      QG_LAUNCHED();
      return QG_OK;
    }
    k_solve<T><<<dim3((unsigned)((g.plane + kSolveTC - 1) / kSolveTC), nsegs), kSolveThreads, solve_smem(g.nseg), on>>>(g, cfg.dz, cfg.Bu, tab_idx, fac_psi, fac_A,
                                                                           du, qs, br, bi, psi, ar, ai, do_psi, do_A, seg0);
    QG_LAUNCHED();
    return QG_OK;
  }

  // Before a step (outside any stream capture): the kept B planes, when
  // they do not hold the transforms of the current B (new handle,
  // qg_set_state of BR or BI, initialisation), are computed from B.
  int prepare() override {
    if (!Qp || q_valid) return QG_OK;
    for (int z0 = 0; z0 < g.n3; z0 += Zb) {
      const int zc = std::min(Zb, g.n3 - z0);
      QG_SWITCH_N(g.n, {
        const dim3 gc((g.K + Tiles<T, NN>::CT) / Tiles<T, NN>::CT, zc);
        k_col_inv<T, NN><<<gc, Tiles<T, NN>::CNT, sm_ci<NN, Tiles<T, NN>::CIP>(Tiles<T, NN>::CINF), st>>>(g, z0, F[F_PSI], F[F_Q], F[F_BR], F[F_BI], S, tw,
                                                                Qp + (size_t)z0 * kNQ * g.n * g.KXP, 2);
        QG_LAUNCHED();
      });
    }
    q_valid = true;     // every step keeps them current from here on
    return QG_OK;
  }

  int run_step(int euler) {
    if (int rc = prepare()) return rc;
    if (!cfg.use_graphs) return enqueue_step(euler);
    if (!gexec[euler]) {
      cudaGraph_t graph = nullptr;
      QG_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      int rc = enqueue_step(euler);
      cudaError_t e = cudaStreamEndCapture(st, &graph);
      if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
      if (e != cudaSuccess) { err = std::string("graph capture: ") + cudaGetErrorString(e); return QG_ERR_CUDA; }
      e = cudaGraphInstantiate(&gexec[euler], graph, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) { err = std::string("graph instantiate: ") + cudaGetErrorString(e); return QG_ERR_CUDA; }
    }
    QG_CK(cudaGraphLaunch(gexec[euler], st));
    return QG_OK;
  }

  // ---- dense drop-in plumbing ---------------------------------------------
  size_t dense_bytes(int nz) const { return (size_t)nz * g.n * (g.n / 2 + 1) * sizeof(double2); }
  int iktxP() const { const int ct = Tile<T>::CT; return ((g.n / 2 + 1 + ct - 1) / ct) * ct; }

  int prep_dense(int nz) {
    if (nz <= 0) { err = "nz must be positive"; return QG_ERR_ARG; }
    if (nz <= dense_nz) return QG_OK;
    QG_CK(cudaStreamSynchronize(st));
    for (auto& p : D) if (p) { cudaFree(p); p = nullptr; }
    for (auto& p : P) if (p) { cudaFree(p); p = nullptr; }
    if (W) { cudaFree(W); W = nullptr; }
    if (dstage) { cudaFree(dstage); dstage = nullptr; }
    for (auto& p : D) QG_CK(cudaMalloc(&p, dense_bytes(nz)));
    for (auto& p : P) QG_CK(cudaMalloc(&p, (size_t)nz * g.n * g.n * sizeof(T)));
    QG_CK(cudaMalloc(&W, (size_t)nz * g.n * iktxP() * sizeof(C)));
    QG_CK(cudaMalloc(&dstage, (size_t)nz * g.n * (g.n + 2) * sizeof(double)));
    dense_nz = nz;
    return QG_OK;
  }

  int d_c2r(const double2* spec, T* phys, int nz) {
    const int CT = Tile<T>::CT;
    QG_SWITCH_N(g.n, {
      k_dcol_inv<T, NN><<<dim3(iktxP() / CT, nz), kThreads, sm_colinv(), st>>>(iktxP(), spec, W, tw);
      QG_LAUNCHED();
      k_drow_c2r<T, NN><<<dim3(g.n / 2, nz), kThreads, sm_drow(), st>>>(iktxP(), W, phys, tw);
      QG_LAUNCHED();
    });
    return QG_OK;
  }

  int d_r2c(const T* phys, double2* spec, int nz) {
    const int CT = Tile<T>::CT;
    QG_SWITCH_N(g.n, {
      k_drow_r2c<T, NN><<<dim3(g.n / 2, nz), kThreads, sm_drow(), st>>>(iktxP(), phys, W, tw);
      QG_LAUNCHED();
      k_dcol_fwd<T, NN><<<dim3(iktxP() / CT, nz), kThreads, sm_colinv(), st>>>(iktxP(), W, spec, tw);
      QG_LAUNCHED();
    });
    return QG_OK;
  }

  int ensure_tmp() {
    const size_t fbytes = (size_t)g.n3 * g.plane * sizeof(C);
    for (auto& p : tmpF) if (!p) { QG_CK(cudaMalloc(&p, fbytes)); QG_CK(cudaMemsetAsync(p, 0, fbytes, st)); }
    return QG_OK;
  }

  int upload_compact(const double* kvar, C* dst) {
    const size_t bytes = dense_bytes(g.n3);
    int rc = ensure(&stage, &stage_bytes, bytes);
    if (rc) return rc;
    QG_CK(cudaMemcpyAsync(stage, kvar, bytes, cudaMemcpyDefault, st));
    k_dense_to_compact<T><<<grid_for((long long)g.n3 * g.plane), 256, 0, st>>>(g, 0, g.n3, (const double2*)stage, dst);
    QG_LAUNCHED();
    return QG_OK;
  }

  int download_compact(const C* src, double* kvar, int mode) {
    const size_t bytes = dense_bytes(g.n3);
    int rc = ensure(&stage, &stage_bytes, bytes);
    if (rc) return rc;
    k_compact_to_dense<T><<<grid_for((long long)g.n3 * g.n * (g.n / 2 + 1)), 256, 0, st>>>(g, 0, g.n3, src,
                                                                                           (double2*)stage, mode, cfg.dz);
    QG_LAUNCHED();
    QG_CK(cudaMemcpyAsync(kvar, stage, bytes, cudaMemcpyDefault, st));
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }
};

}  // namespace qg
