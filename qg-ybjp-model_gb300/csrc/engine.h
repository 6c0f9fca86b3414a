// Host-side engine interface shared by the C-ABI (capi.cu) and the two
// precision instantiations (engine_fp32.cu, engine_fp64.cu).
#pragma once
#include <string>
#include <vector>
#include "../../include/qgybj.h"

namespace qg {

// Tables built once on the host from the configuration (init.f90:17-264).
struct HostTables {
  int n, n3, K, KX, KY, KXP, kmax2;
  // a stack of `members` ensemble members of nseg levels each (n3 = members
  // * nseg): the per-level tables below (du, cu, cl, r2, factors) describe
  // one member's levels, the integrating factors are [members][plane] and
  // mpar holds {delt, 0.5/(Bu Ro), Ro, W2F} per member.  One run: nseg = n3,
  // members = 1, mpar empty.
  int nseg = 0, members = 1;
  std::vector<double> mpar;
  long long plane;
  std::vector<double> e1, e2, e1w, e2w;     // [plane] integrating factors
  std::vector<double> tw;                   // [2n] cos, sin of -2 pi m / n interleaved
  std::vector<int> tab_idx;                 // [plane] distinct-kh2 row, -1 = inactive column
  std::vector<double> fac_psi, fac_A;       // [ndistinct][n3][2] {f_i, 1/d'_i}
  int ndistinct;
  std::vector<double> du;                   // [n3] upper diagonal rho_ut a / rho_st
  std::vector<double> cu, cl;               // [n3] init_q coefficients of psi(z+1), psi(z-1)
  std::vector<double> r2;                   // [n3] N^2 at za(iz)
  bool rho_unit = true;                     // rho_ut = rho_st = 1: symmetric vertical operators
  // omega equation (elliptic.f90:463-567), unstaggered levels iz = 0..n3-2:
  // d = -(om_t1 + dz^2 kh2 / a), upper om_du, lower om_dl; om_a = a_ell_ut
  std::vector<double> om_t1, om_du, om_dl, om_a;
};

struct EngineBase {
  virtual ~EngineBase() {}
  std::string err;
  virtual int init(const qg_config& cfg, const HostTables& t) = 0;
  virtual int set_state(int field, const double* kvar, int level0, int nlev) = 0;
  virtual int get_state(int field, double* kvar, int level0, int nlev) = 0;
  virtual int init_state(int apply_sumB, int q_from_psi) = 0;
  // the same on the members of levels [z0, z0 + nz) of a stack, and the
  // release of what the initialisation kept (see Engine::init_state_range)
  virtual int init_state_range(int z0, int nz, int apply_sumB, int q_from_psi) = 0;
  virtual void release_init_buffers() = 0;
  // work that must precede a step and cannot be captured with it (launched
  // on the engine's stream); run before capturing enqueue() into a graph
  virtual int prepare() = 0;
  // levels per member and members of this engine (a stack holds several)
  virtual int levels_per_member() const = 0;
  virtual int member_count() const = 0;
  virtual int step(int euler) = 0;
  virtual int steps_async(int nsteps, int euler) = 0;
  virtual int synchronize() = 0;
  // status flags raised on the device since the last check (the stream must
  // have drained): QG_ERR_TIMEOUT, QG_ERR_NONFINITE or QG_OK
  virtual int check_waits() = 0;
  // runs k_wait_expire on the stream; QG_ERR_TIMEOUT expected
  virtual int selftest_wait() = 0;
  virtual void* stream() = 0;
  virtual int diagnostics(qg_energy* out) = 0;
  virtual int diagnostics_range(int z0, int nz, qg_energy* out) = 0;
  virtual int diagnostics_async() = 0;
  virtual int diagnostics_wait(qg_energy* out) = 0;
  virtual int profile_step(int euler, double* ms, int* launches, int nclasses) = 0;
  // enqueue one step on the engine's stream without synchronising or graph
  // replay (used when an ensemble captures its members into one graph)
  virtual int enqueue(int euler) = 0;
  // levels per phase-A batch: current value and re-selection (drops graphs)
  virtual int batch_levels() const = 0;
  virtual int set_batch_levels(int zb) = 0;
  // phase-A batches in flight at once: current value and re-selection (drops graphs)
  virtual int batch_lanes() const = 0;
  virtual int set_batch_lanes(int lanes) = 0;
  // columns per CTA of the column solves (16, 32, 64): current value and re-selection
  virtual int solve_columns() const = 0;
  virtual int set_solve_columns(int tc) = 0;
  // adjoint (FP64 engines only)
  virtual int adjoint_run(const double* q0, const double* BR0, const double* BI0, int nsteps, int ckpt_every,
                          int objective, double* J, double* gq, double* gR, double* gI) {
    err = "the adjoint needs an FP64 handle";
    return QG_ERR_UNSUPPORTED;
  }
  virtual int adjoint_step(int euler, const double* const* X, const double* const* lX, double* const* Xn,
                           double* const* lXo) {
    err = "the adjoint needs an FP64 handle";
    return QG_ERR_UNSUPPORTED;
  }
  // real-space FP32 output of the dumps: which = 0 psi (out0), 1 B, 2 LA (out0 = R, out1 = I)
  virtual int dump_real(int which, float* out0, float* out1, int level0, int nlev, double s1, double s2) = 0;
  // omega equation: right-hand side (derivatives.f90:1469-1586), solve
  // (elliptic.f90:463-567), and w from the resident psi
  virtual int omega_eqn_rhs(const double* psik, double* rhs) = 0;
  virtual int omega_equation(const double* rhs, double* wk) = 0;
  virtual int omega_from_state(double* wk) = 0;
  virtual int fft_r2c(const double* rvar, double* kvar, int nz) = 0;
  virtual int fft_c2r(const double* kvar, double* rvar, int nz) = 0;
  virtual int convol_waqg(const double* uk, const double* vk, const double* qk, const double* BRk, const double* BIk,
                          double* nqk, double* nBRk, double* nBIk, int nz) = 0;
  virtual int refraction_waqg(const double* BRk, const double* BIk, const double* psik, double* rBRk, double* rBIk,
                              int nz) = 0;
  virtual int compute_qw(const double* BRk, const double* BIk, double* qwk, int nz) = 0;
  virtual int psi_solver(const double* qstar, double* psik) = 0;
  virtual int A_solver(const double* bk, double* ak, double* ck) = 0;
};

EngineBase* make_engine_fp32();
EngineBase* make_engine_fp64();

bool supported_n(int n);

// Error text of calls made without a handle (qg_create, qg_fft_c2r_noalloc),
// returned by qg_last_error(NULL) on the calling thread.
void set_handleless_error(const std::string& msg);
// mismatches of the integer FP32<->FP64 conversions of the mixed solve
// against the hardware conversions (engine_fp32.cu)
int selftest_conversions(int device, long long* bad32, long long* bad64, std::string& err);

}  // namespace qg
