// C-ABI entry points (include/qgybj.h) and the host-side tables built once per
// handle: dealiasing mask (init.f90:17-80), integrating factors
// (main_waqg.f90:246-247), base state (init.f90:177-264) and the DGTSV
// elimination factors of the two vertical operators (elliptic.f90:177-189).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#include "engine.h"

struct qg_handle {
  qg::EngineBase* eng = nullptr;
  std::string err;
  // a member of an ensemble stack: levels [z0, z0 + nz) of an engine that the
  // ensemble owns (state I/O, initialisation and diagnostics of that member)
  bool view = false;
  int z0 = 0, nz = 0;
};

namespace {
thread_local std::string g_create_err;

int fail(qg_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg; else g_create_err = msg;
  return code;
}

// Correctly rounded float32 of a non-negative integer (nearest-even): the
// value of the default-REAL power (1.*k)**(2.*ilap) of the reference.
float f32_round(unsigned __int128 m) {
  int bits = 0;
  for (unsigned __int128 t = m; t; t >>= 1) ++bits;
  if (bits <= 24) return (float)(unsigned long long)m;
  const int e = bits - 24;
  unsigned __int128 q = m >> e;
  const unsigned __int128 r = m - (q << e);
  const unsigned __int128 half = (unsigned __int128)1 << (e - 1);
  if (r > half || (r == half && (q & 1))) q += 1;
  return std::ldexp((float)(unsigned long long)q, e);
}

float powk(int k, int ex) {
  unsigned __int128 p = 1;
  for (int i = 0; i < ex; ++i) p *= (unsigned __int128)(unsigned)k;
  return f32_round(p);
}

bool finite_all(const double* a, int n) {
  for (int i = 0; i < n; ++i) if (!std::isfinite(a[i])) return false;
  return true;
}

int build_tables(const qg_config& c, qg::HostTables& t, std::string& err) {
  const int n = c.n1, n3 = c.n3;
  const int iktx = n / 2 + 1, ikty = n, kty = n / 2;
  // --- mask L exactly as init_arrays (init.f90:32-80) ---------------------
  const double twopi = 4.0 * std::asin(1.0);
  const float thr_f = (float)(int)((float)n / 3.0f + 0.5f) - 0.5f;
  const double thr = (double)thr_f;
  std::vector<int> kya(ikty);
  for (int iky = 1; iky <= ikty; ++iky) {
    int jj = iky - 1;
    if (iky > kty) jj -= 2 * kty;
    if (iky == kty + 1) jj = 0;
    if (iky > 2 * kty) jj = 0;
    kya[iky - 1] = jj;
  }
  std::vector<unsigned char> L((size_t)ikty * iktx);
  int kmax2 = -1, K = 0;
  for (int iky = 0; iky < ikty; ++iky) {
    for (int kx = 0; kx < iktx; ++kx) {
      const int ky = kya[iky];
      const double kh = (double)std::sqrt((float)(kx * kx + ky * ky));
      int l = 1;
      if (iky + 1 == kty + 1) l = 0;
      else if (kx == 0 && ky < 0) l = 0;
      else if ((kh * twopi / twopi) > thr) l = 0;
      L[(size_t)iky * iktx + kx] = (unsigned char)l;
      if (l) { kmax2 = std::max(kmax2, kx * kx + ky * ky); K = std::max(K, kx); }
    }
  }
  // the compact layout relies on L being the disk kx^2+ky^2 <= kmax2 (minus kx=0,ky<0)
  for (int iky = 0; iky < ikty; ++iky)
    for (int kx = 0; kx < iktx; ++kx) {
      const int ky = kya[iky];
      const bool disk = iky != kty && kx * kx + ky * ky <= kmax2 && !(kx == 0 && ky < 0);
      if (disk != (bool)L[(size_t)iky * iktx + kx]) { err = "dealiasing mask is not a disk"; return QG_ERR_UNSUPPORTED; }
    }
  t.n = n; t.n3 = n3; t.K = K; t.KX = K + 1; t.KY = 2 * K + 1;
  t.KXP = ((K + 1 + 7) / 8) * 8;
  t.kmax2 = kmax2;
  t.plane = (long long)t.KY * t.KXP;
  // --- integrating factors (main_waqg.f90:246-247, 371-372) ---------------
  t.e1.assign(t.plane, 0.0); t.e2.assign(t.plane, 0.0); t.e1w.assign(t.plane, 0.0); t.e2w.assign(t.plane, 0.0);
  for (int r = 0; r < t.KY; ++r) {
    const int ky = r <= K ? r : r - t.KY;
    const int aky = ky < 0 ? -ky : ky;
    for (int kx = 0; kx <= K; ++kx) {
      const float s1 = powk(kx, 2 * c.ilap1) + powk(aky, 2 * c.ilap1);
      const float s2 = powk(kx, 2 * c.ilap2) + powk(aky, 2 * c.ilap2);
      const float s1w = powk(kx, 2 * c.ilap1w) + powk(aky, 2 * c.ilap1w);
      const float s2w = powk(kx, 2 * c.ilap2w) + powk(aky, 2 * c.ilap2w);
      const double IF = c.delt * (c.nuh1 * (double)s1 + c.nuh2 * (double)s2);
      const double IFw = c.delt * (c.nuh1w * (double)s1w + c.nuh2w * (double)s2w);
      const long long m = (long long)r * t.KXP + kx;
      t.e1[m] = std::exp(-IF); t.e2[m] = std::exp(-2 * IF);
      t.e1w[m] = std::exp(-IFw); t.e2w[m] = std::exp(-2 * IFw);
    }
  }
  // --- twiddles W_n^m = exp(-2 pi i m/n) ---------------------------------
  t.tw.assign(2 * (size_t)n, 0.0);
  for (int m = 0; m < n; ++m) {
    double cs, sn;
    if ((4 * m) % n == 0) {
      const int q = (4 * m) / n;
      const double C4[4] = {1, 0, -1, 0}, S4[4] = {0, 1, 0, -1};
      cs = C4[q]; sn = S4[q];
    } else {
      const double th = twopi * (double)m / (double)n;
      cs = std::cos(th); sn = std::sin(th);
    }
    t.tw[2 * m] = cs; t.tw[2 * m + 1] = -sn;
  }
  // --- base state and vertical operators ---------------------------------
  std::vector<double> a(c.a_ell_ut, c.a_ell_ut + n3), ru(n3, 1.0), rs(n3, 1.0);
  if (c.rho_ut) ru.assign(c.rho_ut, c.rho_ut + n3);
  if (c.rho_st) rs.assign(c.rho_st, c.rho_st + n3);
  t.om_t1.assign(n3, 0.0); t.om_du.assign(n3, 0.0); t.om_dl.assign(n3, 0.0); t.om_a = a;
  for (int i = 0; i + 1 < n3; ++i) {
    t.om_t1[i] = (ru[i] * (rs[i + 1] + rs[i])) / (rs[i + 1] * rs[i]);
    if (i + 2 < n3) { t.om_du[i] = ru[i + 1] / rs[i + 1]; t.om_dl[i] = ru[i] / rs[i + 1]; }
  }
  t.rho_unit = true;
  for (int i = 0; i < n3; ++i) t.rho_unit = t.rho_unit && ru[i] == 1.0 && rs[i] == 1.0;
  t.du.assign(n3, 0.0); t.cu.assign(n3, 0.0); t.cl.assign(n3, 0.0); t.r2.assign(n3, 0.0);
  for (int i = 0; i < n3; ++i) {
    if (i < n3 - 1) t.du[i] = ru[i] * a[i] / rs[i];
    t.cu[i] = i < n3 - 1 ? ru[i] * a[i] / rs[i] : 0.0;
    t.cl[i] = i > 0 ? ru[i - 1] * a[i - 1] / rs[i] : 0.0;
    t.r2[i] = c.r_2ut ? c.r_2ut[i] : c.Bu / a[i];
  }
  // distinct kh^2 of active columns (L=1, kh^2 != 0), elliptic.f90:171
  std::map<int, int> idx;
  for (int r = 0; r < t.KY; ++r) {
    const int ky = r <= K ? r : r - t.KY;
    for (int kx = 0; kx <= K; ++kx) {
      const int kh2 = kx * kx + ky * ky;
      if (kh2 != 0 && kh2 <= kmax2 && !(kx == 0 && ky < 0)) idx[kh2] = 0;
    }
  }
  int nd = 0;
  for (auto& kv : idx) kv.second = nd++;
  t.ndistinct = nd;
  t.tab_idx.assign(t.plane, -1);
  for (int r = 0; r < t.KY; ++r) {
    const int ky = r <= K ? r : r - t.KY;
    for (int kx = 0; kx <= K; ++kx) {
      const int kh2 = kx * kx + ky * ky;
      if (kh2 != 0 && kh2 <= kmax2 && !(kx == 0 && ky < 0)) t.tab_idx[(size_t)r * t.KXP + kx] = idx[kh2];
    }
  }
  t.fac_psi.assign((size_t)nd * n3 * 4, 0.0);
  t.fac_A.assign((size_t)nd * n3 * 4, 0.0);
  std::vector<double> d(n3), dl(n3), du(n3);
  // FP64 path: {f_i, d'_i, 0, 0} for DGTSV's exact arithmetic;
  // mixed path: {f_i, s/d'_i, u_i/d'_i, 0} with s the RHS scaling of the operator
  const bool exact = c.precision == QG_PREC_FP64;
  for (auto& kv : idx) {
    for (int op = 0; op < 2; ++op) {
      const double kdz = op == 0 ? (double)kv.first * c.dz * c.dz : (double)kv.first * c.dz * c.dz / 4.0;
      for (int i = 0; i < n3; ++i) {
        if (i == 0) {
          d[i] = -(ru[0] * a[0] / rs[0] + kdz);
          du[i] = ru[0] * a[0] / rs[0];
        } else if (i == n3 - 1) {
          d[i] = -(ru[i - 1] * a[i - 1] / rs[i] + kdz);
          dl[i - 1] = ru[i - 1] * a[i - 1] / rs[i];
        } else {
          d[i] = -((ru[i] * a[i] + ru[i - 1] * a[i - 1]) / rs[i] + kdz);
          du[i] = ru[i] * a[i] / rs[i];
          dl[i - 1] = ru[i - 1] * a[i - 1] / rs[i];
        }
      }
      // DGTSV elimination order without row interchanges
      double* out = (op == 0 ? t.fac_psi.data() : t.fac_A.data()) + (size_t)kv.second * n3 * 4;
      const double s = op == 0 ? c.dz * c.dz : c.dz * c.dz * c.Bu;
      double dp = d[0];
      for (int i = 0; i < n3 - 1; ++i) {
        if (dp == 0.0) { err = "zero pivot in tridiagonal factorisation (kh2=" + std::to_string(kv.first) + ")"; return QG_ERR_PIVOT; }
        if (std::fabs(dp) < std::fabs(dl[i])) {
          err = "tridiagonal factorisation needs a row interchange (kh2=" + std::to_string(kv.first) + ")";
          return QG_ERR_PIVOT;
        }
        const double f = dl[i] / dp;
        out[4 * i] = f;
        out[4 * i + 1] = exact ? dp : s / dp;
        out[4 * i + 2] = exact ? 0.0 : du[i] / dp;
        dp = d[i + 1] - f * du[i];
      }
      if (dp == 0.0 || !std::isfinite(dp)) { err = "zero pivot in tridiagonal factorisation"; return QG_ERR_PIVOT; }
      out[4 * (n3 - 1)] = 0.0;
      out[4 * (n3 - 1) + 1] = exact ? dp : s / dp;
      out[4 * (n3 - 1) + 2] = 0.0;
    }
  }
  return QG_OK;
}

}  // namespace

namespace qg {
void set_handleless_error(const std::string& msg) { g_create_err = msg; }
bool supported_n(int n) { return n == 16 || n == 32 || n == 64 || n == 128 || n == 256 || n == 512 || n == 1024; }
}  // namespace qg

extern "C" {

int qg_config_defaults(qg_config* c) {
  if (!c) return QG_ERR_ARG;
  std::memset(c, 0, sizeof *c);
  c->precision = QG_PREC_MIXED;
  c->ybj_plus = 1;
  c->inviscid = 1;
  c->ilap1 = c->ilap1w = 2;
  c->ilap2 = c->ilap2w = 6;
  c->use_graphs = 1;
  c->solve_columns = 0;
  return QG_OK;
}

// the checks of qg_create; QG_OK or the status with its text in g_create_err
static int validate_config(const qg_config& c) {
  if (c.n1 != c.n2) return fail(nullptr, QG_ERR_UNSUPPORTED, "n1 must equal n2");
  if (!qg::supported_n(c.n1)) return fail(nullptr, QG_ERR_UNSUPPORTED, "n1 must be a power of two in [16,1024]");
  if (c.n3 < 2) return fail(nullptr, QG_ERR_ARG, "n3 must be >= 2");
  if (c.n3 > 1024) return fail(nullptr, QG_ERR_UNSUPPORTED, "n3 must be <= 1024 (solve checkpoints in shared memory)");
  if (c.precision != QG_PREC_FP64 && c.precision != QG_PREC_MIXED) return fail(nullptr, QG_ERR_ARG, "bad precision");
  if (c.ybj_plus != 0 && c.ybj_plus != 1) return fail(nullptr, QG_ERR_ARG, "ybj_plus must be 0 or 1");
  if (!c.a_ell_ut) return fail(nullptr, QG_ERR_ARG, "a_ell_ut is required");
  if (!(c.dz > 0) || !(c.Bu > 0) || !(c.Ro > 0)) return fail(nullptr, QG_ERR_ARG, "dz, Bu and Ro must be positive");
  const double sc[] = {c.dz, c.Bu, c.Ro, c.W2F, c.delt, c.gamma, c.nuh1, c.nuh2, c.nuh1w, c.nuh2w, c.nuz};
  if (!finite_all(sc, (int)(sizeof sc / sizeof sc[0])) || !finite_all(c.a_ell_ut, c.n3) ||
      (c.rho_ut && !finite_all(c.rho_ut, c.n3)) || (c.rho_st && !finite_all(c.rho_st, c.n3)) ||
      (c.r_2ut && !finite_all(c.r_2ut, c.n3)))
    return fail(nullptr, QG_ERR_NONFINITE, "non-finite configuration value");
  if (c.ilap1 < 0 || c.ilap2 < 0 || c.ilap1w < 0 || c.ilap2w < 0 || c.ilap1 > 9 || c.ilap2 > 9 || c.ilap1w > 9 ||
      c.ilap2w > 9)
    return fail(nullptr, QG_ERR_ARG, "ilap out of range [0,9]");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || c.device < 0 || c.device >= ndev)
    return fail(nullptr, QG_ERR_CUDA, "no CUDA device with that ordinal");
  return QG_OK;
}

// a handle whose engine is built from c and the tables t
static int create_from_tables(const qg_config& c, const qg::HostTables& t, qg_handle** out) {
  qg_handle* h = new qg_handle();
  h->eng = c.precision == QG_PREC_FP64 ? qg::make_engine_fp64() : qg::make_engine_fp32();
  const int rc = h->eng->init(c, t);
  if (rc) {
    g_create_err = h->eng->err;
    delete h->eng;
    delete h;
    return rc;
  }
  *out = h;
  return QG_OK;
}

int qg_create(const qg_config* cfg, qg_handle** out) {
  if (!cfg || !out) return fail(nullptr, QG_ERR_ARG, "null argument");
  *out = nullptr;
  int rc = validate_config(*cfg);
  if (rc) return rc;
  qg::HostTables t;
  std::string err;
  rc = build_tables(*cfg, t, err);
  if (rc) return fail(nullptr, rc, err);
  return create_from_tables(*cfg, t, out);
}

int qg_destroy(qg_handle* h) {
  if (!h) return QG_ERR_ARG;
  if (!h->view) delete h->eng;    // a member view leaves its stack to the ensemble
  delete h;
  return QG_OK;
}

int qg_selftest_conversions(int device, long long* mismatches32, long long* mismatches64) {
  if (!mismatches32 || !mismatches64) return fail(nullptr, QG_ERR_ARG, "qg_selftest_conversions: null pointer");
  std::string e;
  const int rc = qg::selftest_conversions(device, mismatches32, mismatches64, e);
  if (rc) return fail(nullptr, rc, e);
  return QG_OK;
}

const char* qg_last_error(const qg_handle* h) {
  if (!h) return g_create_err.c_str();
  if (!h->err.empty()) return h->err.c_str();
  return h->eng ? h->eng->err.c_str() : "";
}

#define QG_ENTRY(h)                       \
  if (!(h) || !(h)->eng) return QG_ERR_ARG; \
  (h)->err.clear();
// calls that act on a whole run: refused on a member of an ensemble stack
#define QG_WHOLE(h)                                                                                     \
  if ((h)->view)                                                                                        \
    return fail(h, QG_ERR_UNSUPPORTED, "this call acts on a whole run; the handle is a member of an "   \
                                       "ensemble stack (step and solve it through the ensemble)");
// level range of a member view: [level0, level0 + nlev) of the member, shifted to the stack
#define QG_LEVELS(h, level0, nlev)                                                                      \
  if ((h)->view) {                                                                                      \
    if ((level0) < 0 || (nlev) <= 0 || (level0) + (nlev) > (h)->nz)                                      \
      return fail(h, QG_ERR_ARG, "bad level range for this member");                                    \
    (level0) += (h)->z0;                                                                                \
  }

static int fwd(qg_handle* h, int rc) {
  if (rc && h->err.empty()) h->err = h->eng->err;
  return rc;
}

int qg_set_state(qg_handle* h, int field, const double* kvar, int level0, int nlev) {
  QG_ENTRY(h);
  QG_LEVELS(h, level0, nlev);
  return fwd(h, h->eng->set_state(field, kvar, level0, nlev));
}
int qg_get_state(qg_handle* h, int field, double* kvar, int level0, int nlev) {
  QG_ENTRY(h);
  QG_LEVELS(h, level0, nlev);
  return fwd(h, h->eng->get_state(field, kvar, level0, nlev));
}
int qg_init_state(qg_handle* h, int apply_sumB, int q_from_psi) {
  QG_ENTRY(h);
  if (h->view) return fwd(h, h->eng->init_state_range(h->z0, h->nz, apply_sumB, q_from_psi));
  return fwd(h, h->eng->init_state(apply_sumB, q_from_psi));
}
int qg_step(qg_handle* h, int euler_first) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  return fwd(h, h->eng->step(euler_first));
}
int qg_steps_async(qg_handle* h, int nsteps, int euler_first) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (nsteps < 0) return fail(h, QG_ERR_ARG, "nsteps must be >= 0");
  return fwd(h, h->eng->steps_async(nsteps, euler_first));
}
int qg_synchronize(qg_handle* h) {
  QG_ENTRY(h);
  return fwd(h, h->eng->synchronize());
}
int qg_selftest_wait(qg_handle* h) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  return fwd(h, h->eng->selftest_wait());
}
int qg_get_stream(qg_handle* h, void** stream) {
  QG_ENTRY(h);
  if (!stream) return fail(h, QG_ERR_ARG, "null stream pointer");
  *stream = h->eng->stream();
  return QG_OK;
}
int qg_diagnostics_fp64(qg_handle* h, qg_energy* out) {
  QG_ENTRY(h);
  if (!out) return fail(h, QG_ERR_ARG, "null output");
  if (h->view) return fwd(h, h->eng->diagnostics_range(h->z0, h->nz, out));
  return fwd(h, h->eng->diagnostics(out));
}
int qg_diagnostics_fp64_async(qg_handle* h) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  return fwd(h, h->eng->diagnostics_async());
}
int qg_diagnostics_fp64_wait(qg_handle* h, qg_energy* out) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (!out) return fail(h, QG_ERR_ARG, "null output");
  return fwd(h, h->eng->diagnostics_wait(out));
}
int qg_profile_step(qg_handle* h, int euler_first, double* ms, int* launches, int nclasses) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (!ms || !launches || nclasses <= 0) return fail(h, QG_ERR_ARG, "null output or nclasses <= 0");
  return fwd(h, h->eng->profile_step(euler_first, ms, launches, nclasses));
}
int qg_adjoint_run(qg_handle* h, const double* q0, const double* BR0, const double* BI0, int nsteps, int ckpt_every,
                   int objective, double* J, double* gq, double* gR, double* gI) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (!q0 || !BR0 || !BI0 || !J || nsteps < 1 || ckpt_every < 1) return fail(h, QG_ERR_ARG, "qg_adjoint_run: bad arguments");
  if (objective != QG_OBJ_LA_SUBVOLUME) return fail(h, QG_ERR_ARG, "qg_adjoint_run: unknown objective");
  if ((gq || gR || gI) && !(gq && gR && gI)) return fail(h, QG_ERR_ARG, "qg_adjoint_run: pass all three gradients or none");
  return fwd(h, h->eng->adjoint_run(q0, BR0, BI0, nsteps, ckpt_every, objective, J, gq, gR, gI));
}
int qg_adjoint_step(qg_handle* h, int euler_first, const double* const* X, const double* const* lX, double* const* Xn,
                    double* const* lXo) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (!X) return fail(h, QG_ERR_ARG, "qg_adjoint_step: null state");
  for (int i = 0; i < 6; ++i) if (!X[i]) return fail(h, QG_ERR_ARG, "qg_adjoint_step: null state field");
  if (lXo && !lX) return fail(h, QG_ERR_ARG, "qg_adjoint_step: lX_out needs lX");
  return fwd(h, h->eng->adjoint_step(euler_first, X, lX, Xn, lXo));
}
int qg_fft_r2c(qg_handle* h, const double* rvar, double* kvar, int nz) {
  QG_ENTRY(h);
  if (!rvar || !kvar) return fail(h, QG_ERR_ARG, "null pointer");
  return fwd(h, h->eng->fft_r2c(rvar, kvar, nz));
}
int qg_fft_c2r(qg_handle* h, const double* kvar, double* rvar, int nz) {
  QG_ENTRY(h);
  if (!rvar || !kvar) return fail(h, QG_ERR_ARG, "null pointer");
  return fwd(h, h->eng->fft_c2r(kvar, rvar, nz));
}
int qg_convol_waqg(qg_handle* h, const double* uk, const double* vk, const double* qk, const double* BRk,
                   const double* BIk, double* nqk, double* nBRk, double* nBIk, int nz) {
  QG_ENTRY(h);
  if (!uk || !vk || !qk || !BRk || !BIk || !nqk || !nBRk || !nBIk) return fail(h, QG_ERR_ARG, "null pointer");
  return fwd(h, h->eng->convol_waqg(uk, vk, qk, BRk, BIk, nqk, nBRk, nBIk, nz));
}
int qg_refraction_waqg(qg_handle* h, const double* BRk, const double* BIk, const double* psik, double* rBRk,
                       double* rBIk, int nz) {
  QG_ENTRY(h);
  if (!BRk || !BIk || !psik || !rBRk || !rBIk) return fail(h, QG_ERR_ARG, "null pointer");
  return fwd(h, h->eng->refraction_waqg(BRk, BIk, psik, rBRk, rBIk, nz));
}
int qg_compute_qw(qg_handle* h, const double* BRk, const double* BIk, double* qwk, int nz) {
  QG_ENTRY(h);
  if (!BRk || !BIk || !qwk) return fail(h, QG_ERR_ARG, "null pointer");
  return fwd(h, h->eng->compute_qw(BRk, BIk, qwk, nz));
}
int qg_dump_psi(qg_handle* h, float* out, int level0, int nlev, double U_scale, double L_scale) {
  QG_ENTRY(h);
  QG_LEVELS(h, level0, nlev);
  if (!out) return fail(h, QG_ERR_ARG, "qg_dump_psi: null pointer");
  return fwd(h, h->eng->dump_real(0, out, nullptr, level0, nlev, U_scale, L_scale));
}
int qg_dump_la(qg_handle* h, float* outR, float* outI, int level0, int nlev, double Uw_scale, int la) {
  QG_ENTRY(h);
  QG_LEVELS(h, level0, nlev);
  if (!outR || !outI) return fail(h, QG_ERR_ARG, "qg_dump_la: null pointer");
  return fwd(h, h->eng->dump_real(la ? 2 : 1, outR, outI, level0, nlev, Uw_scale, 1.0));
}
int qg_omega_eqn_rhs(qg_handle* h, const double* psik, double* rhs) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (!psik || !rhs) return fail(h, QG_ERR_ARG, "qg_omega_eqn_rhs: null pointer");
  return fwd(h, h->eng->omega_eqn_rhs(psik, rhs));
}
int qg_omega_equation(qg_handle* h, const double* rhs, double* wk) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (!rhs || !wk) return fail(h, QG_ERR_ARG, "qg_omega_equation: null pointer");
  return fwd(h, h->eng->omega_equation(rhs, wk));
}
int qg_omega(qg_handle* h, double* wk) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (!wk) return fail(h, QG_ERR_ARG, "qg_omega: null pointer");
  return fwd(h, h->eng->omega_from_state(wk));
}
int qg_psi_solver(qg_handle* h, const double* qstar, double* psik) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (!qstar || !psik) return fail(h, QG_ERR_ARG, "null pointer");
  return fwd(h, h->eng->psi_solver(qstar, psik));
}
int qg_A_solver_ybj_plus(qg_handle* h, const double* bk, double* ak, double* ck) {
  QG_ENTRY(h);
  QG_WHOLE(h);
  if (!bk || !ak) return fail(h, QG_ERR_ARG, "null pointer");
  return fwd(h, h->eng->A_solver(bk, ak, ck));
}

// ---- ensembles ----------------------------------------------------------------
// Members of one shape, precision, physics switches and vertical operator
// are stacked in z into one engine (a "stack": each member a segment of
// n3 levels, with its own time step, Rossby number, W2F and integrating
// factors), so that every kernel of the step runs once per stack instead of
// once per member.  The step graph advances the runs: stacks and the
// members that share their shape with no other.
struct qg_ensemble {
  std::vector<qg_handle*> members;    // per member: its own handle, or a view of its stack
  std::vector<qg_handle*> runs;       // stacks and unstacked members (owned)
  std::vector<long long> cells;       // n1*n2*n3 of each run (lane balancing)
  cudaStream_t master = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;      // per run
  int lanes = 8;                      // concurrent chains of runs in the step graph
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  std::string err;
};

namespace {
bool same_doubles(const double* a, const double* b, int n) {
  if (!a || !b) return a == b;
  return std::memcmp(a, b, (size_t)n * sizeof(double)) == 0;
}
// members that can share one stack: everything but the time step, Ro, W2F
// and the hyperdiffusion coefficients equal (YBJ+ only: the regular-YBJ A
// is a vertical integral over one run's column)
bool stackable(const qg_config& a, const qg_config& b) {
  return a.n1 == b.n1 && a.n2 == b.n2 && a.n3 == b.n3 && a.precision == b.precision && a.device == b.device &&
         a.ybj_plus == 1 && b.ybj_plus == 1 && a.fixed_flow == b.fixed_flow && a.no_feedback == b.no_feedback &&
         a.passive_scalar == b.passive_scalar && a.linear == b.linear && a.no_dispersion == b.no_dispersion &&
         a.inviscid == b.inviscid && a.dz == b.dz && a.Bu == b.Bu && a.gamma == b.gamma && a.nuz == b.nuz &&
         a.ilap1 == b.ilap1 && a.ilap2 == b.ilap2 && a.ilap1w == b.ilap1w && a.ilap2w == b.ilap2w &&
         a.solve_columns == b.solve_columns && same_doubles(a.a_ell_ut, b.a_ell_ut, a.n3) &&
         same_doubles(a.rho_ut, b.rho_ut, a.n3) && same_doubles(a.rho_st, b.rho_st, a.n3) &&
         same_doubles(a.r_2ut, b.r_2ut, a.n3);
}
}  // namespace

static int ens_fail(qg_ensemble* e, int code, const std::string& msg) {
  if (e) e->err = msg;
  return code;
}

#define ENS_CK(call)                                                                       \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return ens_fail(e, QG_ERR_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
  } while (0)

int qg_ensemble_destroy(qg_ensemble* e) {
  if (!e) return QG_ERR_ARG;
  if (e->master) cudaStreamSynchronize(e->master);
  for (auto& g : e->gexec) if (g) cudaGraphExecDestroy(g);
  for (auto* h : e->members) if (h && h->view) qg_destroy(h);
  for (auto* h : e->runs) qg_destroy(h);
  for (auto ev : e->join) cudaEventDestroy(ev);
  if (e->fork) cudaEventDestroy(e->fork);
  if (e->master) cudaStreamDestroy(e->master);
  delete e;
  return QG_OK;
}

int qg_ensemble_create(const qg_config* cfgs, int nmembers, qg_ensemble** out) {
  if (!cfgs || !out || nmembers <= 0) return fail(nullptr, QG_ERR_ARG, "qg_ensemble_create: bad arguments");
  *out = nullptr;
  for (int m = 1; m < nmembers; ++m)
    if (cfgs[m].device != cfgs[0].device) return fail(nullptr, QG_ERR_ARG, "ensemble members must share one device");
  qg_ensemble* e = new qg_ensemble();
  e->members.assign(nmembers, nullptr);
  // group the members into stacks (first member of each group as its key)
  std::vector<std::vector<int>> groups;
  for (int m = 0; m < nmembers; ++m) {
    size_t k = 0;
    while (k < groups.size() && !stackable(cfgs[groups[k][0]], cfgs[m])) ++k;
    if (k == groups.size()) groups.push_back({});
    groups[k].push_back(m);
  }
  for (const auto& grp : groups) {
    const int m0 = grp[0], M = (int)grp.size();
    qg_config c = cfgs[m0];
    c.use_graphs = 0;          // runs are replayed through the ensemble graph
    qg_handle* h = nullptr;
    int rc = QG_OK;
    std::string where = "member " + std::to_string(m0) + ": ";
    if (M == 1) {
      rc = qg_create(&c, &h);
    } else {
      qg::HostTables t;
      std::string err;
      for (int k = 0; k < M && !rc; ++k) {
        const qg_config& cm = cfgs[grp[k]];
        where = "member " + std::to_string(grp[k]) + ": ";
        if ((rc = validate_config(cm))) break;
        qg::HostTables tk;
        if ((rc = build_tables(cm, tk, err))) { g_create_err = err; break; }
        if (k == 0) {
          t = std::move(tk);
        } else {
          t.e1.insert(t.e1.end(), tk.e1.begin(), tk.e1.end());
          t.e2.insert(t.e2.end(), tk.e2.begin(), tk.e2.end());
          t.e1w.insert(t.e1w.end(), tk.e1w.begin(), tk.e1w.end());
          t.e2w.insert(t.e2w.end(), tk.e2w.begin(), tk.e2w.end());
        }
        t.mpar.insert(t.mpar.end(), {cm.delt, 0.5 / (cm.Bu * cm.Ro), cm.Ro, cm.W2F});
      }
      if (!rc) {
        t.nseg = c.n3;
        t.members = M;
        t.n3 = M * c.n3;
        c.n3 = t.n3;
        c.levels_per_batch = 0;    // the stack's own batch depth
        rc = create_from_tables(c, t, &h);
      }
    }
    if (rc) {
      const std::string msg = where + g_create_err;
      qg_ensemble_destroy(e);
      return fail(nullptr, rc, msg);
    }
    e->runs.push_back(h);
    e->cells.push_back((long long)c.n1 * c.n2 * c.n3);
    for (int k = 0; k < M; ++k) {
      if (M == 1) { e->members[grp[k]] = h; continue; }
      qg_handle* v = new qg_handle();
      v->eng = h->eng;
      v->view = true;
      v->z0 = k * cfgs[m0].n3;
      v->nz = cfgs[m0].n3;
      e->members[grp[k]] = v;
    }
  }
  if (cudaSetDevice(cfgs[0].device) != cudaSuccess || cudaStreamCreateWithFlags(&e->master, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming) != cudaSuccess) {
    qg_ensemble_destroy(e);
    return fail(nullptr, QG_ERR_CUDA, "qg_ensemble_create: stream/event creation failed");
  }
  e->join.resize(e->runs.size());
  for (auto& ev : e->join) cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  *out = e;
  return QG_OK;
}

int qg_ensemble_member(qg_ensemble* e, int member, qg_handle** h) {
  if (!e || !h || member < 0 || member >= (int)e->members.size()) return ens_fail(e, QG_ERR_ARG, "bad member index");
  *h = e->members[member];
  return QG_OK;
}

// One step of every member as one graph: members are dealt to `lanes`
// chains (largest first, each to the lane with the fewest cells so far);
// the chains run concurrently, the members of a chain one after another,
// which bounds how many members' scratch planes compete for L2 at once.
static int ens_capture(qg_ensemble* e, int euler) {
  cudaGraph_t graph = nullptr;
  const int nm = (int)e->runs.size();
  const int L = std::max(1, std::min(e->lanes, nm));
  std::vector<int> order(nm);
  for (int m = 0; m < nm; ++m) order[m] = m;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return e->cells[a] > e->cells[b]; });
  std::vector<long long> load(L, 0);
  std::vector<int> tail(L, -1);       // last member of each lane (-1: the fork)
  ENS_CK(cudaStreamBeginCapture(e->master, cudaStreamCaptureModeThreadLocal));
  int rc = QG_OK;
  if (cudaEventRecord(e->fork, e->master) != cudaSuccess) { rc = QG_ERR_CUDA; e->err = "ensemble fork failed"; }
  for (int k = 0; k < nm && !rc; ++k) {
    const int m = order[k];
    int lane = 0;
    for (int l = 1; l < L; ++l) if (load[l] < load[lane]) lane = l;
    cudaStream_t ms = (cudaStream_t)e->runs[m]->eng->stream();
    cudaEvent_t dep = tail[lane] < 0 ? e->fork : e->join[tail[lane]];
    if (cudaStreamWaitEvent(ms, dep, 0) != cudaSuccess) { rc = QG_ERR_CUDA; e->err = "ensemble fork failed"; break; }
    rc = e->runs[m]->eng->enqueue(euler);
    if (rc) { e->err = "run " + std::to_string(m) + ": " + e->runs[m]->eng->err; break; }
    if (cudaEventRecord(e->join[m], ms) != cudaSuccess) { rc = QG_ERR_CUDA; e->err = "ensemble join failed"; break; }
    tail[lane] = m;
    load[lane] += e->cells[m];
  }
  for (int l = 0; l < L && !rc; ++l)
    if (tail[l] >= 0 && cudaStreamWaitEvent(e->master, e->join[tail[l]], 0) != cudaSuccess) {
      rc = QG_ERR_CUDA;
      e->err = "ensemble join failed";
    }
  cudaError_t ce = cudaStreamEndCapture(e->master, &graph);
  if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
  if (ce != cudaSuccess) return ens_fail(e, QG_ERR_CUDA, std::string("ensemble capture: ") + cudaGetErrorString(ce));
  ce = cudaGraphInstantiate(&e->gexec[euler], graph, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) return ens_fail(e, QG_ERR_CUDA, std::string("ensemble instantiate: ") + cudaGetErrorString(ce));
  return QG_OK;
}

int qg_ensemble_step(qg_ensemble* e, int nsteps, int euler_first) {
  if (!e || nsteps < 0) return ens_fail(e, QG_ERR_ARG, "bad arguments");
  e->err.clear();
  for (auto* r : e->runs) {                                  // outside any capture
    r->eng->release_init_buffers();
    const int rc = r->eng->prepare();
    if (rc) return ens_fail(e, rc, r->eng->err);
  }
  for (int i = 0; i < nsteps; ++i) {
    const int k = (euler_first && i == 0) ? 1 : 0;
    if (!e->gexec[k]) {
      int rc = ens_capture(e, k);
      if (rc) return rc;
    }
    ENS_CK(cudaGraphLaunch(e->gexec[k], e->master));
  }
  return QG_OK;
}

int qg_ensemble_set_lanes(qg_ensemble* e, int lanes) {
  if (!e || lanes < 1) return ens_fail(e, QG_ERR_ARG, "qg_ensemble_set_lanes: lanes must be >= 1");
  ENS_CK(cudaStreamSynchronize(e->master));
  for (auto& x : e->gexec)
    if (x) { cudaGraphExecDestroy(x); x = nullptr; }
  e->lanes = lanes;
  return QG_OK;
}

int qg_ensemble_synchronize(qg_ensemble* e) {
  if (!e) return QG_ERR_ARG;
  ENS_CK(cudaStreamSynchronize(e->master));
  // every member's device-raised status (expired wait, non-finite q*)
  int first = QG_OK;
  for (size_t m = 0; m < e->runs.size(); ++m) {
    const int rc = e->runs[m]->eng->check_waits();
    if (rc && !first) {
      first = rc;
      const int nm = e->runs[m]->eng->member_count();
      e->err = (nm > 1 ? "stack of " + std::to_string(nm) + " members (run " + std::to_string(m) + "): "
                       : "run " + std::to_string(m) + ": ") + e->runs[m]->eng->err;
    }
  }
  return first;
}

int qg_ensemble_get_stream(qg_ensemble* e, void** stream) {
  if (!e || !stream) return ens_fail(e, QG_ERR_ARG, "null argument");
  *stream = (void*)e->master;
  return QG_OK;
}

const char* qg_ensemble_last_error(const qg_ensemble* e) { return e ? e->err.c_str() : ""; }

int qg_ensemble_profile_step(qg_ensemble* e, int euler_first, double* ms, int* launches, int nclasses) {
  if (!e || !ms || !launches || nclasses <= 0) return ens_fail(e, QG_ERR_ARG, "qg_ensemble_profile_step: bad arguments");
  ENS_CK(cudaStreamSynchronize(e->master));
  for (int i = 0; i < nclasses; ++i) { ms[i] = 0.0; launches[i] = 0; }
  std::vector<double> rm(nclasses);
  std::vector<int> rl(nclasses);
  for (size_t r = 0; r < e->runs.size(); ++r) {
    e->runs[r]->eng->release_init_buffers();
    const int rc = e->runs[r]->eng->profile_step(euler_first, rm.data(), rl.data(), nclasses);
    if (rc) return ens_fail(e, rc, "run " + std::to_string(r) + ": " + e->runs[r]->eng->err);
    for (int i = 0; i < nclasses; ++i) { ms[i] += rm[i]; launches[i] += rl[i]; }
  }
  return QG_OK;
}

// ---- autotuner -------------------------------------------------------------
int qg_autotune(const qg_config* cfg, int nsteps, qg_tuning* out) {
  if (!cfg || !out || nsteps <= 0) return fail(nullptr, QG_ERR_ARG, "qg_autotune: bad arguments");
  std::memset(out, 0, sizeof *out);
  qg_config c = *cfg;
  c.use_graphs = 1;
  qg_handle* h = nullptr;
  int rc = qg_create(&c, &h);
  if (rc) return rc;
  // candidate depths: powers of two and depths whose kernel grids fill an
  // integral number of waves well, capped by a 1.25 GB scratch budget (past
  // L2: deep batches trade scratch traffic for fuller waves, longer
  // persistent row kernels and fewer launches, which the timing settles)
  std::vector<int> cand;
  const int n = c.n1, n3 = c.n3;
  const size_t cbytes = c.precision == QG_PREC_FP64 ? 16 : 8;
  const int K = (int)((float)(int)((float)n / 3.0f + 0.5f) - 0.5f);
  const size_t per_level = (size_t)6 * n * (((K + 1 + 7) / 8) * 8) * cbytes;
  const int zmax = (int)std::max<size_t>(1, std::min<size_t>((size_t)n3, (size_t)(1280u << 20) / per_level));
  for (int z : {1, 2, 4, 8, 13, 16, 20, 26, 32, 43, 64, 86, 128, 192, 256})
    if (z <= zmax && (int)cand.size() < 16) cand.push_back(z);
  cudaStream_t st = (cudaStream_t)h->eng->stream();
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double best = 1e300;
  int bestz = cand.empty() ? 1 : cand[0];
  for (int z : cand) {
    rc = h->eng->set_batch_levels(z);
    if (!rc) rc = h->eng->steps_async(2, 1);          // warm-up, graph capture
    if (!rc) rc = h->eng->synchronize();
    if (rc) break;
    cudaEventRecord(a, st);
    rc = h->eng->steps_async(nsteps, 0);
    cudaEventRecord(b, st);
    if (!rc) rc = h->eng->synchronize();
    if (rc) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    const double per = ms / nsteps;
    const int zeff = h->eng->batch_levels();
    out->candidates[out->ncandidates] = zeff;
    out->candidate_ms[out->ncandidates] = per;
    out->ncandidates++;
    if (per < best) { best = per; bestz = zeff; }
  }
  // block shape of the column solves at the chosen batch depth
  int best_tc = h->eng->solve_columns();
  if (!rc) rc = h->eng->set_batch_levels(bestz);
  for (int tc : {16, 32, 64}) {
    if (rc) break;
    rc = h->eng->set_solve_columns(tc);
    if (!rc) rc = h->eng->steps_async(2, 1);
    if (!rc) rc = h->eng->synchronize();
    if (rc) break;
    cudaEventRecord(a, st);
    rc = h->eng->steps_async(nsteps, 0);
    cudaEventRecord(b, st);
    if (!rc) rc = h->eng->synchronize();
    if (rc) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    const double per = ms / nsteps;
    out->solve_candidates[out->nsolve] = tc;
    out->solve_candidate_ms[out->nsolve] = per;
    out->nsolve++;
    if (per < best) { best = per; best_tc = tc; }
  }
  std::string err = rc ? h->eng->err : "";
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  qg_destroy(h);
  if (rc) return fail(nullptr, rc, "qg_autotune: " + err);
  out->levels_per_batch = bestz;
  out->solve_columns = best_tc;
  out->ms_per_step = best;
  return QG_OK;
}

}  // extern "C"
