// FP64 instantiation: every operation of the step in double precision, plus
// the hand-written adjoint of the step (reverse sweep with checkpoints).
//
// The adjoint works on the reference's dense spectral layout and mirrors,
// primitive by primitive, the transposes of the step's operations: c2r/r2c
// on the retained modes, i k multipliers, physical products, the symmetric
// tridiagonal inversions, the leapfrog/Robert-Asselin/integrating-factor
// update.  The forward states it linearises about are recomputed inside each
// checkpoint segment with the step kernels.
#include <cmath>
#include <initializer_list>
#include <vector>
#include "adjoint_kernels.cuh"
#include "engine_impl.cuh"

namespace qg {

class AdjEngine final : public Engine<double> {
  using C = double2;
  enum { NSPEC = 17, NPHYS = 28, NST = 9 };

 public:
  ~AdjEngine() override {
    free_list(owned);
    free_list(scratch);
  }

  int init(const qg_config& c, const HostTables& t) override {
    rho_unit = t.rho_unit;
    return Engine<double>::init(c, t);
  }

  int adjoint_run(const double* q0, const double* BR0, const double* BI0, int nsteps, int every, int objective,
                  double* J, double* gq, double* gR, double* gI) override {
    int rc = ensure_adj();
    if (rc) return rc;
    ScratchScope scope(this);
    const size_t sb = spec_bytes();
    // initial carried state and its derived fields
    std::vector<C*> st0 = alloc_state();
    if (st0.empty()) return QG_ERR_NOMEM;
    QG_CK(cudaMemcpyAsync(st0[0], q0, sb, cudaMemcpyDefault, st));
    QG_CK(cudaMemcpyAsync(st0[2], BR0, sb, cudaMemcpyDefault, st));
    QG_CK(cudaMemcpyAsync(st0[3], BI0, sb, cudaMemcpyDefault, st));
    for (int f : {0, 2, 3}) if ((rc = lin(st0[f], 0, {term(st0[f], 1, 0, 0)}))) return rc;
    QG_CK(cudaMemcpyAsync(st0[1], st0[0], sb, cudaMemcpyDeviceToDevice, st));
    QG_CK(cudaMemcpyAsync(st0[4], st0[2], sb, cudaMemcpyDeviceToDevice, st));
    QG_CK(cudaMemcpyAsync(st0[5], st0[3], sb, cudaMemcpyDeviceToDevice, st));
    if ((rc = derived(st0[0], st0[2], st0[3], st0[6], st0[7], st0[8]))) return rc;
    // forward sweep, checkpoints every `every` steps
    std::vector<std::vector<C*>> ck;
    ck.push_back(st0);
    if ((rc = import_state(st0))) return rc;
    for (int i = 0; i < nsteps; ++i) {
      if ((rc = run_step(i == 0 ? 1 : 0))) return rc;
      if ((i + 1) % every == 0 && i + 1 < nsteps) {
        std::vector<C*> s = alloc_state();
        if (s.empty()) return QG_ERR_NOMEM;
        if ((rc = export_state(s))) return rc;
        ck.push_back(s);
      }
    }
    std::vector<C*> fin = alloc_state();
    if (fin.empty()) return QG_ERR_NOMEM;
    if ((rc = export_state(fin))) return rc;
    // objective and its gradient with respect to the final B
    std::vector<C*> lam = alloc_fields(6), lam2 = alloc_fields(6);
    if (lam.empty() || lam2.empty()) return QG_ERR_NOMEM;
    if ((rc = objective_value(fin, J, gq ? lam : std::vector<C*>()))) return rc;
    if (gq) {
      // reverse sweep segment by segment
      std::vector<std::vector<C*>> seg(every);
      for (auto& s : seg) { s = alloc_state(); if (s.empty()) return QG_ERR_NOMEM; }
      for (int c = (int)ck.size() - 1; c >= 0; --c) {
        const int s0 = c * every, s1 = std::min(s0 + every, nsteps);
        if ((rc = copy_state(ck[c], seg[0]))) return rc;
        if ((rc = import_state(ck[c]))) return rc;
        for (int i = s0; i < s1 - 1; ++i) {
          if ((rc = run_step(i == 0 ? 1 : 0))) return rc;
          if ((rc = export_state(seg[i - s0 + 1]))) return rc;
        }
        for (int i = s1 - 1; i >= s0; --i) {
          if ((rc = step_T(seg[i - s0], i == 0, lam, lam2))) return rc;
          std::swap(lam, lam2);
        }
      }
      // X0 = (q0, q0, B0, B0): gradients add the current and old components
      if ((rc = lin(lam2[0], 0, {term(lam[0], 1, 0, 0), term(lam[1], 1, 0, 0)})) ||
          (rc = lin(lam2[1], 0, {term(lam[2], 1, 0, 0), term(lam[4], 1, 0, 0)})) ||
          (rc = lin(lam2[2], 0, {term(lam[3], 1, 0, 0), term(lam[5], 1, 0, 0)})))
        return rc;
      QG_CK(cudaMemcpyAsync(gq, lam2[0], sb, cudaMemcpyDefault, st));
      QG_CK(cudaMemcpyAsync(gR, lam2[1], sb, cudaMemcpyDefault, st));
      QG_CK(cudaMemcpyAsync(gI, lam2[2], sb, cudaMemcpyDefault, st));
    }
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

  int adjoint_step(int euler, const double* const* X, const double* const* lX, double* const* Xn,
                   double* const* lXo) override {
    int rc = ensure_adj();
    if (rc) return rc;
    ScratchScope scope(this);
    const size_t sb = spec_bytes();
    std::vector<C*> s = alloc_state();
    if (s.empty()) return QG_ERR_NOMEM;
    for (int f = 0; f < 6; ++f) {
      QG_CK(cudaMemcpyAsync(s[f], X[f], sb, cudaMemcpyDefault, st));
      if ((rc = lin(s[f], 0, {term(s[f], 1, 0, 0)}))) return rc;
    }
    if ((rc = derived(s[0], s[2], s[3], s[6], s[7], s[8]))) return rc;
    if (lXo) {
      std::vector<C*> a = alloc_fields(6), b = alloc_fields(6);
      if (a.empty() || b.empty()) return QG_ERR_NOMEM;
      for (int f = 0; f < 6; ++f) {
        QG_CK(cudaMemcpyAsync(a[f], lX[f], sb, cudaMemcpyDefault, st));
        if ((rc = lin(a[f], 0, {term(a[f], 1, 0, 0)}))) return rc;
      }
      if ((rc = step_T(s, euler != 0, a, b))) return rc;
      for (int f = 0; f < 6; ++f) if (lXo[f]) QG_CK(cudaMemcpyAsync(lXo[f], b[f], sb, cudaMemcpyDefault, st));
    }
    if (Xn) {
      if ((rc = import_state(s)) || (rc = run_step(euler ? 1 : 0)) || (rc = export_state(s))) return rc;
      for (int f = 0; f < 6; ++f) if (Xn[f]) QG_CK(cudaMemcpyAsync(Xn[f], s[f], sb, cudaMemcpyDefault, st));
    }
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

 private:
  C* Sb[NSPEC] = {};
  double* Pb[NPHYS] = {};
  double* tab[4] = {};
  C* tmpC[3] = {};
  double* part = nullptr;
  std::vector<double> part_h;
  std::vector<void*> owned;    // buffers kept for the handle's lifetime
  std::vector<void*> scratch;  // checkpoints and segment states of one call
  bool ready = false, rho_unit = true;
  static constexpr int kObjBlocks = 512;

  static void free_list(std::vector<void*>& v) {
    for (void* p : v) cudaFree(p);
    v.clear();
  }
  // frees one call's checkpoint storage when the call returns (cudaFree
  // waits for the work that still uses it)
  struct ScratchScope {
    AdjEngine* e;
    explicit ScratchScope(AdjEngine* x) : e(x) {}
    ~ScratchScope() {
      cudaStreamSynchronize(e->st);
      free_list(e->scratch);
    }
  };

  size_t spec_bytes() const { return (size_t)g.n3 * g.n * (g.n / 2 + 1) * sizeof(C); }
  long long totS() const { return (long long)g.n3 * g.n * (g.n / 2 + 1); }
  long long totP() const { return (long long)g.n3 * g.n * g.n; }

  template <typename P>
  int grab(P** p, size_t bytes, bool keep = true) {
    void* q = nullptr;
    QG_CK(cudaMalloc(&q, bytes));
    (keep ? owned : scratch).push_back(q);
    *p = static_cast<P*>(q);
    return QG_OK;
  }

  std::vector<C*> alloc_fields(int k) {
    std::vector<C*> v(k, nullptr);
    for (auto& p : v) if (grab(&p, spec_bytes(), false)) return {};
    return v;
  }
  std::vector<C*> alloc_state() { return alloc_fields(NST); }

  int ensure_adj() {
    if (ready) return QG_OK;
    // the transposes below use psi_solver and A_solver as self-adjoint
    // (rho = 1) and cover the step without vertical diffusion, with psi
    // and A derived from the carried state
    if (!rho_unit) { err = "the adjoint needs rho_ut = rho_st = 1 (symmetric vertical operators)"; return QG_ERR_UNSUPPORTED; }
    if (sp.use_dq) { err = "the adjoint covers the inviscid vertical step (nuz = 0 or inviscid = 1)"; return QG_ERR_UNSUPPORTED; }
    if (cfg.fixed_flow || cfg.passive_scalar) {
      err = "the adjoint needs fixed_flow = 0 and passive_scalar = 0";
      return QG_ERR_UNSUPPORTED;
    }
    int rc = prep_dense(g.n3);
    if (rc) return rc;
    for (auto& p : Sb) if ((rc = grab(&p, spec_bytes()))) return rc;
    for (auto& p : Pb) if ((rc = grab(&p, (size_t)totP() * sizeof(double)))) return rc;
    const size_t tb = (size_t)g.n * (g.n / 2 + 1) * sizeof(double);
    const double* src[4] = {e1, e2, e1w, e2w};
    for (int i = 0; i < 4; ++i) {
      if ((rc = grab(&tab[i], tb))) return rc;
      k_table_to_dense<double><<<grid_for((long long)g.n * (g.n / 2 + 1)), 256, 0, st>>>(g, src[i], tab[i]);
      QG_LAUNCHED();
    }
    for (auto& p : tmpC) {
      if ((rc = grab(&p, (size_t)g.n3 * g.plane * sizeof(C)))) return rc;
      QG_CK(cudaMemsetAsync(p, 0, (size_t)g.n3 * g.plane * sizeof(C), st));
    }
    if ((rc = grab(&part, kObjBlocks * sizeof(double)))) return rc;
    part_h.assign(kObjBlocks, 0.0);
    ready = true;
    return QG_OK;
  }

  // ---- primitives ----------------------------------------------------------
  static SpecTerm term(const C* in, double sr, double si, int mult, const double* t = nullptr) {
    SpecTerm s;
    s.in = in; s.sr = sr; s.si = si; s.mult = mult; s.tab = t;
    return s;
  }
  int lin(C* out, int acc, std::initializer_list<SpecTerm> ts) {
    SpecTerm t[3] = {term(nullptr, 0, 0, 0), term(nullptr, 0, 0, 0), term(nullptr, 0, 0, 0)};
    int k = 0;
    for (const auto& x : ts) t[k++] = x;
    k_spec_lin<<<grid_for(totS()), 256, 0, st>>>(g.n, g.kmax2, totS(), k, t[0], t[1], t[2], acc, out);
    QG_LAUNCHED();
    return QG_OK;
  }
  int Cf(const C* X, double* x) { return d_c2r(X, x, g.n3); }       // X holds only retained modes
  int CTf(const double* y, C* out, int acc) {
    int rc = d_r2c(y, Sb[15], g.n3);
    if (rc) return rc;
    k_ct_weights<<<grid_for(totS()), 256, 0, st>>>(g.n, g.kmax2, totS(), (double)g.n * g.n, Sb[15], acc, out);
    QG_LAUNCHED();
    return QG_OK;
  }
  int RTf(const C* Y, double* x) {
    k_rt_prep<<<grid_for(totS()), 256, 0, st>>>(g.n, g.kmax2, totS(), 0.5 / ((double)g.n * g.n), Y, Sb[16]);
    QG_LAUNCHED();
    return d_c2r(Sb[16], x, g.n3);
  }
  int pacc(double* out, const double* x, const double* y, double s, int acc) {
    k_phys_acc<<<grid_for(totP()), 256, 0, st>>>(totP(), x, y, s, acc, out);
    QG_LAUNCHED();
    return QG_OK;
  }
  int inv(const C* in, C* out, bool psi_op) {
    k_dense_to_compact<double><<<grid_for((long long)g.n3 * g.plane), 256, 0, st>>>(g, 0, g.n3, in, tmpC[0]);
    QG_LAUNCHED();
    int rc = psi_op ? solve_generic(tmpC[0], nullptr, nullptr, tmpC[1], nullptr, nullptr, 1, 0)
                    : solve_generic(nullptr, tmpC[0], tmpC[0], nullptr, tmpC[1], tmpC[2], 0, 1);
    if (rc) return rc;
    k_compact_to_dense<double><<<grid_for(totS()), 256, 0, st>>>(g, 0, g.n3, tmpC[1], out, 0, cfg.dz);
    QG_LAUNCHED();
    return QG_OK;
  }

  // psi = psi_solver(q - q^w(B)), A = A_solver(B)
  int derived(const C* q, const C* BR, const C* BI, C* psi, C* AR, C* AI) {
    int rc;
    if (!cfg.fixed_flow) {
      if (!cfg.no_feedback) {
        if ((rc = compute_qw(reinterpret_cast<const double*>(BR), reinterpret_cast<const double*>(BI),
                             reinterpret_cast<double*>(Sb[13]), g.n3)))
          return rc;
        if ((rc = lin(Sb[14], 0, {term(q, 1, 0, 0), term(Sb[13], -1, 0, 0)}))) return rc;
      } else if ((rc = lin(Sb[14], 0, {term(q, 1, 0, 0)}))) {
        return rc;
      }
      if ((rc = inv(Sb[14], psi, true))) return rc;
    } else {
      QG_CK(cudaMemsetAsync(psi, 0, spec_bytes(), st));
    }
    if ((rc = inv(BR, AR, false)) || (rc = inv(BI, AI, false))) return rc;
    return QG_OK;
  }

  // ---- engine state <-> dense fields ---------------------------------------
  int import_state(const std::vector<C*>& s) {
    const int ids[NST] = {QG_Q, QG_QOLD, QG_BR, QG_BI, QG_BROLD, QG_BIOLD, QG_PSI, QG_AR, QG_AI};
    for (int f = 0; f < NST; ++f) {
      int rc = set_state(ids[f], reinterpret_cast<const double*>(s[f]), 0, g.n3);
      if (rc) return rc;
    }
    return QG_OK;
  }
  int export_state(const std::vector<C*>& s) {
    const int ids[NST] = {QG_Q, QG_QOLD, QG_BR, QG_BI, QG_BROLD, QG_BIOLD, QG_PSI, QG_AR, QG_AI};
    for (int f = 0; f < NST; ++f) {
      int rc = get_state(ids[f], reinterpret_cast<double*>(s[f]), 0, g.n3);
      if (rc) return rc;
    }
    return QG_OK;
  }
  int copy_state(const std::vector<C*>& a, const std::vector<C*>& b) {
    for (int f = 0; f < NST; ++f) QG_CK(cudaMemcpyAsync(b[f], a[f], spec_bytes(), cudaMemcpyDeviceToDevice, st));
    return QG_OK;
  }

  int obj_first_level() const {
    int z0 = 0;
    while (z0 < g.n3 && ((double)z0 + 0.5) / g.n3 < 0.8) ++z0;
    return z0;
  }

  // J = 1/2 sum_W |C(B + kh^2 A/(4 Bu))|^2 and, when lam is given, dJ/dB in lam[2], lam[3]
  int objective_value(const std::vector<C*>& s, double* J, const std::vector<C*>& lam) {
    int rc;
    const double k4 = 0.25 / cfg.Bu;
    double* LR = Pb[0];
    double* LI = Pb[1];
    if ((rc = lin(Sb[0], 0, {term(s[2], 1, 0, 0), term(s[7], k4, 0, 3)})) || (rc = Cf(Sb[0], LR))) return rc;
    if ((rc = lin(Sb[0], 0, {term(s[3], 1, 0, 0), term(s[8], k4, 0, 3)})) || (rc = Cf(Sb[0], LI))) return rc;
    const int z0 = obj_first_level();
    k_obj_partial<<<kObjBlocks, 256, 0, st>>>(g.n, g.n3, z0, LR, LI, part);
    QG_LAUNCHED();
    QG_CK(cudaMemcpyAsync(part_h.data(), part, kObjBlocks * sizeof(double), cudaMemcpyDeviceToHost, st));
    QG_CK(cudaStreamSynchronize(st));
    double acc = 0.0;
    for (double v : part_h) acc += v;
    *J = 0.5 * acc;
    if (lam.empty()) return QG_OK;
    for (int f = 0; f < 6; ++f) QG_CK(cudaMemsetAsync(lam[f], 0, spec_bytes(), st));
    for (int c = 0; c < 2; ++c) {
      double* Lx = c == 0 ? LR : LI;
      k_obj_window<<<grid_for(totP()), 256, 0, st>>>(g.n, g.n3, z0, Lx);
      QG_LAUNCHED();
      // grad = g + A_solver(kh^2/(4 Bu) g), g = C^T(W L)
      if ((rc = CTf(Lx, Sb[1], 0)) || (rc = lin(Sb[2], 0, {term(Sb[1], k4, 0, 3)})) || (rc = inv(Sb[2], Sb[3], false)) ||
          (rc = lin(lam[2 + c], 0, {term(Sb[1], 1, 0, 0), term(Sb[3], 1, 0, 0)})))
        return rc;
    }
    return QG_OK;
  }

  // ---- adjoint of one step at the state s (9 fields) ----------------------
  int step_T(const std::vector<C*>& s, bool first, const std::vector<C*>& l1, const std::vector<C*>& lo) {
    int rc;
    const double gm = cfg.gamma, dt = cfg.delt, cd = 0.5 / (cfg.Bu * cfg.Ro);
    C* q = s[0]; C* BR = s[2]; C* BI = s[3]; C* psi = s[6];
    C *lq = lo[0], *lr = lo[1], *lBR = lo[2], *lBI = lo[3], *lcR = lo[4], *lcI = lo[5];
    C *lqp = Sb[0], *lBRp = Sb[1], *lBIp = Sb[2], *lNq = Sb[3], *lTR = Sb[4], *lTI = Sb[5];
    C *lAR = Sb[6], *lAI = Sb[7], *lrBR = Sb[8], *lrBI = Sb[9], *lpsi = Sb[10], *tA = Sb[11], *tB = Sb[12],
      *tC = Sb[13], *w = Sb[14];
    if (first) {
      // r1 = q0, c1 = B0 ; q1 = e1 (q0 - dt Nq) ; B1 = e1w (B0 - dt T)
      if ((rc = lin(lq, 0, {term(l1[1], 1, 0, 0), term(l1[0], 1, 0, 4, tab[0])})) ||
          (rc = lin(lBR, 0, {term(l1[4], 1, 0, 0), term(l1[2], 1, 0, 4, tab[2])})) ||
          (rc = lin(lBI, 0, {term(l1[5], 1, 0, 0), term(l1[3], 1, 0, 4, tab[2])})))
        return rc;
      for (C* z : {lr, lcR, lcI}) QG_CK(cudaMemsetAsync(z, 0, spec_bytes(), st));
      if ((rc = lin(lNq, 0, {term(l1[0], -dt, 0, 4, tab[0])})) || (rc = lin(lTR, 0, {term(l1[2], -dt, 0, 4, tab[2])})) ||
          (rc = lin(lTI, 0, {term(l1[3], -dt, 0, 4, tab[2])})))
        return rc;
    } else {
      // Robert-Asselin filter and leapfrog
      if ((rc = lin(lqp, 0, {term(l1[0], 1, 0, 0), term(l1[1], gm, 0, 0)})) ||
          (rc = lin(lBRp, 0, {term(l1[2], 1, 0, 0), term(l1[4], gm, 0, 0)})) ||
          (rc = lin(lBIp, 0, {term(l1[3], 1, 0, 0), term(l1[5], gm, 0, 0)})) ||
          (rc = lin(lq, 0, {term(l1[1], 1 - 2 * gm, 0, 0)})) || (rc = lin(lBR, 0, {term(l1[4], 1 - 2 * gm, 0, 0)})) ||
          (rc = lin(lBI, 0, {term(l1[5], 1 - 2 * gm, 0, 0)})) ||
          (rc = lin(lr, 0, {term(l1[1], gm, 0, 0), term(lqp, 1, 0, 4, tab[1])})) ||
          (rc = lin(lcR, 0, {term(l1[4], gm, 0, 0), term(lBRp, 1, 0, 4, tab[3])})) ||
          (rc = lin(lcI, 0, {term(l1[5], gm, 0, 0), term(lBIp, 1, 0, 4, tab[3])})) ||
          (rc = lin(lNq, 0, {term(lqp, -2 * dt, 0, 4, tab[0])})) || (rc = lin(lTR, 0, {term(lBRp, -2 * dt, 0, 4, tab[2])})) ||
          (rc = lin(lTI, 0, {term(lBIp, -2 * dt, 0, 4, tab[2])})))
        return rc;
    }
    const double disp = (cfg.no_dispersion || cfg.passive_scalar) ? 0.0 : 1.0;
    const double refr = cfg.passive_scalar ? 0.0 : 1.0;
    const double adv = cfg.linear ? 0.0 : 1.0;
    // T_R = NBR + c kh2 AI - rBI/2 ; T_I = NBI - c kh2 AR + rBR/2
    if ((rc = lin(lAI, 0, {term(lTR, disp * cd, 0, 3)})) || (rc = lin(lAR, 0, {term(lTI, -disp * cd, 0, 3)})) ||
        (rc = lin(lrBI, 0, {term(lTR, -0.5 * refr, 0, 0)})) || (rc = lin(lrBR, 0, {term(lTI, 0.5 * refr, 0, 0)})))
      return rc;
    // physical fields of the step
    double *u = Pb[0], *v = Pb[1], *Z = Pb[2], *Qp = Pb[3], *BRp = Pb[4], *BIp = Pb[5];
    double *lu = Pb[6], *lv = Pb[7], *lZ = Pb[8], *lQ = Pb[9], *lBRr = Pb[10], *lBIr = Pb[11];
    double *lUX = Pb[12], *lVX = Pb[13], *lZBR = Pb[14], *lZBI = Pb[15];
    if ((rc = lin(tA, 0, {term(psi, 0, -1, 2)})) || (rc = Cf(tA, u)) || (rc = lin(tA, 0, {term(psi, 0, 1, 1)})) ||
        (rc = Cf(tA, v)) || (rc = lin(tA, 0, {term(psi, -1, 0, 3)})) || (rc = Cf(tA, Z)) || (rc = Cf(q, Qp)) ||
        (rc = Cf(BR, BRp)) || (rc = Cf(BI, BIp)))
      return rc;
    const C* lNs[3] = {lNq, lTR, lTI};
    double* Xps[3] = {Qp, BRp, BIp};
    double* lXps[3] = {lQ, lBRr, lBIr};
    for (int k = 0; k < 3; ++k) {
      // N = P[i kx R(u X) + i ky R(v X)]
      if ((rc = lin(tA, 0, {term(lNs[k], 0, -adv, 1)})) || (rc = RTf(tA, lUX)) ||
          (rc = lin(tA, 0, {term(lNs[k], 0, -adv, 2)})) || (rc = RTf(tA, lVX)) ||
          (rc = pacc(lu, lUX, Xps[k], 1.0, k > 0)) || (rc = pacc(lv, lVX, Xps[k], 1.0, k > 0)) ||
          (rc = pacc(lXps[k], lUX, u, 1.0, 0)) || (rc = pacc(lXps[k], lVX, v, 1.0, 1)))
        return rc;
    }
    // rB = P R(Z B)
    if ((rc = RTf(lrBR, lZBR)) || (rc = RTf(lrBI, lZBI)) || (rc = pacc(lZ, lZBR, BRp, 1.0, 0)) ||
        (rc = pacc(lZ, lZBI, BIp, 1.0, 1)) || (rc = pacc(lBRr, lZBR, Z, 1.0, 1)) || (rc = pacc(lBIr, lZBI, Z, 1.0, 1)))
      return rc;
    if ((rc = CTf(lQ, lq, 1)) || (rc = CTf(lBRr, lBR, 1)) || (rc = CTf(lBIr, lBI, 1))) return rc;
    // psi -> u (-i ky), v (i kx), zeta (-kh2): transposes i ky, -i kx, -kh2
    if ((rc = CTf(lu, tA, 0)) || (rc = CTf(lv, tB, 0)) || (rc = CTf(lZ, tC, 0)) ||
        (rc = lin(lpsi, 0, {term(tA, 0, 1, 2), term(tB, 0, -1, 1), term(tC, -1, 0, 3)})))
      return rc;
    // derived fields: A = A_solver(B) (symmetric), psi = psi_solver(q - q^w(B))
    if ((rc = inv(lAR, tA, false)) || (rc = lin(lBR, 1, {term(tA, 1, 0, 0)})) || (rc = inv(lAI, tA, false)) ||
        (rc = lin(lBI, 1, {term(tA, 1, 0, 0)})))
      return rc;
    if (!cfg.fixed_flow) {
      if ((rc = inv(lpsi, w, true)) || (rc = lin(lq, 1, {term(w, 1, 0, 0)}))) return rc;
      if (!cfg.no_feedback && (rc = qw_T(BRp, BIp, BR, BI, w, lBR, lBI))) return rc;
    }
    return QG_OK;
  }

  // lBR, lBI += transpose of the linearised q^w at B, applied to -w
  int qw_T(const double* brr, const double* bir, const C* BR, const C* BI, const C* w, C* lBR, C* lBI) {
    int rc;
    const double s = cfg.Ro * cfg.W2F;
    C *tA = Sb[11], *tB = Sb[12], *tC = Sb[13];
    double *BRx = Pb[16], *BRy = Pb[17], *BIx = Pb[18], *BIy = Pb[19], *lP1 = Pb[20], *lP2 = Pb[21];
    double *a = Pb[22], *b = Pb[23], *c = Pb[24];
    if ((rc = lin(tA, 0, {term(BR, 0, 1, 1)})) || (rc = Cf(tA, BRx)) || (rc = lin(tA, 0, {term(BR, 0, 1, 2)})) ||
        (rc = Cf(tA, BRy)) || (rc = lin(tA, 0, {term(BI, 0, 1, 1)})) || (rc = Cf(tA, BIx)) ||
        (rc = lin(tA, 0, {term(BI, 0, 1, 2)})) || (rc = Cf(tA, BIy)))
      return rc;
    // q^w = s P R(P1) - s kh2/4 P R(P2) applied to lqw = -w
    if ((rc = lin(tA, 0, {term(w, -s, 0, 0)})) || (rc = RTf(tA, lP1)) || (rc = lin(tA, 0, {term(w, 0.25 * s, 0, 3)})) ||
        (rc = RTf(tA, lP2)))
      return rc;
    // P1 = BRy BIx - BRx BIy ; P2 = BR^2 + BI^2
    // BR: (BRx, BRy, br) adjoints = (-lP1 BIy, lP1 BIx, 2 br lP2)
    if ((rc = pacc(a, lP1, BIy, -1.0, 0)) || (rc = pacc(b, lP1, BIx, 1.0, 0)) || (rc = pacc(c, brr, lP2, 2.0, 0)) ||
        (rc = CTf(a, tA, 0)) || (rc = CTf(b, tB, 0)) || (rc = CTf(c, tC, 0)) ||
        (rc = lin(lBR, 1, {term(tA, 0, -1, 1), term(tB, 0, -1, 2), term(tC, 1, 0, 0)})))
      return rc;
    // BI: (BIx, BIy, bi) adjoints = (lP1 BRy, -lP1 BRx, 2 bi lP2)
    if ((rc = pacc(a, lP1, BRy, 1.0, 0)) || (rc = pacc(b, lP1, BRx, -1.0, 0)) || (rc = pacc(c, bir, lP2, 2.0, 0)) ||
        (rc = CTf(a, tA, 0)) || (rc = CTf(b, tB, 0)) || (rc = CTf(c, tC, 0)) ||
        (rc = lin(lBI, 1, {term(tA, 0, -1, 1), term(tB, 0, -1, 2), term(tC, 1, 0, 0)})))
      return rc;
    return QG_OK;
  }
};

EngineBase* make_engine_fp64() { return new AdjEngine(); }

}  // namespace qg
