// FP64 instantiation: every operation of the step in double precision, plus
// the hand-written adjoint of the step (reverse sweep with checkpoints).
//
// The adjoint runs on the compact layout with fused kernels
// (adjoint_kernels.cuh): per batch of levels, y-inverse FFTs of the forward
// and adjoint fields, one row kernel for the transposed products, y-forward
// FFTs with the transposed time update; the symmetric FP64 solves of the
// step; then the transpose of q^w.  The forward states it linearises about
// are recomputed inside each checkpoint segment with the step itself.
#include <cmath>
#include <initializer_list>
#include <vector>
#include "adjoint_kernels.cuh"
#include "engine_impl.cuh"

namespace qg {

class AdjEngine final : public Engine<double> {
  using C = double2;
  // dense buffers of the objective (reference layout)
  enum { NSPEC = 7, NPHYS = 2 };
  // compact adjoint fields
  enum { A_LPSI = 0, A_LAR, A_LAI, A_W, A_LBRA, A_LBIA, A_QW, A_QSTAR, A_N };

 public:
  ~AdjEngine() override {
    free_list(owned);
    free_list(scratch);
    if (SA) cudaFree(SA);
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
    // initial carried state in the engine's fields, psi and A derived from it
    if ((rc = set_state(QG_Q, q0, 0, g.n3)) || (rc = set_state(QG_BR, BR0, 0, g.n3)) ||
        (rc = set_state(QG_BI, BI0, 0, g.n3)))
      return rc;
    const size_t fb = field_bytes();
    QG_CK(cudaMemcpyAsync(F[F_QO], F[F_Q], fb, cudaMemcpyDeviceToDevice, st));
    QG_CK(cudaMemcpyAsync(F[F_BRO], F[F_BR], fb, cudaMemcpyDeviceToDevice, st));
    QG_CK(cudaMemcpyAsync(F[F_BIO], F[F_BI], fb, cudaMemcpyDeviceToDevice, st));
    if ((rc = derive())) return rc;
    // forward sweep, checkpoints (the 9 fields of the engine) every `every` steps
    std::vector<std::vector<C*>> ck;
    {
      std::vector<C*> s = alloc_fields(kCk);
      if (s.empty()) return QG_ERR_NOMEM;
      if ((rc = save(s, kCk))) return rc;
      ck.push_back(s);
    }
    for (int i = 0; i < nsteps; ++i) {
      if ((rc = run_step(i == 0 ? 1 : 0))) return rc;
      if ((i + 1) % every == 0 && i + 1 < nsteps) {
        std::vector<C*> s = alloc_fields(kCk);
        if (s.empty()) return QG_ERR_NOMEM;
        if ((rc = save(s, kCk))) return rc;
        ck.push_back(s);
      }
    }
    // objective at the final state and its gradient with respect to B
    if ((rc = objective_value(J, gq != nullptr))) return rc;
    if (!gq) {
      QG_CK(cudaStreamSynchronize(st));
      return QG_OK;
    }
    // reverse sweep: recompute each segment's states (q, BR, BI, psi), then
    // apply the transposed steps in reverse order
    std::vector<std::vector<C*>> seg(every);
    for (int k = 1; k < every; ++k) {
      seg[k] = alloc_fields(4);
      if (seg[k].empty()) return QG_ERR_NOMEM;
    }
    for (int c = (int)ck.size() - 1; c >= 0; --c) {
      const int s0 = c * every, s1 = std::min(s0 + every, nsteps);
      seg[0] = {ck[c][0], ck[c][2], ck[c][3], ck[c][6]};
      if (s1 - s0 > 1 && (rc = restore(ck[c]))) return rc;
      for (int i = s0; i < s1 - 1; ++i) {
        if ((rc = run_step(i == 0 ? 1 : 0))) return rc;
        if ((rc = save(seg[i - s0 + 1], 4))) return rc;
      }
      for (int i = s1 - 1; i >= s0; --i) {
        const std::vector<C*>& X = seg[i - s0];
        if ((rc = step_T(X[0], X[1], X[2], X[3], i == 0, lamA, lamB))) return rc;
        std::swap(lamA, lamB);
      }
    }
    // X0 = (q0, q0, B0, B0): the gradients add the current and old components
    const long long tot = (long long)g.n3 * g.plane;
    double* outs[3] = {gq, gR, gI};
    const int a[3] = {0, 2, 3}, b[3] = {1, 4, 5};
    for (int k = 0; k < 3; ++k) {
      k_adj_sum<<<grid_for(tot), 256, 0, st>>>(g, tot, lamA[a[k]], lamA[b[k]], 1.0, lamB[0]);
      QG_LAUNCHED();
      if ((rc = download_compact(lamB[0], outs[k], 0))) return rc;
    }
    return QG_OK;
  }

  int adjoint_step(int euler, const double* const* X, const double* const* lX, double* const* Xn,
                   double* const* lXo) override {
    int rc = ensure_adj();
    if (rc) return rc;
    ScratchScope scope(this);
    const int ids[6] = {QG_Q, QG_QOLD, QG_BR, QG_BI, QG_BROLD, QG_BIOLD};
    for (int f = 0; f < 6; ++f)
      if ((rc = set_state(ids[f], X[f], 0, g.n3))) return rc;
    if ((rc = derive())) return rc;
    if (lXo) {
      for (int f = 0; f < 6; ++f)
        if ((rc = upload_compact(lX[f], lamA[f]))) return rc;
      if ((rc = step_T(F[F_Q], F[F_BR], F[F_BI], F[F_PSI], euler != 0, lamA, lamB))) return rc;
      for (int f = 0; f < 6; ++f)
        if (lXo[f] && (rc = download_compact(lamB[f], lXo[f], 0))) return rc;
    }
    if (Xn) {
      if ((rc = run_step(euler ? 1 : 0))) return rc;
      for (int f = 0; f < 6; ++f)
        if (Xn[f] && (rc = get_state(ids[f], Xn[f], 0, g.n3))) return rc;
    }
    QG_CK(cudaStreamSynchronize(st));
    return QG_OK;
  }

 private:
  static constexpr int kCk = 9;          // q, qo, BR, BI, BRo, BIo, psi, AR, AI
  static constexpr int kObjBlocks = 512;
  double2* Sb[NSPEC] = {};
  double* Pb[NPHYS] = {};
  double2* tmpC[3] = {};
  std::vector<C*> lamA, lamB;
  C* Af[A_N] = {};
  C* SA = nullptr;                       // adjoint scratch planes, same shape as S
  int sa_levels = 0;
  double* part = nullptr;
  std::vector<double> part_h;
  std::vector<void*> owned;              // buffers kept for the handle's lifetime
  std::vector<void*> scratch;            // checkpoints and segment states of one call
  bool ready = false, rho_unit = true;

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

  size_t field_bytes() const { return (size_t)g.n3 * g.plane * sizeof(C); }
  size_t spec_bytes() const { return (size_t)g.n3 * g.n * (g.n / 2 + 1) * sizeof(double2); }
  long long totS() const { return (long long)g.n3 * g.n * (g.n / 2 + 1); }
  long long totP() const { return (long long)g.n3 * g.n * g.n; }

  template <typename P>
  int grab(P** p, size_t bytes, bool keep) {
    void* q = nullptr;
    QG_CK(cudaMalloc(&q, bytes));
    (keep ? owned : scratch).push_back(q);
    *p = static_cast<P*>(q);
    return QG_OK;
  }
  std::vector<C*> alloc_fields(int k) {
    std::vector<C*> v(k, nullptr);
    for (auto& p : v) if (grab(&p, field_bytes(), false)) return {};
    return v;
  }

  template <int NN> static constexpr size_t sm_col4() {
    return (size_t)(NN + 4 * Tiles<double, NN>::CT * Tiles<double, NN>::LD) * sizeof(C);
  }

  int ensure_adj() {
    if (ready) return QG_OK;
    // the transposes use psi_solver and A_solver as self-adjoint (rho = 1)
    // and cover the step without vertical diffusion, with psi and A
    // derived from the carried state
    if (!rho_unit) { err = "the adjoint needs rho_ut = rho_st = 1 (symmetric vertical operators)"; return QG_ERR_UNSUPPORTED; }
    if (sp.use_dq) { err = "the adjoint covers the inviscid vertical step (nuz = 0 or inviscid = 1)"; return QG_ERR_UNSUPPORTED; }
    if (!cfg.ybj_plus) { err = "the adjoint covers the YBJ+ step (ybj_plus = 1)"; return QG_ERR_UNSUPPORTED; }
    if (cfg.fixed_flow || cfg.passive_scalar) {
      err = "the adjoint needs fixed_flow = 0 and passive_scalar = 0";
      return QG_ERR_UNSUPPORTED;
    }
    int rc = prep_dense(g.n3);
    if (rc) return rc;
    for (auto& p : Sb) if ((rc = grab(&p, spec_bytes(), true))) return rc;
    for (auto& p : Pb) if ((rc = grab(&p, (size_t)totP() * sizeof(double), true))) return rc;
    for (auto& p : tmpC) {
      if ((rc = grab(&p, field_bytes(), true))) return rc;
      QG_CK(cudaMemsetAsync(p, 0, field_bytes(), st));
    }
    lamA.assign(6, nullptr);
    lamB.assign(6, nullptr);
    for (auto& p : lamA) if ((rc = grab(&p, field_bytes(), true))) return rc;
    for (auto& p : lamB) if ((rc = grab(&p, field_bytes(), true))) return rc;
    for (auto& p : Af) {
      if ((rc = grab(&p, field_bytes(), true))) return rc;
      QG_CK(cudaMemsetAsync(p, 0, field_bytes(), st));
    }
    if ((rc = grab(&part, kObjBlocks * sizeof(double), true))) return rc;
    part_h.assign(kObjBlocks, 0.0);
    const int mx = cudaFuncAttributeMaxDynamicSharedMemorySize;
    QG_SWITCH_N(g.n, {
      QG_CK(cudaFuncSetAttribute(k_adj_col_inv<NN>, (cudaFuncAttribute)mx, (int)sm_col6<NN>()));
      QG_CK(cudaFuncSetAttribute(k_adj_row<NN>, (cudaFuncAttribute)mx, (int)sm_row7<NN>()));
      QG_CK(cudaFuncSetAttribute(k_adj_col_fwd<NN>, (cudaFuncAttribute)mx, (int)sm_col6<NN>()));
      QG_CK(cudaFuncSetAttribute(k_adj_qw_col_inv<NN>, (cudaFuncAttribute)mx, (int)sm_col6<NN>()));
      QG_CK(cudaFuncSetAttribute(k_adj_qw_row<NN>, (cudaFuncAttribute)mx, (int)sm_row4<NN>()));
      QG_CK(cudaFuncSetAttribute(k_adj_qw_col_fwd<NN>, (cudaFuncAttribute)mx, (int)sm_col4<NN>()));
    });
    ready = true;
    return QG_OK;
  }

  // ---- engine state <-> checkpoint fields ----------------------------------
  // k = 4: (q, BR, BI, psi); k = 9: (q, qo, BR, BI, BRo, BIo, psi, AR, AI)
  int save(const std::vector<C*>& s, int k) {
    const int f4[4] = {F_Q, F_BR, F_BI, F_PSI};
    const int f9[9] = {F_Q, F_QO, F_BR, F_BI, F_BRO, F_BIO, F_PSI, F_AR, F_AI};
    for (int i = 0; i < k; ++i)
      QG_CK(cudaMemcpyAsync(s[i], F[k == 4 ? f4[i] : f9[i]], field_bytes(), cudaMemcpyDeviceToDevice, st));
    return QG_OK;
  }
  int restore(const std::vector<C*>& s) {
    const int f9[9] = {F_Q, F_QO, F_BR, F_BI, F_BRO, F_BIO, F_PSI, F_AR, F_AI};
    for (int i = 0; i < kCk; ++i)
      QG_CK(cudaMemcpyAsync(F[f9[i]], s[i], field_bytes(), cudaMemcpyDeviceToDevice, st));
    return QG_OK;
  }

  // psi = psi_solver(q - q^w(B)), A = A_solver(B) from the engine's q, BR, BI
  int derive() {
    int rc;
    const long long tot = (long long)g.n3 * g.plane;
    const C* qs = F[F_Q];
    if (need_qw) {
      k_compact_to_dense<double><<<grid_for(totS()), 256, 0, st>>>(g, 0, g.n3, F[F_BR], Sb[0], 0, cfg.dz);
      QG_LAUNCHED();
      k_compact_to_dense<double><<<grid_for(totS()), 256, 0, st>>>(g, 0, g.n3, F[F_BI], Sb[1], 0, cfg.dz);
      QG_LAUNCHED();
      if ((rc = compute_qw(reinterpret_cast<const double*>(Sb[0]), reinterpret_cast<const double*>(Sb[1]),
                           reinterpret_cast<double*>(Sb[2]), g.n3)))
        return rc;
      k_dense_to_compact<double><<<grid_for(tot), 256, 0, st>>>(g, 0, g.n3, Sb[2], Af[A_QW]);
      QG_LAUNCHED();
      k_adj_sum<<<grid_for(tot), 256, 0, st>>>(g, tot, F[F_Q], Af[A_QW], -1.0, Af[A_QSTAR]);
      QG_LAUNCHED();
      qs = Af[A_QSTAR];
    }
    return solve_generic(qs, F[F_BR], F[F_BI], F[F_PSI], F[F_AR], F[F_AI], 1, 1);
  }

  // ---- the objective (reference layout) -------------------------------------
  static SpecTerm term(const double2* in, double sr, double si, int mult, const double* t = nullptr) {
    SpecTerm s;
    s.in = in; s.sr = sr; s.si = si; s.mult = mult; s.tab = t;
    return s;
  }
  int lin(double2* out, int acc, std::initializer_list<SpecTerm> ts) {
    SpecTerm t[3] = {term(nullptr, 0, 0, 0), term(nullptr, 0, 0, 0), term(nullptr, 0, 0, 0)};
    int k = 0;
    for (const auto& x : ts) t[k++] = x;
    k_spec_lin<<<grid_for(totS()), 256, 0, st>>>(g.n, g.kmax2, totS(), k, t[0], t[1], t[2], acc, out);
    QG_LAUNCHED();
    return QG_OK;
  }
  // C^T y = w_k F(y) on the retained modes
  int CTf(const double* y, double2* out) {
    int rc = d_r2c(y, Sb[6], g.n3);
    if (rc) return rc;
    k_ct_weights<<<grid_for(totS()), 256, 0, st>>>(g.n, g.kmax2, totS(), (double)g.n * g.n, Sb[6], 0, out);
    QG_LAUNCHED();
    return QG_OK;
  }
  // A_solver on a dense field
  int A_inv(const double2* in, double2* out) {
    k_dense_to_compact<double><<<grid_for((long long)g.n3 * g.plane), 256, 0, st>>>(g, 0, g.n3, in, tmpC[0]);
    QG_LAUNCHED();
    int rc = solve_generic(nullptr, tmpC[0], tmpC[0], nullptr, tmpC[1], tmpC[2], 0, 1);
    if (rc) return rc;
    k_compact_to_dense<double><<<grid_for(totS()), 256, 0, st>>>(g, 0, g.n3, tmpC[1], out, 0, cfg.dz);
    QG_LAUNCHED();
    return QG_OK;
  }

  int obj_first_level() const {
    int z0 = 0;
    while (z0 < g.n3 && ((double)z0 + 0.5) / g.n3 < 0.8) ++z0;
    return z0;
  }

  // J = 1/2 sum_W |C(B + kh^2 A/(4 Bu))|^2 at the engine's state
  // (diagnostics.f90:1698-1706 for LA); with grad, lamA = dJ/dX at the final X
  int objective_value(double* J, bool grad) {
    int rc;
    const double k4 = 0.25 / cfg.Bu;
    const int src[4] = {F_BR, F_BI, F_AR, F_AI};
    for (int i = 0; i < 4; ++i) {
      k_compact_to_dense<double><<<grid_for(totS()), 256, 0, st>>>(g, 0, g.n3, F[src[i]], Sb[i], 0, cfg.dz);
      QG_LAUNCHED();
    }
    // Sb[4], Sb[5]: LA of the real and imaginary parts
    if ((rc = lin(Sb[4], 0, {term(Sb[0], 1, 0, 0), term(Sb[2], k4, 0, 3)})) ||
        (rc = lin(Sb[5], 0, {term(Sb[1], 1, 0, 0), term(Sb[3], k4, 0, 3)})) || (rc = d_c2r(Sb[4], Pb[0], g.n3)) ||
        (rc = d_c2r(Sb[5], Pb[1], g.n3)))
      return rc;
    const int z0 = obj_first_level();
    k_obj_partial<<<kObjBlocks, 256, 0, st>>>(g.n, g.n3, z0, Pb[0], Pb[1], part);
    QG_LAUNCHED();
    QG_CK(cudaMemcpyAsync(part_h.data(), part, kObjBlocks * sizeof(double), cudaMemcpyDeviceToHost, st));
    QG_CK(cudaStreamSynchronize(st));
    double acc = 0.0;
    for (double v : part_h) acc += v;
    *J = 0.5 * acc;
    if (!grad) return QG_OK;
    for (int f = 0; f < 6; ++f) QG_CK(cudaMemsetAsync(lamA[f], 0, field_bytes(), st));
    for (int c = 0; c < 2; ++c) {
      k_obj_window<<<grid_for(totP()), 256, 0, st>>>(g.n, g.n3, z0, Pb[c]);
      QG_LAUNCHED();
      // dJ/dB = g + A_solver(kh^2/(4 Bu) g), g = C^T(W LA)
      if ((rc = CTf(Pb[c], Sb[0])) || (rc = lin(Sb[1], 0, {term(Sb[0], k4, 0, 3)})) || (rc = A_inv(Sb[1], Sb[2])) ||
          (rc = lin(Sb[3], 0, {term(Sb[0], 1, 0, 0), term(Sb[2], 1, 0, 0)})))
        return rc;
      k_dense_to_compact<double><<<grid_for((long long)g.n3 * g.plane), 256, 0, st>>>(g, 0, g.n3, Sb[3],
                                                                                    lamA[2 + c]);
      QG_LAUNCHED();
    }
    return QG_OK;
  }

  // ---- the transposed step --------------------------------------------------
  // lo = (d step / d X)^T li at the state whose q, BR, BI, psi are given
  int step_T(const C* q, const C* BR, const C* BI, const C* psi, bool first, const std::vector<C*>& li,
             const std::vector<C*>& lo) {
    if (sa_levels < Zb) {    // the batch depth can change with set_batch_levels
      if (SA) { QG_CK(cudaStreamSynchronize(st)); cudaFree(SA); SA = nullptr; sa_levels = 0; }
      QG_CK(cudaMalloc(&SA, (size_t)Zb * kNScr * g.n * g.KXP * sizeof(C)));
      sa_levels = Zb;
    }
    AdjP p;
    p.dt = cfg.delt;
    p.gam = cfg.gamma;
    p.cdisp = sp.disp ? 0.5 / (cfg.Bu * cfg.Ro) : 0.0;
    p.adv = sp.adv ? 1.0 : 0.0;
    p.refr = sp.refr ? 1.0 : 0.0;
    p.s = cfg.Ro * cfg.W2F;
    p.first = first ? 1 : 0;
    AdjIn L;
    AdjOut O;
    for (int f = 0; f < 6; ++f) { L.l[f] = li[f]; O.l[f] = lo[f]; }
    O.lpsi = Af[A_LPSI]; O.lAR = Af[A_LAR]; O.lAI = Af[A_LAI];
    for (int z0 = 0; z0 < g.n3; z0 += Zb) {
      const int zc = std::min(Zb, g.n3 - z0);
      QG_SWITCH_N(g.n, {
        const dim3 gc(g.KXP / Tiles<double, NN>::CT, zc), gr(g.n / Tiles<double, NN>::RT, zc);
        k_col_inv<double, NN><<<gc, Tiles<double, NN>::CNT, sm_ci<NN, Tiles<double, NN>::CIP>(Tiles<double, NN>::CINF), st>>>(g, z0, psi, q, BR, BI, S, tw, nullptr, 0);
        QG_LAUNCHED();
        k_adj_col_inv<NN><<<gc, kColThreads, sm_col6<NN>(), st>>>(g, p, z0, L, e1, e2, e1w, e2w, SA, tw);
        QG_LAUNCHED();
        k_adj_row<NN><<<gr, kThreadsB, sm_row7<NN>(), st>>>(g, p, S, SA, tw);
        QG_LAUNCHED();
        k_adj_col_fwd<NN><<<gc, kColThreads, sm_col6<NN>(), st>>>(g, p, z0, L, O, e1, e2, e1w, e2w, SA, tw);
        QG_LAUNCHED();
      });
    }
    int rc = solve_generic(Af[A_LPSI], Af[A_LAR], Af[A_LAI], Af[A_W], Af[A_LBRA], Af[A_LBIA], 1, 1);
    if (rc) return rc;
    for (int z0 = 0; z0 < g.n3; z0 += Zb) {
      const int zc = std::min(Zb, g.n3 - z0);
      QG_SWITCH_N(g.n, {
        const dim3 gc(g.KXP / Tiles<double, NN>::CT, zc), gr(g.n / Tiles<double, NN>::RT, zc);
        if (need_qw) {
          k_adj_qw_col_inv<NN><<<gc, kColThreads, sm_col6<NN>(), st>>>(g, z0, BR, BI, Af[A_W], S, tw);
          QG_LAUNCHED();
          k_adj_qw_row<NN><<<gr, kThreadsB, sm_row4<NN>(), st>>>(g, p, S, tw);
          QG_LAUNCHED();
        }
        k_adj_qw_col_fwd<NN><<<gc, kColThreads, sm_col4<NN>(), st>>>(g, z0, need_qw ? 1 : 0, lo[0], lo[2], lo[3],
                                                                     Af[A_W], Af[A_LBRA], Af[A_LBIA], S, tw);
        QG_LAUNCHED();
      });
    }
    return QG_OK;
  }
};

EngineBase* make_engine_fp64() { return new AdjEngine(); }

}  // namespace qg
