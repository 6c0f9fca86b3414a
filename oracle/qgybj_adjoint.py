"""FP64 CPU adjoint of the QG-YBJ+ step — TEST INFRASTRUCTURE ONLY.

The reverse-mode derivative of the step restated in oracle/qgybj_oracle.py,
built from the exact transposes of its primitives, used to check the CUDA
adjoint.  The reference has no adjoint; what is differentiated is the step of
main_waqg.f90:197-467 (YBJ+, inviscid vertical diffusion) with the carried
state X = (q, q_old, B, B_old) and psi, A derived from it.

Inner products: spectral vectors hold the L=1 modes, <X, Y> = sum Re(conj X) Y
over those modes (real and imaginary parts as independent reals); physical
fields use sum x*y over the grid.

Primitives and transposes (N = n1 = n2):
  C   (c2r of a masked spectrum, realit included):  C^T y = mask(2 N^2 R y),
      except the (0,0) mode: N^2 Re(R y)_00 (its imaginary part does not enter C)
  P R (r2c then mask):                            (P R)^T Y = C(Y') / (2 N^2),
      Y' = Y with the (0,0) entry doubled
  multiplication by i k:                          transpose = multiplication by -i k
  real multipliers, masks:                        self-adjoint
  psi_solver / A_solver (symmetric matrices):     self-adjoint
"""
from __future__ import annotations

import numpy as np

from .qgybj_oracle import Model, State


class Adjoint:
    def __init__(self, model: Model):
        if not (np.all(np.asarray(model.p.rho_ut) == 1) and np.all(np.asarray(model.p.rho_st) == 1)):
            raise ValueError("the adjoint uses the symmetry of the vertical operators (rho = 1)")
        self.m = model
        g = model.grid
        self.N2 = float(model.p.n1 * model.p.n2)
        self.Lb = model.Lb
        self.kx, self.ky, self.kh2 = g.kx, g.ky, model.kh2f

    # -- primitives ---------------------------------------------------------
    def mask(self, X):
        return np.where(self.Lb, X, 0)

    def C(self, X):
        return self.m.fft_c2r(self.mask(X))

    def CT(self, y):
        Y = self.m.fft_r2c(y)
        out = 2.0 * self.N2 * Y
        out[..., 0, 0] = self.N2 * Y[..., 0, 0].real
        return self.mask(out)

    def R(self, x):
        return self.mask(self.m.fft_r2c(x))

    def RT(self, Y):
        Y = self.mask(Y).copy()
        Y[..., 0, 0] = 2.0 * Y[..., 0, 0].real
        return self.m.fft_c2r(Y) / (2.0 * self.N2)

    def psi_inv(self, X):      # psi = M^-1 dz^2 X (psi_solver), symmetric
        return self.m.psi_solver(X)

    def A_inv(self, X):        # A = M_A^-1 dz^2 Bu X (A_solver_ybj_plus), symmetric
        return self.m.A_solver_ybj_plus(X)[0]

    # -- forward pieces (same arithmetic as the oracle) -----------------------
    def derived(self, q, BR, BI):
        p = self.m.p
        qw = self.m.compute_qw(BR, BI) if p.no_feedback == 0 else np.zeros_like(q)
        psi = self.psi_inv(self.mask(q - qw)) if p.fixed_flow == 0 else None
        return psi, self.A_inv(BR), self.A_inv(BI)

    def step(self, X, first: bool):
        """X = (q, r, BR, BI, cR, cI) -> next X (r, c: filtered old levels)."""
        q, r, BR, BI, cR, cI = X
        psi, AR, AI = self.derived(q, BR, BI)
        s = State(q=q, qo=(q if first else r), BR=BR, BI=BI, BRo=(BR if first else cR), BIo=(BI if first else cI),
                  psi=psi, AR=AR, AI=AI, CR=np.zeros_like(q), CI=np.zeros_like(q))
        m = self.m
        s2 = m.step_euler(s) if first else m.step_leapfrog(s)
        return (s2.q, s2.qo, s2.BR, s2.BI, s2.BRo, s2.BIo)

    # -- adjoint of the derived fields ---------------------------------------
    def derived_T(self, q, BR, BI, lpsi, lAR, lAI):
        """Transpose of (q, BR, BI) -> (psi, AR, AI) at the given state."""
        p, m = self.m.p, self.m
        lq = np.zeros_like(q)
        lBR = self.A_inv(lAR)
        lBI = self.A_inv(lAI)
        if p.fixed_flow == 0 and lpsi is not None:
            w = self.mask(self.psi_inv(self.mask(lpsi)))
            lq = lq + w
            if p.no_feedback == 0:
                dR, dI = self.qw_T(BR, BI, -w)
                lBR, lBI = lBR + dR, lBI + dI
        return lq, lBR, lBI

    def qw_T(self, BR, BI, lqw):
        """Transpose of the linearisation of compute_qw at (BR, BI)."""
        p = self.m.p
        kx, ky, kh2 = self.kx, self.ky, self.kh2
        s = p.Ro * p.W2F
        C, CT = self.C, self.CT
        BRx, BRy = C(1j * kx * BR), C(1j * ky * BR)
        BIx, BIy = C(1j * kx * BI), C(1j * ky * BI)
        brr, bir = C(BR), C(BI)
        lP1 = self.RT(s * lqw)                       # qw = s P R(P1) - s 1/4 kh2 P R(P2)
        lP2 = self.RT(-0.25 * kh2 * s * lqw)
        # P1 = BRy BIx - BRx BIy ; P2 = BR^2 + BI^2
        lBRy, lBIx = lP1 * BIx, lP1 * BRy
        lBRx, lBIy = -lP1 * BIy, -lP1 * BRx
        lbr, lbi = 2.0 * brr * lP2, 2.0 * bir * lP2
        lBR = -1j * kx * CT(lBRx) - 1j * ky * CT(lBRy) + CT(lbr)
        lBI = -1j * kx * CT(lBIx) - 1j * ky * CT(lBIy) + CT(lbi)
        return self.mask(lBR), self.mask(lBI)

    # -- adjoint of one step ---------------------------------------------------
    def step_T(self, X, first: bool, lX):
        """Transpose of the step's Jacobian at X applied to lX (both 6-tuples)."""
        m, p = self.m, self.m.p
        q, r, BR, BI, cR, cI = X
        lq1, lr1, lBR1, lBI1, lcR1, lcI1 = (self.mask(a) for a in lX)
        psi, AR, AI = self.derived(q, BR, BI)
        g = p.gamma
        dt = p.delt
        c = 0.5 / (p.Bu * p.Ro)
        kx, ky, kh2 = self.kx, self.ky, self.kh2
        e1, e2, e1w, e2w = m.e1, m.e2, m.e1w, m.e2w
        lq = np.zeros_like(q); lr = np.zeros_like(q)
        lBR = np.zeros_like(q); lBI = np.zeros_like(q)
        lcR = np.zeros_like(q); lcI = np.zeros_like(q)
        if first:
            # r1 = q0, c1 = B0; q1 = e1 (q0 - dt Nq); B1 = e1w (B0 - dt TB)
            lq += lr1; lBR += lcR1; lBI += lcI1
            lqp, lBRp, lBIp = lq1, lBR1, lBI1
            lq += e1 * lqp; lBR += e1w * lBRp; lBI += e1w * lBIp
            lNq = -dt * e1 * lqp
            lTR = -dt * e1w * lBRp
            lTI = -dt * e1w * lBIp
        else:
            # filter: r1 = q + g (r - 2 q + q1); c1 likewise
            lq += (1 - 2 * g) * lr1; lr += g * lr1
            lBR += (1 - 2 * g) * lcR1; lcR += g * lcR1
            lBI += (1 - 2 * g) * lcI1; lcI += g * lcI1
            lqp = lq1 + g * lr1
            lBRp = lBR1 + g * lcR1
            lBIp = lBI1 + g * lcI1
            # leapfrog: q1 = e2 r - 2dt e1 Nq ; BR1 = e2w cR - 2dt e1w (NBR + c kh2 AI - rBI/2) ...
            lr += e2 * lqp; lcR += e2w * lBRp; lcI += e2w * lBIp
            lNq = -2 * dt * e1 * lqp
            lTR = -2 * dt * e1w * lBRp
            lTI = -2 * dt * e1w * lBIp
        lNq, lTR, lTI = (self.mask(a) for a in (lNq, lTR, lTI))
        # TR = NBR + c kh2 AI - rBI/2 ; TI = NBI - c kh2 AR + rBR/2
        if p.linear == 1:
            lNq = np.zeros_like(lNq); lNBR = np.zeros_like(lNq); lNBI = np.zeros_like(lNq)
        else:
            lNBR, lNBI = lTR, lTI
        disp = 0.0 if (p.no_dispersion or p.passive_scalar) else 1.0
        lAI = disp * c * kh2 * lTR
        lAR = -disp * c * kh2 * lTI
        refr = 0.0 if p.passive_scalar else 1.0
        lrBI = -0.5 * refr * lTR
        lrBR = 0.5 * refr * lTI
        # physical fields of step n
        C, CT, RT = self.C, self.CT, self.RT
        u, v, Z = C(-1j * ky * psi), C(1j * kx * psi), C(-kh2 * psi)
        Qp, BRp, BIp = C(q), C(BR), C(BI)
        lu = np.zeros_like(u); lv = np.zeros_like(u); lZ = np.zeros_like(u)
        lQ = np.zeros_like(u); lBRr = np.zeros_like(u); lBIr = np.zeros_like(u)
        for lN, Xp, lXp in ((lNq, Qp, lQ), (lNBR, BRp, lBRr), (lNBI, BIp, lBIr)):
            lUX = RT(-1j * kx * lN)          # N = P[ikx R(u X) + iky R(v X)]
            lVX = RT(-1j * ky * lN)
            lu += lUX * Xp; lv += lVX * Xp
            lXp += lUX * u + lVX * v
        lZBR, lZBI = RT(lrBR), RT(lrBI)      # rB = P R(Z B)
        lZ += lZBR * BRp + lZBI * BIp
        lBRr += lZBR * Z; lBIr += lZBI * Z
        lq += CT(lQ); lBR += CT(lBRr); lBI += CT(lBIr)
        lpsi = 1j * ky * CT(lu) - 1j * kx * CT(lv) - kh2 * CT(lZ)   # transposes of -i ky, i kx, -kh2
        dq, dR, dI = self.derived_T(q, BR, BI, self.mask(lpsi), self.mask(lAR), self.mask(lAI))
        lq += dq; lBR += dR; lBI += dI
        return tuple(self.mask(a) for a in (lq, lr, lBR, lBI, lcR, lcI))


def inner(a, b, Lb) -> float:
    """Euclidean inner product of two tuples of masked spectral fields."""
    return float(sum(np.sum(np.where(Lb, (np.conj(x) * y).real, 0.0)) for x, y in zip(a, b)))


# ---------------------------------------------------------------------------
# objective and reverse sweep with checkpoints
# ---------------------------------------------------------------------------
def subvolume_mask(n: int, n3: int) -> np.ndarray:
    """Central quarter of the horizontal domain (x, y in [n/4, 3n/4)) and the
    top 20 % of the depth (staggered levels zs >= 0.8), float [n3][n][n]."""
    W = np.zeros((n3, n, n))
    zs = (np.arange(n3) + 0.5) / n3
    W[np.ix_(zs >= 0.8, np.arange(n // 4, 3 * n // 4), np.arange(n // 4, 3 * n // 4))] = 1.0
    return W


class Objective:
    """J = sum over the subvolume of 1/2 |LA|^2, LA = B + kh^2 A / (4 Bu)
    (diagnostics.f90:1698-1706), in physical space."""

    def __init__(self, adj: Adjoint):
        self.a = adj
        p = adj.m.p
        self.W = subvolume_mask(p.n1, p.n3)
        self.k = 0.25 * adj.kh2 / p.Bu

    def value(self, BR, BI) -> float:
        a = self.a
        LR = a.C(BR + self.k * a.A_inv(BR))
        LI = a.C(BI + self.k * a.A_inv(BI))
        return 0.5 * float(np.sum(self.W * (LR * LR + LI * LI)))

    def grad(self, BR, BI):
        a = self.a
        out = []
        for B in (BR, BI):
            g = a.CT(self.W * a.C(B + self.k * a.A_inv(B)))
            out.append(a.mask(g + a.A_inv(self.k * g)))
        return out


def run_forward(adj: Adjoint, q0, BR0, BI0, nsteps: int):
    X = (q0, q0, BR0, BI0, BR0, BI0)
    traj = [X]
    for i in range(nsteps):
        X = adj.step(X, i == 0)
        traj.append(X)
    return traj


def gradient(adj: Adjoint, q0, BR0, BI0, nsteps: int, every: int = 10):
    """J after nsteps and its gradient with respect to (q0, BR0, BI0), with
    checkpoints every `every` steps and recomputation inside each segment."""
    obj = Objective(adj)
    ck = {0: (q0, q0, BR0, BI0, BR0, BI0)}
    X = ck[0]
    for i in range(nsteps):
        X = adj.step(X, i == 0)
        if (i + 1) % every == 0 and i + 1 < nsteps:
            ck[i + 1] = X
    J = obj.value(X[2], X[3])
    gR, gI = obj.grad(X[2], X[3])
    z = np.zeros_like(q0)
    lX = (z, z, gR, gI, z, z)
    for s0 in sorted(ck, reverse=True):
        s1 = min(s0 + every, nsteps)
        seg = [ck[s0]]
        for i in range(s0, s1 - 1):
            seg.append(adj.step(seg[-1], i == 0))
        for i in range(s1 - 1, s0 - 1, -1):
            lX = adj.step_T(seg[i - s0], i == 0, lX)
    lq, lr, lBR, lBI, lcR, lcI = lX
    return J, (adj.mask(lq + lr), adj.mask(lBR + lcR), adj.mask(lBI + lcI))
