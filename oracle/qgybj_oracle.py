"""FP64 CPU restatement of one QG-YBJ+ time step (numpy + scipy.fft).

TEST INFRASTRUCTURE ONLY.  This module is the oracle the CUDA path is checked
against.  It may be imported by ``tests/``, by ``__graft_entry__.smoke()`` and
by the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` and by
nothing else; the product path never routes through it.

Parity status: **parity unpinned** against the Fortran reference itself.  The
reference (Fortran 90 + MPI + FFTW/MKL + LAPACK + netCDF) cannot be compiled in
this environment and ships no tests, fixtures or golden vectors.  The oracle is
pinned instead by known-answer tests that the reference's own discrete
operators imply (init_q <-> psi_solver round trip, single-mode FFTs, single-mode
Jacobians, DGTSV agreement with LAPACK, conservation of sum|B|^2 by advection
and refraction, linear dispersion rotation).

Array conventions (C order, identical in memory to the Fortran arrays):
  spectral  complex128[nz][ikty][iktx]  == Fortran kvar(iktx, ikty, nz)
  physical  float64  [nz][n2][n1]       == Fortran rvar(1:n1, n2, nz)
ky runs in FFT order: kya = [0 .. n/2-1, 0*, -n/2+1 .. -1] where 0* is the
ky = -n/2 row, forced to 0 and masked (init.f90:35-41).

Every function cites the reference routine (file:line) it restates.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field, replace

import numpy as np
import scipy.fft as sfft

_WORKERS = int(os.environ.get("QGYBJ_ORACLE_WORKERS", "1"))


def set_workers(n: int) -> None:
    """Threads used by scipy.fft inside the oracle (1 = scalar port)."""
    global _WORKERS
    _WORKERS = max(1, int(n))


# Floating type the 2D FFTs compute in: float64 (the reference's FFTW in
# double precision), or np.longdouble for a sensitivity check: the transforms
# then round differently (80-bit extended on x86-64) while every other
# operation stays FP64, so the difference between the two runs measures how
# far FP64 roundoff of the transforms alone carries through the step.
_FFT_DTYPE = np.float64


def set_fft_dtype(dtype) -> None:
    global _FFT_DTYPE
    _FFT_DTYPE = np.dtype(dtype).type


# ---------------------------------------------------------------------------
# L0: grid, dealiasing mask, base state, integrating-factor tables
# ---------------------------------------------------------------------------

def float32_round_int(m: int) -> float:
    """Correctly rounded (nearest-even) float32 value of a non-negative integer.

    Used for ``(1.*kx)**(2.*ilap)``: default-REAL power of an integer
    (main_waqg.f90:246-247, 371-372).  The exact integer power rounded once to
    float32 is what a correctly rounded powf returns.
    """
    if m < (1 << 24):
        return float(np.float32(m))
    e = m.bit_length() - 24
    q, r = divmod(m, 1 << e)
    half = 1 << (e - 1)
    if r > half or (r == half and (q & 1)):
        q += 1
    return float(np.float32(q * (1 << e)))


@dataclass
class Grid:
    """Wavenumbers, mask and kh^2 (init.f90:17-80, init_arrays)."""
    n1: int
    n2: int
    n3: int
    kxa: np.ndarray = field(init=False)
    kya: np.ndarray = field(init=False)
    L: np.ndarray = field(init=False)      # int32 [ikty][iktx]
    kh2: np.ndarray = field(init=False)    # int64 [ikty][iktx]
    kx: np.ndarray = field(init=False)     # float64 [1][iktx] broadcastable
    ky: np.ndarray = field(init=False)     # float64 [ikty][1]

    def __post_init__(self):
        n1, n2 = self.n1, self.n2
        if n1 != n2 or n1 % 2:
            raise ValueError("n1 must equal n2 and be even")
        iktx, ikty, kty = n1 // 2 + 1, n2, n2 // 2
        self.iktx, self.ikty = iktx, ikty
        self.kxa = np.arange(iktx, dtype=np.int64)
        kya = np.empty(ikty, dtype=np.int64)
        for iky in range(1, ikty + 1):          # init.f90:35-41
            jj = iky - 1
            if iky > kty:
                jj -= 2 * kty
            if iky == kty + 1:
                jj = 0
            if iky > 2 * kty:
                jj = 0
            kya[iky - 1] = jj
        self.kya = kya
        KX, KY = np.meshgrid(self.kxa, kya)      # [ikty][iktx]
        kh2 = KX * KX + KY * KY
        # init.f90:51-74: kh = sqrt(real(kx*kx+ky*ky)) in default REAL,
        # threshold ifix(float(n1)/3.+0.5)-0.5 in default REAL.
        kh = np.sqrt(kh2.astype(np.float32)).astype(np.float64)
        thr = float(int(np.float32(n1) / np.float32(3.0) + np.float32(0.5))) - 0.5
        L = np.ones((ikty, iktx), dtype=np.int32)
        twopi = 4.0 * math.asin(1.0)
        for iky in range(ikty):
            for ikx in range(iktx):
                kx, ky = int(KX[iky, ikx]), int(KY[iky, ikx])
                if iky + 1 == kty + 1:
                    L[iky, ikx] = 0
                elif kx < 0:
                    L[iky, ikx] = 0
                elif kx == 0 and ky < 0:
                    L[iky, ikx] = 0
                elif iky + 1 > 2 * kty:
                    L[iky, ikx] = 0
                elif (kh[iky, ikx] * twopi / twopi) > thr:
                    L[iky, ikx] = 0
        self.L = L
        self.kh2 = kh2
        self.kx = self.kxa.astype(np.float64)[None, :]
        self.ky = kya.astype(np.float64)[:, None]
        self.threshold = thr
        self.kmax = int(math.floor(thr))

    @property
    def Lb(self) -> np.ndarray:
        return self.L.astype(bool)


def integrating_factor(grid: Grid, delt: float, nuh1: float, nuh2: float,
                       ilap1: int, ilap2: int) -> np.ndarray:
    """int_factor per (ky, kx) (main_waqg.f90:246-247 and 371-372).

    ``delt*(nuh1*((1.*kx)**(2.*ilap1)+(1.*ky)**(2.*ilap1)) + nuh2*(...))``:
    each power and the inner sum are default REAL (float32); the products
    with nuh* and delt are double precision.
    """
    ikty, iktx = grid.L.shape
    out = np.empty((ikty, iktx), dtype=np.float64)
    px1 = [float32_round_int(int(k) ** (2 * ilap1)) for k in range(max(iktx, ikty))]
    px2 = [float32_round_int(int(k) ** (2 * ilap2)) for k in range(max(iktx, ikty))]
    for iky in range(ikty):
        ky = abs(int(grid.kya[iky]))
        for ikx in range(iktx):
            kx = int(grid.kxa[ikx])
            s1 = float(np.float32(px1[kx]) + np.float32(px1[ky]))
            s2 = float(np.float32(px2[kx]) + np.float32(px2[ky]))
            out[iky, ikx] = delt * (nuh1 * s1 + nuh2 * s2)
    return out


@dataclass
class Params:
    """Physical/numerical parameters (parameters_test1.f90:45-113)."""
    n1: int
    n2: int
    n3: int
    dz: float
    Bu: float
    Ro: float
    W2F: float
    delt: float
    gamma: float
    nuh1: float
    nuh2: float
    ilap1: int
    ilap2: int
    nuh1w: float
    nuh2w: float
    ilap1w: int
    ilap2w: int
    nuz: float
    a_ell_ut: np.ndarray          # [n3] Bu/N^2 at za(iz)=iz*dz (init.f90:253)
    rho_ut: np.ndarray | None = None
    rho_st: np.ndarray | None = None
    r_2ut: np.ndarray | None = None   # N^2 at za(iz) (wave PE diagnostic)
    inviscid: int = 1
    linear: int = 0
    no_dispersion: int = 0
    passive_scalar: int = 0
    fixed_flow: int = 0
    no_feedback: int = 0
    ybj_plus: int = 1

    def __post_init__(self):
        n3 = self.n3
        if self.rho_ut is None:
            self.rho_ut = np.ones(n3)
        if self.rho_st is None:
            self.rho_st = np.ones(n3)
        if self.r_2ut is None:
            self.r_2ut = self.Bu / np.asarray(self.a_ell_ut, dtype=np.float64)
        self.a_ell_ut = np.asarray(self.a_ell_ut, dtype=np.float64)


class Model:
    """Tables shared by all routines (init_arrays / init_base_state)."""

    def __init__(self, p: Params):
        if p.n3 < 2:
            raise ValueError("n3 must be >= 2")
        self.p = p
        self.grid = Grid(p.n1, p.n2, p.n3)
        g = self.grid
        IF = integrating_factor(g, p.delt, p.nuh1, p.nuh2, p.ilap1, p.ilap2)
        IFw = integrating_factor(g, p.delt, p.nuh1w, p.nuh2w, p.ilap1w, p.ilap2w)
        self.e1 = np.array([[math.exp(-x) for x in row] for row in IF])
        self.e2 = np.array([[math.exp(-2 * x) for x in row] for row in IF])
        self.e1w = np.array([[math.exp(-x) for x in row] for row in IFw])
        self.e2w = np.array([[math.exp(-2 * x) for x in row] for row in IFw])
        self.IF, self.IFw = IF, IFw
        self.Lb = g.Lb
        self.kh2f = g.kh2.astype(np.float64)

    # -- spectral transforms (fft.f90) -------------------------------------
    def fft_r2c(self, r: np.ndarray) -> np.ndarray:
        """fft.f90:55-66: per-level 2D r2c, then divided by n1*n2."""
        if _FFT_DTYPE is not np.float64:
            k = sfft.rfft2(r.astype(_FFT_DTYPE), axes=(-2, -1), norm="forward", workers=_WORKERS)
            return k.astype(np.complex128)
        return sfft.rfft2(r, axes=(-2, -1), norm="forward", workers=_WORKERS)

    def realit(self, k: np.ndarray) -> np.ndarray:
        """fft.f90:88-107: k(1, n-iky+2) = conj(k(1, iky)) for iky=2..n/2."""
        k = k.copy()
        n2 = self.p.n2
        m = np.arange(1, n2 // 2)
        k[..., n2 - m, 0] = np.conj(k[..., m, 0])
        return k

    def fft_c2r(self, k: np.ndarray) -> np.ndarray:
        """fft.f90:71-83: realit, then unnormalised per-level 2D c2r."""
        k = self.realit(k)
        if _FFT_DTYPE is not np.float64:
            kd = k.astype(np.result_type(_FFT_DTYPE, np.complex64))
            r = sfft.irfft2(kd, s=(self.p.n2, self.p.n1), axes=(-2, -1), norm="forward", workers=_WORKERS)
            return r.astype(np.float64)
        return sfft.irfft2(k, s=(self.p.n2, self.p.n1), axes=(-2, -1),
                           norm="forward", workers=_WORKERS)

    # -- transform-method terms (derivatives.f90) --------------------------
    def compute_velo(self, psik):
        """derivatives.f90:1295-1338 (u and v only; w=0, b unused by the step)."""
        g = self.grid
        uk = np.where(self.Lb, -(1j * g.ky) * psik, 0)
        vk = np.where(self.Lb, (1j * g.kx) * psik, 0)
        return uk, vk

    def _ik_combine(self, utermk, vtermk):
        g = self.grid
        return np.where(self.Lb, (1j * g.kx) * utermk + (1j * g.ky) * vtermk, 0)

    def convol_waqg(self, uk, vk, qk, BRk, BIk):
        """derivatives.f90:607-803: flux-form J(psi,X) for X = q, BR, BI."""
        ur, vr = self.fft_c2r(uk), self.fft_c2r(vk)
        out = []
        for X in (qk, BRk, BIk):
            xr = self.fft_c2r(X)
            ut = self.fft_r2c(ur * xr)
            vt = self.fft_r2c(vr * xr)
            out.append(self._ik_combine(ut, vt))
        return tuple(out)

    def refraction_waqg(self, BRk, BIk, psik):
        """derivatives.f90:810-900: rB = F(zeta*B), zeta = -kh^2 psi."""
        zetak = np.where(self.Lb, -self.kh2f * psik, 0)
        zr = self.fft_c2r(zetak)
        brr, bir = self.fft_c2r(BRk), self.fft_c2r(BIk)
        rBRk = np.where(self.Lb, self.fft_r2c(zr * brr), 0)
        rBIk = np.where(self.Lb, self.fft_r2c(zr * bir), 0)
        return rBRk, rBIk

    def compute_qw(self, BRk, BIk):
        """derivatives.f90:906-1032: Xie-Vanneste feedback q^w.

        The reference zeroes BRyk twice (line 936) and never zeroes BIyk; the
        intent (all four derivative fields zero where L=0) is taken here.
        """
        g, Lb = self.grid, self.Lb
        BRx = self.fft_c2r(np.where(Lb, (1j * g.kx) * BRk, 0))
        BRy = self.fft_c2r(np.where(Lb, (1j * g.ky) * BRk, 0))
        BIx = self.fft_c2r(np.where(Lb, (1j * g.kx) * BIk, 0))
        BIy = self.fft_c2r(np.where(Lb, (1j * g.ky) * BIk, 0))
        qwr = BRy * BIx - BRx * BIy
        brr, bir = self.fft_c2r(BRk), self.fft_c2r(BIk)
        tempk = self.fft_r2c(brr * brr + bir * bir)
        qwk = self.fft_r2c(qwr)
        qwk = np.where(Lb, qwk - 0.25 * self.kh2f * tempk, 0)
        return qwk * self.p.Ro * self.p.W2F

    def dissipation_q_nv(self, qok):
        """derivatives.f90:1877-1926: nuz * d2q/dz2 with one-sided ends."""
        nuz, dz = self.p.nuz, self.p.dz
        d = np.zeros_like(qok)
        d[1:-1] = nuz * (qok[2:] - 2.0 * qok[1:-1] + qok[:-2]) / (dz * dz)
        d[0] = nuz * (qok[1] - qok[0]) / (dz * dz)
        d[-1] = nuz * (qok[-2] - qok[-1]) / (dz * dz)
        return np.where(self.Lb, d, 0)

    def sumB(self, BRk, BIk):
        """derivatives.f90:1073-1118: remove the vertical mean of B where kh>0."""
        sel = self.Lb & (self.grid.kh2 > 0)
        n3 = self.p.n3
        aR = BRk.sum(axis=0) / n3
        aI = BIk.sum(axis=0) / n3
        return np.where(sel, BRk - aR, BRk), np.where(sel, BIk - aI, BIk)

    # -- vertical elliptic inversions (elliptic.f90) -----------------------
    def _tridiag(self, kh2dz2: np.ndarray):
        """Matrix of psi_solver / A_solver_ybj_plus (elliptic.f90:177-189)."""
        p = self.p
        a, ru, rs = p.a_ell_ut, p.rho_ut, p.rho_st
        n3 = p.n3
        ncol = kh2dz2.shape[0]
        d = np.empty((n3, ncol))
        du = np.empty((n3 - 1, ncol))
        dl = np.empty((n3 - 1, ncol))
        for iz in range(n3):
            if iz == 0:
                d[iz] = -(ru[0] * a[0] / rs[0] + kh2dz2)
                du[0] = ru[0] * a[0] / rs[0]
            elif iz == n3 - 1:
                d[iz] = -(ru[iz - 1] * a[iz - 1] / rs[iz] + kh2dz2)
                dl[iz - 1] = ru[iz - 1] * a[iz - 1] / rs[iz]
            else:
                d[iz] = -((ru[iz] * a[iz] + ru[iz - 1] * a[iz - 1]) / rs[iz] + kh2dz2)
                du[iz] = ru[iz] * a[iz] / rs[iz]
                dl[iz - 1] = ru[iz - 1] * a[iz - 1] / rs[iz]
        return dl, d, du

    def _solve_columns(self, rhs: np.ndarray, quarter: bool, scale: float):
        """Solve per (ky,kx) column; kh2==0 or L==0 columns are set to 0."""
        p, g = self.p, self.grid
        sel = self.Lb & (g.kh2 != 0)
        iy, ix = np.nonzero(sel)
        kh2 = g.kh2[iy, ix].astype(np.float64)
        if quarter:
            kh2dz2 = kh2 * p.dz * p.dz / 4.0
        else:
            kh2dz2 = kh2 * p.dz * p.dz
        cols = rhs[:, iy, ix]                      # [n3][ncol]
        br = scale * cols.real
        bi = scale * cols.imag
        dl, d, du = self._tridiag(kh2dz2)
        xr = dgtsv_nopivot(dl.copy(), d.copy(), du.copy(), br)
        xi = dgtsv_nopivot(dl, d, du, bi)
        out = np.zeros_like(rhs)
        out[:, iy, ix] = xr + 1j * xi
        return out

    def psi_solver(self, qstar):
        """elliptic.f90:145-247: d/dz(a dpsi/dz) - kh^2 psi = q*, Neumann ends."""
        dz = self.p.dz
        return self._solve_columns(qstar, quarter=False, scale=dz * dz)

    def A_solver_ybj_plus(self, Bk):
        """elliptic.f90:346-460: d/dz(a dA/dz) - kh^2/4 A = Bu B; C = A_z."""
        p = self.p
        Ak = self._solve_columns(Bk, quarter=True, scale=p.dz * p.dz * p.Bu)
        Ck = np.zeros_like(Ak)
        Ck[:-1] = (Ak[1:] - Ak[:-1]) / p.dz
        return Ak, Ck

    def init_q(self, psik):
        """init.f90:591-652: discrete q from psi (the psi_solver operator)."""
        p, g = self.p, self.grid
        a, ru, rs, dz = p.a_ell_ut, p.rho_ut, p.rho_st, p.dz
        n3 = p.n3
        kdz = self.kh2f * dz * dz
        q = np.zeros_like(psik)
        for iz in range(n3):
            if iz == 0:
                c0 = ru[0] * a[0] / rs[0]
                val = c0 * psik[1] - (c0 + kdz) * psik[0]
            elif iz == n3 - 1:
                cm = ru[iz - 1] * a[iz - 1] / rs[iz]
                val = -(cm + kdz) * psik[iz] + cm * psik[iz - 1]
            else:
                cp = ru[iz] * a[iz] / rs[iz]
                cm = ru[iz - 1] * a[iz - 1] / rs[iz]
                val = cp * psik[iz + 1] - ((ru[iz] * a[iz] + ru[iz - 1] * a[iz - 1]) / rs[iz] + kdz) * psik[iz] \
                    + cm * psik[iz - 1]
            q[iz] = np.where(self.Lb, val, 0)
        return q / (dz * dz)

    # -- the time step (main_waqg.f90) --------------------------------------
    def tendencies(self, s: "State"):
        """Nonlinear, refraction and dissipation terms of one step
        (main_waqg.f90:202-230 / 331-356)."""
        p = self.p
        uk, vk = self.compute_velo(s.psi)
        nq, nBR, nBI = self.convol_waqg(uk, vk, s.q, s.BR, s.BI)
        rBR, rBI = self.refraction_waqg(s.BR, s.BI, s.psi)
        dq = self.dissipation_q_nv(s.qo)
        if p.inviscid == 1:
            dq = np.zeros_like(dq)
        if p.linear == 1:
            nq = np.zeros_like(nq); nBR = np.zeros_like(nBR); nBI = np.zeros_like(nBI)
        AR, AI = s.AR, s.AI
        if p.no_dispersion == 1 or p.passive_scalar == 1:
            AR = np.zeros_like(AR); AI = np.zeros_like(AI)
        if p.passive_scalar == 1:
            rBR = np.zeros_like(rBR); rBI = np.zeros_like(rBI)
        return nq, nBR, nBI, rBR, rBI, dq, AR, AI

    def invert(self, s: "State", tend=None) -> "State":
        """q* = q - q^w, psi and A inversions (main_waqg.f90:421-462).
        Regular YBJ (ybj_plus = 0): sumB on B^{n+1}, then A from the vertical
        integral of B and sigma of this step's tendencies `tend` =
        (nBR, nBI, rBR, rBI) (main_waqg.f90:449-460)."""
        p = self.p
        psi, AR, AI, CR, CI = s.psi, s.AR, s.AI, s.CR, s.CI
        if p.fixed_flow == 0:
            if p.no_feedback == 1:
                qw = np.zeros_like(s.q)
            else:
                qw = self.compute_qw(s.BR, s.BI)
            qstar = np.where(self.Lb, s.q - qw, qw)
            psi = self.psi_solver(qstar)
        if p.passive_scalar == 0:
            if p.ybj_plus == 1:
                AR, CR = self.A_solver_ybj_plus(s.BR)
                AI, CI = self.A_solver_ybj_plus(s.BI)
            else:
                BR, BI = self.sumB(s.BR, s.BI)
                s = replace(s, BR=BR, BI=BI)
                sig1, sig2 = self.compute_sigma(*tend)
                AR, CR = self.compute_A(s.BR, sig1)
                AI, CI = self.compute_A(s.BI, sig2)
        return replace(s, psi=psi, AR=AR, AI=AI, CR=CR, CI=CI)

    # -- regular YBJ (ybj_plus = 0) ------------------------------------------
    def compute_sigma(self, nBR, nBI, rBR, rBI):
        """derivatives.f90:1037-1068: sigma = Bu Ro sum_z ((rBR + 2 nBI)/kh2,
        (rBI - 2 nBR)/kh2) where kh2 > 0 and L = 1 (vertical integral of A)."""
        p = self.p
        sel = self.Lb & (self.grid.kh2 > 0)
        kh2 = np.where(sel, self.kh2f, 1.0)
        s1 = np.zeros(nBR.shape[1:], dtype=complex)
        s2 = np.zeros(nBR.shape[1:], dtype=complex)
        for z in range(nBR.shape[0]):
            s1 = s1 + np.where(sel, (rBR[z] + 2 * nBI[z]) / kh2, 0)
            s2 = s2 + np.where(sel, (rBI[z] - 2 * nBR[z]) / kh2, 0)
        return s1 * p.Bu * p.Ro, s2 * p.Bu * p.Ro

    def compute_A(self, Bk, sigma):
        """derivatives.f90:1141-1264: A~(1) = 0, A~(iz) = A~(iz-1) + sumB r_2ut(iz-1) dz^2
        with sumB the running vertical sum of B; A = A~ + (sigma - sum A~)/n3 where
        kh2 > 0 and L = 1, else 0; C = A_z (0 at the top)."""
        p = self.p
        n3, dz = p.n3, p.dz
        r2 = np.asarray(p.r_2ut, dtype=np.float64)
        sel = self.Lb & (self.grid.kh2 > 0)
        At = np.zeros_like(Bk)
        sumB = Bk[0].copy()
        sumA = np.zeros(Bk.shape[1:], dtype=complex)
        for iz in range(1, n3):
            At[iz] = At[iz - 1] + sumB * r2[iz - 1] * dz * dz
            sumA = sumA + At[iz]
            sumB = sumB + Bk[iz]
        A = np.where(sel, At + (sigma - sumA) / n3, 0)
        C = np.zeros_like(A)
        C[:-1] = (A[1:] - A[:-1]) / dz
        return A, C

    def step_euler(self, s: "State") -> "State":
        """First step, forward Euler (main_waqg.f90:197-317)."""
        p = self.p
        nq, nBR, nBI, rBR, rBI, dq, AR, AI = self.tendencies(s)
        c = 0.5 / (p.Bu * p.Ro)
        kh2 = self.kh2f
        dt = p.delt
        qo, BRo, BIo = s.q, s.BR, s.BI
        q = (qo - dt * nq + dt * dq) * self.e1
        BR = (BRo - dt * nBR - dt * c * kh2 * AI + dt * 0.5 * rBI) * self.e1w
        BI = (BIo - dt * nBI + dt * c * kh2 * AR - dt * 0.5 * rBR) * self.e1w
        Lb = self.Lb
        q, BR, BI = (np.where(Lb, x, 0) for x in (q, BR, BI))
        s2 = replace(s, q=q, BR=BR, BI=BI, qo=qo.copy(), BRo=BRo.copy(), BIo=BIo.copy())
        return self.invert(s2, (nBR, nBI, rBR, rBI))

    def step_leapfrog(self, s: "State") -> "State":
        """Leapfrog + Robert-Asselin filter (main_waqg.f90:326-467)."""
        p = self.p
        nq, nBR, nBI, rBR, rBI, dq, AR, AI = self.tendencies(s)
        c = 0.5 / (p.Bu * p.Ro)
        kh2 = self.kh2f
        dt2 = 2 * p.delt
        e1, e2, e1w, e2w = self.e1, self.e2, self.e1w, self.e2w
        qt = s.qo * e2 - dt2 * nq * e1 + dt2 * dq * e2
        BRt = s.BRo * e2w - dt2 * (nBR + c * kh2 * AI - 0.5 * rBI) * e1w
        BIt = s.BIo * e2w - dt2 * (nBI - c * kh2 * AR + 0.5 * rBR) * e1w
        Lb = self.Lb
        qt, BRt, BIt = (np.where(Lb, x, 0) for x in (qt, BRt, BIt))
        g = p.gamma
        qo = np.where(Lb, s.q + g * (s.qo - 2 * s.q + qt), 0)
        BRo = np.where(Lb, s.BR + g * (s.BRo - 2 * s.BR + BRt), 0)
        BIo = np.where(Lb, s.BI + g * (s.BIo - 2 * s.BI + BIt), 0)
        s2 = replace(s, q=qt, BR=BRt, BI=BIt, qo=qo, BRo=BRo, BIo=BIo)
        return self.invert(s2, (nBR, nBI, rBR, rBI))

    def step(self, s: "State", first: bool) -> "State":
        return self.step_euler(s) if first else self.step_leapfrog(s)

    def run(self, s: "State", nsteps: int, first: bool = True) -> "State":
        for i in range(nsteps):
            s = self.step(s, first and i == 0)
        return s

    # -- output path: real-space FP32 fields of the netCDF dumps -------------
    def dump_psi(self, psik: np.ndarray, U_scale: float, L_scale: float) -> np.ndarray:
        """ncdump_psi (IO_ncf.f90:35-58): c2r of psi, times U_scale*L_scale
        (left to right in FP64), rounded to FP32; [nz][n2][n1], x fastest."""
        r = self.fft_c2r(psik)
        return ((r * U_scale) * L_scale).astype(np.float32)

    def la_from_b(self, Bk: np.ndarray, Ak: np.ndarray) -> np.ndarray:
        """YBJ+ B -> LA on the retained modes (diagnostics.f90:1698-1727):
        LA = B + 0.25*kh2*A/Bu, evaluated left to right; zero where L=0."""
        return np.where(self.Lb, Bk + ((0.25 * self.kh2f) * Ak) / self.p.Bu, 0)

    def dump_la(self, BRk, BIk, ARk, AIk, Uw_scale: float, la: bool):
        """ncdump_la (IO_ncf.f90:137-158): c2r of BR and BI (or of LA when
        `la`), times Uw_scale, rounded to FP32; [nz][n2][n1] each."""
        if la:
            BRk, BIk = self.la_from_b(BRk, ARk), self.la_from_b(BIk, AIk)
        return ((self.fft_c2r(BRk) * Uw_scale).astype(np.float32),
                (self.fft_c2r(BIk) * Uw_scale).astype(np.float32))

    # -- omega equation (vertical velocity diagnostic) ----------------------
    def omega_eqn_rhs(self, psik):
        """derivatives.f90:1469-1586: rhs = r2c(2 (bx xy - by xx)) with
        bx, by = i kx, i ky psi_z; xx, xy = -i kx, -i ky kh2 psi_avg on the
        unstaggered level between z and z+1 (psi_z = 0, psi_avg = psi at the top)."""
        g, Lb, dz = self.grid, self.Lb, self.p.dz
        kx, ky, kh2 = g.kx, g.ky, self.kh2f
        rz = np.zeros_like(psik)
        rz[:-1] = np.where(Lb, (psik[1:] - psik[:-1]) / dz, 0)
        bx = np.where(Lb, 1j * kx * rz, 0)
        by = np.where(Lb, 1j * ky * rz, 0)
        xx = np.zeros_like(psik)
        xy = np.zeros_like(psik)
        xx[:-1] = np.where(Lb, -1j * kx * kh2 * 0.5 * (psik[1:] + psik[:-1]), 0)
        xy[:-1] = np.where(Lb, -1j * ky * kh2 * 0.5 * (psik[1:] + psik[:-1]), 0)
        xx[-1] = np.where(Lb, -1j * kx * kh2 * psik[-1], 0)
        xy[-1] = np.where(Lb, -1j * ky * kh2 * psik[-1], 0)
        bxr, byr, xxr, xyr = (self.fft_c2r(a) for a in (bx, by, xx, xy))
        return self.fft_r2c(2.0 * (bxr * xyr - byr * xxr))

    def omega_equation(self, rhs):
        """elliptic.f90:463-567: per column (kh2 != 0, L = 1) the n3-1
        unstaggered levels, d = -(rho_ut(rho_st1 + rho_st0)/(rho_st1 rho_st0)
        + dz^2 kh2/a), du = rho_ut(iz+1)/rho_st(iz+1), dl = rho_ut(iz-1)/rho_st(iz),
        rhs dz^2 q, DGTSV; w = 0 at the top level and elsewhere."""
        p, g = self.p, self.grid
        n3, dz = p.n3, p.dz
        a = np.asarray(p.a_ell_ut, dtype=np.float64)
        ru = np.asarray(p.rho_ut, dtype=np.float64) * np.ones(n3)
        rs = np.asarray(p.rho_st, dtype=np.float64) * np.ones(n3)
        w = np.zeros_like(rhs)
        act = self.Lb & (g.kh2 != 0)
        if n3 < 2 or not act.any():
            return w
        kh2 = g.kh2[act].astype(np.float64)
        m = n3 - 1
        t1 = (ru[:m] * (rs[1:] + rs[:m])) / (rs[1:] * rs[:m])
        d = np.stack([-(t1[i] + ((dz * dz) * kh2) / a[i]) for i in range(m)])
        du = np.array([ru[i + 1] / rs[i + 1] for i in range(m - 1)])[:, None] * np.ones_like(kh2)
        dl = np.array([ru[i] / rs[i + 1] for i in range(m - 1)])[:, None] * np.ones_like(kh2)
        br = (dz * dz) * rhs[:m].real[:, act]
        bi = (dz * dz) * rhs[:m].imag[:, act]
        xr = dgtsv_nopivot(dl.copy(), d.copy(), du.copy(), br)
        xi = dgtsv_nopivot(dl.copy(), d.copy(), du.copy(), bi)
        w[:m][:, act] = xr + 1j * xi
        return w

    # -- FP64 diagnostics (diagnostics.f90) ---------------------------------
    def diagnostics(self, s: "State") -> dict:
        """Domain-integrated energies and enstrophy.

        wave_energy (diagnostics.f90:647-743): WKE, WPE, WCE without the
        Uw_scale^2 factor; diag_zentrum rotational part (16-211): flow KE and
        PE from psi; enstrophy (1262-1363): <zeta_z^2> and <omega_H^2>.
        Each vertical sum is divided by n3.  Accumulation is FP64.
        """
        p, g, Lb = self.p, self.grid, self.Lb
        kh2 = self.kh2f
        n3, dz, Bu = p.n3, p.dz, p.Bu
        ab = lambda z: (z.real * z.real + z.imag * z.imag)
        Lf = Lb.astype(np.float64)
        # waves
        kz = (ab(s.BR) + ab(s.BI)) * Lf
        k_p = kz.sum(axis=(1, 2)) - 0.5 * (ab(s.BR[:, 0, 0]) + ab(s.BI[:, 0, 0]))
        r2 = np.asarray(p.r_2ut)
        p_p = ((0.5 / (r2 * Bu))[:, None, None] * (kh2 * (ab(s.CR) + ab(s.CI))) * Lf).sum(axis=(1, 2))
        c_p = ((1.0 / 8.0) * (1.0 / (Bu * Bu)) * kh2 * kh2 * (ab(s.AR) + ab(s.AI)) * Lf).sum(axis=(1, 2))
        # flow (rotational part of diag_zentrum)
        ke = (kh2 * ab(s.psi) * Lf).sum(axis=(1, 2))
        b = np.zeros_like(s.psi)
        b[:-1] = (s.psi[1:] - s.psi[:-1]) / dz
        pe = ((Bu / r2)[:, None, None] * ab(b) * Lf).sum(axis=(1, 2))
        pe = pe - 0.5 * (Bu / r2) * ab(b[:, 0, 0])
        # enstrophy: zeta_z = -kh2 psi; omega_H from vertical shear of (u,v)
        ws = (2.0 * kh2 * kh2 * ab(s.psi) * Lf).sum(axis=(1, 2))
        wu = (2.0 * kh2 * ab(b) * Lf).sum(axis=(1, 2))
        wu[-1] = 0.0
        return {
            "wke": float(k_p.sum() / n3), "wpe": float(p_p.sum() / n3), "wce": float(c_p.sum() / n3),
            "ke": float(ke.sum() / n3), "pe": float(pe.sum() / n3),
            "zeta2": float(ws.sum() / n3), "omegah2": float(wu.sum() / n3),
        }


def dgtsv_nopivot(dl, d, du, b):
    """LAPACK DGTSV (NRHS=1) elimination order, vectorised over columns.

    Gaussian elimination of a tridiagonal system as published in LAPACK's
    dgtsv: FACT = DL(I)/D(I); D(I+1) -= FACT*DU(I); B(I+1) -= FACT*B(I); then
    back substitution B(N) /= D(N); B(I) = (B(I) - DU(I)*B(I+1)) / D(I).  The
    matrices of psi_solver / A_solver_ybj_plus are diagonally dominant, so the
    row-interchange branch of DGTSV is never taken; this is asserted.  A zero
    pivot raises (DGTSV's INFO > 0, elliptic.f90:192).  Inputs are modified.
    """
    n = d.shape[0]
    b = np.array(b, dtype=np.float64, copy=True)
    for i in range(n - 1):
        if np.any(np.abs(d[i]) < np.abs(dl[i])):
            raise ArithmeticError("row interchange required (matrix not diagonally dominant)")
        if np.any(d[i] == 0):
            raise ZeroDivisionError(f"DGTSV zero pivot at row {i + 1}")
        fact = dl[i] / d[i]
        d[i + 1] = d[i + 1] - fact * du[i]
        b[i + 1] = b[i + 1] - fact * b[i]
    if np.any(d[n - 1] == 0):
        raise ZeroDivisionError(f"DGTSV zero pivot at row {n}")
    b[n - 1] = b[n - 1] / d[n - 1]
    if n > 1:
        b[n - 2] = (b[n - 2] - du[n - 2] * b[n - 1]) / d[n - 2]
    for i in range(n - 3, -1, -1):
        b[i] = (b[i] - du[i] * b[i + 1]) / d[i]
    return b


@dataclass
class State:
    """Prognostic and diagnostic spectral fields (main_waqg.f90:15-60)."""
    q: np.ndarray
    qo: np.ndarray
    BR: np.ndarray
    BI: np.ndarray
    BRo: np.ndarray
    BIo: np.ndarray
    psi: np.ndarray
    AR: np.ndarray
    AI: np.ndarray
    CR: np.ndarray
    CI: np.ndarray

    FIELDS = ("q", "qo", "BR", "BI", "BRo", "BIo", "psi", "AR", "AI", "CR", "CI")

    def copy(self) -> "State":
        return State(**{f: getattr(self, f).copy() for f in self.FIELDS})


def initial_state(model: Model, psik: np.ndarray, BRk: np.ndarray,
                  BIk: np.ndarray | None = None, apply_sumB: bool = True) -> State:
    """Initialisation sequence of main_waqg.f90:125-147 on given psi and B:
    sumB, A=0 at t=0 replaced by the A inversion of B, q = init_q(psi)."""
    if BIk is None:
        BIk = np.zeros_like(BRk)
    if apply_sumB:
        BRk, BIk = model.sumB(BRk, BIk)
    q = model.init_q(psik) if model.p.fixed_flow == 0 else np.zeros_like(psik)
    z = np.zeros_like(psik)
    s = State(q=q, qo=q.copy(), BR=BRk.copy(), BI=BIk.copy(), BRo=BRk.copy(), BIo=BIk.copy(),
              psi=psik.copy(), AR=z.copy(), AI=z.copy(), CR=z.copy(), CI=z.copy())
    if model.p.passive_scalar == 0 and model.p.ybj_plus == 1:
        AR, CR = model.A_solver_ybj_plus(s.BR)
        AI, CI = model.A_solver_ybj_plus(s.BI)
        s = replace(s, AR=AR, AI=AI, CR=CR, CI=CI)
    # regular YBJ: A at t = 0 is the initial-condition field (zero here unless
    # the caller sets it), as generate_fields_stag provides it (main_waqg.f90:124-127)
    return s
