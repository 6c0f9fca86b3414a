"""Known-answer tests that pin the FP64 oracle (CPU only).

The reference ships no tests or golden vectors, so the oracle is pinned by
identities its own discrete operators imply."""
from __future__ import annotations

import math

import numpy as np
import pytest
import scipy.linalg.lapack as lapack

from oracle import qgybj_oracle as orc
from qgybj.config import CONFIGS, dealias_mask, kmax, model_parameters, scaled
from tests.helpers import oracle_for, oracle_params, random_masked, rel_l2


def small_model(n=32, n3=16, strat="constant", **flags):
    rc = scaled(CONFIGS["c1" if strat == "exponential" else "c0"], n, n3)
    return oracle_for(rc, **flags)


# --- L0: grid and tables -----------------------------------------------------
@pytest.mark.parametrize("n", [16, 32, 64, 128, 256, 512])
def test_mask_is_two_thirds_disk(n):
    g = orc.Grid(n, n, 4)
    thr = int(np.float32(n) / np.float32(3.0) + np.float32(0.5)) - 0.5
    kx, ky = np.meshgrid(g.kxa, g.kya)
    expect = (kx * kx + ky * ky < thr * thr) & ~((kx == 0) & (ky < 0))
    expect[n // 2, :] = False
    assert (g.L.astype(bool) == expect).all()
    assert g.kmax == kmax(n) == math.floor(thr)
    assert (dealias_mask(n) == g.L.astype(bool)).all()
    assert g.kya[n // 2] == 0 and g.kya[n - 1] == -1 and g.kya[n // 2 - 1] == n // 2 - 1


def test_retained_fraction_512():
    g = orc.Grid(512, 512, 2)
    assert int(g.L.sum()) == 45681


def test_float32_power_rounding():
    for k in range(0, 600, 7):
        for e in (2, 4, 12):
            exact = k ** e
            got = orc.float32_round_int(exact)
            # nearest float32: no other float32 is closer
            f = np.float32(got)
            up = np.nextafter(f, np.float32(np.inf))
            dn = np.nextafter(f, np.float32(0))
            assert abs(float(f) - exact) <= abs(float(up) - exact)
            assert abs(float(f) - exact) <= abs(float(dn) - exact)


def test_integrating_factor_values():
    g = orc.Grid(64, 64, 4)
    IF = orc.integrating_factor(g, 0.5, 1e-3, 2e-9, 2, 6)
    # kx=3, ky=-5
    iky = int(np.nonzero(g.kya == -5)[0][0])
    s1 = float(np.float32(81.0) + np.float32(625.0))
    s2 = float(np.float32(3.0 ** 12) + np.float32(5.0 ** 12))
    assert IF[iky, 3] == 0.5 * (1e-3 * s1 + 2e-9 * s2)


# --- L2: transforms ------------------------------------------------------------
def test_fft_single_mode():
    m, s, ic, p = small_model(16, 2)
    n = 16
    x = 2 * np.pi * np.arange(n) / n
    X, Y = np.meshgrid(x, x)  # [y][x]
    r = np.stack([np.sin(X) * np.sin(Y), np.cos(2 * X)])
    k = m.fft_r2c(r)
    # sin x sin y = -(1/4)(e^{i(x+y)} - e^{i(x-y)} - e^{-i(x-y)} + e^{-i(x+y)})
    assert abs(k[0, 1, 1] - (-0.25)) < 1e-15
    assert abs(k[0, n - 1, 1] - 0.25) < 1e-15
    assert abs(k[1, 0, 2] - 0.5) < 1e-15
    k2 = k.copy()
    k2[0, 1, 1] = 0; k2[0, n - 1, 1] = 0; k2[1, 0, 2] = 0
    assert np.abs(k2).max() < 1e-15
    assert np.abs(m.fft_c2r(k) - r).max() < 1e-14


def test_fft_roundtrip_masked():
    m, s, ic, p = small_model(32, 3)
    k = random_masked(32, 3, 7)
    k[:, 0, 0] = k[:, 0, 0].real
    back = m.fft_r2c(m.fft_c2r(k))
    assert rel_l2(np.where(m.Lb, back, 0), k) < 1e-14


def test_realit_kx0_column():
    m, s, ic, p = small_model(16, 2)
    k = np.zeros((1, 16, 9), complex)
    k[0, 3, 0] = 2 + 1j
    r = m.fft_c2r(k)
    y = 2 * np.pi * np.arange(16) / 16
    expect = 2 * np.real((2 + 1j) * np.exp(1j * 3 * y))[:, None] * np.ones((1, 16))
    assert np.abs(r[0] - expect).max() < 1e-13


# --- L3: transform-method terms --------------------------------------------
def test_jacobian_single_modes():
    """psi = cos x, q = cos y: J(psi,q) = psi_x q_y - psi_y q_x = sin x sin y."""
    m, s, ic, p = small_model(16, 2)
    n = 16
    psi = np.zeros((1, n, 9), complex); psi[0, 0, 1] = 0.5
    q = np.zeros((1, n, 9), complex); q[0, 1, 0] = 0.5
    uk, vk = m.compute_velo(psi)
    nq, _, _ = m.convol_waqg(uk, vk, q, q, q)
    x = 2 * np.pi * np.arange(n) / n
    X, Y = np.meshgrid(x, x)
    expect = m.fft_r2c((np.sin(X) * np.sin(Y))[None])
    assert np.abs(nq - expect).max() < 1e-15


def _inner(m, a, b):
    """Parseval volume mean of a*b for two real fields held on the L modes."""
    w = 2.0 * np.where(m.Lb, 1.0, 0.0)
    w[0, 0] = 1.0
    return float((w * (np.conj(a) * b).real).sum())


def test_advection_and_refraction_conserve_wave_action():
    m, s, ic, p = small_model(32, 4)
    psi = random_masked(32, 4, 1)
    psi[:, 0, 0] = 0
    BR, BI = random_masked(32, 4, 2), random_masked(32, 4, 3)
    BR[:, 0, 0] = BR[:, 0, 0].real; BI[:, 0, 0] = BI[:, 0, 0].real
    uk, vk = m.compute_velo(psi)
    _, nBR, nBI = m.convol_waqg(uk, vk, BR, BR, BI)
    rBR, rBI = m.refraction_waqg(BR, BI, psi)
    adv = _inner(m, BR, nBR) + _inner(m, BI, nBI)
    ref = _inner(m, BR, -0.5 * rBI) + _inner(m, BI, 0.5 * rBR)
    scale = _inner(m, BR, BR) * np.abs(psi).max() * 32
    assert abs(adv) < 1e-12 * scale
    assert abs(ref) < 1e-12 * scale


def test_qw_of_uniform_wave_is_zero():
    m, s, ic, p = small_model(16, 3)
    BR = np.zeros((3, 16, 9), complex); BR[:, 0, 0] = [1.0, 2.0, 3.0]
    qw = m.compute_qw(BR, np.zeros_like(BR))
    assert np.abs(qw).max() < 1e-15


# --- L3: vertical inversions --------------------------------------------------
def test_dgtsv_matches_lapack():
    rng = np.random.Generator(np.random.PCG64(5))
    n, ncol = 50, 7
    du = rng.uniform(0.5, 2.0, (n - 1, ncol))
    dl = du.copy()
    d = -(np.vstack([du, np.zeros((1, ncol))]) + np.vstack([np.zeros((1, ncol)), dl]) + rng.uniform(0.01, 1, (n, ncol)))
    b = rng.standard_normal((n, ncol))
    x = orc.dgtsv_nopivot(dl.copy(), d.copy(), du.copy(), b)
    for c in range(ncol):
        _, _, _, xr, info = lapack.dgtsv(dl[:, c], d[:, c], du[:, c], b[:, c])
        assert info == 0
        assert rel_l2(x[:, c], xr) < 1e-14


def test_dgtsv_zero_pivot_raises():
    d = np.array([[0.0], [1.0]])
    with pytest.raises(ZeroDivisionError):
        orc.dgtsv_nopivot(np.array([[0.0]]), d, np.array([[1.0]]), np.ones((2, 1)))


@pytest.mark.parametrize("strat", ["constant", "exponential"])
def test_init_q_psi_solver_roundtrip(strat):
    m, s, ic, p = small_model(32, 16, strat)
    psi = random_masked(32, 16, 11)
    psi[:, 0, 0] = 0
    q = m.init_q(psi)
    back = m.psi_solver(q)
    assert rel_l2(back, psi) < (1e-12 if strat == "constant" else 1e-8)


def test_A_solver_operator():
    m, s, ic, p = small_model(32, 16)
    A = random_masked(32, 16, 12)
    A[:, 0, 0] = 0
    pp = m.p
    # B = (1/Bu) [d/dz(a dA/dz) - kh^2/4 A]  with Neumann ends
    a = pp.a_ell_ut
    dz = pp.dz
    kh2 = m.kh2f
    B = np.zeros_like(A)
    for iz in range(pp.n3):
        up = a[iz] * (A[iz + 1] - A[iz]) if iz < pp.n3 - 1 else 0
        dn = a[iz - 1] * (A[iz] - A[iz - 1]) if iz > 0 else 0
        B[iz] = ((up - dn) / dz ** 2 - 0.25 * kh2 * A[iz]) / pp.Bu
    B = np.where(m.Lb, B, 0)
    A2, C2 = m.A_solver_ybj_plus(B)
    assert rel_l2(A2, A) < 1e-11
    assert rel_l2(C2[:-1], (A[1:] - A[:-1]) / dz) < 1e-10
    assert np.abs(C2[-1]).max() == 0


def test_sumB_removes_vertical_mean():
    m, s, ic, p = small_model(16, 4)
    BR, BI = random_masked(16, 4, 3), random_masked(16, 4, 4)
    R, I = m.sumB(BR, BI)
    sel = m.Lb & (m.grid.kh2 > 0)
    assert np.abs(R.sum(axis=0)[sel]).max() < 1e-13
    assert np.allclose(R[:, 0, 0], BR[:, 0, 0])


# --- time stepping ---------------------------------------------------------------
def test_linear_dispersion_rotation():
    """psi = 0, one horizontal mode times a discrete vertical eigenmode: B
    rotates with the frequency (0.5/(Bu Ro)) kh^2 s, s = A/B of the A
    inversion; compare with a scalar restatement of Euler + leapfrog + filter.
    The wave feedback is off so that no flow develops."""
    m, s, ic, p = small_model(32, 16, no_feedback=1)
    pp = m.p
    n3, dz = pp.n3, pp.dz
    kx, iky, ky = 3, 2, 2
    zs = (np.arange(n3) + 0.5) / n3
    mode = 2
    prof = np.cos(mode * np.pi * zs)
    B0 = np.zeros((n3, 32, 17), complex)
    B0[:, iky, kx] = prof * (0.3 + 0.1j)
    z = np.zeros_like(B0)
    st = orc.State(q=z.copy(), qo=z.copy(), BR=B0.copy(), BI=z.copy(), BRo=B0.copy(), BIo=z.copy(), psi=z.copy(),
                   AR=z.copy(), AI=z.copy(), CR=z.copy(), CI=z.copy())
    st = m.invert(st)
    a = pp.a_ell_ut[0]
    lam = -4 * a * math.sin(mode * math.pi / (2 * n3)) ** 2
    kh2 = kx * kx + ky * ky
    sfac = pp.Bu * dz * dz / (lam - kh2 * dz * dz / 4)
    assert np.allclose(st.AR[:, iky, kx], sfac * st.BR[:, iky, kx], rtol=1e-10, atol=1e-14)
    w = (0.5 / (pp.Bu * pp.Ro)) * kh2 * sfac
    e1, e2 = m.e1w[iky, kx], m.e2w[iky, kx]
    dt, g = pp.delt, pp.gamma
    # scalar restatement on (br, bi) = amplitudes of the profile
    br, bi = complex(B0[0, iky, kx]), 0j
    br_o, bi_o = br, bi
    # Euler
    brn = (br - dt * w * bi) * e1
    bin_ = (bi + dt * w * br) * e1
    br_o, bi_o, br, bi = br, bi, brn, bin_
    st = m.step_euler(st)
    for _ in range(20):
        brt = br_o * e2 - 2 * dt * (w * bi) * e1
        bit = bi_o * e2 - 2 * dt * (-w * br) * e1
        br_o = br + g * (br_o - 2 * br + brt)
        bi_o = bi + g * (bi_o - 2 * bi + bit)
        br, bi = brt, bit
        st = m.step_leapfrog(st)
    assert abs(st.BR[0, iky, kx] - br) < 1e-12 * abs(br)
    assert abs(st.BI[0, iky, kx] - bi) < 1e-12 * abs(bi)


def test_zero_state_stays_zero():
    m, s, ic, p = small_model(16, 4)
    z = np.zeros((4, 16, 9), complex)
    st = orc.State(**{f: z.copy() for f in orc.State.FIELDS})
    st = m.run(st, 3)
    for f in orc.State.FIELDS:
        assert np.abs(getattr(st, f)).max() == 0


def test_step_keeps_fields_masked_and_finite():
    m, s, ic, p = small_model(32, 8)
    s = m.run(s, 4)
    for f in ("q", "qo", "BR", "BI", "psi", "AR", "AI"):
        a = getattr(s, f)
        assert np.isfinite(a).all()
        assert np.abs(np.where(m.Lb, 0, a)).max() == 0


def test_diagnostics_wave_energy_of_uniform_wave():
    m, s, ic, p = small_model(16, 8)
    d = m.diagnostics(s)
    prof = ic.BR[:, 0, 0].real
    assert abs(d["wke"] - 0.5 * np.mean(prof ** 2)) < 1e-14
    assert d["ke"] > 0 and d["zeta2"] > 0


# --- output path (netCDF dumps) --------------------------------------------------
def test_dump_single_mode_layout_and_scaling():
    """A single (kx=1, ky=0) mode dumps as 2 Re(a e^{ix}) times the scales,
    varying along the last (x) axis, in float32 (IO_ncf.f90:47-52)."""
    m, s, ic, p = small_model(16, 2)
    n = 16
    k = np.zeros((2, n, n // 2 + 1), dtype=complex)
    k[:, 0, 1] = 0.5 - 0.25j
    U, L = 0.25, 5e4
    out = m.dump_psi(k, U, L)
    assert out.dtype == np.float32 and out.shape == (2, n, n)
    x = 2 * np.pi * np.arange(n) / n
    exp = (2 * (0.5 * np.cos(x) + 0.25 * np.sin(x)) * U * L).astype(np.float32)
    assert np.allclose(out[0, 3], exp, rtol=1e-6, atol=1e-3)
    assert np.array_equal(out[0, 0], out[0, 5])          # no y dependence


def test_la_from_b_adds_a_on_retained_modes_only():
    """LA = B + 0.25 kh2 A / Bu where L=1 and 0 elsewhere (diagnostics.f90:1698-1727)."""
    m, s, ic, p = small_model(32, 2)
    B = random_masked(32, 2, 5, masked=False)
    A = random_masked(32, 2, 6, masked=False)
    la = m.la_from_b(B, A)
    Lb = m.Lb
    kh2 = m.kh2f
    assert np.array_equal(la[:, ~Lb], np.zeros_like(la[:, ~Lb]))
    assert np.allclose(la[:, Lb], (B + 0.25 * kh2 * A / m.p.Bu)[:, Lb], rtol=0, atol=1e-14)
    # kh = 0: LA = B (horizontally uniform waves are their own LA)
    assert la[0, 0, 0] == B[0, 0, 0]
    R, I = m.dump_la(B * Lb, B * Lb, A * Lb, A * Lb, 2.5e-5, la=False)
    assert np.array_equal(R, I)


# --- omega equation ----------------------------------------------------------------
def test_omega_rhs_two_modes_known_answer():
    """psi = A(z) cos x + B(z) cos y: 2 J(psi_z, lap psi) = 2 sin x sin y
    (Abar B' - A' Bbar) with the discrete vertical difference and average, so
    the (1, +-1) modes carry -/+ c/2 and every other mode is zero."""
    m, s, ic, p = small_model(16, 6)
    n, n3, dz = 16, 6, m.p.dz
    z = np.arange(n3)
    A = 1.0 + 0.3 * z
    B = np.cos(0.7 * z)
    psik = np.zeros((n3, n, n // 2 + 1), dtype=complex)
    psik[:, 0, 1] = A / 2
    psik[:, 1, 0] = B / 2
    rhs = m.omega_eqn_rhs(psik)
    c = np.zeros(n3)
    c[:-1] = 0.5 * (A[1:] + A[:-1]) * (B[1:] - B[:-1]) / dz - (A[1:] - A[:-1]) / dz * 0.5 * (B[1:] + B[:-1])
    assert np.allclose(rhs[:, 1, 1], -0.5 * c, atol=1e-13)
    assert np.allclose(rhs[:, n - 1, 1], 0.5 * c, atol=1e-13)
    rest = rhs.copy()
    rest[:, 1, 1] = 0
    rest[:, n - 1, 1] = 0
    assert np.abs(rest).max() < 1e-13
    # a single horizontal mode has no Jacobian with its own Laplacian
    only = psik.copy()
    only[:, 1, 0] = 0
    assert np.abs(m.omega_eqn_rhs(only)).max() < 1e-13


@pytest.mark.parametrize("strat", ["constant", "exponential"])
def test_omega_equation_inverts_its_operator(strat):
    """Apply the tridiagonal operator of elliptic.f90:463-567 to a random w
    (zero at the top level, kh2 != 0, L = 1) and solve it back."""
    m, s, ic, p = small_model(32, 12, strat)
    n3, dz = m.p.n3, m.p.dz
    g = m.grid
    act = m.Lb & (g.kh2 != 0)
    w = random_masked(32, n3, 11) * act
    w[-1] = 0
    a = np.asarray(m.p.a_ell_ut)
    kh2 = m.kh2f
    rhs = np.zeros_like(w)
    for i in range(n3 - 1):
        v = -(2.0 + dz * dz * kh2 / a[i]) * w[i]
        if i > 0:
            v = v + w[i - 1]
        if i < n3 - 2:
            v = v + w[i + 1]
        rhs[i] = np.where(act, v / (dz * dz), 0)
    got = m.omega_equation(rhs)
    assert rel_l2(got, w) < 1e-11
    assert np.abs(got[-1]).max() == 0


# --- regular YBJ (ybj_plus = 0) ----------------------------------------------------
def test_compute_A_inverts_the_regular_ybj_operator():
    """compute_A (derivatives.f90:1141-1264) returns A with
    d/dz (A_z / N^2) = B on the interior levels (discretely) and vertical
    mean sigma/n3, for B of zero vertical mean (as sumB leaves it)."""
    m, s, ic, p = small_model(16, 10, "exponential", ybj_plus=0)
    n3, dz = m.p.n3, m.p.dz
    r2 = np.asarray(m.p.r_2ut)
    sel = m.Lb & (m.grid.kh2 > 0)
    B = random_masked(16, n3, 7) * sel
    B = B - B.mean(axis=0)
    sigma = random_masked(16, 1, 8)[0] * sel
    A, C = m.compute_A(B, sigma)
    for iz in range(1, n3 - 1):
        lhs = (A[iz + 1] - A[iz]) / (dz * dz * r2[iz]) - (A[iz] - A[iz - 1]) / (dz * dz * r2[iz - 1])
        assert np.allclose(np.where(sel, lhs, 0), B[iz], rtol=0, atol=1e-9 * np.abs(B).max())
    assert np.allclose(A.sum(axis=0), sigma, atol=1e-12 * max(1.0, np.abs(sigma).max()))
    assert np.abs(A[:, ~sel]).max() == 0


def test_regular_ybj_step_keeps_zero_vertical_mean_of_B():
    m, s, ic, p = small_model(16, 8, ybj_plus=0)
    s = m.run(s, 3, first=True)
    sel = m.Lb & (m.grid.kh2 > 0)
    assert np.abs(s.BR.sum(axis=0)[sel]).max() < 1e-13 * max(1.0, np.abs(s.BR).max())
    assert np.isfinite(s.AR).all() and np.abs(s.AR).max() > 0
