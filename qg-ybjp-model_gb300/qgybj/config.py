"""Run configurations and the seeded initial-condition generator.

The reference reads its parameters from a compiled module
(parameters_test1.f90) and its initial conditions from netCDF files that it
does not ship; the configurations here state the same quantities explicitly
and generate synthetic, seeded initial conditions with the shapes and
spectra the benchmark configurations describe.

Conventions (all nondimensional, as in parameters_test1.f90:45-74):
  horizontal domain 2*pi periodic, n x n points, 2/3 dealiasing;
  unit depth, n3 staggered levels zs = (iz-1/2) dz, interfaces za = iz dz;
  a_ell_ut(iz) = Bu / N^2(za(iz)) (init.f90:253), rho = 1;
  hyperdiffusion int_factor = delt*nuh1*(kx^4+ky^4) with nuh1 set so that
  int_factor = if_kt at (kx=K, ky=0), K the largest retained wavenumber.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np


# ---------------------------------------------------------------------------
# grid helpers (init.f90:32-80)
# ---------------------------------------------------------------------------
def wavenumbers(n: int):
    """kxa [iktx], kya [ikty] in FFT order with ky=-n/2 set to 0."""
    kxa = np.arange(n // 2 + 1)
    kya = np.empty(n, dtype=np.int64)
    for iky in range(1, n + 1):
        jj = iky - 1
        if iky > n // 2:
            jj -= n
        if iky == n // 2 + 1:
            jj = 0
        kya[iky - 1] = jj
    return kxa, kya


def dealias_mask(n: int) -> np.ndarray:
    """L [ikty][iktx] (bool) as init_arrays computes it."""
    kxa, kya = wavenumbers(n)
    KX, KY = np.meshgrid(kxa, kya)
    kh = np.sqrt((KX * KX + KY * KY).astype(np.float32)).astype(np.float64)
    thr = float(int(np.float32(n) / np.float32(3.0) + np.float32(0.5))) - 0.5
    L = kh <= thr
    L[n // 2, :] = False
    L[(KX == 0) & (KY < 0)] = False
    return L


def kmax(n: int) -> int:
    return int(math.floor(float(int(np.float32(n) / np.float32(3.0) + np.float32(0.5))) - 0.5))


# ---------------------------------------------------------------------------
@dataclass
class RunConfig:
    name: str
    n: int
    n3: int
    precision: str = "fp64"          # "fp64" | "mixed"
    steps: int = 100
    seed: int = 0
    k0: float = 3.0                  # peak of the eddy spectrum
    Ro: float = 0.1
    Bu: float = 1.0
    W2F: float = 1.0
    wave_depth: float = 0.1          # e-folding depth of the surface wave profile
    stratification: str = "constant"  # "constant" | "exponential"
    strat_scale: float = 0.1         # N^2 = exp((z-1)/strat_scale) for "exponential"
    gamma: float = 0.0010000000474974513   # single-precision literal 1e-3 (parameters_test1.f90:87)
    cfl: float = 0.2
    if_kt: float = 0.1
    ilap: int = 2
    delt: float | None = None        # derived from the CFL number when None
    levels_per_batch: int = 0
    solve_columns: int = 0
    use_graphs: int = 1
    extra: dict = field(default_factory=dict)

    @property
    def dz(self) -> float:
        return 1.0 / self.n3

    def n2_profile(self, z: np.ndarray) -> np.ndarray:
        if self.stratification == "constant":
            return np.ones_like(z)
        if self.stratification == "exponential":
            return np.exp((z - 1.0) / self.strat_scale)
        raise ValueError(self.stratification)

    def a_ell_ut(self) -> np.ndarray:
        za = np.arange(1, self.n3 + 1) * self.dz
        return self.Bu / self.n2_profile(za)

    def r_2ut(self) -> np.ndarray:
        za = np.arange(1, self.n3 + 1) * self.dz
        return self.n2_profile(za)

    def hyperdiffusion(self, delt: float) -> float:
        K = kmax(self.n)
        return self.if_kt / (delt * float(K) ** (2 * self.ilap))


# the configurations of the benchmark (64^2x64 CPU case, 256^2x128 FP64,
# 512^2x256 mixed precision, ensemble members, adjoint case)
CONFIGS = {
    "c0": RunConfig("c0_64x64x64_fp64", 64, 64, "fp64", steps=200, seed=0, k0=3.0),
    # levels_per_batch, solve_columns: the choices of qg_autotune on GB300 for these sizes
    # (0: the library's default depth)
    "c1": RunConfig("c1_256x256x128_fp64", 256, 128, "fp64", steps=200, seed=1, k0=6.0,
                    stratification="exponential", levels_per_batch=0, solve_columns=16),
    "c2": RunConfig("c2_512x512x256_mixed", 512, 256, "mixed", steps=100, seed=2, k0=8.0,
                    stratification="exponential", levels_per_batch=256, solve_columns=16),
    "c4": RunConfig("c4_128x128x64_fp64", 128, 64, "fp64", steps=50, seed=4, k0=3.0),
}


def ensemble_members() -> list[RunConfig]:
    """64 uneven members: 24 at 64^2x32, 24 at 128^2x64, 16 at 256^2x128;
    seed 1000+m each, Ro and wave depth ~ U[0.05, 0.2] drawn from seed 999."""
    rng = np.random.Generator(np.random.PCG64(999))
    ro = rng.uniform(0.05, 0.2, 64)
    wd = rng.uniform(0.05, 0.2, 64)
    sizes = [(64, 32)] * 24 + [(128, 64)] * 24 + [(256, 128)] * 16
    out = []
    for m, (n, n3) in enumerate(sizes):
        out.append(RunConfig(f"c3_m{m:02d}_{n}x{n}x{n3}", n, n3, "mixed", steps=100, seed=1000 + m, k0=8.0,
                             Ro=float(ro[m]), wave_depth=float(wd[m]), stratification="exponential"))
    return out


def scaled(rc: RunConfig, n: int, n3: int, steps: int | None = None) -> RunConfig:
    """Same recipe at another resolution (used for small parity cases)."""
    return replace(rc, name=f"{rc.name}@{n}x{n}x{n3}", n=n, n3=n3, steps=rc.steps if steps is None else steps,
                   delt=None)


# ---------------------------------------------------------------------------
# initial conditions
# ---------------------------------------------------------------------------
@dataclass
class InitialCondition:
    psi: np.ndarray      # complex128 [n3][n][n/2+1]
    BR: np.ndarray
    BI: np.ndarray
    delt: float
    umax: float


def make_initial_condition(rc: RunConfig) -> InitialCondition:
    """Seeded random-phase eddies plus a horizontally uniform surface wave.

    psi: |psi_k| ~ exp(-(k/k0)^2/2)/k (energy spectrum ~ k exp(-(k/k0)^2)),
    independent uniform phases for a barotropic part and a first-baroclinic
    part of equal energy, scaled so rms(zeta) = 1
    (flow Rossby number = Ro).  B = exp(-((1-zs)/wave_depth)^2) at kh=0
    (LA = B there, wave velocity amplitude 1, W2F = 1).  delt from the
    advective CFL number on the initial velocity.
    """
    n, n3 = rc.n, rc.n3
    L = dealias_mask(n)
    kxa, kya = wavenumbers(n)
    KX, KY = np.meshgrid(kxa, kya)
    kh2 = (KX * KX + KY * KY).astype(np.float64)
    k = np.sqrt(kh2)
    sel = L & (kh2 > 0)
    amp = np.zeros_like(k)
    amp[sel] = np.exp(-0.5 * (k[sel] / rc.k0) ** 2) / k[sel]
    rng = np.random.Generator(np.random.PCG64(rc.seed))
    ph_bt = rng.uniform(0.0, 2.0 * np.pi, size=k.shape)
    ph_bc = rng.uniform(0.0, 2.0 * np.pi, size=k.shape)
    P_bt = amp * np.exp(1j * ph_bt)
    P_bc = amp * np.exp(1j * ph_bc)
    zs = (np.arange(1, n3 + 1) - 0.5) * rc.dz
    vert = first_baroclinic_mode(rc)
    psi = P_bt[None] + vert[:, None, None] * P_bc[None]
    psi = np.where(L[None], psi, 0)
    # rms vorticity over the volume
    z2 = (kh2 * kh2)[None] * (psi.real ** 2 + psi.imag ** 2)
    msq = (2.0 * z2.sum(axis=(1, 2)) - z2[:, 0, 0]).mean()
    psi = psi / math.sqrt(msq)
    # CFL
    import scipy.fft as sfft
    uk = np.where(L[None], -(1j * KY)[None] * psi, 0)
    vk = np.where(L[None], (1j * KX)[None] * psi, 0)

    def c2r(a):
        a = a.copy()
        m = np.arange(1, n // 2)
        a[..., n - m, 0] = np.conj(a[..., m, 0])
        return sfft.irfft2(a, s=(n, n), axes=(-2, -1), norm="forward", workers=-1)

    ur, vr = c2r(uk), c2r(vk)
    umax = float(np.sqrt(ur * ur + vr * vr).max())
    dx = 2.0 * np.pi / n
    delt = rc.delt if rc.delt is not None else rc.cfl * dx / umax
    BR = np.zeros((n3, n, n // 2 + 1), dtype=np.complex128)
    BR[:, 0, 0] = np.exp(-((1.0 - zs) / rc.wave_depth) ** 2)
    BI = np.zeros_like(BR)
    return InitialCondition(psi=psi.astype(np.complex128), BR=BR, BI=BI, delt=float(delt), umax=umax)


def la_from_b(n: int, Bu: float, Bk: np.ndarray, Ak: np.ndarray) -> np.ndarray:
    """YBJ+ wave field LA = B + kh^2 A / (4 Bu) on the retained modes, zero
    elsewhere (diagnostics.f90:1698-1706), for arrays in the reference
    layout [nz][n][n/2+1]."""
    kxa, kya = wavenumbers(n)
    KX, KY = np.meshgrid(kxa, kya)
    kh2 = (KX * KX + KY * KY).astype(np.float64)
    return np.where(dealias_mask(n)[None], Bk + ((0.25 * kh2)[None] * Ak) / Bu, 0)


def first_baroclinic_mode(rc: RunConfig) -> np.ndarray:
    """First baroclinic eigenvector of the discrete vertical operator of
    psi_solver (elliptic.f90:177-189 without the kh^2 term, Neumann ends),
    normalised to mean square 1 and positive at the bottom.  For constant
    N^2 it is sqrt(2) cos(pi zs)."""
    from scipy.linalg import eigh_tridiagonal
    a = rc.a_ell_ut()
    n3 = rc.n3
    d = np.empty(n3)
    d[0] = -a[0]
    d[1:-1] = -(a[1:-1] + a[:-2])
    d[-1] = -a[-2]
    w, v = eigh_tridiagonal(d, a[:-1])
    phi = v[:, -2]                       # eigenvalues ascending: -2 = first nonzero
    phi = phi / np.sqrt(np.mean(phi * phi))
    return phi if phi[0] > 0 else -phi


def model_parameters(rc: RunConfig, delt: float) -> dict:
    """Scalar parameters shared by the library configuration and the oracle."""
    nuh = rc.hyperdiffusion(delt)
    return dict(n1=rc.n, n2=rc.n, n3=rc.n3, dz=rc.dz, Bu=rc.Bu, Ro=rc.Ro, W2F=rc.W2F, delt=delt, gamma=rc.gamma,
                nuh1=nuh, nuh2=0.0, ilap1=rc.ilap, ilap2=6, nuh1w=nuh, nuh2w=0.0, ilap1w=rc.ilap, ilap2w=6,
                nuz=0.0, a_ell_ut=rc.a_ell_ut(), r_2ut=rc.r_2ut())
