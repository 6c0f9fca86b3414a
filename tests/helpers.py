"""Shared test helpers: oracle construction from a run configuration,
error norms, random masked spectral fields."""
from __future__ import annotations

import numpy as np

from oracle import qgybj_oracle as orc
from qgybj.config import RunConfig, dealias_mask, make_initial_condition, model_parameters


def oracle_params(params: dict, **flags) -> orc.Params:
    keys = ("n1", "n2", "n3", "dz", "Bu", "Ro", "W2F", "delt", "gamma", "nuh1", "nuh2", "ilap1", "ilap2",
            "nuh1w", "nuh2w", "ilap1w", "ilap2w", "nuz", "a_ell_ut")
    kw = {k: params[k] for k in keys}
    kw["r_2ut"] = params.get("r_2ut")
    kw.update(flags)
    return orc.Params(**kw)


def oracle_for(rc: RunConfig, **flags):
    ic = make_initial_condition(rc)
    params = model_parameters(rc, ic.delt)
    model = orc.Model(oracle_params(params, **flags))
    state = orc.initial_state(model, ic.psi, ic.BR, ic.BI)
    return model, state, ic, params


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    nb = np.linalg.norm(b)
    if nb == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)


def random_masked(n: int, nz: int, seed: int, masked: bool = True) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    a = rng.standard_normal((nz, n, n // 2 + 1)) + 1j * rng.standard_normal((nz, n, n // 2 + 1))
    if masked:
        a = np.where(dealias_mask(n)[None], a, 0)
    return a


def random_physical(n: int, nz: int, seed: int) -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.standard_normal((nz, n, n))


def hermitian_consistent(k: np.ndarray) -> np.ndarray:
    """Spectrum of a real field: the r2c of its c2r (kx=0 column Hermitian,
    DC and Nyquist entries real)."""
    import scipy.fft as sfft
    n = k.shape[-2]
    r = sfft.irfft2(k, s=(n, n), axes=(-2, -1), norm="forward")
    return sfft.rfft2(r, axes=(-2, -1), norm="forward")
