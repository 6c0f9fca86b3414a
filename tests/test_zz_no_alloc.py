"""The allocation-free transform qg_fft_c2r_noalloc against qg_fft_c2r.

Some callers cannot allocate device memory (a host with a fixed device
memory budget shared with other processes, or a loop that cannot afford the
device-wide synchronisation of cudaFree).  qg_fft_c2r_noalloc serves them:
the caller passes device buffers it already owns and the transform keeps its
intermediate plane in the library's static device scratch.  This file is
collected last so that a failure here leaves every other test already run.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from qgybj import Simulation, lib
from qgybj._lib import QG_ERR_ARG, QG_ERR_UNSUPPORTED
from qgybj.config import CONFIGS, make_initial_condition, model_parameters, scaled
from oracle import qgybj_oracle as orc
from tests.helpers import oracle_params, random_masked, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-13   # FP64, same tolerance as the other FP64 transform tests


def _noalloc(torch, spec: np.ndarray, n: int) -> np.ndarray:
    nz = spec.shape[0]
    kdev = torch.from_numpy(spec.view(np.float64).copy()).cuda()
    rdev = torch.full((nz, n, n + 2), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib().qg_fft_c2r_noalloc(C.c_void_p(kdev.data_ptr()), C.c_void_p(rdev.data_ptr()), n, nz, None)
    assert rc == 0, lib().qg_last_error(None)
    torch.cuda.synchronize()
    return rdev.cpu().numpy()


@pytest.mark.parametrize("n,nz", [(64, 5), (512, 7)])
def test_noalloc_c2r_matches_handle_path_on_two_calls(n, nz):
    torch = pytest.importorskip("torch")
    rc = scaled(CONFIGS["c0"], n, 4)
    ic = make_initial_condition(rc)
    params = model_parameters(rc, ic.delt)
    sim = Simulation(params, "fp64")
    model = orc.Model(oracle_params(params))
    for seed in (11, 12):        # two calls in a row, different inputs
        spec = random_masked(n, nz, seed, masked=False)
        expect = sim.fft_c2r(spec)
        got = _noalloc(torch, spec, n)
        assert np.isfinite(got).all()
        assert rel_l2(got[:, :, :n], expect[:, :, :n]) <= TOL
        assert np.abs(got[:, :, n:]).max() == 0
        # and directly against the oracle's c2r (fft.f90:71-83, realit included)
        assert rel_l2(got[:, :, :n], model.fft_c2r(spec)) <= TOL
    sim.close()


def test_noalloc_rejects_what_it_cannot_do():
    torch = pytest.importorskip("torch")
    k = torch.zeros((2, 1024, 513, 2), dtype=torch.float64, device="cuda")
    r = torch.zeros((2, 1024, 1026), dtype=torch.float64, device="cuda")
    assert lib().qg_fft_c2r_noalloc(C.c_void_p(k.data_ptr()), C.c_void_p(r.data_ptr()), 1024, 2, None) \
        == QG_ERR_UNSUPPORTED
    assert b"8 MiB" in lib().qg_last_error(None)
    host = np.zeros((1, 64, 33), dtype=np.complex128)
    hr = np.zeros((1, 64, 66))
    assert lib().qg_fft_c2r_noalloc(host.ctypes.data, hr.ctypes.data, 64, 1, None) == QG_ERR_ARG
    # complex input read in 16-byte pairs: an input offset by one double is refused, not launched
    k64 = torch.zeros((1, 64, 33, 2), dtype=torch.float64, device="cuda")
    r64 = torch.zeros((1, 64, 66), dtype=torch.float64, device="cuda")
    assert lib().qg_fft_c2r_noalloc(C.c_void_p(k64.data_ptr() + 8), C.c_void_p(r64.data_ptr()), 64, 1, None) \
        == QG_ERR_ARG
    assert b"16-byte aligned" in lib().qg_last_error(None)
    assert lib().qg_fft_c2r_noalloc(C.c_void_p(k64.data_ptr()), C.c_void_p(r64.data_ptr() + 4), 64, 1, None) \
        == QG_ERR_ARG
    torch.cuda.synchronize()
