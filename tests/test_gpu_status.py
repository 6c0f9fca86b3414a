"""Status codes the device raises: non-finite inputs and a blown-up run.

The reference prints and carries on when a solve fails (elliptic.f90:192)
and would write NaN into its dumps after a blow-up; through the C-ABI a NaN
or infinity on a retained mode of a qg_set_state input, and a step whose
q* (= q - q^w) is no longer finite, come back as QG_ERR_NONFINITE.  The
failures are made on the host (a NaN planted in the uploaded array, a time
step twenty times the CFL limit); no kernel is made to fault.
"""
from __future__ import annotations

import numpy as np
import pytest

from qgybj import QgError, Simulation
from qgybj._lib import QG_ERR_NONFINITE
from qgybj.config import CONFIGS, make_initial_condition, model_parameters, scaled

pytestmark = pytest.mark.gpu


def _sim(precision, dt_factor=1.0, n=32, n3=16):
    rc = scaled(CONFIGS["c0"], n, n3)
    ic = make_initial_condition(rc)
    return Simulation(model_parameters(rc, ic.delt * dt_factor), precision), ic


def _init(sim, ic):
    sim.set_state("psi", ic.psi)
    sim.set_state("BR", ic.BR)
    sim.set_state("BI", ic.BI)
    sim.init_state(True, True)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_set_state_reports_nonfinite_retained_modes(precision):
    sim, ic = _sim(precision)
    n = sim.n
    for bad in (np.nan, np.inf, -np.inf):
        psi = ic.psi.copy()
        psi[3, 1, 2] = complex(bad, 0.0)          # kx=2, ky=1: retained
        with pytest.raises(QgError) as e:
            sim.set_state("psi", psi)
        assert e.value.status == QG_ERR_NONFINITE
        BR = ic.BR.copy()
        BR[5, n - 2, 1] = complex(0.0, bad)       # kx=1, ky=-2: retained (imaginary part)
        with pytest.raises(QgError) as e:
            sim.set_state("BR", BR)
        assert e.value.status == QG_ERR_NONFINITE
    # modes outside the retained set are discarded unread: no error
    psi = ic.psi.copy()
    psi[3, n // 2, 2] = np.nan                    # the ky = -n/2 row
    psi[4, 0, n // 2] = np.inf                    # kx = n/2, beyond the 2/3 disk
    sim.set_state("psi", psi)
    # a clean upload after a refused one succeeds and the handle steps
    _init(sim, ic)
    sim.step(True)
    sim.step(False)
    assert np.isfinite(sim.get_state("q")).all()
    sim.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_blow_up_reports_nonfinite(precision):
    """dt at 20x the advective CFL limit: the leapfrog grows by ~1e10 per
    step (the oracle passes 1e44 within 5 steps at 32^2x16) until q* is no
    longer finite; qg_step then returns QG_ERR_NONFINITE, and the same
    handle runs a sane state afterwards."""
    sim, ic = _sim(precision, dt_factor=20.0)
    _init(sim, ic)
    raised = None
    try:
        sim.step(True)
        for _ in range(200):
            sim.step(False)
    except QgError as e:
        raised = e
    assert raised is not None and raised.status == QG_ERR_NONFINITE
    assert b"non-finite q*" in str(raised).encode()
    # asynchronous steps report it at qg_synchronize
    _init(sim, ic)
    sim.steps_async(200, True)
    with pytest.raises(QgError) as e:
        sim.synchronize()
    assert e.value.status == QG_ERR_NONFINITE
    sim.close()
    # a fresh handle with a sane time step reports nothing
    sim, ic = _sim(precision)
    _init(sim, ic)
    sim.steps_async(20, True)
    sim.synchronize()
    sim.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_async_diagnostics_pipelined_with_steps(precision):
    """qg_diagnostics_fp64_async followed at once by a step: the integrals
    are those of the state before the step, and the step is not disturbed
    (bitwise against synchronous diagnostics and an undisturbed run)."""
    a, ic = _sim(precision)
    b, _ = _sim(precision)
    _init(a, ic)
    _init(b, ic)
    a.steps_async(3, True)
    b.steps_async(3, True)
    ref = [b.diagnostics_fp64()]
    a.diagnostics_fp64_async()
    a.step(False)
    got = [a.diagnostics_fp64_wait()]
    for _ in range(3):
        a.diagnostics_fp64_async()
        a.step(False)
        got.append(a.diagnostics_fp64_wait())
    for _ in range(4):
        b.step(False)
        ref.append(b.diagnostics_fp64())
    assert got == ref[:4]
    for f in ("q", "psi", "BR", "BI", "AR", "AI"):
        assert np.array_equal(a.get_state(f), b.get_state(f)), f
    with pytest.raises(QgError):
        a.diagnostics_fp64_wait()          # nothing pending
    a.close()
    b.close()
