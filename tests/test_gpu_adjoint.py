"""CUDA adjoint (FP64) through the C-ABI against the CPU adjoint of
oracle/qgybj_adjoint.py, dot-product tests of one step and central
differences of the objective.

Tolerances: one adjoint step vs the CPU transpose 1e-11 (relative L2 per
field); J 1e-12 and its gradient 1e-10 over several steps; dot-product and
finite-difference checks 1e-6 (their own truncation error is ~1e-8)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.qgybj_adjoint import Adjoint, gradient, inner
from qgybj import Simulation
from qgybj._lib import QG_ERR_UNSUPPORTED, QgError
from qgybj.config import CONFIGS, scaled
from tests.helpers import oracle_for, random_masked, rel_l2

pytestmark = pytest.mark.gpu

N, NZ = 32, 8


@pytest.fixture(scope="module")
def setup():
    model, st, ic, params = oracle_for(scaled(CONFIGS["c4"], N, NZ))
    adj = Adjoint(model)
    sim = Simulation(params, "fp64")
    X = (st.q, st.qo, st.BR + 0.3 * random_masked(N, NZ, 21), st.BI + 0.3 * random_masked(N, NZ, 22), st.BRo, st.BIo)
    X = tuple(adj.mask(a) for a in X)
    yield adj, sim, X, st
    sim.close()


def _rand6(seed):
    return tuple(random_masked(N, NZ, seed + i) for i in range(6))


@pytest.mark.parametrize("first", [True, False])
def test_step_transpose_matches_cpu(setup, first):
    adj, sim, X, _ = setup
    lam = _rand6(200)
    Xn, lo = sim.adjoint_step(X, lam, euler_first=first)
    ref_n = adj.step(X, first)
    ref_l = adj.step_T(X, first, lam)
    for a, b in zip(Xn, ref_n):
        assert rel_l2(a, b) <= 1e-12
    for k, (a, b) in enumerate(zip(lo, ref_l)):
        if np.linalg.norm(b) == 0:
            assert np.linalg.norm(a) == 0
        else:
            assert rel_l2(a, b) <= 1e-11, (k, rel_l2(a, b))


@pytest.mark.parametrize("first", [True, False])
def test_step_dot_product(setup, first):
    adj, sim, X, _ = setup
    dX = _rand6(100)
    lam = _rand6(300)
    eps = 1e-5
    Xp, _ = sim.adjoint_step(tuple(a + eps * d for a, d in zip(X, dX)), euler_first=first)
    Xm, _ = sim.adjoint_step(tuple(a - eps * d for a, d in zip(X, dX)), euler_first=first)
    tl = tuple((p - m) / (2 * eps) for p, m in zip(Xp, Xm))
    _, lo = sim.adjoint_step(X, lam, euler_first=first, forward=False)
    lhs, rhs = inner(tl, lam, adj.Lb), inner(dX, lo, adj.Lb)
    assert abs(lhs - rhs) <= 1e-6 * max(abs(lhs), abs(rhs))


def test_gradient_matches_cpu_and_differences(setup):
    adj, sim, _, st = setup
    q0 = st.q
    BR0 = adj.mask(st.BR + 0.01 * random_masked(N, NZ, 23))
    BI0 = adj.mask(st.BI + 0.01 * random_masked(N, NZ, 24))
    nsteps, every = 7, 3
    J, g = sim.adjoint_run(q0, BR0, BI0, nsteps, every)
    Jr, gr = gradient(adj, q0, BR0, BI0, nsteps, every)
    assert abs(J - Jr) <= 1e-12 * abs(Jr)
    for a, b in zip(g, gr):
        assert rel_l2(a, b) <= 1e-10
    # checkpoint spacing does not change the result
    J1, g1 = sim.adjoint_run(q0, BR0, BI0, nsteps, 1)
    assert J1 == J
    for a, b in zip(g1, g):
        assert rel_l2(a, b) <= 1e-13
    for k in range(2):
        d = tuple(random_masked(N, NZ, 400 + 3 * k + i) for i in range(3))
        nrm = np.sqrt(inner(d, d, adj.Lb))
        d = tuple(x / nrm for x in d)
        h = 1e-6
        Jp = sim.adjoint_run(q0 + h * d[0], BR0 + h * d[1], BI0 + h * d[2], nsteps, every, gradient=False)
        Jm = sim.adjoint_run(q0 - h * d[0], BR0 - h * d[1], BI0 - h * d[2], nsteps, every, gradient=False)
        fd = (Jp - Jm) / (2 * h)
        ad = inner(d, g, adj.Lb)
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_adjoint_refuses_mixed_and_vertical_diffusion():
    model, st, ic, params = oracle_for(scaled(CONFIGS["c4"], 16, 4))
    with Simulation(params, "mixed") as sim:
        with pytest.raises(QgError) as e:
            sim.adjoint_run(st.q, st.BR, st.BI, 2, 1)
        assert e.value.status == QG_ERR_UNSUPPORTED
    p2 = dict(params, nuz=1e-3)
    with Simulation(p2, "fp64", flags={"inviscid": 0}) as sim:
        with pytest.raises(QgError) as e:
            sim.adjoint_run(st.q, st.BR, st.BI, 2, 1)
        assert e.value.status == QG_ERR_UNSUPPORTED


def test_c4_full_size_gradient():
    """128^2 x 64, 50 steps, checkpoints every 10: central differences along
    8 seeded random unit directions (step 1e-6) and the dot-product test of
    one step at this size."""
    from qgybj.config import dealias_mask, make_initial_condition, model_parameters
    rc = CONFIGS["c4"]
    ic = make_initial_condition(rc)
    params = model_parameters(rc, ic.delt)
    n, nz = rc.n, rc.n3
    Lb = dealias_mask(n)[None]
    with Simulation(params, "fp64") as sim:
        sim.set_state("psi", ic.psi); sim.set_state("BR", ic.BR); sim.set_state("BI", ic.BI)
        sim.init_state(True, True)
        q0, BR0, BI0 = sim.get_state("q"), sim.get_state("BR"), sim.get_state("BI")
        J, g = sim.adjoint_run(q0, BR0, BI0, rc.steps, 10)
        errs = []
        for k in range(8):
            d = tuple(random_masked(n, nz, 1000 + 3 * k + i) for i in range(3))
            nrm = np.sqrt(inner(d, d, Lb))
            d = tuple(x / nrm for x in d)
            h = 1e-6
            Jp = sim.adjoint_run(q0 + h * d[0], BR0 + h * d[1], BI0 + h * d[2], rc.steps, 10, gradient=False)
            Jm = sim.adjoint_run(q0 - h * d[0], BR0 - h * d[1], BI0 - h * d[2], rc.steps, 10, gradient=False)
            fd = (Jp - Jm) / (2 * h)
            ad = inner(d, g, Lb)
            errs.append(abs(fd - ad) / abs(ad))
        assert max(errs) <= 1e-6, errs
        # one step: <TL dX, lam> = <dX, ADJ lam>
        X = (q0, q0, BR0, BI0, BR0, BI0)
        dX = tuple(random_masked(n, nz, 2000 + i) for i in range(6))
        lam = tuple(random_masked(n, nz, 3000 + i) for i in range(6))
        eps = 1e-6
        for first in (True, False):
            Xp, _ = sim.adjoint_step(tuple(a + eps * b for a, b in zip(X, dX)), euler_first=first)
            Xm, _ = sim.adjoint_step(tuple(a - eps * b for a, b in zip(X, dX)), euler_first=first)
            tl = tuple((p - m) / (2 * eps) for p, m in zip(Xp, Xm))
            _, lo = sim.adjoint_step(X, lam, euler_first=first, forward=False)
            lhs, rhs = inner(tl, lam, Lb), inner(dX, lo, Lb)
            assert abs(lhs - rhs) <= 1e-6 * max(abs(lhs), abs(rhs)), (first, lhs, rhs)
