"""The CPU adjoint (oracle/qgybj_adjoint.py) against central differences:
dot-product (tangent-linear / adjoint) tests of one step and gradient checks
of the objective over several steps, FP64."""
from __future__ import annotations

import numpy as np
import pytest

from oracle.qgybj_adjoint import Adjoint, Objective, gradient, inner, run_forward
from qgybj.config import CONFIGS, make_initial_condition, model_parameters, scaled
from tests.helpers import oracle_for, random_masked


@pytest.fixture(scope="module")
def setup():
    model, st, ic, params = oracle_for(scaled(CONFIGS["c4"], 32, 8))
    adj = Adjoint(model)
    X = (st.q, st.qo, st.BR + 0.3 * random_masked(32, 8, 21), st.BI + 0.3 * random_masked(32, 8, 22), st.BRo, st.BIo)
    X = tuple(adj.mask(a) for a in X)
    return adj, X


def _rand6(seed, scale=1.0):
    return tuple(scale * random_masked(32, 8, seed + i) for i in range(6))


@pytest.mark.parametrize("first", [True, False])
def test_step_dot_product(setup, first):
    adj, X = setup
    dX = _rand6(100)
    lam = _rand6(200)
    eps = 1e-5
    Xp = adj.step(tuple(a + eps * d for a, d in zip(X, dX)), first)
    Xm = adj.step(tuple(a - eps * d for a, d in zip(X, dX)), first)
    tl = tuple((p - m) / (2 * eps) for p, m in zip(Xp, Xm))
    lhs = inner(tl, lam, adj.Lb)
    rhs = inner(dX, adj.step_T(X, first, lam), adj.Lb)
    assert abs(lhs - rhs) <= 1e-7 * max(abs(lhs), abs(rhs))


def test_gradient_matches_central_differences(setup):
    adj, X = setup
    model, st, ic, params = oracle_for(scaled(CONFIGS["c4"], 32, 8))
    q0 = st.q
    BR0 = adj.mask(st.BR + 0.01 * random_masked(32, 8, 23))
    BI0 = adj.mask(st.BI + 0.01 * random_masked(32, 8, 24))
    nsteps = 6
    J, (gq, gR, gI) = gradient(adj, q0, BR0, BI0, nsteps, every=4)
    obj = Objective(adj)
    rng = np.random.Generator(np.random.PCG64(40))
    for k in range(3):
        d = tuple(random_masked(32, 8, 300 + 3 * k + i) for i in range(3))
        nrm = np.sqrt(inner(d, d, adj.Lb))
        d = tuple(x / nrm for x in d)
        h = 1e-6
        Jp = obj.value(*run_forward(adj, q0 + h * d[0], BR0 + h * d[1], BI0 + h * d[2], nsteps)[-1][2:4])
        Jm = obj.value(*run_forward(adj, q0 - h * d[0], BR0 - h * d[1], BI0 - h * d[2], nsteps)[-1][2:4])
        fd = (Jp - Jm) / (2 * h)
        ad = inner(d, (gq, gR, gI), adj.Lb)
        assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-300), (fd, ad)
