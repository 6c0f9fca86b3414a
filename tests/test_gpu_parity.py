"""CUDA path vs the FP64 oracle, through the C-ABI (libqgybj.so).

Tolerances (relative L2 per field):
  FP64 path: 1e-12 (1e-11 for single exponential-stratification inversions,
             whose condition number is ~1e5 larger; full-size runs in
             test_gpu_fullsize.py state their bar from the oracle's own
             FP64 roundoff floor);
  mixed path (FP32 transforms/update, FP64 solves): 1e-5 after 100 steps,
             2e-6 for single routine calls.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import qgybj_oracle as orc
from qgybj import Simulation
from qgybj._lib import QG_ERR_ARG, QG_ERR_NONFINITE, QG_ERR_PIVOT, QG_ERR_UNSUPPORTED, QgError
from qgybj.config import CONFIGS, make_initial_condition, model_parameters, scaled
from tests.helpers import oracle_params, random_masked, random_physical, rel_l2

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "mixed": 2e-6}
FIELDS = ("q", "qo", "BR", "BI", "BRo", "BIo", "psi", "AR", "AI")


def pair(rc, precision, flags=None, **kw):
    flags = flags or {}
    ic = make_initial_condition(rc)
    params = model_parameters(rc, ic.delt)
    if "nuz" in flags:
        params["nuz"] = flags.pop("nuz")
    model = orc.Model(oracle_params(params, **flags))
    st = orc.initial_state(model, ic.psi, ic.BR, ic.BI)
    sim = Simulation(params, precision, flags=flags, **kw)
    sim.set_state("psi", ic.psi)
    sim.set_state("BR", ic.BR)
    sim.set_state("BI", ic.BI)
    sim.init_state(True, True)
    return model, st, sim


def compare(sim, st, tol, fields=FIELDS):
    errs = {f: rel_l2(sim.get_state(f), getattr(st, f)) for f in fields}
    bad = {f: e for f, e in errs.items() if not e <= tol}
    assert not bad, f"fields above {tol}: {bad} (all: {errs})"
    return errs


# --- transforms ------------------------------------------------------------------
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n", [16, 64, 128, 256, 512])
def test_fft_dropins(precision, n):
    rc = scaled(CONFIGS["c0"], n, 4)
    model, st, sim = pair(rc, precision)
    r = random_physical(n, 3, 1)
    rp = np.zeros((3, n, n + 2)); rp[:, :, :n] = r
    k = sim.fft_r2c(rp)
    assert rel_l2(k, model.fft_r2c(r)) < TOL[precision]
    spec = random_masked(n, 3, 2, masked=False)        # unmasked, Nyquist row included
    back = sim.fft_c2r(spec)
    ref = model.fft_c2r(spec)
    assert rel_l2(back[:, :, :n], ref) < TOL[precision]
    assert np.abs(back[:, :, n:]).max() == 0
    sim.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_transform_method_dropins(precision):
    n, nz = 64, 3
    rc = scaled(CONFIGS["c0"], n, 4)
    model, st, sim = pair(rc, precision)
    psi = random_masked(n, nz, 3); psi[:, 0, 0] = 0
    q = random_masked(n, nz, 4)
    BR, BI = random_masked(n, nz, 5, masked=False), random_masked(n, nz, 6, masked=False)
    uk, vk = model.compute_velo(psi)
    got = sim.convol_waqg(uk, vk, q, BR, BI)
    exp = model.convol_waqg(uk, vk, q, BR, BI)
    for a, b in zip(got, exp):
        assert rel_l2(a, b) < TOL[precision]
    got = sim.refraction_waqg(BR, BI, psi)
    exp = model.refraction_waqg(BR, BI, psi)
    for a, b in zip(got, exp):
        assert rel_l2(a, b) < TOL[precision]
    assert rel_l2(sim.compute_qw(BR, BI), model.compute_qw(BR, BI)) < TOL[precision]
    sim.close()


@pytest.mark.parametrize("strat", ["c0", "c1"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solver_dropins(strat, precision):
    rc = scaled(CONFIGS[strat], 64, 32)
    model, st, sim = pair(rc, precision)
    q = random_masked(64, 32, 7)
    # FP64: DGTSV's arithmetic is reproduced exactly; mixed: FP32 inputs,
    # and C = A_z (a difference) loses a further two digits
    tol, tolc = (1e-15, 1e-15) if precision == "fp64" else (2e-6, 1e-4)
    assert rel_l2(sim.psi_solver(q), model.psi_solver(q)) <= tol
    A, Cz = sim.A_solver_ybj_plus(q)
    Ae, Ce = model.A_solver_ybj_plus(q)
    assert rel_l2(A, Ae) <= tol and rel_l2(Cz, Ce) <= tolc
    sim.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_init_state(precision):
    rc = scaled(CONFIGS["c1"], 32, 16)
    model, st, sim = pair(rc, precision)
    tol = 1e-11 if precision == "fp64" else 2e-6
    compare(sim, st, tol, FIELDS + ("CR", "CI"))
    sim.close()


# --- full steps -----------------------------------------------------------------
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_steps_small(precision):
    rc = scaled(CONFIGS["c0"], 32, 16)
    model, st, sim = pair(rc, precision)
    sim.step(euler_first=True)
    st = model.step(st, True)
    for _ in range(9):
        sim.step(False)
        st = model.step(st, False)
    compare(sim, st, 1e-12 if precision == "fp64" else 1e-5)
    got = sim.diagnostics_fp64()
    exp = model.diagnostics(st)
    for k, v in exp.items():
        assert abs(got[k] - v) <= (1e-12 if precision == "fp64" else 1e-5) * abs(v) + 1e-300, k
    sim.close()


@pytest.mark.parametrize("strat", ["c0", "c1"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_step_solves_equal_dropin_solvers(strat, precision):
    """The step's column solves (over the retained columns only; on the
    mixed path with per-column copies of the elimination factors) equal the
    drop-in solvers (every column, the per-kh^2 factor tables) bitwise on
    the same right-hand sides: A from B after the update, psi from q*
    (exponential N^2, c1: the ill-conditioned small-kh columns included)."""
    rc = scaled(CONFIGS[strat], 64, 32)
    model, st, sim = pair(rc, precision)
    sim.step(True)
    BR = sim.get_state("BR")
    assert np.array_equal(sim.get_state("AR"), sim.A_solver_ybj_plus(BR)[0])
    qs = sim.get_state("qstar")
    assert np.array_equal(sim.get_state("psi"), sim.psi_solver(qs))
    sim.close()


@pytest.mark.parametrize("scale", [1.0, 1e25, 1e-30])
def test_mixed_diagnostics_are_fp64_sums_of_the_fp32_state(scale):
    """The mixed engine forms the seven diagnostic sums of its FP32 state in
    FP32-pair arithmetic (exact products, TwoSum accumulation) and
    recomputes a thread's sums in FP64 where a pair overflows.  They equal
    the FP64 sums of that same FP32 state within 1e-12 relative, plus an
    absolute 2^-100 per mode for values whose squares underflow FP32.
    Scale 1e25: squares overflow FP32 and the FP64 recomputation runs;
    1e-30: squares underflow and only the absolute bound holds."""
    rc = scaled(CONFIGS["c1"], 64, 16)
    model, st, sim = pair(rc, "mixed")
    sim.step(True)
    sim.step()
    sim.step()
    s = st.copy()
    for f in ("psi", "BR", "BI", "AR", "AI"):
        v = sim.get_state(f)
        if scale != 1.0:
            sim.set_state(f, v * scale)
            v = sim.get_state(f)                  # the FP32-rounded values
        setattr(s, f, v)
    for c, a in (("CR", "AR"), ("CI", "AI")):
        A = getattr(s, a)
        C = np.zeros_like(A)
        C[:-1] = (A[1:] - A[:-1]) / model.p.dz
        setattr(s, c, C)
    exp = model.diagnostics(s)
    got = sim.diagnostics_fp64()
    nmodes = s.psi.size
    for k, v in exp.items():
        assert np.isfinite(got[k]), k
        assert abs(got[k] - v) <= 1e-12 * abs(v) + nmodes * 2.0 ** -100, (k, got[k], v)
    sim.close()


@pytest.mark.parametrize("n", [128, 256, 512])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_steps_each_row_kernel_path(precision, n):
    """10 steps at n = 128 (row transforms through shared memory), 256
    (radices 8 x 4 x 8, inverse and forward row transforms fused in
    registers) and 512 (8 x 8 x 8, fused, spectra split by warp shuffles),
    exponential stratification, against the oracle."""
    rc = scaled(CONFIGS["c1"], n, 6)
    model, st, sim = pair(rc, precision)
    sim.steps_async(10, True)
    sim.synchronize()
    st = model.run(st, 10, first=True)
    compare(sim, st, 1e-12 if precision == "fp64" else 1e-5)
    sim.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_state_reload_matches_fresh_run(precision):
    """A handle that has stepped, then gets a new state (qg_set_state of
    every prognostic field, with and without qg_init_state), steps exactly as
    a fresh handle given that state: the step's data kept from one step to
    the next (the y-inverse transforms of B in the mixed path) follow the
    state the host sets (bitwise)."""
    rc = scaled(CONFIGS["c1"], 64, 12)
    ic1 = make_initial_condition(rc)
    rc2 = scaled(CONFIGS["c1"], 64, 12)
    rc2.seed = 23
    ic2 = make_initial_condition(rc2)
    params = model_parameters(rc, ic1.delt)

    def init(sim, ic):
        sim.set_state("psi", ic.psi); sim.set_state("BR", ic.BR); sim.set_state("BI", ic.BI)
        sim.init_state(True, True)

    a, b = Simulation(params, precision), Simulation(params, precision)
    init(a, ic1)
    a.steps_async(3, True)
    init(a, ic2)                                 # new state through qg_set_state + qg_init_state
    a.steps_async(4, True)
    init(b, ic2)
    b.steps_async(4, True)
    a.synchronize(); b.synchronize()
    for f in FIELDS:
        assert np.array_equal(a.get_state(f), b.get_state(f)), f
    # every prognostic field set directly (no initialisation), mid-run
    saved = {f: b.get_state(f) for f in FIELDS}
    b.steps_async(2, False)
    a.steps_async(5, False)
    for f, v in saved.items():
        a.set_state(f, v)
    a.steps_async(2, False)
    a.synchronize(); b.synchronize()
    for f in FIELDS:
        assert np.array_equal(a.get_state(f), b.get_state(f)), f
    a.close(); b.close()


def test_c0_fp64_200_steps():
    """64^2 x 64, FP64, 200 leapfrog steps: relative L2 <= 1e-12 per field."""
    rc = CONFIGS["c0"]
    model, st, sim = pair(rc, "fp64")
    sim.step(True)
    sim.steps_async(rc.steps - 1, False)
    sim.synchronize()
    st = model.run(st, rc.steps, first=True)
    compare(sim, st, 1e-12)
    sim.close()


def test_c0_mixed_100_steps():
    rc = CONFIGS["c0"]
    model, st, sim = pair(rc, "mixed")
    sim.steps_async(100, True)
    sim.synchronize()
    st = model.run(st, 100, first=True)
    compare(sim, st, 1e-5)
    sim.close()


@pytest.mark.parametrize("flags", [
    {"linear": 1}, {"no_feedback": 1}, {"fixed_flow": 1}, {"passive_scalar": 1}, {"no_dispersion": 1},
    {"inviscid": 0, "nuz": 3e-4}, {"ybj_plus": 0}, {"ybj_plus": 0, "linear": 1},
])
def test_physics_switches(flags):
    rc = scaled(CONFIGS["c0"], 32, 8)
    model, st, sim = pair(rc, "fp64", dict(flags))
    st = model.run(st, 4, first=True)
    sim.steps_async(4, True)
    sim.synchronize()
    compare(sim, st, 1e-12)
    sim.close()


def test_batching_and_graphs_are_bitwise_invariant():
    rc = scaled(CONFIGS["c1"], 64, 12)
    outs = []
    for lpb, graphs in ((0, 1), (1, 0), (5, 1)):
        model, st, sim = pair(rc, "mixed", levels_per_batch=lpb, use_graphs=graphs)
        sim.steps_async(3, True)
        sim.synchronize()
        outs.append([sim.get_state(f) for f in FIELDS])
        sim.close()
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            assert np.array_equal(a, b)


# --- full sizes: tests/test_gpu_fullsize.py ----------------------------------------


# --- error statuses ---------------------------------------------------------------
def _params(n=32, n3=8):
    rc = scaled(CONFIGS["c0"], n, n3)
    ic = make_initial_condition(rc)
    return model_parameters(rc, ic.delt)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_output_dumps(precision, tmp_path):
    """qg_dump_psi / qg_dump_la (ncdump_psi, ncdump_la; LA conversion of the
    slice diagnostics) against the oracle applied to the handle's own
    spectral state: float32 outputs, rel. L2 <= 1e-7 (FP64) / 2e-6 (mixed)."""
    from qgybj.io import read_dump
    rc = scaled(CONFIGS["c0"], 32, 8)
    model, st, sim = pair(rc, precision)
    sim.step(True)
    for _ in range(3):
        sim.step()
    tol = 1e-7 if precision == "fp64" else 2e-6
    U, L, Uw = 0.25, float(np.float32(6.28318530718 * 5e4)) / (2 * np.pi), float(np.float32(2.5e-5))
    psi, BR, BI = sim.get_state("psi"), sim.get_state("BR"), sim.get_state("BI")
    AR, AI = sim.get_state("AR"), sim.get_state("AI")
    got = sim.dump_psi(U, L)
    assert got.dtype == np.float32 and got.shape == (8, 32, 32)
    assert rel_l2(got.astype(np.float64), model.dump_psi(psi, U, L).astype(np.float64)) <= tol
    for la in (False, True):
        gr, gi = sim.dump_la(Uw, la)
        er, ei = model.dump_la(BR, BI, AR, AI, Uw, la)
        assert rel_l2(gr.astype(np.float64), er.astype(np.float64)) <= tol
        assert rel_l2(gi.astype(np.float64), ei.astype(np.float64)) <= tol
    # a level sub-range is the same slice of the full dump
    part = sim.dump_psi(U, L, level0=2, nlev=3)
    assert np.array_equal(part, got[2:5])
    # files
    p1, p2 = sim.write_dumps(tmp_path, 0, 1.5, U, L, Uw)
    d, t = read_dump(p1)
    assert np.array_equal(d["psi"], got) and t == float(np.float32(1.5 * L / U))
    d, _ = read_dump(p2)
    assert np.array_equal(d["LAr"], sim.dump_la(Uw)[0])
    with pytest.raises(QgError) as e:
        sim.dump_psi(U, L, level0=6, nlev=3)
    assert e.value.status == QG_ERR_ARG
    sim.close()


@pytest.mark.parametrize("strat", ["c0", "c1"])
def test_omega_equation(strat):
    """qg_omega_eqn_rhs / qg_omega_equation (FP64 drop-ins) and qg_omega (from
    the resident psi) against the oracle: rhs 1e-12, solve 1e-13 (DGTSV order
    reproduced), w from the state 1e-12 (constant N^2) / 1e-10 (exponential
    stratification, whose columns are ill-conditioned at small kh)."""
    rc = scaled(CONFIGS[strat], 32, 12)
    model, st, sim = pair(rc, "fp64")
    sim.step(True)
    sim.step()
    psi = sim.get_state("psi")
    rhs = sim.omega_eqn_rhs(psi)
    exp_rhs = model.omega_eqn_rhs(psi)
    assert rel_l2(rhs, exp_rhs) <= 1e-12
    w = sim.omega_equation(exp_rhs)
    assert rel_l2(w, model.omega_equation(exp_rhs)) <= 1e-13
    assert np.abs(w[-1]).max() == 0
    tol = 1e-12 if strat == "c0" else 1e-10
    assert rel_l2(sim.omega(), model.omega_equation(exp_rhs)) <= tol
    sim.close()


def test_error_statuses():
    p = _params()
    with pytest.raises(QgError) as e:
        Simulation(dict(p, n2=64), "fp64")
    assert e.value.status == QG_ERR_UNSUPPORTED
    with pytest.raises(QgError) as e:
        Simulation(dict(p, n1=48, n2=48), "fp64")
    assert e.value.status == QG_ERR_UNSUPPORTED
    with pytest.raises(QgError) as e:
        Simulation(dict(p, delt=float("nan")), "fp64")
    assert e.value.status == QG_ERR_NONFINITE
    with pytest.raises(QgError) as e:
        Simulation(dict(p, a_ell_ut=-np.ones(8)), "fp64")
    assert e.value.status == QG_ERR_PIVOT
    with pytest.raises(QgError) as e:
        Simulation(p, "fp64", flags={"ybj_plus": 2})
    assert e.value.status == QG_ERR_ARG
    sim = Simulation(p, "fp64")
    with pytest.raises(QgError) as e:
        sim.set_state("CR", np.zeros((8, 32, 17), complex))
    assert e.value.status == QG_ERR_ARG
    with pytest.raises(QgError) as e:
        sim.set_state("q", np.zeros((9, 32, 17), complex))
    assert e.value.status == QG_ERR_ARG
    # a valid call after errors still works
    sim.step(True)
    sim.close()


# --- ensembles and the autotuner ----------------------------------------------------
def test_ensemble_members_match_standalone_runs():
    """Uneven members advanced by one graph launch per step give, member by
    member, bit-identical fields to the same runs made alone."""
    from qgybj import Ensemble
    rcs = [scaled(CONFIGS["c0"], 32, 8), scaled(CONFIGS["c1"], 64, 16), scaled(CONFIGS["c0"], 32, 12)]
    rcs[2].seed = 7
    ics = [make_initial_condition(rc) for rc in rcs]
    params = [model_parameters(rc, ic.delt) for rc, ic in zip(rcs, ics)]
    ens = Ensemble(params, "mixed")
    for sim, ic in zip(ens.members, ics):
        sim.set_state("psi", ic.psi); sim.set_state("BR", ic.BR); sim.set_state("BI", ic.BI)
        sim.init_state(True, True)
    # steps with different numbers of concurrent member chains
    ens.set_lanes(1)
    ens.step(2, euler_first=True)
    ens.set_lanes(2)
    ens.step(2)
    ens.set_lanes(8)
    ens.step(1)
    ens.synchronize()
    for sim, p, ic in zip(ens.members, params, ics):
        alone = Simulation(p, "mixed")
        alone.set_state("psi", ic.psi); alone.set_state("BR", ic.BR); alone.set_state("BI", ic.BI)
        alone.init_state(True, True)
        alone.steps_async(5, True)
        alone.synchronize()
        for f in FIELDS:
            assert np.array_equal(sim.get_state(f), alone.get_state(f)), f
        alone.close()
    ens.close()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_ensemble_stack_matches_standalone_runs(precision):
    """Members of one shape are stacked in z into one engine (each kernel of
    the step runs once for all of them); each member, with its own seed,
    Rossby number, wave depth and time step, still gives bit-identical
    fields and diagnostics to the same run made alone.  A member of another
    shape runs beside the stack."""
    from dataclasses import replace

    from qgybj import Ensemble
    base = scaled(CONFIGS["c1"], 64, 16)
    rcs = [replace(base, seed=11 + k, Ro=0.05 + 0.05 * k, wave_depth=0.08 + 0.04 * k) for k in range(3)]
    rcs.append(scaled(CONFIGS["c0"], 32, 8))
    ics = [make_initial_condition(rc) for rc in rcs]
    params = [model_parameters(rc, ic.delt) for rc, ic in zip(rcs, ics)]
    assert len({p["delt"] for p in params[:3]}) == 3          # the stacked members differ in dt
    ens = Ensemble(params, precision)
    for sim, ic in zip(ens.members, ics):
        sim.set_state("psi", ic.psi); sim.set_state("BR", ic.BR); sim.set_state("BI", ic.BI)
        sim.init_state(True, True)
    with pytest.raises(QgError) as e:                           # a member of a stack steps with its stack
        ens.members[0].step(True)
    assert e.value.status == QG_ERR_UNSUPPORTED
    ens.step(1, euler_first=True)
    ens.set_lanes(1)
    ens.step(3)
    ens.synchronize()
    for sim, p, ic in zip(ens.members, params, ics):
        alone = Simulation(p, precision)
        alone.set_state("psi", ic.psi); alone.set_state("BR", ic.BR); alone.set_state("BI", ic.BI)
        alone.init_state(True, True)
        alone.steps_async(4, True)
        alone.synchronize()
        for f in FIELDS + ("CR", "CI"):
            assert np.array_equal(sim.get_state(f), alone.get_state(f)), f
        assert sim.diagnostics_fp64() == alone.diagnostics_fp64()
        alone.close()
    ens.close()


def test_autotune_picks_a_timed_candidate():
    from qgybj import autotune
    rc = scaled(CONFIGS["c1"], 128, 32)
    ic = make_initial_condition(rc)
    t = autotune(model_parameters(rc, ic.delt), "mixed", nsteps=2)
    assert t["levels_per_batch"] in t["candidates"]
    assert set(t["solve_candidates"]) == {16, 32, 64} and t["solve_columns"] in t["solve_candidates"]
    assert t["ms_per_step"] == min(list(t["candidates"].values()) + list(t["solve_candidates"].values())) > 0
    # the tuned block shape is accepted by the library and gives the same results
    rc2 = scaled(CONFIGS["c0"], 32, 8)
    ic2 = make_initial_condition(rc2)
    p2 = model_parameters(rc2, ic2.delt)
    outs = []
    for tc in (16, 64):
        sim = Simulation(p2, "mixed", solve_columns=tc)
        sim.set_state("psi", ic2.psi); sim.set_state("BR", ic2.BR); sim.set_state("BI", ic2.BI)
        sim.init_state(True, True)
        sim.steps_async(3, True)
        sim.synchronize()
        outs.append(sim.get_state("psi"))
        sim.close()
    assert np.array_equal(outs[0], outs[1])
    with pytest.raises(QgError):
        Simulation(p2, "mixed", solve_columns=48)


def test_integer_conversions_match_hardware():
    """The FP32 <-> FP64 conversions the mixed path's FP64 solves and
    diagnostics do with integer operations equal the hardware conversions
    bit for bit: every FP32 pattern, 2^32 FP64 patterns with rounding ties."""
    import ctypes as C

    from qgybj._lib import QG_OK, lib
    a, b = C.c_longlong(-1), C.c_longlong(-1)
    assert lib().qg_selftest_conversions(0, C.byref(a), C.byref(b)) == QG_OK
    assert (a.value, b.value) == (0, 0)


def test_bounded_wait_expiry_reports_timeout():
    """A device-side wait that nothing completes gives up after its bound
    (~0.5 s of SM clocks) and the call returns QG_ERR_TIMEOUT; the handle then
    still steps and matches the oracle.  No GPU fault is involved."""
    from qgybj._lib import QG_ERR_TIMEOUT, lib
    rc = scaled(CONFIGS["c0"], 32, 8)
    model, st, sim = pair(rc, "mixed")
    assert lib().qg_selftest_wait(sim.h) == QG_ERR_TIMEOUT
    sim.steps_async(3, True)
    sim.synchronize()
    st = model.run(st, 3, first=True)
    compare(sim, st, TOL["mixed"])
    sim.close()
