"""Host-side mirror of the reference's use of its step routines.

``Simulation`` owns one library handle and exposes the routines of the
reference under their Fortran names (fft_r2c, fft_c2r, convol_waqg,
refraction_waqg, compute_qw, psi_solver, A_solver_ybj_plus, sumB/init_q via
init_state) with numpy arrays in the reference's memory layout, plus the
resident-state interface (set_state/get_state/step) that replaces the time
loop of main_waqg.f90.  Status codes other than QG_OK raise QgError.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import FIELDS, QG_PREC_FP64, QG_PREC_MIXED, QgConfig, QgEnergy, QgError, QgTuning, check, lib, ptr
from .config import RunConfig, make_initial_condition, model_parameters


def _arr(a, n3=None):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def make_config(params: dict, precision: str = "fp64", device: int = 0, levels_per_batch: int = 0,
                use_graphs: int = 1, flags: dict | None = None, solve_columns: int = 0):
    """qg_config of a parameter dict; returns (config, arrays kept alive)."""
    cfg = QgConfig()
    check(lib().qg_config_defaults(C.byref(cfg)))
    cfg.n1, cfg.n2, cfg.n3 = int(params["n1"]), int(params["n2"]), int(params["n3"])
    cfg.precision = QG_PREC_FP64 if precision == "fp64" else QG_PREC_MIXED
    cfg.device = device
    for k in ("dz", "Bu", "Ro", "W2F", "delt", "gamma", "nuh1", "nuh2", "nuh1w", "nuh2w", "nuz"):
        setattr(cfg, k, float(params.get(k, 0.0)))
    for k in ("ilap1", "ilap2", "ilap1w", "ilap2w"):
        setattr(cfg, k, int(params.get(k, 2)))
    for k, v in (flags or {}).items():
        setattr(cfg, k, int(v))
    keep = []
    for k in ("a_ell_ut", "rho_ut", "rho_st", "r_2ut"):
        v = params.get(k)
        if v is not None:
            a = np.ascontiguousarray(v, dtype=np.float64)
            keep.append(a)
            setattr(cfg, k, a.ctypes.data_as(C.POINTER(C.c_double)))
    cfg.levels_per_batch = levels_per_batch
    cfg.use_graphs = use_graphs
    cfg.solve_columns = solve_columns
    return cfg, keep


def autotune(params: dict, precision: str = "mixed", device: int = 0, nsteps: int = 3) -> dict:
    """qg_autotune: fastest phase-A batch depth for these parameters."""
    cfg, keep = make_config(params, precision, device)
    t = QgTuning()
    check(lib().qg_autotune(C.byref(cfg), int(nsteps), C.byref(t)))
    return {"levels_per_batch": t.levels_per_batch, "solve_columns": t.solve_columns, "ms_per_step": t.ms_per_step,
            "candidates": {t.candidates[i]: t.candidate_ms[i] for i in range(t.ncandidates)},
            "solve_candidates": {t.solve_candidates[i]: t.solve_candidate_ms[i] for i in range(t.nsolve)}}


class Simulation:
    def __init__(self, params: dict, precision: str = "fp64", device: int = 0, levels_per_batch: int = 0,
                 use_graphs: int = 1, flags: dict | None = None, _handle=None, solve_columns: int = 0):
        L = lib()
        self.n, self.n3 = int(params["n1"]), int(params["n3"])
        self.precision = precision
        if _handle is not None:          # a member handle owned by an Ensemble
            self.h, self._owned, self._keep = _handle, False, []
            self.cfg, _ = make_config(params, precision, device, levels_per_batch, use_graphs, flags, solve_columns)
            return
        self._owned = True
        self.cfg, self._keep = make_config(params, precision, device, levels_per_batch, use_graphs, flags,
                                           solve_columns)
        h = C.c_void_p()
        check(L.qg_create(C.byref(self.cfg), C.byref(h)))
        self.h = h

    # -- lifecycle -------------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            if getattr(self, "_owned", True):
                lib().qg_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, st):
        check(st, self.h)

    @property
    def spectral_shape(self):
        return (self.n3, self.n, self.n // 2 + 1)

    # -- resident state ----------------------------------------------------------
    def set_state(self, name: str, kvar, level0: int = 0):
        if isinstance(kvar, np.ndarray):
            kvar = np.ascontiguousarray(kvar, dtype=np.complex128)
            nlev = kvar.shape[0]
        else:
            nlev = kvar.shape[0]
        self._ck(lib().qg_set_state(self.h, FIELDS[name], ptr(kvar), level0, nlev))

    def get_state(self, name: str, level0: int = 0, nlev: int | None = None, out=None):
        nlev = self.n3 - level0 if nlev is None else nlev
        if out is None:
            out = np.empty((nlev, self.n, self.n // 2 + 1), dtype=np.complex128)
        self._ck(lib().qg_get_state(self.h, FIELDS[name], ptr(out), level0, nlev))
        return out

    def init_state(self, apply_sumB: bool = True, q_from_psi: bool = True):
        self._ck(lib().qg_init_state(self.h, int(apply_sumB), int(q_from_psi)))

    def step(self, euler_first: bool = False):
        self._ck(lib().qg_step(self.h, int(euler_first)))

    def steps_async(self, nsteps: int, euler_first: bool = False):
        self._ck(lib().qg_steps_async(self.h, int(nsteps), int(euler_first)))

    def synchronize(self):
        self._ck(lib().qg_synchronize(self.h))

    def stream(self) -> int:
        s = C.c_void_p()
        self._ck(lib().qg_get_stream(self.h, C.byref(s)))
        return int(s.value or 0)

    def diagnostics_fp64(self) -> dict:
        e = QgEnergy()
        self._ck(lib().qg_diagnostics_fp64(self.h, C.byref(e)))
        return {k: getattr(e, k) for k, _ in QgEnergy._fields_}

    def diagnostics_fp64_async(self):
        """Queue the FP64 integrals of the current state (collect them with
        diagnostics_fp64_wait; a step may be queued in between)."""
        self._ck(lib().qg_diagnostics_fp64_async(self.h))

    def diagnostics_fp64_wait(self) -> dict:
        e = QgEnergy()
        self._ck(lib().qg_diagnostics_fp64_wait(self.h, C.byref(e)))
        return {k: getattr(e, k) for k, _ in QgEnergy._fields_}

    def profile_step(self, euler_first: bool = False) -> dict:
        """One step with CUDA events around each launch: {class: (ms, launches)}."""
        from ._lib import KERNEL_CLASSES
        n = len(KERNEL_CLASSES)
        ms = (C.c_double * n)()
        cnt = (C.c_int * n)()
        self._ck(lib().qg_profile_step(self.h, int(euler_first), ms, cnt, n))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(KERNEL_CLASSES)}

    # -- routine-level drop-ins --------------------------------------------------
    def fft_r2c(self, rvar: np.ndarray) -> np.ndarray:
        rvar = np.ascontiguousarray(rvar, dtype=np.float64)
        nz = rvar.shape[0]
        assert rvar.shape[1:] == (self.n, self.n + 2)
        out = np.empty((nz, self.n, self.n // 2 + 1), dtype=np.complex128)
        self._ck(lib().qg_fft_r2c(self.h, ptr(rvar), ptr(out), nz))
        return out

    def fft_c2r(self, kvar: np.ndarray) -> np.ndarray:
        kvar = np.ascontiguousarray(kvar, dtype=np.complex128)
        nz = kvar.shape[0]
        out = np.empty((nz, self.n, self.n + 2), dtype=np.float64)
        self._ck(lib().qg_fft_c2r(self.h, ptr(kvar), ptr(out), nz))
        return out

    def _c(self, a):
        return np.ascontiguousarray(a, dtype=np.complex128)

    def convol_waqg(self, uk, vk, qk, BRk, BIk):
        ins = [self._c(a) for a in (uk, vk, qk, BRk, BIk)]
        nz = ins[0].shape[0]
        outs = [np.empty_like(ins[0]) for _ in range(3)]
        self._ck(lib().qg_convol_waqg(self.h, *[ptr(a) for a in ins], *[ptr(a) for a in outs], nz))
        return tuple(outs)

    def refraction_waqg(self, BRk, BIk, psik):
        ins = [self._c(a) for a in (BRk, BIk, psik)]
        nz = ins[0].shape[0]
        outs = [np.empty_like(ins[0]) for _ in range(2)]
        self._ck(lib().qg_refraction_waqg(self.h, *[ptr(a) for a in ins], *[ptr(a) for a in outs], nz))
        return tuple(outs)

    def compute_qw(self, BRk, BIk):
        ins = [self._c(a) for a in (BRk, BIk)]
        out = np.empty_like(ins[0])
        self._ck(lib().qg_compute_qw(self.h, ptr(ins[0]), ptr(ins[1]), ptr(out), ins[0].shape[0]))
        return out

    def psi_solver(self, qstar):
        q = self._c(qstar)
        out = np.empty_like(q)
        self._ck(lib().qg_psi_solver(self.h, ptr(q), ptr(out)))
        return out

    def A_solver_ybj_plus(self, bk):
        b = self._c(bk)
        a, c = np.empty_like(b), np.empty_like(b)
        self._ck(lib().qg_A_solver_ybj_plus(self.h, ptr(b), ptr(a), ptr(c)))
        return a, c

    # -- output path (the netCDF dumps' real-space FP32 fields) ----------------------
    def dump_psi(self, U_scale: float, L_scale: float, level0: int = 0, nlev: int | None = None):
        """psi in physical space, dimensional, float32 [nz][n][n] (ncdump_psi)."""
        nlev = self.n3 - level0 if nlev is None else nlev
        out = np.empty((nlev, self.n, self.n), dtype=np.float32)
        self._ck(lib().qg_dump_psi(self.h, ptr(out), level0, nlev, float(U_scale), float(L_scale)))
        return out

    def dump_la(self, Uw_scale: float, la: bool = False, level0: int = 0, nlev: int | None = None):
        """Real and imaginary wave fields in physical space, float32 (ncdump_la:
        B; with la=True the YBJ+ LA = B + kh^2 A/(4 Bu))."""
        nlev = self.n3 - level0 if nlev is None else nlev
        outR = np.empty((nlev, self.n, self.n), dtype=np.float32)
        outI = np.empty_like(outR)
        self._ck(lib().qg_dump_la(self.h, ptr(outR), ptr(outI), level0, nlev, float(Uw_scale), int(la)))
        return outR, outI

    def write_dumps(self, directory, count: int, time: float, U_scale: float, L_scale: float, Uw_scale: float):
        """psiNNN and laNNN dumps as ncdump_psi / ncdump_la write them (raw
        binary + JSON sidecar, qgybj.io); returns the two .bin paths."""
        from .io import dump_time_seconds, write_dump
        ts = dump_time_seconds(time, L_scale, U_scale)
        p1 = write_dump(directory, "psi", count, {"psi": self.dump_psi(U_scale, L_scale)}, ts)
        lr, li = self.dump_la(Uw_scale)
        p2 = write_dump(directory, "la", count, {"LAr": lr, "LAi": li}, ts)
        return p1, p2

    # -- omega equation (vertical velocity) ------------------------------------------
    def omega_eqn_rhs(self, psik):
        p = self._c(psik)
        out = np.empty_like(p)
        self._ck(lib().qg_omega_eqn_rhs(self.h, ptr(p), ptr(out)))
        return out

    def omega_equation(self, rhs):
        r = self._c(rhs)
        out = np.empty_like(r)
        self._ck(lib().qg_omega_equation(self.h, ptr(r), ptr(out)))
        return out

    def omega(self):
        """w (spectral, dense layout) from the resident psi."""
        out = np.empty(self.spectral_shape, dtype=np.complex128)
        self._ck(lib().qg_omega(self.h, ptr(out)))
        return out

    # -- adjoint (FP64 handles) ------------------------------------------------------
    def adjoint_run(self, q0, BR0, BI0, nsteps: int, ckpt_every: int = 10, gradient: bool = True):
        """J = 1/2 sum over the central quarter and top fifth of |LA|^2 after
        nsteps from (q0, B0), and its gradient with respect to (q0, BR0, BI0)."""
        ins = [self._c(a) for a in (q0, BR0, BI0)]
        J = C.c_double()
        outs = [np.empty_like(ins[0]) for _ in range(3)] if gradient else [None] * 3
        self._ck(lib().qg_adjoint_run(self.h, *[ptr(a) for a in ins], int(nsteps), int(ckpt_every), 0, C.byref(J),
                                      *[ptr(a) for a in outs]))
        return (J.value, tuple(outs)) if gradient else J.value

    def adjoint_step(self, X, lX=None, euler_first: bool = False, forward: bool = True):
        """One step from the carried state X = (q, q_old, BR, BI, BR_old, BI_old):
        returns (next X or None, transpose of the step's Jacobian at X applied to lX or None)."""
        Xs = [self._c(a) for a in X]
        Xa = (C.c_void_p * 6)(*[ptr(a) for a in Xs])
        Xn = [np.empty_like(Xs[0]) for _ in range(6)] if forward else None
        lo = None
        if lX is not None:
            lXs = [self._c(a) for a in lX]
            la = (C.c_void_p * 6)(*[ptr(a) for a in lXs])
            lo = [np.empty_like(Xs[0]) for _ in range(6)]
        self._ck(lib().qg_adjoint_step(self.h, int(euler_first), Xa, la if lX is not None else None,
                                       (C.c_void_p * 6)(*[ptr(a) for a in Xn]) if forward else None,
                                       (C.c_void_p * 6)(*[ptr(a) for a in lo]) if lo is not None else None))
        return (tuple(Xn) if forward else None), (tuple(lo) if lo is not None else None)


def simulation_for(rc: RunConfig, device: int = 0, precision: str | None = None):
    """Handle and initial condition of a run configuration: the
    initialisation of main_waqg.f90:117-147 with the seeded generator in
    place of generate_fields_stag / ncread_*."""
    ic = make_initial_condition(rc)
    params = model_parameters(rc, ic.delt)
    sim = Simulation(params, precision or rc.precision, device=device, levels_per_batch=rc.levels_per_batch,
                     solve_columns=rc.solve_columns,
                     use_graphs=rc.use_graphs)
    sim.set_state("psi", ic.psi)
    sim.set_state("BR", ic.BR)
    sim.set_state("BI", ic.BI)
    sim.init_state(apply_sumB=True, q_from_psi=True)
    return sim, ic, params


class Ensemble:
    """Independent runs of possibly different sizes advanced by one CUDA graph
    launch per step (qg_ensemble_*).  ``members[m]`` is a Simulation view of
    member m for state I/O; call synchronize() before touching members after
    step()."""

    def __init__(self, params_list: list[dict], precision: str = "mixed", device: int = 0,
                 levels_per_batch: list[int] | None = None, solve_columns: list[int] | None = None):
        L = lib()
        n = len(params_list)
        cfgs = (QgConfig * n)()
        self._keep = []
        for m, p in enumerate(params_list):
            lpb = levels_per_batch[m] if levels_per_batch else 0
            c, keep = make_config(p, precision, device, lpb, solve_columns=solve_columns[m] if solve_columns else 0)
            cfgs[m] = c
            self._keep += keep
        e = C.c_void_p()
        st = L.qg_ensemble_create(cfgs, n, C.byref(e))
        if st:
            raise QgError(st, (L.qg_last_error(None) or b"").decode())
        self.e = e
        self.members = []
        for m, p in enumerate(params_list):
            h = C.c_void_p()
            self._ck(L.qg_ensemble_member(self.e, m, C.byref(h)))
            self.members.append(Simulation(p, precision, device, _handle=h))

    def _ck(self, st):
        if st:
            raise QgError(st, (lib().qg_ensemble_last_error(self.e) or b"").decode())

    def step(self, nsteps: int = 1, euler_first: bool = False):
        self._ck(lib().qg_ensemble_step(self.e, int(nsteps), int(euler_first)))

    def profile_step(self, euler_first: bool = False) -> dict:
        """One step of every run with CUDA events around each launch:
        {class: (ms, launches)} summed over the runs."""
        from ._lib import KERNEL_CLASSES
        n = len(KERNEL_CLASSES)
        ms = (C.c_double * n)()
        cnt = (C.c_int * n)()
        self._ck(lib().qg_ensemble_profile_step(self.e, int(euler_first), ms, cnt, n))
        return {k: (ms[i], cnt[i]) for i, k in enumerate(KERNEL_CLASSES)}

    def set_lanes(self, lanes: int):
        """Runs (stacks of same-shape members, or single members) the step
        graph advances concurrently (qg_ensemble_set_lanes)."""
        self._ck(lib().qg_ensemble_set_lanes(self.e, int(lanes)))

    def synchronize(self):
        self._ck(lib().qg_ensemble_synchronize(self.e))

    def stream(self) -> int:
        s = C.c_void_p()
        self._ck(lib().qg_ensemble_get_stream(self.e, C.byref(s)))
        return int(s.value or 0)

    def close(self):
        if getattr(self, "e", None):
            for m in self.members:
                m.h = None
            lib().qg_ensemble_destroy(self.e)
            self.e = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
