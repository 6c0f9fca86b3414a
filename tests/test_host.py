"""Host-side checks that need no GPU: the C-ABI library loads and exports
every declared entry point, the ctypes struct layout matches the header,
and the run configurations / initial-condition generator behave."""
from __future__ import annotations

import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import qgybj
from qgybj import _lib
from qgybj.config import CONFIGS, dealias_mask, ensemble_members, kmax, make_initial_condition, model_parameters, scaled

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "qgybj.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(qg_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    L = qgybj.lib()
    decl = declared_functions()
    assert len(decl) >= 19
    for name in decl:
        assert hasattr(L, name), name
    assert set(decl) == set(_lib.EXPORTS)


def test_struct_layout_matches_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "abi"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(ROOT / "tests" / "abi_layout.c"), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    assert int(out.pop("sizeof")) == C.sizeof(_lib.QgConfig)
    assert int(out.pop("energy")) == C.sizeof(_lib.QgEnergy)
    assert int(out.pop("tuning")) == C.sizeof(_lib.QgTuning)
    for f, off in out.items():
        assert getattr(_lib.QgConfig, f).offset == int(off), f


def test_create_without_device_reports_status():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present; covered by the gpu tests")
    rc = scaled(CONFIGS["c0"], 16, 4)
    ic = make_initial_condition(rc)
    with pytest.raises(qgybj.QgError) as e:
        qgybj.Simulation(model_parameters(rc, ic.delt), "fp64")
    assert e.value.status == _lib.QG_ERR_CUDA


def test_error_status_text():
    cfg = _lib.QgConfig()
    assert qgybj.lib().qg_config_defaults(C.byref(cfg)) == 0
    assert cfg.ybj_plus == 1 and cfg.inviscid == 1 and cfg.use_graphs == 1
    h = C.c_void_p()
    cfg.n1, cfg.n2, cfg.n3 = 32, 64, 8
    assert qgybj.lib().qg_create(C.byref(cfg), C.byref(h)) == _lib.QG_ERR_UNSUPPORTED
    assert b"n1 must equal n2" in qgybj.lib().qg_last_error(None)
    assert qgybj.lib().qg_step(None, 0) == _lib.QG_ERR_ARG


@pytest.mark.parametrize("name", ["c0", "c1", "c4"])
def test_initial_condition_properties(name):
    rc = CONFIGS[name] if name != "c1" else scaled(CONFIGS["c1"], 64, 32)
    ic = make_initial_condition(rc)
    L = dealias_mask(rc.n)
    assert np.abs(np.where(L[None], 0, ic.psi)).max() == 0
    kxa = np.arange(rc.n // 2 + 1)
    kya = np.fft.fftfreq(rc.n, 1.0 / rc.n).astype(int)
    kh2 = (kxa[None, :] ** 2 + kya[:, None] ** 2).astype(float)
    z2 = kh2[None] ** 2 * np.abs(ic.psi) ** 2
    msq = (2 * z2.sum(axis=(1, 2)) - z2[:, 0, 0]).mean()
    assert abs(msq - 1.0) < 1e-12
    zs = (np.arange(rc.n3) + 0.5) / rc.n3
    assert np.allclose(ic.BR[:, 0, 0].real, np.exp(-((1 - zs) / rc.wave_depth) ** 2))
    assert ic.delt > 0 and ic.umax > 0
    p = model_parameters(rc, ic.delt)
    K = kmax(rc.n)
    assert abs(p["delt"] * p["nuh1"] * K ** 4 - rc.if_kt) < 1e-12


def test_exponential_stratification_profile():
    rc = CONFIGS["c2"]
    a = rc.a_ell_ut()
    assert a.shape == (256,)
    assert abs(a[-1] - 1.0) < 1e-15 and abs(a[0] - np.exp(10 * (1 - 1 / 256))) < 1e-9


def test_ensemble_members():
    m = ensemble_members()
    assert len(m) == 64
    sizes = [(r.n, r.n3) for r in m]
    assert sizes.count((64, 32)) == 24 and sizes.count((128, 64)) == 24 and sizes.count((256, 128)) == 16
    assert all(0.05 <= r.Ro <= 0.2 and 0.05 <= r.wave_depth <= 0.2 for r in m)
    assert len({r.seed for r in m}) == 64


def test_dump_files_round_trip(tmp_path):
    """qgybj.io writes psiNNN/laNNN dumps as float32 [z][y][x] plus a JSON
    sidecar (names and time as the netCDF files carry them) and reads them back."""
    from qgybj.io import dump_time_seconds, read_dump, write_dump
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal((4, 8, 8)).astype(np.float32), rng.standard_normal((4, 8, 8)).astype(np.float32)
    ts = dump_time_seconds(12.5, 5e4, 0.25)
    assert ts == float(np.float32(12.5 * 5e4 / 0.25))
    p = write_dump(tmp_path, "la", 7, {"LAr": a, "LAi": b}, ts)
    assert p.name == "la007.out.bin"
    got, t = read_dump(p)
    assert t == ts and list(got) == ["LAr", "LAi"]
    assert np.array_equal(got["LAr"], a) and np.array_equal(got["LAi"], b)
    with pytest.raises(ValueError):
        write_dump(tmp_path, "x", 0, {"a": a, "b": b[:2]}, ts)
