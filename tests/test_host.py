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
    structs = {"qg_config": _lib.QgConfig, "qg_tuning": _lib.QgTuning, "qg_energy": _lib.QgEnergy}
    for name, cls in structs.items():
        assert int(out.pop(f"sizeof.{name}")) == C.sizeof(cls), name
    seen = set()
    for key, off in out.items():
        name, f = key.split(".")
        assert getattr(structs[name], f).offset == int(off), key
        seen.add(name)
    assert seen == set(structs)


def test_noalloc_pointer_checks(tmp_path):
    """The argument checks of qg_fft_c2r_noalloc (csrc/noalloc_check.h) on
    every branch, host-only: device memory of the current GPU passes; host
    memory, another GPU's memory and misaligned pointers are refused."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "check.cc"
    src.write_text(r'''
#include <stdio.h>
#include "noalloc_check.h"
int main() {
  alignas(16) static char buf[64];
  const void* a16 = buf; const void* a8 = buf + 8;
  printf("%d %d %d %d %d %d %d %d\n",
         qgna::check_pointer(2, 0, 0, a16, 16),   /* device memory, current GPU */
         qgna::check_pointer(3, 1, 0, a16, 16),   /* managed memory: any GPU */
         qgna::check_pointer(0, -1, 0, a16, 16),  /* unregistered host memory */
         qgna::check_pointer(1, 0, 0, a16, 16),   /* page-locked host memory */
         qgna::check_pointer(2, 1, 0, a16, 16),   /* another GPU's memory */
         qgna::check_pointer(2, 0, 0, a8, 16),    /* 8-byte aligned complex input */
         qgna::check_pointer(2, 0, 0, a8, 8),     /* 8-byte aligned real output */
         qgna::check_pointer(2, 0, 0, buf + 4, 8));
  return 0;
}
''')
    exe = tmp_path / "check"
    subprocess.run([cxx, "-std=c++17", "-I", str(ROOT / "qg-ybjp-model_gb300" / "csrc"), str(src), "-o", str(exe)],
                   check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    ok, not_dev, other, misaligned = 0, 1, 2, 3
    assert got == [ok, ok, not_dev, not_dev, other, misaligned, ok, misaligned]


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


_BAD_CONFIGS = [
    # (field, value, status, message fragment): qg_create validates on the
    # host, before any device call
    ("n2", 64, "QG_ERR_UNSUPPORTED", b"n1 must equal n2"),
    ("n1", 48, "QG_ERR_UNSUPPORTED", b"power of two"),
    ("n3", 1, "QG_ERR_ARG", b"n3 must be >= 2"),
    ("n3", 2048, "QG_ERR_UNSUPPORTED", b"n3 must be <= 1024"),
    ("precision", 7, "QG_ERR_ARG", b"bad precision"),
    ("ybj_plus", 2, "QG_ERR_ARG", b"ybj_plus must be 0 or 1"),
    ("a_ell_ut", None, "QG_ERR_ARG", b"a_ell_ut is required"),
    ("dz", 0.0, "QG_ERR_ARG", b"must be positive"),
    ("Ro", -1.0, "QG_ERR_ARG", b"must be positive"),
    ("delt", float("nan"), "QG_ERR_NONFINITE", b"non-finite"),
    ("nuh1", float("inf"), "QG_ERR_NONFINITE", b"non-finite"),
    ("ilap2", 12, "QG_ERR_ARG", b"ilap out of range"),
]


@pytest.mark.parametrize("field,value,status,msg", _BAD_CONFIGS)
def test_create_rejects_bad_configuration(field, value, status, msg):
    """qg_create's configuration checks (csrc/capi.cu:validate_config): each
    rule returns its status and message with no handle made."""
    from qgybj.model import make_config
    rc = scaled(CONFIGS["c0"], 32, 8)
    ic = make_initial_condition(rc)
    cfg, keep = make_config(model_parameters(rc, ic.delt), "fp64")
    if field == "n1":
        cfg.n1 = cfg.n2 = value
    elif field == "a_ell_ut":
        cfg.a_ell_ut = None
    else:
        setattr(cfg, field, value)
    h = C.c_void_p()
    assert qgybj.lib().qg_create(C.byref(cfg), C.byref(h)) == getattr(_lib, status)
    assert not h.value
    assert msg in qgybj.lib().qg_last_error(None)


def test_create_rejects_non_finite_profile():
    from qgybj.model import make_config
    rc = scaled(CONFIGS["c1"], 32, 8)
    ic = make_initial_condition(rc)
    params = model_parameters(rc, ic.delt)
    a = np.array(params["a_ell_ut"], dtype=np.float64)
    a[3] = np.nan
    params = dict(params, a_ell_ut=a)
    cfg, keep = make_config(params, "mixed")
    h = C.c_void_p()
    assert qgybj.lib().qg_create(C.byref(cfg), C.byref(h)) == _lib.QG_ERR_NONFINITE


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
