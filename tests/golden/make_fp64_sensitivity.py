"""How far FP64 roundoff alone carries through the step: the evidence behind
the FP64 tolerance of the exponentially stratified runs.

Runs the FP64 oracle on a configuration's seeded initial condition three ways
and records, at a few step counts, the per-field relative L2 distance of
  ext: the same run with the 2D FFTs in extended precision (np.longdouble:
       80-bit on x86-64) and every other operation in FP64;
  ulp: the same run from a psi perturbed by one unit in the last place on
       every retained mode (seeded signs);
to the plain FP64 run.  Either distance is a floor under the agreement two
correct FP64 implementations of the step (this CUDA path, the Fortran
reference with MKL's FFTW and DGTSV, or the oracle on another machine) can
reach, because they differ from each other by roundoff of the same size.

  python tests/golden/make_fp64_sensitivity.py c1 [--steps 200] [--workers 8]

writes tests/golden/fp64_sensitivity_<config>.json.  C0 (constant N^2) is
the control: its distances stay near 1e-14.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import platform
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
for _p in (str(ROOT), str(ROOT / "qg-ybjp-model_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

FIELDS = ("psi", "q", "LAr", "LAi", "BR", "BI")


def fields_of(model, st):
    return {"psi": st.psi, "q": st.q, "BR": st.BR, "BI": st.BI,
            "LAr": model.la_from_b(st.BR, st.AR), "LAi": model.la_from_b(st.BI, st.AI)}


def run(kind: str, cfg: str, steps: int, marks: list[int], workers: int, out_dir: str):
    import numpy as np

    from oracle import qgybj_oracle as orc
    from qgybj.config import CONFIGS
    from tests.helpers import oracle_for

    orc.set_workers(workers)
    if kind == "ext":
        orc.set_fft_dtype(np.longdouble)
    model, st, ic, params = oracle_for(CONFIGS[cfg])
    if kind == "ulp":
        rng = np.random.Generator(np.random.PCG64(12345))
        psi = ic.psi.copy()
        sgn = np.where(rng.random(psi.shape) < 0.5, -1.0, 1.0)
        re = np.nextafter(psi.real, psi.real + sgn * np.inf)
        sgn = np.where(rng.random(psi.shape) < 0.5, -1.0, 1.0)
        im = np.nextafter(psi.imag, psi.imag + sgn * np.inf)
        psi = np.where(model.Lb[None], re + 1j * im, psi)
        st = orc.initial_state(model, psi, ic.BR, ic.BI)
    t0 = time.time()
    for i in range(steps):
        st = model.step(st, i == 0)
        if i + 1 in marks:
            np.savez(os.path.join(out_dir, f"{kind}_{i + 1}.npz"), **fields_of(model, st))
    return kind, time.time() - t0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("config", choices=("c0", "c1"))
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--workers", type=int, default=max(1, (os.cpu_count() or 3) // 3))
    ap.add_argument("--scratch", default=None, help="directory for the intermediate states")
    args = ap.parse_args(argv)
    import tempfile

    import numpy as np

    marks = sorted({m for m in (1, 2, 10, 50, 100, 200) if m <= args.steps} | {args.steps})
    scratch = args.scratch or tempfile.mkdtemp(prefix="qg_sens_")
    ctx = mp.get_context("spawn")
    with ctx.Pool(3) as pool:
        res = pool.starmap(run, [(k, args.config, args.steps, marks, args.workers, scratch)
                                 for k in ("base", "ext", "ulp")])
    secs = dict(res)
    out = {"config": args.config, "steps": args.steps, "marks": marks,
           "platform": f"{platform.machine()} {platform.system()}, numpy {np.__version__}",
           "longdouble_mantissa_bits": int(np.finfo(np.longdouble).nmant) + 1,
           "seconds": secs, "relL2": {}}
    for k in ("ext", "ulp"):
        out["relL2"][k] = {}
        for m in marks:
            a = np.load(os.path.join(scratch, f"base_{m}.npz"))
            b = np.load(os.path.join(scratch, f"{k}_{m}.npz"))
            out["relL2"][k][str(m)] = {f: float(np.linalg.norm(b[f] - a[f]) / np.linalg.norm(a[f])) for f in FIELDS}
    path = HERE / f"fp64_sensitivity_{args.config}.json"
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(path)


if __name__ == "__main__":
    main()
