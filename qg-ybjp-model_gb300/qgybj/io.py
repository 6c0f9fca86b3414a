"""Raw-binary stand-in for the reference's netCDF dumps (IO_ncf.f90).

The reference writes psiNNN.out.nc (variable "psi") and laNNN.out.nc
(variables "LAr", "LAi"), each a float32 (x, y, z) array with x fastest,
plus the dump time in seconds.  No netCDF library is available here, so the
same arrays go to NAME+NNN.out.bin (the variables one after another, float32
little-endian, C order [z][y][x]) with a JSON sidecar NAME+NNN.out.json
holding the dimensions, the variable names and byte offsets, and the time.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np


def dump_time_seconds(time: float, L_scale: float, U_scale: float) -> float:
    """time_seconds = time*L_scale/U_scale stored as a default REAL (IO_ncf.f90:32)."""
    return float(np.float32(time * L_scale / U_scale))


def write_dump(directory, name: str, count: int, variables: dict, time_seconds: float) -> Path:
    """Write one dump; returns the path of the .bin file."""
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    stem = f"{name}{count:03d}.out"
    meta = {"time": time_seconds, "variables": [], "dims": None}
    off = 0
    with open(d / f"{stem}.bin", "wb") as f:
        for vname, arr in variables.items():
            a = np.ascontiguousarray(arr, dtype="<f4")
            nz, ny, nx = a.shape
            dims = {"x": nx, "y": ny, "z": nz}
            if meta["dims"] is None:
                meta["dims"] = dims
            elif meta["dims"] != dims:
                raise ValueError("variables of one dump must share their dimensions")
            f.write(a.tobytes())
            meta["variables"].append({"name": vname, "dtype": "float32", "offset": off, "order": "z,y,x"})
            off += a.nbytes
    (d / f"{stem}.json").write_text(json.dumps(meta, indent=1))
    return d / f"{stem}.bin"


def read_dump(path) -> tuple[dict, float]:
    """Read a dump written by write_dump: ({name: float32 [z][y][x]}, time)."""
    p = Path(path)
    meta = json.loads(p.with_suffix(".json").read_text())
    dims = meta["dims"]
    shape = (dims["z"], dims["y"], dims["x"])
    raw = p.read_bytes()
    out = {}
    for v in meta["variables"]:
        n = int(np.prod(shape))
        out[v["name"]] = np.frombuffer(raw, dtype="<f4", count=n, offset=v["offset"]).reshape(shape).copy()
    return out, meta["time"]
