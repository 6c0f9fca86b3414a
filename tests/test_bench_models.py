"""The byte and flop models bench.py reports its roofline and transform rate
on (CPU only): the retained-mode field passes of the 512^2 x 256 step, the
dominant kernel's passes, the fields-plus-planes traffic model and the
transform count of each precision path."""
from __future__ import annotations

import bench
from qgybj.config import dealias_mask, kmax

N, N3 = 512, 256


def test_step_moves_22_field_passes_of_the_retained_modes():
    fld = int(dealias_mask(N).sum()) * 8
    assert int(dealias_mask(N).sum()) == 45681
    a = bench.algorithmic_bytes(N, N3, N3, "mixed")
    assert a["step"] == 22 * fld * N3 == 2058203136
    assert a["col_update"] == 14 * fld * N3
    # q is read again by k_col_inv and k_col_qw: 24 passes over the kernels
    # on the mixed path (k_col_inv reads psi and q only), 26 in FP64
    per_level = lambda p: sum(bench.algorithmic_bytes(N, N3, 1, p)[k] for k in ("col_inv", "col_update", "col_qw")) \
        + bench.algorithmic_bytes(N, 1, 1, p)["solve"]
    assert per_level("mixed") == 24 * fld
    assert per_level("fp64") == 26 * 2 * fld


def test_traffic_model_counts_fields_and_planes():
    fld = int(dealias_mask(N).sum()) * 8
    pln = N * (kmax(N) + 1) * 8
    t = bench.traffic_model(N, 1, "mixed")
    assert t["col_inv"] == 2 * fld + 4 * pln          # B's planes kept from the previous update
    assert t["col_update"] == 14 * fld + 10 * pln
    assert bench.traffic_model(N, 1, "fp64")["col_inv"] == 4 * 2 * fld + 6 * 2 * pln


def test_transform_count_per_path():
    m = bench.transform_flops(N, N3, "mixed")
    f = bench.transform_flops(N, N3, "fp64")
    per = m["per_complex_fft"]
    assert per == 64 * 56 + 2 * 64 * (56 + 7 * 6)       # 512 = 8 x 8 x 8
    K = kmax(N)
    assert m["transforms"] == (16 * (K + 1) + 11 * N) * per * N3
    assert f["transforms"] == (18 * (K + 1) + 11 * N) * per * N3
    assert abs((f["transforms"] + f["solve_fp64"]) / 1e9 - 36.31) < 0.01
