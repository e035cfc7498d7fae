"""Host-side logic of the quench protocols and the ground-state grid
(finite_ed.jl:437-650, gs_benchmark.jl:28-175): parameter order, sectors and
CSV layout.  No GPU."""
import csv

import numpy as np

from lgt_gb300 import ed, gs_grid, protocols


def test_param_grid_order_is_julia_vec_order():
    # [(m=m, g=g) for m in MASS_LIST, g in G_LIST] |> vec: m runs fastest
    assert len(gs_grid.PARAM_GRID) == 25
    assert gs_grid.PARAM_GRID[0] == (0.25, 0.25)
    assert gs_grid.PARAM_GRID[1] == (0.5, 0.25)
    assert gs_grid.PARAM_GRID[4] == (4.0, 0.25)
    assert gs_grid.PARAM_GRID[5] == (0.25, 0.5)
    assert gs_grid.PARAM_GRID[24] == (4.0, 4.0)


def test_quench_a_sector():
    g = ed.string_charges(3, 4)  # iy_str = 2
    expect = np.zeros((3, 4), np.int32)
    expect[0, 1], expect[1, 1] = 1, -2
    np.testing.assert_array_equal(g, expect)
    assert -g.sum() == 1  # one fermion


def test_float_text_matches_julia_shortest_repr():
    assert protocols._fmt(0.5) == "0.5"
    assert protocols._fmt(2.0) == "2.0"
    assert protocols._fmt(1e-5) == "1.0e-5"
    assert protocols._fmt(-3.25e-12) == "-3.25e-12"
    assert protocols._fmt(1.5e20) == "1.5e20"


def test_quench_csv_layout(tmp_path):
    data = [dict(t=0.0, nf_mean=0.5, nf_even=0.25, nf_odd=0.75, E2_mean=0.0, plaq_mean=9.0),
            dict(t=0.02, nf_mean=0.5, nf_even=0.3, nf_odd=0.7, E2_mean=1e-5, plaq_mean=9.0)]
    p = protocols.write_csv(str(tmp_path / "x_data.csv"), protocols.data_to_rows(data))
    rows = list(csv.reader(open(p)))
    assert rows[0] == ["t", "nf_mean", "nf_even", "nf_odd", "E2_mean"]
    assert rows[2] == ["0.02", "0.5", "0.3", "0.7", "1.0e-5"]


def test_batched_quench_csv_has_value_column(tmp_path):
    step = [dict(t=0.0, nf_mean=0.5, nf_even=0.5, nf_odd=0.5, E2_mean=0.0)] * 2
    data = [step, step]  # 2 steps, K = 2
    p = protocols._save(str(tmp_path), "q", data, 2, "m_final", np.array([0.1, 0.3]))
    rows = list(csv.reader(open(p)))
    assert rows[0][0] == "m_final" and len(rows) == 1 + 4
    assert [r[0] for r in rows[1:]] == ["0.1", "0.1", "0.3", "0.3"]


def test_grid_row_schema_with_missing_peps(tmp_path):
    r = gs_grid._row(7, 0.5, 0.5, 3, 4, 1, -12.5, dict(nf_mean=0.5, nf_even=0.2, nf_odd=0.8,
                                                       E2_mean=0.1), 72211, 0.25)
    p = gs_grid.write_row(str(tmp_path / "gs_benchmark_007.csv"), r)
    rows = list(csv.reader(open(p)))
    assert tuple(rows[0]) == gs_grid.COLUMNS
    row = dict(zip(rows[0], rows[1]))
    assert row["task_id"] == "7" and row["ed_basis_dim"] == "72211"
    assert row["ed_E0"] == "-12.5" and row["peps_nf_mean"] == "" and row["d_cdw"] == ""
    assert row["D_bond"] == "4" and row["tau_ite"] == "0.05"
