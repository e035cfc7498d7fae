"""Ground-state benchmark grid of the reference (gs_benchmark.jl:28-175), ED
side, on the GPU library.

The reference sweeps a 5 x 5 (m, g) grid on the 3x4 staggered sector as a
SLURM array, one task per point, each writing a one-row CSV
``gs_benchmark_<idx>.csv``.  Here ``run_one_point`` is that task and
``run_grid`` maps the whole sweep (or any subset of task ids) onto one
K-batched ground-state solve on one shared basis, then writes the same
one-row CSVs.  Columns follow the reference's schema; the PEPS columns and
the PEPS - ED differences are written empty (``missing``), because the PEPS
solver is not part of this library.  ``ed_time_s`` of a batched run is the
batch's wall time divided by its number of points.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

from . import ed
from .protocols import _fmt

MASS_LIST = [0.25, 0.5, 1.0, 2.0, 4.0]
G_LIST = [0.25, 0.5, 1.0, 2.0, 4.0]
# [(m, g) for m in MASS_LIST, g in G_LIST] |> vec: m runs fastest
PARAM_GRID = [(m, g) for g in G_LIST for m in MASS_LIST]

BENCH_NX, BENCH_NY, BENCH_DG = 3, 4, 1
BENCH_D_BOND, BENCH_D_MAX = 4, 12
BENCH_T_HOP, BENCH_TAU, BENCH_N_ITE, BENCH_MU_ITE = 1.0, 0.05, 300, 0.0

COLUMNS = ("task_id", "m", "g", "t_hop", "nx", "ny", "dg", "D_bond", "D_max", "tau_ite", "n_ite",
           "mu_ite", "peps_nf_mean", "peps_nf_even", "peps_nf_odd", "peps_E2_mean", "peps_S_h",
           "peps_S_v", "peps_S_mean", "peps_time_s", "ed_E0", "ed_nf_mean", "ed_nf_even",
           "ed_nf_odd", "ed_E2_mean", "ed_basis_dim", "ed_time_s", "d_nf_mean", "d_nf_even",
           "d_nf_odd", "d_E2_mean", "d_cdw")


def _cell(v):
    if v is None:
        return ""  # missing
    if isinstance(v, (float, np.floating)):
        return _fmt(v)
    return str(v)


def write_row(path, row):
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(path, "w") as f:
        f.write(",".join(COLUMNS) + "\n")
        f.write(",".join(_cell(row.get(c)) for c in COLUMNS) + "\n")
    return path


def _row(task_id, m, g, nx, ny, dg, E0, obs, dim, seconds):
    return dict(task_id=task_id, m=float(m), g=float(g), t_hop=BENCH_T_HOP, nx=nx, ny=ny, dg=dg,
                D_bond=BENCH_D_BOND, D_max=BENCH_D_MAX, tau_ite=BENCH_TAU, n_ite=BENCH_N_ITE,
                mu_ite=BENCH_MU_ITE, ed_E0=float(E0), ed_nf_mean=float(obs["nf_mean"]),
                ed_nf_even=float(obs["nf_even"]), ed_nf_odd=float(obs["nf_odd"]),
                ed_E2_mean=float(obs["E2_mean"]), ed_basis_dim=int(dim),
                ed_time_s=float(seconds))


def run_grid(task_ids=None, out_dir="results/gs_bench", *, nx=BENCH_NX, ny=BENCH_NY,
             dg=BENCH_DG, precision="fp64", model="ref", write=True):
    """ED ground states of the grid points ``task_ids`` (1-based, default
    all 25) in one batched solve; returns the rows (dicts) in task order."""
    ids = list(range(1, len(PARAM_GRID) + 1)) if task_ids is None else [int(i) for i in task_ids]
    for i in ids:
        if not 1 <= i <= len(PARAM_GRID):
            raise ValueError("task_id=%d outside 1..%d" % (i, len(PARAM_GRID)))
    ms = np.array([PARAM_GRID[i - 1][0] for i in ids])
    gs = np.array([PARAM_GRID[i - 1][1] for i in ids])
    t0 = time.perf_counter()
    states, key_dict = ed.build_basis(nx, ny, dg, ed.staggered_charges(nx, ny))
    H = ed.build_hamiltonian(states, key_dict, nx, ny, dg, g=gs, t=BENCH_T_HOP, m=ms, model=model)
    try:
        E0, psi = ed.find_ground_state(H, precision=precision, as_complex=False)
    finally:
        H.close()
    E0 = np.atleast_1d(E0)
    psi = psi.reshape(len(states), len(ids))
    obs = ed.measure_ED(psi, states, nx, ny, dg, 0.0)
    obs = obs if isinstance(obs, list) else [obs]
    per_point = (time.perf_counter() - t0) / len(ids)
    rows = []
    for q, i in enumerate(ids):
        r = _row(i, ms[q], gs[q], nx, ny, dg, E0[q], obs[q], len(states), per_point)
        rows.append(r)
        if write:
            write_row(os.path.join(out_dir, "gs_benchmark_%03d.csv" % i), r)
    return rows


def run_one_point(task_id, out_dir="results/gs_bench", **kw):
    """One SLURM-array task (gs_benchmark.jl:86-175), ED side."""
    return run_grid([task_id], out_dir, **kw)[0]


def _parse_args(argv):
    if not argv:
        raise SystemExit("Usage: python -m lgt_gb300.gs_grid <task_id|all> [--out-dir DIR]")
    task = argv[0]
    out_dir = "results/gs_bench"
    i = 1
    while i < len(argv):
        if argv[i] == "--out-dir" and i + 1 < len(argv):
            out_dir = argv[i + 1]
            i += 2
        else:
            i += 1
    return task, out_dir


def main(argv=None):
    task, out_dir = _parse_args(sys.argv[1:] if argv is None else argv)
    if task == "all":
        run_grid(None, out_dir)
    else:
        run_one_point(int(task), out_dir)
    return 0


if __name__ == "__main__":
    sys.exit(main())
