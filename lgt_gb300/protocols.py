"""Quench protocols A, B and C of the reference ED driver and their CSV output
(finite_ed.jl:437-445, 491-650), on the GPU library.

Each ``run_quench_*_ED`` keeps the reference's keyword names and defaults
(lattice 3x4, dg = 1, g = t = 1, m = 2, dt = 0.02, 2 steps; ED_* constants at
finite_ed.jl:60-65), builds the sector, prepares the initial state, evolves
with ``evolve_ED`` and writes ``<results_dir>/<label>_data.csv`` with the
columns of ``data_to_df_ED`` (t, nf_mean, nf_even, nf_odd, E2_mean).  The
ED-vs-PEPS plots of the reference are not produced (plotting is outside this
library).

Batched form (this library's addition): the post-quench coupling of B and C
(``m_final``, ``g_final``) may be a sequence of K values.  All K quenches then
share one basis and run as one K-point Krylov panel; the CSV gets one block
of rows per value, with the value in a leading column.
"""
from __future__ import annotations

import csv
import os
import sys

import numpy as np

from . import ed

ED_NX, ED_NY, ED_DG = 3, 4, 1
ED_G_COUP, ED_T_HOP, ED_M_MASS = 1.0, 1.0, 2.0

COLUMNS = ("t", "nf_mean", "nf_even", "nf_odd", "E2_mean")


def data_to_rows(data):
    """data_to_df_ED (finite_ed.jl:437-445): one row per measurement."""
    return [{c: float(d[c]) for c in COLUMNS} for d in data]


def _fmt(v):
    # shortest round-trip text of a Float64, as Julia prints it
    r = repr(float(v))
    if "e" in r:
        mant, ex = r.split("e")
        if "." not in mant:
            mant += ".0"
        r = "%se%d" % (mant, int(ex))
    return r


def write_csv(path, rows, columns=COLUMNS):
    """CSV with a header line and one line per row (CSV.write layout)."""
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    with open(path, "w", newline="") as f:
        w = csv.writer(f, lineterminator="\n")
        w.writerow(columns)
        for r in rows:
            w.writerow([_fmt(r[c]) if isinstance(r[c], (float, np.floating)) else r[c]
                        for c in columns])
    return path


def _per_point(data, K):
    """evolve_ED output for K points -> K lists of dicts."""
    if K == 1:
        return [data]
    return [[step[k] for step in data] for k in range(K)]


def _save(results_dir, label, data, K, key=None, values=None):
    path = os.path.join(results_dir, "%s_data.csv" % label)
    if K == 1:
        return write_csv(path, data_to_rows(data))
    rows = []
    for k, series in enumerate(_per_point(data, K)):
        for r in data_to_rows(series):
            rows.append(dict({key: float(values[k])}, **r))
    return write_csv(path, rows, (key,) + COLUMNS)


def run_quench_A_ED(*, nx=ED_NX, ny=ED_NY, dg=ED_DG, g=ED_G_COUP, t=ED_T_HOP, m=ED_M_MASS,
                    dt=0.02, n_steps=2, results_dir="results", label="finite_ed_quench_A",
                    precision="fp64", model="ref", write=True):
    """Quench A, string breaking (finite_ed.jl:491-543): sector
    g(1,iy_str) = +1, g(2,iy_str) = -2 (iy_str = ny / 2), initial state
    n_f(2,iy_str) = 1, e_R(1,iy_str) = +1, evolved at (g, t, m)."""
    gq = ed.string_charges(nx, ny)
    states, key_dict = ed.build_basis(nx, ny, dg, gq)
    psi0 = ed.string_state(states)
    H = ed.build_hamiltonian(states, key_dict, nx, ny, dg, g=g, t=t, m=m, model=model)
    try:
        data = ed.evolve_ED(psi0, H, states, nx, ny, dg, dt=dt, n_steps=n_steps,
                            precision=precision)
    finally:
        H.close()
    if write:
        _save(results_dir, label, data, 1)
    return data


def run_quench_B_ED(*, nx=ED_NX, ny=ED_NY, dg=ED_DG, g=ED_G_COUP, t=ED_T_HOP, m_init=5.0,
                    m_final=0.1, dt=0.02, n_steps=2, results_dir="results",
                    label="finite_ed_quench_B", precision="fp64", model="ref", write=True):
    """Quench B, mass quench m_init -> m_final (finite_ed.jl:549-599):
    staggered sector, ground state at m_init, evolved at m_final.
    ``m_final`` may be a sequence (one batched panel)."""
    mf = np.atleast_1d(np.asarray(m_final, dtype=float))
    states, key_dict = ed.build_basis(nx, ny, dg, ed.staggered_charges(nx, ny))
    E0, psi0 = ed.ite_ground_state_ED(states, key_dict, nx, ny, dg, g=g, t=t, m=m_init,
                                      model=model, precision=precision)
    K = len(mf)
    H = ed.build_hamiltonian(states, key_dict, nx, ny, dg, g=g, t=t,
                             m=mf if K > 1 else float(mf[0]), model=model)
    try:
        start = psi0 if K == 1 else np.repeat(psi0[:, None], K, axis=1)
        data = ed.evolve_ED(start, H, states, nx, ny, dg, dt=dt, n_steps=n_steps,
                            precision=precision)
    finally:
        H.close()
    if write:
        _save(results_dir, label, data, K, "m_final", mf)
    return data


def run_quench_C_ED(*, nx=ED_NX, ny=ED_NY, dg=ED_DG, t=ED_T_HOP, m=ED_M_MASS, g_init=2.0,
                    g_final=0.5, dt=0.02, n_steps=2, results_dir="results",
                    label="finite_ed_quench_C", precision="fp64", model="ref", write=True):
    """Quench C, coupling quench g_init -> g_final (finite_ed.jl:605-650):
    staggered sector, ground state at g_init, evolved at g_final.
    ``g_final`` may be a sequence (one batched panel)."""
    gf = np.atleast_1d(np.asarray(g_final, dtype=float))
    states, key_dict = ed.build_basis(nx, ny, dg, ed.staggered_charges(nx, ny))
    E0, psi0 = ed.ite_ground_state_ED(states, key_dict, nx, ny, dg, g=g_init, t=t, m=m,
                                      model=model, precision=precision)
    K = len(gf)
    H = ed.build_hamiltonian(states, key_dict, nx, ny, dg, g=gf if K > 1 else float(gf[0]),
                             t=t, m=m, model=model)
    try:
        start = psi0 if K == 1 else np.repeat(psi0[:, None], K, axis=1)
        data = ed.evolve_ED(start, H, states, nx, ny, dg, dt=dt, n_steps=n_steps,
                            precision=precision)
    finally:
        H.close()
    if write:
        _save(results_dir, label, data, K, "g_final", gf)
    return data


def main(argv=None):
    """finite_ed.jl main (:656-690): quench id 0 (all), 1 (A), 2 (B), 3 (C);
    CSVs go to ./results."""
    argv = sys.argv[1:] if argv is None else argv
    qid = int(argv[0]) if argv else 0
    results_dir = os.path.join(os.getcwd(), "results")
    os.makedirs(results_dir, exist_ok=True)
    if qid in (0, 1):
        run_quench_A_ED(results_dir=results_dir)
    if qid in (0, 2):
        run_quench_B_ED(results_dir=results_dir)
    if qid in (0, 3):
        run_quench_C_ED(results_dir=results_dir)
    return 0


if __name__ == "__main__":
    sys.exit(main())
