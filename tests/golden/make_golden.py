"""Generates the golden fixtures in tests/golden/ from the CPU oracle.

The reference ships no goldens (NoaFeldman/LGT has no test suite) and Julia
is not available, so these vectors come from the oracle (oracle/), whose
integer layer is pinned by the full tensor-product construction of
oracle/fullspace.py and by the reference sector dimensions.  Re-run with
``python tests/golden/make_golden.py`` after an intentional oracle change.

Each fixture NAME.npz holds, for one lattice / sector / model / coupling:
order_keys, ref_keys, indptr, indices, data (CSR of H, the reference's CSC
arrays), E0, psi (sign fixed: largest entry positive), nf_grid, E2_grid,
plaq_grid, and evolved observables of a short quench from the staggered
product state (when that state is in the sector).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

CASES = [
    # name, nx, ny, dg, sector, model, g, t, m
    ("stag3x2_ref", 3, 2, 1, "stag", "ref", 1.0, 1.0, 0.5),
    ("stag3x2_pjw", 3, 2, 1, "stag", "pjw", 1.0, 1.0, 0.5),
    ("stag2x2_pjw", 2, 2, 1, "stag", "pjw", 0.7, 1.2, 0.3),
    ("stag4x2_ref", 4, 2, 1, "stag", "ref", 0.8, 1.0, 0.5),
    ("stag4x2_pjw", 4, 2, 1, "stag", "pjw", 0.8, 1.0, 0.5),
    ("string3x4_ref", 3, 4, 1, "string", "ref", 1.0, 1.0, 2.0),
    ("stag3x2_dg2_pjw", 3, 2, 2, "stag", "pjw", 1.3, 1.0, 0.4),
]

QUENCH_STEPS, QUENCH_DT = 10, 0.05


def charges(nx, ny, kind):
    return O.staggered_charges(nx, ny) if kind == "stag" else O.string_charges(nx, ny)


def make(name, nx, ny, dg, kind, model, g, t, m):
    b = O.build_basis(nx, ny, dg, charges(nx, ny, kind))
    H = O.build_hamiltonian(b, g=g, t=t, m=m, model=model)
    E0, psi = O.ground_state(H)
    ms = O.measure(psi, b)
    out = dict(nx=nx, ny=ny, dg=dg, g=g, t=t, m=m, model=model, sector=kind,
               order_keys=b.order_keys, ref_keys=b.ref_keys, indptr=H.indptr.astype(np.int64),
               indices=H.indices.astype(np.int32), data=H.data, E0=E0, psi=psi,
               nf_grid=ms["nf_grid"], E2_grid=ms["E2_grid"], plaq_grid=ms["plaq_grid"])
    if kind == "stag":
        i0 = O.staggered_product_index(b)
        v = np.zeros(b.dim, np.complex128)
        v[i0] = 1.0
        _, data = O.evolve(v, H, b, dt=QUENCH_DT, n_steps=QUENCH_STEPS)
        out["quench_E2"] = np.array([d["E2_mean"] for d in data])
        out["quench_nf_even"] = np.array([d["nf_even"] for d in data])
        out["quench_plaq"] = np.array([d["plaq_mean"] for d in data])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    return b.dim


if __name__ == "__main__":
    for case in CASES:
        print(case[0], make(*case))
