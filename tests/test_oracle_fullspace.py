"""Pins the oracle's conventions to the reference's own operator definitions.

The sector Hamiltonian of the oracle (finite_ed.jl recursion, plus the PJW
terms) must equal the full tensor-product Hamiltonian assembled from the
reference's local operators and term lists, projected onto the sector; the
sector must be closed under H (Gauss law); and the lowest eigenvalue of the
Gauss-penalised full-space H (the method of the reference's dense
self-tests selftest_mps_lgt / selftest_plaqjw) must equal the sector E0.
"""
import numpy as np
import pytest

from oracle import fullspace as F


@pytest.mark.parametrize("nx,ny", [(2, 2), (3, 2), (2, 3)])
@pytest.mark.parametrize("model", ["ref", "pjw"])
@pytest.mark.parametrize("g,t,m", [(0.8, 1.1, 0.37), (1.7, 0.6, -0.9)])
def test_sector_projection_equals_oracle(oracle, nx, ny, model, g, t, m):
    b = oracle.build_basis(nx, ny, 1, oracle.staggered_charges(nx, ny))
    Hs = oracle.build_hamiltonian(b, g=g, t=t, m=m, model=model)
    Hf = F.hamiltonian(nx, ny, 1, g=g, t=t, m=m, model=model)
    idx = F.sector_indices(b)
    P = Hf[idx][:, idx]
    assert abs(P - Hs).max() <= 1e-14
    # the sector is invariant under H: no amplitude leaks out of it
    col = abs(Hf[:, idx]).sum()
    assert col == pytest.approx(abs(P).sum(), rel=1e-14)


@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_penalised_dense_selftest(oracle, model):
    """selftest_plaqjw / selftest_mps_lgt method at 2x2 (Hilbert dim 1296):
    lowest eigenvalue of H + Lambda sum_i (G_i - g_i)^2 == sector E0."""
    nx, ny, g, t, m = 2, 2, 1.0, 1.0, 0.5
    gch = oracle.staggered_charges(nx, ny)
    Hf = F.hamiltonian(nx, ny, 1, g=g, t=t, m=m, model=model).toarray()
    Hf += np.diag(F.gauss_penalty_diag(nx, ny, 1, gch, 20.0))
    e_dense = np.linalg.eigvalsh(Hf)[0]
    b = oracle.build_basis(nx, ny, 1, gch)
    e_sector = oracle.ground_state(oracle.build_hamiltonian(b, g=g, t=t, m=m, model=model))[0]
    assert e_dense == pytest.approx(e_sector, abs=1e-10)
