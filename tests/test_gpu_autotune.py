"""Autotuner: the Krylov drivers time their H*psi kernel candidates and
reduction block counts per operator shape, keep the fastest, and give the
same results as the built-in choice (oracle bars of the solver tests)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_choice_is_reported_and_cached(oracle, lgt):
    gq = oracle.staggered_charges(4, 3)
    ob = oracle.build_basis(4, 3, 1, gq)
    gb = lgt.build_basis(4, 3, 1, gq)[0]
    gs = np.array([0.6, 1.1, 1.7, 2.4])
    H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=0.4)
    for ncomp in (1, 2):
        for prec in ("fp64", "fp32_mixed"):
            c = H.autotune(ncomp, prec)
            assert c["measured"]
            assert c["hpsi_kernel"] in ("generic", "fixed_vpl1", "fixed_vpl2", "fixed_wide",
                                        "table_vpl1", "table_vpl2", "table_wide")
            assert c["reduce_blocks"] in (304, 608, 912, 1216)
            assert 0.0 < c["hpsi_ms"] < 1e3 and 0.0 < c["reduce_ms"] < 1e3
            assert H.autotune(ncomp, prec) == c  # cached for the process
    # solves with the tuned kernels meet the oracle bars
    E0, psi = lgt.find_ground_state(H, tol=1e-12, solver="panel", as_complex=False)
    for k in range(4):
        E0o = oracle.ground_state(oracle.build_hamiltonian(ob, g=gs[k], t=1.0, m=0.4))[0]
        assert abs(E0[k] - E0o) <= 1e-10 * abs(E0o)
    H.close()


def test_autotune_disabled_keeps_rules(lgt, monkeypatch):
    monkeypatch.setenv("LGT_AUTOTUNE", "0")
    gb = lgt.build_basis(3, 4, 1, lgt.staggered_charges(3, 4))[0]
    H = lgt.build_hamiltonian(gb, g=[0.5, 0.9, 1.3], t=1.0, m=0.2)  # K = 3: a fresh shape
    c = H.autotune(1, "fp64")
    assert not c["measured"] and c["hpsi_kernel"] == "rule" and c["reduce_blocks"] == 608
    H.close()


def test_destroy_basis_before_hamiltonian(oracle, lgt):
    """Handles may be released in any order: the basis stays alive while a
    Hamiltonian made from it exists."""
    gb = lgt.build_basis(3, 2, 1, lgt.staggered_charges(3, 2))[0]
    H = lgt.build_hamiltonian(gb, g=1.0, t=1.0, m=0.5)
    gb.close()  # the caller's basis handle goes first
    E0, _ = lgt.find_ground_state(H, tol=1e-12)
    ob = oracle.build_basis(3, 2, 1, oracle.staggered_charges(3, 2))
    E0o = oracle.ground_state(oracle.build_hamiltonian(ob, g=1.0, t=1.0, m=0.5))[0]
    assert abs(E0 - E0o) <= 1e-10 * abs(E0o)
    H.close()
