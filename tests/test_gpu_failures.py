"""Failure paths of the boundary, made on the host (no GPU fault).

The reference stops on @assert: an inconsistent sector (finite_ed.jl:127),
a Lanczos run that did not converge (finite_ed.jl:339) and a missing
initial state (finite_ed.jl:530).  Here they are status codes of the C ABI
that the Python mirror raises as ValueError / NotConverged / KeyError.  Bad
couplings are refused before anything reaches the device, and a refused
update leaves the Hamiltonian as it was.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bad", [math.nan, math.inf, -math.inf])
@pytest.mark.parametrize("which", ["g", "t", "m"])
def test_non_finite_coupling_rejected(lgt, bad, which):
    states, _ = lgt.build_basis(3, 2, 1, lgt.staggered_charges(3, 2), device=0)
    kw = dict(g=[1.0, 0.7], t=1.0, m=0.5)
    kw[which] = [1.0, bad] if which == "g" else bad
    with pytest.raises(ValueError, match="finite"):
        lgt.build_hamiltonian(states, **kw)
    H = lgt.build_hamiltonian(states, g=[1.0, 0.7], t=1.0, m=0.5)
    E_before, _ = lgt.find_ground_state(H, tol=1e-12)
    with pytest.raises(ValueError, match="finite"):
        H.set_couplings(**{which: bad})
    E_after, _ = lgt.find_ground_state(H, tol=1e-12)  # couplings unchanged
    np.testing.assert_allclose(E_after, E_before, rtol=1e-12)
    H.close()
    states.close()


def test_zero_g_only_refused_with_plaquette(lgt, oracle):
    gch = lgt.staggered_charges(3, 2)
    states, _ = lgt.build_basis(3, 2, 1, gch, device=0)
    with pytest.raises(ValueError, match="g != 0"):
        lgt.build_hamiltonian(states, g=0.0, t=1.0, m=0.5, model="pjw")
    # the reference model at g = 0 (no electric energy) is a valid point
    H = lgt.build_hamiltonian(states, g=0.0, t=1.0, m=0.5)
    E0, _ = lgt.find_ground_state(H, tol=1e-12)
    ob = oracle.build_basis(3, 2, 1, gch)
    E0o, _ = oracle.ground_state(oracle.build_hamiltonian(ob, g=0.0, t=1.0, m=0.5))
    assert abs(E0 - E0o) <= 1e-10 * abs(E0o)
    H.close()
    states.close()


@pytest.mark.parametrize("solver", ["cta", "panel"])
@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_not_converged_raises(lgt, solver, precision):
    """maxiter = 1 restart of a 3-vector Krylov space cannot reach 1e-15:
    the call reports NOCONV (the reference's @assert at finite_ed.jl:339)."""
    from lgt_gb300 import _capi as C
    states, _ = lgt.build_basis(4, 2, 1, lgt.staggered_charges(4, 2), device=0)
    H = lgt.build_hamiltonian(states, g=[0.8, 1.3], t=1.0, m=0.5)
    with pytest.raises(C.NotConverged):
        lgt.find_ground_state(H, tol=1e-15, krylovdim=3, maxiter=1, check_every=1,
                              precision=precision, solver=solver)
    # the handle stays usable after the failure
    E0, _ = lgt.find_ground_state(H, tol=1e-12, solver=solver)
    assert np.all(np.isfinite(E0))
    H.close()
    states.close()


def test_inconsistent_sector_and_missing_state(lgt):
    too_many = -2 * np.ones((3, 2), dtype=np.int64)  # N_f = 12 > 6 sites (finite_ed.jl:127)
    with pytest.raises(ValueError, match="Inconsistent sector"):
        lgt.build_basis(3, 2, 1, too_many, device=0)
    states, _ = lgt.build_basis(3, 2, 1, lgt.staggered_charges(3, 2), device=0)
    with pytest.raises(KeyError):
        lgt.string_state(states)  # the string state lives in another sector
    states.close()
