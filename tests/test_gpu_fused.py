"""lgt_ground_state_observe (find_ground_state + measure_ED in one call, the
observables launched before the solve's synchronisation) against the two
calls in turn: the same kernels on the same data, so bitwise the same
energies, states and observables; host and device states; both solvers
(the panel solver runs the two calls in turn)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lgt, C, H, fused, device, precision, K):
    import torch
    lib = C.load()
    o = C.defaults(False)
    o.precision = precision
    N = H.basis.dim
    E0 = np.zeros(K)
    info = C.Info()
    summ = (C.Obs * K)()
    G = H.basis
    nf = np.zeros(K * G.nx * G.ny)
    e2 = np.zeros(K * G.nx * G.ny)
    if device:
        psi = torch.zeros((N, K), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        pp, flags = psi.data_ptr(), C.LGT_DEVICE_PTRS
    else:
        psi = np.zeros((N, K))
        pp, flags = psi.ctypes.data, 0
    if fused:
        C.check(lib.lgt_ground_state_observe(H.handle, o, E0.ctypes.data, pp, None, flags, info,
                                             nf.ctypes.data, e2.ctypes.data, None, summ))
    else:
        C.check(lib.lgt_ground_state(H.handle, o, E0.ctypes.data, pp, None, flags, info))
        C.check(lib.lgt_observe(H.handle, pp, 1, C.LGT_FP64, flags, 0.0, nf.ctypes.data,
                                e2.ctypes.data, None, summ))
    st = psi.cpu().numpy() if device else psi
    return E0, st, np.frombuffer(summ, dtype=np.float64).copy(), nf, e2


@pytest.mark.parametrize("nx,ny,K", [(4, 2, 16), (3, 3, 5), (4, 3, 3)])
@pytest.mark.parametrize("device", [True, False])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_fused_equals_two_calls(oracle, lgt, nx, ny, K, device, prec):
    from lgt_gb300 import _capi as C
    b = lgt.build_basis(nx, ny, 1, lgt.staggered_charges(nx, ny))[0]
    gs = np.linspace(0.6, 1.8, K)
    code = C.LGT_FP32_MIXED if prec == "mixed" else C.LGT_FP64
    H = lgt.build_hamiltonian(b, g=gs, t=1.0, m=0.5)
    a = _run(lgt, C, H, True, device, code, K)
    bb = _run(lgt, C, H, False, device, code, K)
    H.close()
    for x, y in zip(a, bb):
        assert np.array_equal(x, y)
    # and the energies against the FP64 oracle
    ob = oracle.build_basis(nx, ny, 1, oracle.staggered_charges(nx, ny))
    E0o = oracle.ground_state(oracle.build_hamiltonian(ob, g=gs[0], t=1.0, m=0.5))[0]
    assert abs(a[0][0] - E0o) <= 1e-10 * abs(E0o)


@pytest.mark.parametrize("precision", ["fp32_mixed", "fp64"])
@pytest.mark.parametrize("K", [1, 16])
def test_python_measured_wrapper(lgt, precision, K):
    """find_ground_state_measured against find_ground_state + measure_ED
    through the Python API: bitwise the same energies, states and dicts."""
    b = lgt.build_basis(4, 2, 1, lgt.staggered_charges(4, 2))[0]
    gs = np.linspace(0.6, 1.9, K)
    H = lgt.build_hamiltonian(b, g=gs, t=1.0, m=0.5, model="pjw")
    E1, P1, O1 = lgt.find_ground_state_measured(H, precision=precision, as_complex=False)
    E2, P2 = lgt.find_ground_state(H, precision=precision, as_complex=False)
    O2 = lgt.measure_ED(P2, b, 4, 2, 1, 0.0)
    assert np.array_equal(np.atleast_1d(E1), np.atleast_1d(E2))
    assert np.array_equal(P1, P2)
    recs1 = [O1] if K == 1 else O1
    recs2 = [O2] if K == 1 else O2
    assert len(recs1) == len(recs2) == K
    for a, c in zip(recs1, recs2):
        assert set(a) == set(c)
        for key in a:
            assert np.array_equal(np.asarray(a[key]), np.asarray(c[key])), key
    H.close()
