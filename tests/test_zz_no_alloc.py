"""lgt_observe_noalloc through the C ABI against lgt_observe.

lgt_observe_noalloc serves callers that cannot call cudaMalloc (their
device memory is all reserved by their own pool, or an allocation's implicit
synchronisation is not allowed where they call it): it computes the same
observables with a fixed static device scratch instead of allocated buffers.
Both entry points are called on the same device panels; the results must
agree to 1e-11 relative (they differ only in the block partition of the
reduction), on two calls in a row with different states, so that leftovers
of the first call in the shared scratch cannot leak into the second.  The
allocation-free calls run first on a fresh Hamiltonian, with free device
memory checked to be unchanged across them.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _observe(C, lib, H, psi_ptr, ncomp, prec, fn, nx, ny):
    K = H.K
    ns, npl = nx * ny, (nx - 1) * (ny - 1)
    nf = np.zeros(K * ns)
    e2 = np.zeros(K * ns)
    pl = np.zeros(K * npl)
    summ = (C.Obs * K)()
    if fn == "noalloc":
        code = lib.lgt_observe_noalloc(H.handle, ctypes.c_void_p(psi_ptr), ncomp, prec, 0.5,
                                       nf.ctypes.data, e2.ctypes.data, pl.ctypes.data, summ)
    else:
        code = lib.lgt_observe(H.handle, ctypes.c_void_p(psi_ptr), ncomp, prec, C.LGT_DEVICE_PTRS,
                               0.5, nf.ctypes.data, e2.ctypes.data, pl.ctypes.data, summ)
    C.check(code)
    s = np.array([[o.nf_mean, o.nf_even, o.nf_odd, o.E2_mean, o.plaq_mean, o.n_stag, o.norm2, o.t]
                  for o in summ])
    return nf, e2, pl, s


@pytest.mark.parametrize("nx,ny,K,ncomp,dtype", [(3, 4, 128, 1, "fp64"), (4, 2, 8, 2, "fp64"),
                                                  (3, 3, 16, 2, "fp32")])
def test_noalloc_matches_observe_twice(nx, ny, K, ncomp, dtype):
    torch = pytest.importorskip("torch")
    import lgt_gb300 as L
    from lgt_gb300 import _capi as C
    lib = C.load()
    states, _ = L.build_basis(nx, ny, 1, L.staggered_charges(nx, ny), device=0)
    N = len(states)
    tdt = torch.float64 if dtype == "fp64" else torch.float32
    prec = C.LGT_FP64 if dtype == "fp64" else C.LGT_FP32
    gen = torch.Generator(device="cuda").manual_seed(1234)
    psis = []
    for _ in range(2):  # two states, one per call
        psi = torch.randn((N, K, ncomp), dtype=tdt, device="cuda", generator=gen)
        psi /= torch.linalg.vector_norm(psi.double(), dim=(0, 2), keepdim=True).to(tdt)
        psis.append(psi)
    torch.cuda.synchronize()  # the library works on the basis' own stream
    g = np.linspace(0.5, 2.0, K)
    # warm-up on a throw-away Hamiltonian: loads the module and looks up the
    # scratch address (the one-time set-up of the first call on a device)
    H0 = L.build_hamiltonian(states, g=g, t=1.0, m=0.5, model="pjw")
    _observe(C, lib, H0, psis[0].data_ptr(), ncomp, prec, "noalloc", nx, ny)
    H0.close()
    # a fresh Hamiltonian whose own growable buffers have never been used:
    # lgt_observe_noalloc runs on it first and must not change free device
    # memory (no cudaMalloc, no fallback to the handle's buffers)
    H = L.build_hamiltonian(states, g=g, t=1.0, m=0.5, model="pjw")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    got = [_observe(C, lib, H, p.data_ptr(), ncomp, prec, "noalloc", nx, ny) for p in psis]
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0
    for call in range(2):  # two calls in a row, different states
        ref = _observe(C, lib, H, psis[call].data_ptr(), ncomp, prec, "observe", nx, ny)
        again = _observe(C, lib, H, psis[call].data_ptr(), ncomp, prec, "noalloc", nx, ny)
        for a, b, c in zip(got[call], ref, again):
            np.testing.assert_allclose(a, b, rtol=1e-11, atol=1e-13)
            np.testing.assert_array_equal(a, c)  # the same partition: bitwise repeatable
        assert np.allclose(got[call][3][:, 6], 1.0, atol=1e-5)  # norm2 of normalised states
    H.close()
    states.close()


def test_noalloc_rejects_host_pointer():
    pytest.importorskip("torch")
    import lgt_gb300 as L
    from lgt_gb300 import _capi as C
    lib = C.load()
    states, _ = L.build_basis(3, 2, 1, L.staggered_charges(3, 2), device=0)
    H = L.build_hamiltonian(states, g=1.0, t=1.0, m=0.5)
    host = np.zeros(len(states))
    code = lib.lgt_observe_noalloc(H.handle, host.ctypes.data_as(ctypes.c_void_p), 1, C.LGT_FP64,
                                   0.0, None, None, None, None)
    assert code == C.LGT_ERR_ARG
    H.close()
    states.close()
