"""GPU parity: the CUDA library against the CPU oracle, through the C ABI.

Bars: basis, keys, ranks, nonzero pattern and signs
bit-exact; CSR values bit-exact (same summation order as the reference);
H*psi within 1e-12 relative (FP64) / 2e-6 relative (FP32); energies within
1e-10 relative and observables within 1e-9 absolute of the FP64 oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (nx, ny, dg, sector)
CASES = [
    (2, 2, 1, "stag"), (3, 2, 1, "stag"), (2, 3, 1, "stag"), (4, 2, 1, "stag"),
    (2, 4, 1, "stag"), (3, 3, 1, "stag"), (4, 3, 1, "stag"), (3, 4, 1, "stag"),
    (3, 3, 1, "zero"), (4, 2, 1, "string"), (3, 4, 1, "string"),
    (2, 2, 2, "stag"), (3, 2, 2, "stag"), (2, 3, 2, "zero"), (1, 4, 1, "stag"), (4, 1, 1, "stag"),
]


def charges(O, nx, ny, kind):
    if kind == "stag":
        return O.staggered_charges(nx, ny)
    if kind == "string":
        return O.string_charges(nx, ny)
    return np.zeros((nx, ny), np.int32)


_cache = {}


def pair(O, lgt, nx, ny, dg, kind):
    key = (nx, ny, dg, kind)
    if key not in _cache:
        g = charges(O, nx, ny, kind)
        ob = O.build_basis(nx, ny, dg, g)
        gb, kd = lgt.build_basis(nx, ny, dg, g)
        _cache[key] = (ob, gb, kd)
    return _cache[key]


@pytest.mark.parametrize("nx,ny,dg,kind", CASES)
def test_basis_bit_exact(oracle, lgt, nx, ny, dg, kind):
    ob, gb, kd = pair(oracle, lgt, nx, ny, dg, kind)
    assert len(gb) == ob.dim
    np.testing.assert_array_equal(gb.order_keys(), ob.order_keys)
    nf, eR, eU = gb.states()
    np.testing.assert_array_equal(nf, ob.nf)
    np.testing.assert_array_equal(eR, ob.eR)
    np.testing.assert_array_equal(eU, ob.eU)
    if dg == 1:
        np.testing.assert_array_equal(gb.ref_keys(), ob.ref_keys)
        # key_dict: every reference key maps to its 1-based index
        np.testing.assert_array_equal(gb.lookup(ob.ref_keys), np.arange(1, ob.dim + 1))
    np.testing.assert_array_equal(gb.rank(ob.order_keys), np.arange(ob.dim))


def test_lookup_absent_keys(oracle, lgt):
    ob, gb, kd = pair(oracle, lgt, 4, 2, 1, "stag")
    # flip one fermion bit of every key: particle number changes -> absent
    bad = ob.ref_keys ^ 1
    assert np.all(gb.lookup(bad) == 0)
    assert np.all(gb.rank(ob.order_keys | (np.uint64(1) << np.uint64(60))) == -1)
    k0 = int(ob.ref_keys[5])
    assert k0 in kd and kd[k0] == 6


COUPLINGS = [(1.0, 1.0, 0.5), (0.8, 1.3, 0.3), (2.0, 0.7, -1.1)]


@pytest.mark.parametrize("nx,ny,dg,kind", CASES)
@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_csr_export_bit_exact(oracle, lgt, nx, ny, dg, kind, model):
    ob, gb, kd = pair(oracle, lgt, nx, ny, dg, kind)
    g, t, m = COUPLINGS[1]
    H = lgt.build_hamiltonian(gb, kd, nx, ny, dg, g=g, t=t, m=m, model=model)
    Ho = oracle.build_hamiltonian(ob, g=g, t=t, m=m, model=model)
    assert H.nnz() == Ho.nnz
    rp, ci, va = H.export_csr()
    np.testing.assert_array_equal(rp, Ho.indptr)
    np.testing.assert_array_equal(ci, Ho.indices)
    np.testing.assert_array_equal(va, Ho.data)  # bitwise, incl. JW signs
    H.close()


@pytest.mark.parametrize("nx,ny,dg,kind", CASES)
@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_matvec_fp64(oracle, lgt, nx, ny, dg, kind, model):
    ob, gb, kd = pair(oracle, lgt, nx, ny, dg, kind)
    K = len(COUPLINGS)
    gs, ts, ms = (np.array(v) for v in zip(*COUPLINGS))
    H = lgt.build_hamiltonian(gb, g=gs, t=ts, m=ms, model=model)
    rng = np.random.default_rng(nx * 100 + ny * 10 + dg)
    N = ob.dim
    x = rng.standard_normal((N, K))
    xc = rng.standard_normal((N, K)) + 1j * rng.standard_normal((N, K))
    y = H.matvec(x)
    yc = H.matvec(xc)
    for k, (g, t, m) in enumerate(COUPLINGS):
        Ho = oracle.build_hamiltonian(ob, g=g, t=t, m=m, model=model)
        yo = Ho @ x[:, k]
        yco = Ho @ xc[:, k]
        assert np.max(np.abs(y[:, k] - yo)) <= 1e-12 * max(1.0, np.max(np.abs(yo)))
        assert np.max(np.abs(yc[:, k] - yco)) <= 1e-12 * max(1.0, np.max(np.abs(yco)))
    H.close()


@pytest.mark.parametrize("nx,ny", [(3, 2), (4, 2), (3, 3), (4, 3)])
@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_matvec_fp32(oracle, lgt, nx, ny, model):
    ob, gb, kd = pair(oracle, lgt, nx, ny, 1, "stag")
    g, t, m = COUPLINGS[1]
    H = lgt.build_hamiltonian(gb, g=g, t=t, m=m, model=model)
    Ho = oracle.build_hamiltonian(ob, g=g, t=t, m=m, model=model)
    x = np.random.default_rng(7).standard_normal(ob.dim).astype(np.float32)
    y = H.matvec(x, precision="fp32")
    yo = Ho @ x.astype(np.float64)
    assert np.max(np.abs(y - yo)) <= 2e-6 * np.max(np.abs(yo))
    H.close()


def _align(psi, ref):
    ov = np.vdot(ref, psi)
    return psi * (abs(ov) / ov) if ov != 0 else psi


@pytest.mark.parametrize("nx,ny,kind", [(2, 2, "stag"), (3, 2, "stag"), (2, 3, "stag"),
                                         (4, 2, "stag"), (3, 3, "stag"), (4, 2, "string")])
@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_ground_state_fp64(oracle, lgt, nx, ny, kind, model):
    ob, gb, kd = pair(oracle, lgt, nx, ny, 1, kind)
    g, t, m = 1.0, 1.0, 0.5
    H = lgt.build_hamiltonian(gb, g=g, t=t, m=m, model=model)
    Ho = oracle.build_hamiltonian(ob, g=g, t=t, m=m, model=model)
    E0o, psio = oracle.ground_state(Ho)
    E0, psi, info = lgt.find_ground_state(H, tol=1e-12, return_info=True)
    assert abs(E0 - E0o) <= 1e-10 * abs(E0o)
    assert info["residual"] <= 1e-11
    psi = _align(psi, psio)
    gap = np.diff(oracle.spectrum_low(Ho, 2))[0]
    if gap > 1e-6:
        assert np.linalg.norm(psi - psio) <= 1e-9 / min(gap, 1.0) + 1e-10
        mo = oracle.measure(psio, ob)
        mg = lgt.measure_ED(psi, gb, nx, ny, 1, 0.0)
        for key in ("nf_mean", "nf_even", "nf_odd", "E2_mean", "plaq_mean", "n_stag"):
            assert abs(mg[key] - mo[key]) <= 1e-9, key
        np.testing.assert_allclose(mg["nf_grid"], mo["nf_grid"], atol=1e-9)
        np.testing.assert_allclose(mg["E2_grid"], mo["E2_grid"], atol=1e-9)
        np.testing.assert_allclose(mg["plaq_grid"], mo["plaq_grid"], atol=1e-9)
    H.close()


def test_ground_state_batched_fp64(oracle, lgt):
    """4x2, K = 8 coupling points (g uniform on [0.5, 2]) in one solve."""
    nx, ny = 4, 2
    ob, gb, kd = pair(oracle, lgt, nx, ny, 1, "stag")
    gs = np.random.default_rng(0).uniform(0.5, 2.0, 8)
    for model in ("ref", "pjw"):
        H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=0.5, model=model)
        E0, psi = lgt.find_ground_state(H, tol=1e-12)
        obs = lgt.measure_ED(psi, gb, nx, ny, 1, 0.0)
        for k, g in enumerate(gs):
            Ho = oracle.build_hamiltonian(ob, g=g, t=1.0, m=0.5, model=model)
            E0o, psio = oracle.ground_state(Ho)
            assert abs(E0[k] - E0o) <= 1e-10 * abs(E0o)
            mo = oracle.measure(psio, ob)
            assert abs(obs[k]["E2_mean"] - mo["E2_mean"]) <= 1e-9
            assert abs(obs[k]["plaq_mean"] - mo["plaq_mean"]) <= 1e-9
        H.close()


@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_ground_state_mixed(oracle, lgt, model):
    """FP32 H*psi and Krylov storage, FP64 dots/reorth/tridiagonal, FP64
    Rayleigh quotient: |dE|/|E| <= 1e-10."""
    nx, ny = 4, 2
    ob, gb, kd = pair(oracle, lgt, nx, ny, 1, "stag")
    gs = np.array([0.6, 1.0, 1.7])
    H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=0.5, model=model)
    E0, psi = lgt.find_ground_state(H, precision="fp32_mixed")
    for k, g in enumerate(gs):
        E0o, _ = oracle.ground_state(oracle.build_hamiltonian(ob, g=g, t=1.0, m=0.5, model=model))
        assert abs(E0[k] - E0o) <= 1e-10 * abs(E0o)
    H.close()


@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_evolve_fp64(oracle, lgt, model):
    """Quench from the staggered product state: state and observables after
    each step against exact propagation."""
    nx, ny = 3, 2
    ob, gb, kd = pair(oracle, lgt, nx, ny, 1, "stag")
    H = lgt.build_hamiltonian(gb, g=0.9, t=1.0, m=0.5, model=model)
    Ho = oracle.build_hamiltonian(ob, g=0.9, t=1.0, m=0.5, model=model)
    psi0 = lgt.staggered_product_state(gb)
    i0 = oracle.staggered_product_index(ob)
    assert np.argmax(np.abs(psi0)) == i0
    data, psi, drift = lgt.evolve_ED(psi0, H, gb, nx, ny, 1, dt=0.05, n_steps=20, tol=1e-12,
                                     return_state=True)
    psio, datao = oracle.evolve(psi0, Ho, ob, dt=0.05, n_steps=20)
    assert np.linalg.norm(psi - psio) <= 1e-9
    for d, do in zip(data, datao):
        for key in ("nf_mean", "nf_even", "nf_odd", "E2_mean", "plaq_mean"):
            assert abs(d[key] - do[key]) <= 1e-9, key
        assert abs(d["t"] - do["t"]) < 1e-12
    H.close()
