"""The 4x4 staggered sector (N = 8,563,545; the real-time quench workload)
against the oracle, not against another GPU kernel.

* Basis: every order key, every reference _encode key (at 4x4 _encode fills
  all 64 bits and is negative when the last e_U field is +1,
  finite_ed.jl:80-97) and every state's (n_f, e_R, e_U) are bit-exact;
  key_dict lookups of present and absent keys agree (finite_ed.jl:291-292).
* nnz(H) equals the reference sector's 106,044,513 (reference model) and
  170,273,317 (plaquette + Jordan-Wigner).
* H*psi of the run-time-geometry, fixed-shape and stored-table kernels, FP64
  and FP32, on sampled rows (the oracle builds just those rows with the
  reference's loop body, lgt_oracle.c:orc_ham_rows): 1e-12 relative (FP64),
  2e-6 (FP32), the bars of the smaller lattices.
* One exp(-i H dt) step of the K = 8 quench panel, point 0 against the
  oracle's expm_multiply on the full matrix (finite_ed.jl:405-431): 1e-9
  (FP64), 2e-5 (FP32-mixed) in the state's 2-norm.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N44 = 8_563_545
NNZ44 = {"ref": 106_044_513, "pjw": 170_273_317}
COUPLINGS = [(0.8, 1.3, 0.3), (1.4, 0.9, -0.2)]


@pytest.fixture(scope="module")
def bases(oracle, lgt):
    g = oracle.staggered_charges(4, 4)
    ob = oracle.build_basis(4, 4, 1, g)
    gb = lgt.build_basis(4, 4, 1, g, device=0)[0]
    yield ob, gb
    gb.close()


@pytest.fixture(scope="module")
def sample_rows(bases):
    ob, _ = bases
    rng = np.random.default_rng(4444)
    neg = np.flatnonzero(ob.ref_keys < 0)
    return np.unique(np.r_[0, 1, N44 - 2, N44 - 1, rng.choice(neg, 300, replace=False),
                           rng.integers(0, N44, 3000)])


def test_4x4_basis_bit_exact(bases):
    ob, gb = bases
    assert ob.dim == len(gb) == N44
    np.testing.assert_array_equal(gb.order_keys(), ob.order_keys)
    rk = gb.ref_keys()
    np.testing.assert_array_equal(rk, ob.ref_keys)
    assert np.count_nonzero(rk < 0) > 0  # keys with bit 63 set are present and equal
    nf, eR, eU = gb.states()
    np.testing.assert_array_equal(nf, ob.nf)
    np.testing.assert_array_equal(eR, ob.eR)
    np.testing.assert_array_equal(eU, ob.eU)


def test_4x4_key_dict_lookup(bases, oracle):
    ob, gb = bases
    rng = np.random.default_rng(7)
    idx = np.r_[0, N44 - 1, rng.choice(np.flatnonzero(ob.ref_keys < 0), 500, replace=False),
                rng.integers(0, N44, 5000)]
    np.testing.assert_array_equal(gb.lookup(ob.ref_keys[idx]), idx + 1)
    # keys that are not states: the oracle's dictionary says absent, so must the GPU
    L = oracle.lib()
    cand = rng.integers(-2**63, 2**63 - 1, 4000, dtype=np.int64)
    absent = np.array([k for k in cand if L.orc_basis_lookup(ob._h, int(k) & (2**64 - 1)) < 0])
    assert absent.size > 3000
    np.testing.assert_array_equal(gb.lookup(absent), 0)


@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_4x4_nnz(bases, lgt, model):
    _, gb = bases
    H = lgt.build_hamiltonian(gb, g=1.0, t=1.0, m=0.5, model=model)
    assert H.nnz() == NNZ44[model]
    H.close()


@pytest.mark.parametrize("kernel", ["generic", "fixed", "table"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_4x4_hpsi_sampled_rows_vs_oracle(bases, sample_rows, oracle, lgt, monkeypatch, kernel,
                                         prec, model):
    ob, gb = bases
    if kernel == "fixed":
        monkeypatch.setenv("LGT_HPSI_VARIANT", "3")
    elif kernel == "table":
        monkeypatch.setenv("LGT_HPSI_VARIANT", "6")
    gs, ts, ms = (np.array(v) for v in zip(*COUPLINGS))
    H = lgt.build_hamiltonian(gb, g=gs, t=ts, m=ms, model=model)
    rng = np.random.default_rng(16 + len(model) + len(prec))
    x = rng.standard_normal((N44, 2)) + 1j * rng.standard_normal((N44, 2))
    if prec == "fp32":
        x = x.astype(np.complex64)
    y = H.matvec(x, precision=prec, generic=(kernel == "generic"))
    H.close()
    tol = 1e-12 if prec == "fp64" else 2e-6
    for k, (g, t, m) in enumerate(COUPLINGS):
        R = oracle.hamiltonian_rows(ob, sample_rows, g=g, t=t, m=m, model=model)
        assert R.nnz > 10 * sample_rows.size
        yo = R @ x[:, k].astype(np.complex128)
        err = np.max(np.abs(y[sample_rows, k] - yo))
        assert err <= tol * max(1.0, float(np.max(np.abs(yo)))), (k, err)


QUENCH_G = np.random.default_rng(0).uniform(0.5, 1.5, 8)


@pytest.fixture(scope="module")
def oracle_step(bases, oracle):
    """Point 0 of the quench panel after one step, by the oracle on the full
    4x4 matrix (about 20 s to build, 20 s for expm_multiply)."""
    ob, _ = bases
    v0 = np.zeros(ob.dim, np.complex128)
    v0[oracle.staggered_product_index(ob)] = 1.0
    Ho = oracle.build_hamiltonian(ob, g=QUENCH_G[0], t=1.0, m=0.5)
    assert Ho.nnz == NNZ44["ref"]
    po, do = oracle.evolve(v0, Ho, ob, dt=0.05, n_steps=1)
    return po, do


@pytest.mark.parametrize("precision,tol_state", [("fp64", 1e-9), ("fp32_mixed", 2e-5)])
def test_4x4_quench_step_vs_oracle(bases, oracle_step, lgt, precision, tol_state):
    """The K = 8 quench panel (g uniform on [0.5, 1.5], m = 0.5, staggered
    product state, dt = 0.05), one step; point 0 against the oracle."""
    ob, gb = bases
    H = lgt.build_hamiltonian(gb, g=QUENCH_G, t=1.0, m=0.5)
    v0 = lgt.staggered_product_state(gb)
    data, psi, drift = lgt.evolve_ED(np.stack([v0] * 8, axis=1), H, dt=0.05, n_steps=1,
                                     tol=1e-12, precision=precision, return_state=True)
    H.close()
    po, do = oracle_step
    assert np.linalg.norm(psi[:, 0] - po) <= tol_state
    assert abs(data[1][0]["E2_mean"] - do[1]["E2_mean"]) <= 10 * tol_state
    np.testing.assert_allclose(data[1][0]["nf_grid"], do[1]["nf_grid"], rtol=0,
                               atol=10 * tol_state)
    assert np.all(drift < (1e-12 if precision == "fp64" else 1e-5))
