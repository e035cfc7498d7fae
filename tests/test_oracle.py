"""CPU tests of the oracle: pins against the reference's sector dimensions,
a literal pure-Python copy of build_basis, physics invariants, and the
committed golden fixtures."""
import glob
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))

# reference staggered sectors (dg = 1): dim, nnz(REF), nnz(PJW)
SECTORS = {
    (3, 2): (90, 434, 610),
    (2, 3): (90, 434, 610),
    (4, 2): (645, 4017, 5843),
    (3, 3): (2443, 17027, 25747),
    (4, 3): (72211, 669615, 1042503),
    (3, 4): (72211, 669615, 1042503),
}


@pytest.mark.parametrize("nx,ny", list(SECTORS))
def test_sector_dimensions_and_nnz(oracle, nx, ny):
    dim, nnz_ref, nnz_pjw = SECTORS[(nx, ny)]
    b = oracle.build_basis(nx, ny, 1, oracle.staggered_charges(nx, ny))
    assert b.dim == dim
    assert oracle.build_hamiltonian(b, g=1.0, t=1.0, m=0.5, model="ref").nnz == nnz_ref
    assert oracle.build_hamiltonian(b, g=1.0, t=1.0, m=0.5, model="pjw").nnz == nnz_pjw


@pytest.mark.parametrize("nx,ny,dg,kind", [(2, 2, 1, "stag"), (3, 2, 1, "stag"), (2, 3, 1, "stag"),
                                            (4, 2, 1, "stag"), (3, 3, 1, "zero"),
                                            (3, 3, 1, "string"), (2, 2, 2, "stag"),
                                            (1, 3, 1, "stag"), (3, 1, 1, "stag")])
def test_c_restatement_matches_literal_recursion(oracle, nx, ny, dg, kind):
    if kind == "stag":
        g = oracle.staggered_charges(nx, ny)
    elif kind == "string":
        g = oracle.string_charges(nx, ny)
    else:
        g = np.zeros((nx, ny), np.int32)
    states, keys = oracle.py_build_basis(nx, ny, dg, g, dedup="encode" if dg == 1 else "config")
    b = oracle.build_basis(nx, ny, dg, g)
    assert b.dim == len(states)
    for i, (nf, eR, eU) in enumerate(states):
        assert np.array_equal(b.nf[i], nf)
        assert np.array_equal(b.eR[i], eR)
        assert np.array_equal(b.eU[i], eU)
    if dg == 1:
        assert list(b.ref_keys) == keys
    # discovery order == ascending order keys
    assert np.all(np.diff(b.order_keys.astype(np.uint64)) > 0)


def test_reference_encode_collides_for_dg2(oracle):
    """finite_ed.jl:89,93 write e+1 into 2-bit fields; for dg = 2 distinct
    states share a key and build_basis (:228) drops them.  The oracle and
    the GPU library enumerate the full sector instead."""
    g = oracle.staggered_charges(2, 2)
    lit, _ = oracle.py_build_basis(2, 2, 2, g, dedup="encode")
    full, _ = oracle.py_build_basis(2, 2, 2, g, dedup="config")
    b = oracle.build_basis(2, 2, 2, g)
    assert len(lit) < len(full) == b.dim == 25


def test_inconsistent_sector_raises(oracle):
    g = np.zeros((3, 2), np.int32)
    g[0, 0] = 3  # N_f = -3
    with pytest.raises(ValueError):
        oracle.build_basis(3, 2, 1, g)


def test_encode_4x4_uses_sign_bit(oracle):
    """At 4x4 the reference _encode fills all 64 bits (bit 63 = last e_U
    field); the oracle keeps the Int64 bit pattern."""
    nx, ny = 4, 4
    nf = np.zeros((nx, ny), np.int8)
    eR = np.zeros((nx - 1, ny), np.int8)
    eU = np.zeros((nx, ny - 1), np.int8)
    eU[nx - 1, ny - 2] = 1  # field value 2 -> bit 63
    L = oracle.lib()
    k = L.orc_encode(nx, ny, oracle._ptr(np.asfortranarray(nf)), oracle._ptr(np.asfortranarray(eR)),
                     oracle._ptr(np.asfortranarray(eU)))
    assert k < 0


@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_hamiltonian_invariants(oracle, model):
    nx, ny = 4, 2
    b = oracle.build_basis(nx, ny, 1, oracle.staggered_charges(nx, ny))
    H = oracle.build_hamiltonian(b, g=0.9, t=1.1, m=0.37, model=model)
    assert abs(H - H.T).max() == 0.0
    # staggered product state: E = 0, n_f = 1 on odd sites (stag = -1)
    i0 = oracle.staggered_product_index(b)
    n_odd = int(sum((ix + iy) % 2 for ix in range(1, nx + 1) for iy in range(1, ny + 1)))
    assert H[i0, i0] == pytest.approx(-0.37 * n_odd, abs=1e-15)
    # off-diagonal values are exactly -t (with JW sign) or -1/(2g^2)
    off = H.tolil()
    off.setdiag(0)
    off = off.tocsr()
    off.eliminate_zeros()
    vals = np.unique(off.data)
    allowed = {-1.1, 1.1, -1.0 / (2 * 0.81)} if model == "pjw" else {-1.1}
    assert set(np.round(vals, 12)) <= {round(v, 12) for v in allowed} | {0.0}


@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_hellmann_feynman(oracle, model):
    """dE0/dm = sum_s stag(s) <n_f(s)>;  dE0/dg = g <sum E^2> (+ g^-3 <sum(W+W^dag)> for PJW)."""
    nx, ny = 3, 2
    b = oracle.build_basis(nx, ny, 1, oracle.staggered_charges(nx, ny))
    g, t, m, h = 0.9, 1.0, 0.4, 1e-5

    def E(g_, m_):
        return oracle.ground_state(oracle.build_hamiltonian(b, g=g_, t=t, m=m_, model=model))[0]

    E0, psi = oracle.ground_state(oracle.build_hamiltonian(b, g=g, t=t, m=m, model=model))
    ms = oracle.measure(psi, b)
    ns = nx * ny
    dEdm = (E(g, m + h) - E(g, m - h)) / (2 * h)
    assert dEdm == pytest.approx(ms["n_stag"] * ns, abs=1e-7)
    dEdg = (E(g + h, m) - E(g - h, m)) / (2 * h)
    expect = g * ms["E2_mean"] * ns
    if model == "pjw":
        expect += ms["plaq_mean"] * (nx - 1) * (ny - 1) / g**3
    assert dEdg == pytest.approx(expect, abs=1e-7)


def test_evolution_conserves_norm_and_energy(oracle):
    nx, ny = 3, 2
    b = oracle.build_basis(nx, ny, 1, oracle.staggered_charges(nx, ny))
    H = oracle.build_hamiltonian(b, g=1.0, t=1.0, m=0.5, model="pjw")
    v = np.zeros(b.dim, np.complex128)
    v[oracle.staggered_product_index(b)] = 1.0
    psi, data = oracle.evolve(v, H, b, dt=0.1, n_steps=5)
    assert abs(np.linalg.norm(psi) - 1) < 1e-13
    assert abs(np.vdot(psi, H @ psi).real - np.vdot(v, H @ v).real) < 1e-10
    assert len(data) == 6 and data[-1]["t"] == pytest.approx(0.5)


GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_golden(oracle, path):
    z = np.load(path)
    nx, ny, dg = int(z["nx"]), int(z["ny"]), int(z["dg"])
    kind = str(z["sector"])
    g = oracle.staggered_charges(nx, ny) if kind == "stag" else oracle.string_charges(nx, ny)
    b = oracle.build_basis(nx, ny, dg, g)
    np.testing.assert_array_equal(b.order_keys, z["order_keys"])
    np.testing.assert_array_equal(b.ref_keys, z["ref_keys"])
    H = oracle.build_hamiltonian(b, g=float(z["g"]), t=float(z["t"]), m=float(z["m"]),
                                 model=str(z["model"]))
    np.testing.assert_array_equal(H.indptr, z["indptr"])
    np.testing.assert_array_equal(H.indices, z["indices"])
    np.testing.assert_array_equal(H.data, z["data"])
    E0, psi = oracle.ground_state(H)
    assert abs(E0 - float(z["E0"])) <= 1e-12 * abs(float(z["E0"]))


@pytest.mark.parametrize("nx,ny,dg,kind", [(3, 2, 1, "stag"), (4, 2, 1, "stag"), (3, 3, 1, "stag"),
                                            (3, 4, 1, "string"), (2, 2, 2, "stag"),
                                            (3, 2, 2, "stag")])
@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_row_restricted_build_equals_full_build(oracle, nx, ny, dg, kind, model):
    """orc_ham_rows (the sampled-row oracle used at 4x4, where the whole
    matrix is too large for a test) gives exactly the rows of the full
    build: same columns, bitwise the same values, for every row and for a
    random sample with repeats."""
    g = oracle.staggered_charges(nx, ny) if kind == "stag" else oracle.string_charges(nx, ny)
    b = oracle.build_basis(nx, ny, dg, g)
    H = oracle.build_hamiltonian(b, g=0.9, t=1.1, m=0.37, model=model)
    R = oracle.hamiltonian_rows(b, np.arange(b.dim), g=0.9, t=1.1, m=0.37, model=model)
    np.testing.assert_array_equal(R.indptr, H.indptr)
    np.testing.assert_array_equal(R.indices, H.indices)
    np.testing.assert_array_equal(R.data, H.data)
    rows = np.random.default_rng(5).integers(0, b.dim, 40)
    S = oracle.hamiltonian_rows(b, rows, g=0.9, t=1.1, m=0.37, model=model)
    assert (S != H[rows]).nnz == 0
