"""GPU tests of the two ground-state solvers (one CTA per point, and
K-interleaved panels) and of the uneven multi-lattice batch, against the
FP64 oracle.  Tolerances: |dE|/|E| <= 1e-10 (FP64 and FP32-mixed),
observables 1e-9 absolute (FP64), eigenvector 1e-9/gap."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _basis(O, L, nx, ny, kind="stag"):
    g = O.staggered_charges(nx, ny) if kind == "stag" else O.string_charges(nx, ny)
    return O.build_basis(nx, ny, 1, g), L.build_basis(nx, ny, 1, g)[0]


@pytest.mark.parametrize("solver", ["cta", "panel"])
@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
@pytest.mark.parametrize("nx,ny,model", [(3, 2, "ref"), (4, 2, "pjw"), (3, 3, "ref"),
                                          (2, 4, "pjw"), (2, 2, "ref")])
def test_solver_vs_oracle(oracle, lgt, solver, precision, nx, ny, model):
    ob, gb = _basis(oracle, lgt, nx, ny)
    gs = np.array([0.55, 1.0, 1.9])
    ms = np.array([0.5, 0.1, 0.8])
    H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=ms, model=model)
    E0, psi, info = lgt.find_ground_state(H, tol=1e-12, precision=precision, solver=solver,
                                          as_complex=False, return_info=True)
    obs = lgt.measure_ED(psi, gb)
    for k in range(3):
        Ho = oracle.build_hamiltonian(ob, g=gs[k], t=1.0, m=ms[k], model=model)
        E0o, psio = oracle.ground_state(Ho)
        assert abs(E0[k] - E0o) <= 1e-10 * abs(E0o), (k, E0[k], E0o)
        if precision == "fp64":
            gap = np.diff(oracle.spectrum_low(Ho, 2))[0]
            if gap > 1e-3:
                v = psi[:, k] * np.sign(np.dot(psi[:, k], psio))
                assert np.linalg.norm(v - psio) <= 1e-9 / min(gap, 1.0)
                mo = oracle.measure(psio, ob)
                for key in ("E2_mean", "plaq_mean", "nf_even", "nf_odd", "n_stag"):
                    assert abs(obs[k][key] - mo[key]) <= 1e-9, key
        assert info["residual"][k] <= (1e-11 if precision == "fp64" else 1e-3)
    H.close()


def test_cta_and_panel_agree(oracle, lgt):
    ob, gb = _basis(oracle, lgt, 4, 2)
    gs = np.linspace(0.5, 2.0, 16)
    H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=0.5, model="pjw")
    Ec, pc = lgt.find_ground_state(H, tol=1e-12, solver="cta", as_complex=False)
    Ep, pp = lgt.find_ground_state(H, tol=1e-12, solver="panel", as_complex=False)
    np.testing.assert_allclose(Ec, Ep, rtol=1e-12, atol=0)
    ov = np.abs(np.sum(pc * pp, axis=0))
    assert np.all(ov > 1 - 1e-12)
    H.close()


def test_uneven_batch_one_launch(oracle, lgt):
    """3x2, 4x2, 3x3 (one persistent launch, one CTA per point) and 4x3
    (panel solver), 4 (g, m) points each, FP32-mixed."""
    rng = np.random.default_rng(0)
    Hs, obs = [], []
    for nx, ny in [(3, 2), (4, 2), (3, 3), (4, 3)]:
        ob, gb = _basis(oracle, lgt, nx, ny)
        g = np.exp(rng.uniform(np.log(0.3), np.log(3.0), 4))
        m = rng.uniform(0.0, 1.0, 4)
        Hs.append(lgt.build_hamiltonian(gb, g=g, t=1.0, m=m, model="ref"))
        obs.append((ob, g, m))
    res = lgt.find_ground_states(Hs, precision="fp32_mixed")
    for (E0, psi), (ob, g, m) in zip(res, obs):
        for k in range(4):
            E0o = oracle.ground_state(oracle.build_hamiltonian(ob, g=g[k], t=1.0, m=m[k]))[0]
            assert abs(E0[k] - E0o) <= 1e-10 * abs(E0o)
        assert psi.shape == (ob.dim, 4)
    for H in Hs:
        H.close()


def test_string_sector_and_start_vector(oracle, lgt):
    """Quench-A sector; a given start vector (the string state) converges to
    the same ground state."""
    ob, gb = _basis(oracle, lgt, 3, 4, "string")
    H = lgt.build_hamiltonian(gb, g=1.0, t=1.0, m=2.0)
    v0 = lgt.string_state(gb)
    E0, psi = lgt.find_ground_state(H, tol=1e-12, v0=v0.real)
    E0o = oracle.ground_state(oracle.build_hamiltonian(ob, g=1.0, t=1.0, m=2.0))[0]
    assert abs(E0 - E0o) <= 1e-10 * abs(E0o)
    H.close()


@pytest.mark.parametrize("precision,tol_state", [("fp64", 1e-9), ("fp32_mixed", 2e-5)])
@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_quench_4x3_batched(oracle, lgt, precision, tol_state, model):
    """Real-time quench on the 4x3 lattice (N = 72211), two coupling points
    in one panel, from the staggered product state: states after 5 steps of
    dt = 0.05 against exp(-iHt) of the oracle; norm drift and energy
    conservation."""
    ob, gb = _basis(oracle, lgt, 4, 3)
    gs = np.array([0.7, 1.3])
    H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=0.5, model=model)
    v0 = lgt.staggered_product_state(gb)
    p0 = np.stack([v0, v0], axis=1)
    data, psi, drift = lgt.evolve_ED(p0, H, dt=0.05, n_steps=5, tol=1e-12, precision=precision,
                                     return_state=True)
    for k in range(2):
        Ho = oracle.build_hamiltonian(ob, g=gs[k], t=1.0, m=0.5, model=model)
        po, do = oracle.evolve(v0, Ho, ob, dt=0.05, n_steps=5)
        assert np.linalg.norm(psi[:, k] - po) <= tol_state
        assert abs(data[-1][k]["E2_mean"] - do[-1]["E2_mean"]) <= 10 * tol_state
        # every step's record carries measure_ED's site grids (finite_ed.jl:409,421-422)
        for step in (0, 2, 5):
            for key in ("nf_grid", "E2_grid", "plaq_grid"):
                assert data[step][k][key].shape == do[step][key].shape
                np.testing.assert_allclose(data[step][k][key], do[step][key], rtol=0,
                                           atol=10 * tol_state)
            assert abs(data[step][k]["nf_mean"] - data[step][k]["nf_grid"].mean()) <= 1e-12
        e0 = np.vdot(v0, Ho @ v0).real
        e1 = np.vdot(psi[:, k], Ho @ psi[:, k]).real
        assert abs(e1 - e0) <= 100 * tol_state * abs(e0)
    assert np.all(drift < (1e-12 if precision == "fp64" else 1e-5))
    H.close()


@pytest.mark.parametrize("smem", ["0", "1"])
@pytest.mark.parametrize("precision,krylovdim", [("fp32_mixed", 50), ("fp64", 30), ("fp64", 50)])
def test_cta_basis_placement(oracle, lgt, monkeypatch, smem, precision, krylovdim):
    """The per-CTA solver keeps the Krylov basis in shared memory when it
    fits (FP32 at krylovdim 50, FP64 at 30 on the 4x2 sector) and in global
    memory otherwise or with LGT_CTA_BASIS_SMEM=0: same results."""
    monkeypatch.setenv("LGT_CTA_BASIS_SMEM", smem)
    ob, gb = _basis(oracle, lgt, 4, 2)
    gs = np.array([0.5, 0.9, 1.4, 2.0])
    H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=0.5)
    E0, psi = lgt.find_ground_state(H, tol=1e-12, precision=precision, solver="cta",
                                    krylovdim=krylovdim, as_complex=False)
    for k in range(len(gs)):
        Ho = oracle.build_hamiltonian(ob, g=gs[k], t=1.0, m=0.5)
        E0o, psio = oracle.ground_state(Ho)
        assert abs(E0[k] - E0o) <= 1e-10 * abs(E0o), (k, E0[k], E0o)
        assert abs(abs(np.dot(psi[:, k], psio)) - 1.0) <= 1e-8
    H.close()


@pytest.mark.parametrize("solver,nx,ny", [("cta", 4, 2), ("cta", 3, 3), ("panel", 4, 3)])
@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_mixed_with_fp64_refinement(oracle, lgt, solver, nx, ny, model):
    """FP32-mixed solve followed by the FP64 correction (refine_steps: a
    short FP64 Lanczos started from the FP32 solution): observables within
    1e-10 of the FP64 oracle (the unrefined mixed path leaves ~1e-7),
    energies within 1e-12 relative."""
    ob, gb = _basis(oracle, lgt, nx, ny)
    gs, ms = np.array([0.8, 1.5]), np.array([0.3, 0.6])
    H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=ms, model=model)
    E0, psi = lgt.find_ground_state(H, tol=1e-12, precision="fp32_mixed", solver=solver,
                                    refine_steps=20, as_complex=False)
    obs = lgt.measure_ED(psi, gb)
    for k in range(2):
        Ho = oracle.build_hamiltonian(ob, g=gs[k], t=1.0, m=ms[k], model=model)
        E0o, psio = oracle.ground_state(Ho)
        mo = oracle.measure(psio, ob)
        assert abs(E0[k] - E0o) <= 1e-12 * abs(E0o), (k, E0[k], E0o)
        for key in ("E2_mean", "n_stag", "plaq_mean", "nf_even"):
            assert abs(obs[k][key] - mo[key]) <= 1e-10, (k, key, obs[k][key] - mo[key])
    H.close()


@pytest.mark.parametrize("smem", ["0", "1"])
@pytest.mark.parametrize("precision", ["fp32_mixed", "fp64"])
@pytest.mark.parametrize("nx,ny,model", [(4, 2, "ref"), (3, 3, "pjw"), (2, 2, "ref")])
def test_cta_cluster_split(oracle, lgt, monkeypatch, smem, precision, nx, ny, model):
    """Each point on a cluster of two CTAs (LGT_CTA_CLUSTER=2: rows split,
    dot and norm totals exchanged through distributed shared memory, the
    basis kept whole in both CTAs or once in global memory with
    LGT_CTA_BASIS_SMEM=0): energies and states against the FP64 oracle, and
    against the one-CTA solve."""
    monkeypatch.setenv("LGT_CTA_BASIS_SMEM", smem)
    ob, gb = _basis(oracle, lgt, nx, ny)
    gs = np.array([0.5, 0.9, 1.4, 2.0, 1.1])
    H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=0.5, model=model)
    monkeypatch.setenv("LGT_CTA_CLUSTER", "2")
    E2, p2, info = lgt.find_ground_state(H, tol=1e-12, precision=precision, solver="cta",
                                         as_complex=False, return_info=True)
    monkeypatch.setenv("LGT_CTA_CLUSTER", "1")
    E1, p1 = lgt.find_ground_state(H, tol=1e-12, precision=precision, solver="cta",
                                   as_complex=False)
    for k in range(len(gs)):
        Ho = oracle.build_hamiltonian(ob, g=gs[k], t=1.0, m=0.5, model=model)
        E0o, psio = oracle.ground_state(Ho)
        assert abs(E2[k] - E0o) <= 1e-10 * abs(E0o), (k, E2[k], E0o)
        assert abs(abs(np.dot(p2[:, k], psio)) - 1.0) <= 1e-8
        assert abs(E2[k] - E1[k]) <= 1e-10 * abs(E0o)
        assert info["residual"][k] <= (1e-11 if precision == "fp64" else 1e-3)
    H.close()


def test_cta_cluster_uneven_and_refined(oracle, lgt, monkeypatch):
    """Split units in an uneven batch (the 4x2, 3x3 and 3x2 sectors in one
    launch) and the FP64 refinement's second launch from a given start
    vector, both on clusters of two CTAs."""
    monkeypatch.setenv("LGT_CTA_CLUSTER", "2")
    Hs, obs_b = [], []
    for nx, ny in ((4, 2), (3, 3), (3, 2)):
        ob, gb = _basis(oracle, lgt, nx, ny)
        gs = np.array([0.7, 1.6])
        Hs.append(lgt.build_hamiltonian(gb, g=gs, t=1.0, m=0.4))
        obs_b.append((ob, gs))
    res = lgt.find_ground_states(Hs, tol=1e-12, precision="fp32_mixed")
    for (ob, gs), (E0, psi) in zip(obs_b, res):
        for k in range(2):
            Ho = oracle.build_hamiltonian(ob, g=gs[k], t=1.0, m=0.4)
            E0o, _ = oracle.ground_state(Ho)
            assert abs(E0[k] - E0o) <= 1e-10 * abs(E0o)
    E0, psi = lgt.find_ground_state(Hs[0], tol=1e-12, precision="fp32_mixed", solver="cta",
                                    refine_steps=20, as_complex=False)
    ob, gs = obs_b[0]
    for k in range(2):
        Ho = oracle.build_hamiltonian(ob, g=gs[k], t=1.0, m=0.4)
        E0o, _ = oracle.ground_state(Ho)
        assert abs(E0[k] - E0o) <= 1e-12 * abs(E0o)
    for H in Hs:
        H.close()


def _wide_points(n, seed):
    """Couplings of the uneven-batch benchmark: g log-uniform on [0.3, 3]
    (electric or plaquette terms dominating), m uniform on [0, 1]."""
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(0.3), np.log(3.0), n)), rng.uniform(0.0, 1.0, n)


@pytest.mark.parametrize("model", ["ref", "pjw"])
@pytest.mark.parametrize("nx,ny", [(3, 2), (4, 2)])
def test_cta_wide_couplings(oracle, lgt, nx, ny, model):
    """The per-point solver over couplings far from the headline's range
    (electric or plaquette terms dominating) against the oracle's dense
    ground states.  A 3x2 PJW point at g = 2.58 once converged to a wrong
    Ritz pair when beta was taken from the dots (||w||^2 - sum h^2) instead
    of the updated rows' own norm."""
    g, m = _wide_points(16, 0)
    g = np.concatenate([g, [2.583, 0.302, 1.952]])
    m = np.concatenate([m, [0.384, 0.981, 0.028]])
    b = lgt.build_basis(nx, ny, 1, lgt.staggered_charges(nx, ny))[0]
    H = lgt.build_hamiltonian(b, g=g, t=1.0, m=m, model=model)
    ob = oracle.build_basis(nx, ny, 1, oracle.staggered_charges(nx, ny))
    Eo = np.array([oracle.ground_state(oracle.build_hamiltonian(ob, g=gk, t=1.0, m=mk,
                                                                model=model))[0]
                   for gk, mk in zip(g, m)])
    for precision, tol in (("fp32_mixed", 1e-10), ("fp64", 1e-12)):
        E, _ = lgt.find_ground_state(H, precision=precision, solver="cta", as_complex=False)
        assert np.max(np.abs(E - Eo) / np.abs(Eo)) <= tol, precision
    H.close()
