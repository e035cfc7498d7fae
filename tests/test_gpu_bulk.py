"""The Gram-Schmidt kernels that stream the Krylov panels through shared
memory with bulk copies (k_update_bulk, k_multidot_bulk) against the
register-load kernels (k_update_df, k_multidot; LGT_BULK_STREAM=0): the same
rows in the same order with the same double-float arithmetic, so the
FP32-mixed drivers must give bitwise identical results either way.  The 4x3 sector (N = 72211) meets the copy
alignment for every panel width used here."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _both(lgt, monkeypatch, run):
    out = {}
    for bulk in ("1", "0"):
        monkeypatch.setenv("LGT_BULK_STREAM", bulk)
        monkeypatch.setenv("LGT_BULK_DOTS", bulk)  # the streamed dot kernel too
        out[bulk] = run()
    return out["1"], out["0"]


@pytest.mark.parametrize("K", [1, 2, 8])
def test_bulk_update_quench_bitwise(lgt, monkeypatch, K):
    b = lgt.build_basis(4, 3, 1, lgt.staggered_charges(4, 3))[0]
    gs = np.linspace(0.7, 1.3, K)
    v0 = lgt.staggered_product_state(b)
    p0 = np.repeat(v0[:, None], K, axis=1)

    def run():
        H = lgt.build_hamiltonian(b, g=gs, t=1.0, m=0.5)
        data, psi, drift = lgt.evolve_ED(p0, H, dt=0.05, n_steps=3, tol=1e-12,
                                         precision="fp32_mixed", return_state=True)
        H.close()
        recs = [step if isinstance(step, list) else [step] for step in data]  # K = 1: dicts
        return psi, drift, [[d["E2_mean"] for d in step] for step in recs]

    (pa, da, ea), (pb, db, eb) = _both(lgt, monkeypatch, run)
    assert np.array_equal(pa, pb)
    assert np.array_equal(da, db)
    assert ea == eb


@pytest.mark.parametrize("K", [4, 16])
def test_bulk_update_ground_state_bitwise(oracle, lgt, monkeypatch, K):
    b = lgt.build_basis(4, 3, 1, lgt.staggered_charges(4, 3))[0]
    gs = np.linspace(0.6, 1.8, K)

    def run():
        H = lgt.build_hamiltonian(b, g=gs, t=1.0, m=0.5, model="pjw")
        E0, psi = lgt.find_ground_state(H, tol=1e-12, precision="fp32_mixed", solver="panel",
                                        as_complex=False)
        H.close()
        return E0, psi

    (ea, pa), (eb, pb) = _both(lgt, monkeypatch, run)
    assert np.array_equal(ea, eb)
    assert np.array_equal(pa, pb)
    # and the streamed path meets the solver's bar against the FP64 oracle
    ob = oracle.build_basis(4, 3, 1, oracle.staggered_charges(4, 3))
    Ho = oracle.build_hamiltonian(ob, g=gs[0], t=1.0, m=0.5, model="pjw")
    E0o, _ = oracle.ground_state(Ho)
    assert abs(ea[0] - E0o) <= 1e-10 * abs(E0o)


def test_gathered_hpsi_quench(lgt, monkeypatch):
    """The stored-table H*psi with the copy engine gathering the neighbour
    rows (LGT_HPSI_VARIANT=8) inside the FP32-mixed Krylov drivers (the
    panel picked by a device-resident slot index, the table in its
    renumbered row order) against the lane-gathering table kernel (7): the
    same sums in the same order."""
    b = lgt.build_basis(4, 3, 1, lgt.staggered_charges(4, 3))[0]
    gs = np.linspace(0.6, 1.5, 8)
    v0 = lgt.staggered_product_state(b)
    p0 = np.repeat(v0[:, None], 8, axis=1)
    out = {}
    for var in ("8", "7"):
        monkeypatch.setenv("LGT_HPSI_VARIANT", var)
        H = lgt.build_hamiltonian(b, g=gs, t=1.0, m=0.5)
        data, psi, drift = lgt.evolve_ED(p0, H, dt=0.05, n_steps=3, tol=1e-12,
                                         precision="fp32_mixed", return_state=True)
        H.close()
        out[var] = psi
    assert np.max(np.abs(out["8"] - out["7"])) <= 1e-12
