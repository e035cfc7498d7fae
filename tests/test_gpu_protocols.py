"""GPU runs of the quench protocols A/B/C and the ground-state grid against
the FP64 oracle (observables 1e-9 absolute, E0 1e-10 relative)."""
import csv

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("nf_mean", "nf_even", "nf_odd", "E2_mean")


def _check_series(series, ref, tol=1e-9):
    assert len(series) == len(ref)
    for a, b in zip(series, ref):
        assert abs(a["t"] - b["t"]) < 1e-12
        for key in KEYS:
            assert abs(a[key] - b[key]) <= tol, (key, a[key], b[key])


def test_quench_a_default_lattice(oracle, lgt, tmp_path):
    from lgt_gb300 import protocols
    data = protocols.run_quench_A_ED(n_steps=3, results_dir=str(tmp_path))
    g = oracle.string_charges(3, 4)
    ob = oracle.build_basis(3, 4, 1, g)
    Ho = oracle.build_hamiltonian(ob, g=1.0, t=1.0, m=2.0)
    gb = lgt.build_basis(3, 4, 1, g)[0]
    v0 = lgt.string_state(gb)
    _, ref = oracle.evolve(v0, Ho, ob, dt=0.02, n_steps=3)
    _check_series(data, ref)
    rows = list(csv.reader(open(tmp_path / "finite_ed_quench_A_data.csv")))
    assert rows[0] == ["t", "nf_mean", "nf_even", "nf_odd", "E2_mean"] and len(rows) == 5


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32_mixed", 1e-6)])
def test_quench_b_batched(oracle, lgt, tmp_path, precision, tol):
    from lgt_gb300 import protocols
    mf = [0.1, 0.7]
    data = protocols.run_quench_B_ED(nx=3, ny=2, m_final=mf, n_steps=4, dt=0.05,
                                     results_dir=str(tmp_path), precision=precision)
    ob = oracle.build_basis(3, 2, 1, oracle.staggered_charges(3, 2))
    _, psi0 = oracle.ground_state(oracle.build_hamiltonian(ob, g=1.0, t=1.0, m=5.0))
    for k, m in enumerate(mf):
        Ho = oracle.build_hamiltonian(ob, g=1.0, t=1.0, m=m)
        _, ref = oracle.evolve(psi0, Ho, ob, dt=0.05, n_steps=4)
        _check_series([step[k] for step in data], ref, tol)
    rows = list(csv.reader(open(tmp_path / "finite_ed_quench_B_data.csv")))
    assert rows[0][0] == "m_final" and len(rows) == 1 + 2 * 5


def test_quench_c_single(oracle, lgt, tmp_path):
    from lgt_gb300 import protocols
    data = protocols.run_quench_C_ED(nx=4, ny=2, n_steps=3, dt=0.05, results_dir=str(tmp_path))
    ob = oracle.build_basis(4, 2, 1, oracle.staggered_charges(4, 2))
    _, psi0 = oracle.ground_state(oracle.build_hamiltonian(ob, g=2.0, t=1.0, m=2.0))
    Ho = oracle.build_hamiltonian(ob, g=0.5, t=1.0, m=2.0)
    _, ref = oracle.evolve(psi0, Ho, ob, dt=0.05, n_steps=3)
    _check_series(data, ref)


def test_gs_grid_all_points_one_batch(oracle, lgt, tmp_path):
    from lgt_gb300 import gs_grid
    rows = gs_grid.run_grid(None, str(tmp_path), nx=3, ny=2)
    assert [r["task_id"] for r in rows] == list(range(1, 26))
    ob = oracle.build_basis(3, 2, 1, oracle.staggered_charges(3, 2))
    for r in rows:
        Ho = oracle.build_hamiltonian(ob, g=r["g"], t=1.0, m=r["m"])
        E0o, psio = oracle.ground_state(Ho)
        assert abs(r["ed_E0"] - E0o) <= 1e-10 * abs(E0o)
        gap = np.diff(oracle.spectrum_low(Ho, 2))[0]
        if gap > 1e-3:
            mo = oracle.measure(psio, ob)
            for key in KEYS:
                assert abs(r["ed_" + key] - mo[key]) <= 1e-9, key
    files = sorted(p.name for p in tmp_path.iterdir())
    assert files[0] == "gs_benchmark_001.csv" and len(files) == 25
    one = gs_grid.run_one_point(7, str(tmp_path), nx=3, ny=2)
    assert one["m"] == 0.5 and one["g"] == 0.5
    assert abs(one["ed_E0"] - rows[6]["ed_E0"]) <= 1e-10 * abs(rows[6]["ed_E0"])
