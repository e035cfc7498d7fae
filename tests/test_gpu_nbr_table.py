"""GPU parity of the stored-neighbour-table H*psi (nbr_table.cu).

The table is built once per Hamiltonian by the run-time-geometry move
enumeration (any shape, any dg); its kernel gathers with the fixed-shape
kernel's load modes (LGT_HPSI_VARIANT=5, 6, 7: one or two 16-byte vectors
per lane, two as one 32-byte access), or has the copy engine gather the
neighbour rows (8: FP32 panels of 16 columns; other panels fall back to 7).  Bars: 1e-12 relative to max |y|
(FP64) and 2e-6 (FP32) against the FP64 oracle's CSR matrix (reference and
plaquette+JW models), against the run-time-geometry kernel for the JW-only
and plaquette-only models and on the 4x4 lattice; ground states within
1e-10 of the oracle.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COUPLINGS = [(1.0, 1.0, 0.5), (0.8, 1.3, 0.3), (2.0, 0.7, -1.1), (0.55, 1.0, 0.9),
             (1.4, 0.9, 0.0), (0.3, 1.1, 2.0), (1.0, 0.5, -0.4), (2.5, 1.0, 0.7)]

# (nx, ny, dg, sector)
CASES = [(3, 2, 1, "stag"), (2, 3, 1, "zero"), (4, 2, 1, "string"), (3, 3, 1, "stag"),
         (4, 3, 1, "stag"), (3, 4, 1, "string"), (2, 2, 2, "stag"), (3, 2, 2, "stag"),
         (1, 4, 1, "stag"), (4, 1, 1, "stag")]
WIDTHS = {"fp64": [(1, True), (2, True), (4, False)],
          "fp32": [(2, True), (4, True), (8, False), (8, True), (16, False)]}

_cache = {}


def _charges(O, nx, ny, kind):
    if kind == "stag":
        return O.staggered_charges(nx, ny)
    if kind == "string":
        return O.string_charges(nx, ny)
    return np.zeros((nx, ny), np.int32)


def _pair(O, L, nx, ny, dg, kind):
    key = (nx, ny, dg, kind)
    if key not in _cache:
        g = _charges(O, nx, ny, kind)
        _cache[key] = (O.build_basis(nx, ny, dg, g), L.build_basis(nx, ny, dg, g)[0])
    return _cache[key]


def _panel(rng, N, K, cplx, prec):
    x = rng.standard_normal((N, K))
    if cplx:
        x = x + 1j * rng.standard_normal((N, K))
    return x.astype(np.complex64 if cplx else np.float32) if prec == "fp32" else x


def _tol(prec):
    return 1e-12 if prec == "fp64" else 2e-6


@pytest.mark.parametrize("variant", ["5", "6", "7", "8"])
@pytest.mark.parametrize("model", ["ref", "jw", "plaq", "pjw"])
@pytest.mark.parametrize("nx,ny,dg,kind", CASES)
def test_table_vs_oracle(oracle, lgt, nx, ny, dg, kind, model, variant, monkeypatch):
    monkeypatch.setenv("LGT_HPSI_VARIANT", variant)
    ob, gb = _pair(oracle, lgt, nx, ny, dg, kind)
    rng = np.random.default_rng(nx * 100 + ny * 10 + dg)
    Hos = {}
    for prec in ("fp64", "fp32"):
        for K, cplx in WIDTHS[prec]:
            cpl = (COUPLINGS * 2)[:K]  # 16 real columns: the couplings twice
            gs, ts, ms = (np.array(v) for v in zip(*cpl))
            H = lgt.build_hamiltonian(gb, g=gs, t=ts, m=ms, model=model)
            x = _panel(rng, ob.dim, K, cplx, prec)
            y = H.matvec(x, precision=prec)
            if model in ("jw", "plaq"):  # no oracle matrix: the run-time-geometry kernel
                yg = H.matvec(x, precision=prec, generic=True)
                scale = max(1.0, float(np.max(np.abs(yg))))
                assert np.max(np.abs(y - yg)) <= _tol(prec) * scale, (prec, K, cplx)
                H.close()
                continue
            for k in range(K):
                kc = k % len(COUPLINGS)
                if kc not in Hos:
                    g, t, m = COUPLINGS[kc]
                    Hos[kc] = oracle.build_hamiltonian(ob, g=g, t=t, m=m, model=model)
                yo = Hos[kc] @ x[:, k].astype(np.complex128 if cplx else np.float64)
                err = np.max(np.abs(y[:, k] - yo))
                assert err <= _tol(prec) * max(1.0, np.max(np.abs(yo))), (prec, K, cplx, k, err)
            H.close()


@pytest.mark.parametrize("variant,K", [("6", 4), ("7", 4), ("8", 8)])
@pytest.mark.parametrize("model", ["ref", "pjw"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_table_4x4_vs_generic(lgt, model, prec, variant, K, monkeypatch):
    """4x4 staggered sector (N = 8,563,545), K = 4 or 8 complex (8: the
    gathered kernel's panel width)."""
    monkeypatch.setenv("LGT_HPSI_VARIANT", variant)
    st, _ = lgt.build_basis(4, 4, 1, lgt.staggered_charges(4, 4))
    rng = np.random.default_rng(45)
    gs, ts, ms = (np.array(v) for v in zip(*COUPLINGS[:K]))
    H = lgt.build_hamiltonian(st, g=gs, t=ts, m=ms, model=model)
    x = _panel(rng, len(st), K, True, prec)
    y = H.matvec(x, precision=prec)
    yg = H.matvec(x, precision=prec, generic=True)
    assert np.max(np.abs(y - yg)) <= _tol(prec) * max(1.0, float(np.max(np.abs(yg))))
    H.close()


def test_table_disabled_falls_back(oracle, lgt, monkeypatch):
    """With LGT_NBR_TABLE=0 a forced table variant runs the built-in rule."""
    monkeypatch.setenv("LGT_HPSI_VARIANT", "6")
    monkeypatch.setenv("LGT_NBR_TABLE", "0")
    ob, gb = _pair(oracle, lgt, 4, 3, 1, "stag")
    H = lgt.build_hamiltonian(gb, g=[0.9, 1.2], t=1.0, m=0.4)
    x = _panel(np.random.default_rng(7), ob.dim, 2, True, "fp64")
    y = H.matvec(x)
    for k, g in enumerate((0.9, 1.2)):
        yo = oracle.build_hamiltonian(ob, g=g, t=1.0, m=0.4) @ x[:, k]
        assert np.max(np.abs(y[:, k] - yo)) <= 1e-12 * max(1.0, np.max(np.abs(yo)))
    H.close()


@pytest.mark.parametrize("model", ["ref", "pjw"])
def test_table_ground_states(oracle, lgt, model, monkeypatch):
    """Panel Lanczos (FP64 and FP32-mixed) with the table kernel forced."""
    monkeypatch.setenv("LGT_HPSI_VARIANT", "6")
    ob, gb = _pair(oracle, lgt, 4, 3, 1, "stag")
    gs = np.array([0.6, 1.1, 1.7, 2.4])
    H = lgt.build_hamiltonian(gb, g=gs, t=1.0, m=0.3, model=model)
    E0o = [oracle.ground_state(oracle.build_hamiltonian(ob, g=g, t=1.0, m=0.3, model=model))[0]
           for g in gs]
    for prec in ("fp64", "fp32_mixed"):
        E0, _ = lgt.find_ground_state(H, tol=1e-12, solver="panel", precision=prec,
                                      as_complex=False)
        for k in range(len(gs)):
            assert abs(E0[k] - E0o[k]) <= 1e-10 * abs(E0o[k]), (prec, k)
    H.close()


@pytest.mark.parametrize("nx,ny,model", [(4, 3, "ref"), (3, 4, "pjw"), (4, 4, "ref"),
                                          (4, 4, "pjw"), (2, 2, "ref")])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
@pytest.mark.parametrize("order", ["mask", "row"])
def test_row_order_product_bitwise(lgt, monkeypatch, nx, ny, model, prec, order):
    """The renumbered table (breadth-first row order of the hop graph, used
    by the Krylov drivers): the order is a permutation, and H applied to a
    panel kept in that order equals, bit for bit, the reordered product in
    the reference order (same entries, same summation order per row)."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("LGT_TABLE_ORDER", order)
    st, _ = lgt.build_basis(nx, ny, 1, lgt.staggered_charges(nx, ny))
    N = len(st)
    gs, ts, ms = (np.array(v) for v in zip(*COUPLINGS[:2]))
    H = lgt.build_hamiltonian(st, g=gs, t=ts, m=ms, model=model)
    perm = H.row_order()
    assert np.array_equal(np.sort(perm), np.arange(N))
    dt = torch.float64 if prec == "fp64" else torch.float32
    gen = torch.Generator(device="cuda").manual_seed(nx * 10 + ny)
    x = torch.randn((N, 2, 2), dtype=dt, device="cuda", generator=gen)
    y = torch.empty_like(x)
    p = torch.from_numpy(perm.astype(np.int64)).cuda()
    xo = x[p].contiguous()
    yo = torch.empty_like(xo)
    torch.cuda.synchronize()  # the library works on the basis' own stream
    H.matvec_device(x.data_ptr(), y.data_ptr(), 2, prec)
    H.matvec_device(xo.data_ptr(), yo.data_ptr(), 2, prec, row_order=True)
    torch.cuda.synchronize()
    assert torch.equal(yo, y[p])
    H.close()
    st.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32_mixed"])
def test_krylov_row_order_matches_reference_order(lgt, monkeypatch, precision):
    """Krylov drivers with their vectors in the table's mask-segment order
    (default), its row-level order and the reference order
    (LGT_TABLE_ORDER=0), stored-table kernel forced: same ground states and
    evolved states."""
    monkeypatch.setenv("LGT_HPSI_VARIANT", "6")
    st, _ = lgt.build_basis(4, 3, 1, lgt.staggered_charges(4, 3))
    v0 = lgt.staggered_product_state(st)
    res = {}
    for flag in ("mask", "row", "0"):
        monkeypatch.setenv("LGT_TABLE_ORDER", flag)
        H = lgt.build_hamiltonian(st, g=[0.7, 1.3, 0.9, 1.1], t=1.0, m=0.5, model="pjw")
        E0, psi = lgt.find_ground_state(H, tol=1e-12, solver="panel", precision=precision,
                                        as_complex=False)
        _, ps, _ = lgt.evolve_ED(np.stack([v0] * 4, axis=1), H, dt=0.05, n_steps=3, tol=1e-12,
                                 precision=precision, return_state=True)
        res[flag] = (E0, psi, ps)
        H.close()
    tol = 1e-12 if precision == "fp64" else 1e-10
    for flag in ("mask", "row"):
        np.testing.assert_allclose(res[flag][0], res["0"][0], rtol=tol)
        ov = np.abs(np.sum(res[flag][1] * res["0"][1], axis=0))
        assert np.all(ov > 1 - (1e-12 if precision == "fp64" else 1e-8))
        assert np.max(np.abs(res[flag][2] - res["0"][2])) <= (1e-10 if precision == "fp64"
                                                               else 1e-6)
    st.close()
