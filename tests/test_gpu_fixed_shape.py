"""GPU parity of the fixed-shape H*psi kernels (4x3, 3x4 and 4x4 at dg = 1).

Panels with C = K * ncomp a multiple of the vector width run the
compile-time kernels; every load mode (one or two 16-byte vectors per lane,
two vectors as one 32-byte access; forced with LGT_HPSI_VARIANT) and every
column width that changes it is covered, for all four model flags.
Bars: 1e-12 relative to max |y| (FP64) and 2e-6 (FP32) against the FP64
oracle's CSR matrix for the reference and plaquette+JW models; against the
run-time-geometry kernel (itself checked against the oracle in
test_gpu_parity) for the JW-only and plaquette-only models and on the 4x4
lattice, where the oracle's matrix would take minutes to build.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COUPLINGS = [(1.0, 1.0, 0.5), (0.8, 1.3, 0.3), (2.0, 0.7, -1.1), (0.55, 1.0, 0.9),
             (1.4, 0.9, 0.0), (0.3, 1.1, 2.0), (1.0, 0.5, -0.4), (2.5, 1.0, 0.7)]

_cache = {}


def _pair(O, L, nx, ny, kind):
    key = (nx, ny, kind)
    if key not in _cache:
        g = O.staggered_charges(nx, ny) if kind == "stag" else O.string_charges(nx, ny)
        _cache[key] = (O.build_basis(nx, ny, 1, g), L.build_basis(nx, ny, 1, g)[0])
    return _cache[key]


def _panel(rng, N, K, cplx, dtype):
    x = rng.standard_normal((N, K))
    if cplx:
        x = x + 1j * rng.standard_normal((N, K))
    return x.astype(np.complex64 if cplx else np.float32) if dtype == "fp32" else x


def _tol(prec):
    return 1e-12 if prec == "fp64" else 2e-6


# (K, complex): FP64 C = 2, 4, 16; FP32 C = 4, 8, 16
WIDTHS = {"fp64": [(1, True), (2, True), (8, True), (4, False)],
          "fp32": [(2, True), (4, True), (8, True), (8, False)]}


@pytest.mark.parametrize("variant", ["2", "3", "4"])  # one / two vectors, one 32-byte access
@pytest.mark.parametrize("nx,ny,kind", [(4, 3, "stag"), (3, 4, "stag"), (3, 4, "string")])
@pytest.mark.parametrize("model", ["ref", "pjw"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_fixed_vs_oracle(oracle, lgt, nx, ny, kind, model, prec, variant, monkeypatch):
    monkeypatch.setenv("LGT_HPSI_VARIANT", variant)
    ob, gb = _pair(oracle, lgt, nx, ny, kind)
    rng = np.random.default_rng(nx * 10 + ny)
    Hos = {}
    for K, cplx in WIDTHS[prec]:
        gs, ts, ms = (np.array(v) for v in zip(*COUPLINGS[:K]))
        H = lgt.build_hamiltonian(gb, g=gs, t=ts, m=ms, model=model)
        x = _panel(rng, ob.dim, K, cplx, prec)
        y = H.matvec(x, precision=prec)
        for k in range(K):
            if k not in Hos:
                g, t, m = COUPLINGS[k]
                Hos[k] = oracle.build_hamiltonian(ob, g=g, t=t, m=m, model=model)
            yo = Hos[k] @ x[:, k].astype(np.complex128 if cplx else np.float64)
            err = np.max(np.abs(y[:, k] - yo))
            assert err <= _tol(prec) * max(1.0, np.max(np.abs(yo))), (K, cplx, k, err)
        H.close()


@pytest.mark.parametrize("variant", ["2", "3", "4"])
@pytest.mark.parametrize("nx,ny", [(4, 3), (3, 4)])
@pytest.mark.parametrize("model", ["jw", "plaq"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_fixed_vs_generic_models(oracle, lgt, nx, ny, model, prec, variant, monkeypatch):
    monkeypatch.setenv("LGT_HPSI_VARIANT", variant)
    ob, gb = _pair(oracle, lgt, nx, ny, "stag")
    rng = np.random.default_rng(3)
    for K, cplx in WIDTHS[prec]:
        gs, ts, ms = (np.array(v) for v in zip(*COUPLINGS[:K]))
        H = lgt.build_hamiltonian(gb, g=gs, t=ts, m=ms, model=model)
        x = _panel(rng, ob.dim, K, cplx, prec)
        y = H.matvec(x, precision=prec)
        yg = H.matvec(x, precision=prec, generic=True)
        scale = max(1.0, np.max(np.abs(yg)))
        assert np.max(np.abs(y - yg)) <= _tol(prec) * scale, (K, cplx)
        H.close()


@pytest.mark.parametrize("variant", ["3", "4"])
@pytest.mark.parametrize("model", ["ref", "pjw"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_fixed_4x4_vs_generic(lgt, model, prec, variant, monkeypatch):
    """4x4 staggered sector (N = 8,563,545), K = 2 complex and K = 4 complex."""
    monkeypatch.setenv("LGT_HPSI_VARIANT", variant)
    st, _ = lgt.build_basis(4, 4, 1, lgt.staggered_charges(4, 4))
    assert len(st) == 8563545
    rng = np.random.default_rng(44)
    for K in (2, 4):
        gs, ts, ms = (np.array(v) for v in zip(*COUPLINGS[:K]))
        H = lgt.build_hamiltonian(st, g=gs, t=ts, m=ms, model=model)
        x = _panel(rng, len(st), K, True, prec)
        y = H.matvec(x, precision=prec)
        yg = H.matvec(x, precision=prec, generic=True)
        scale = max(1.0, float(np.max(np.abs(yg))))
        assert np.max(np.abs(y - yg)) <= _tol(prec) * scale, K
        H.close()
