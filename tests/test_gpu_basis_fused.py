"""Small sectors build their basis in one launch (k_basis_fused: masks, order
keys, segment starts, low parts, rank tables and their self-check in one
block); LGT_BASIS_FUSED=0 forces the multi-launch build.  Both must give
the same basis bit for bit, the same ranks, and the same H*psi."""
import numpy as np
import pytest

from lgt_gb300 import _capi as C

pytestmark = pytest.mark.gpu

# (nx, ny, dg, sector): candidate spaces up to 2^15 take the one-launch build
SMALL = [
    (2, 2, 1, "stag"), (3, 2, 1, "stag"), (2, 3, 1, "stag"), (4, 2, 1, "stag"),
    (2, 4, 1, "stag"), (3, 3, 1, "stag"), (3, 3, 1, "zero"), (4, 2, 1, "string"),
    (2, 2, 2, "stag"), (3, 2, 2, "stag"), (2, 3, 2, "zero"), (1, 4, 1, "stag"),
    (4, 1, 1, "stag"), (5, 2, 1, "stag"),
]


def _charges(lgt, nx, ny, kind):
    if kind == "stag":
        return lgt.staggered_charges(nx, ny)
    if kind == "string":
        return lgt.string_charges(nx, ny)
    return np.zeros((nx, ny), np.int32)


def _build(lgt, monkeypatch, fused, nx, ny, dg, kind):
    monkeypatch.setenv("LGT_BASIS_FUSED", "1" if fused else "0")
    n0 = C.launch_count()
    b, _ = lgt.build_basis(nx, ny, dg, _charges(lgt, nx, ny, kind))
    return b, C.launch_count() - n0


@pytest.mark.parametrize("nx,ny,dg,kind", SMALL)
def test_fused_basis_matches_multi_launch(lgt, monkeypatch, nx, ny, dg, kind):
    bf, nf_launch = _build(lgt, monkeypatch, True, nx, ny, dg, kind)
    bm, nm_launch = _build(lgt, monkeypatch, False, nx, ny, dg, kind)
    assert nf_launch == 1  # the whole build in one kernel
    assert nm_launch > 1
    assert bf.dim == bm.dim > 0
    keys = bm.order_keys()
    np.testing.assert_array_equal(bf.order_keys(), keys)
    for a, b in zip(bf.states(), bm.states()):
        np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(bf.rank(keys), np.arange(bm.dim))
    absent = keys | (np.uint64(1) << np.uint64(62))
    np.testing.assert_array_equal(bf.rank(absent), bm.rank(absent))
    if dg == 1:
        rk = bm.ref_keys()
        np.testing.assert_array_equal(bf.ref_keys(), rk)
        np.testing.assert_array_equal(bf.lookup(rk), np.arange(1, bm.dim + 1))
    # H*psi through each basis' tables: the same sums
    x = np.random.default_rng(nx * 10 + ny).standard_normal((bm.dim, 2))
    ys = []
    for b in (bf, bm):
        H = lgt.build_hamiltonian(b, g=[0.9, 1.4], t=1.0, m=0.5)
        ys.append(H.matvec(x))
        H.close()
    np.testing.assert_array_equal(ys[0], ys[1])
    bf.close()
    bm.close()


def test_fused_basis_against_oracle(oracle, lgt, monkeypatch):
    """The one-launch build of the headline sector (4x2, staggered) against
    the oracle's basis, keys and lookups."""
    monkeypatch.setenv("LGT_BASIS_FUSED", "1")
    g = oracle.staggered_charges(4, 2)
    ob = oracle.build_basis(4, 2, 1, g)
    gb, kd = lgt.build_basis(4, 2, 1, g)
    np.testing.assert_array_equal(gb.order_keys(), ob.order_keys)
    np.testing.assert_array_equal(gb.ref_keys(), ob.ref_keys)
    np.testing.assert_array_equal(gb.lookup(ob.ref_keys), np.arange(1, ob.dim + 1))
    assert kd[int(ob.ref_keys[7])] == 8


def test_bases_reuse_streams(lgt):
    """Bases created and dropped in a loop (their streams reused) keep
    giving the same basis."""
    g = lgt.staggered_charges(3, 3)
    ref = None
    for _ in range(40):
        b, _ = lgt.build_basis(3, 3, 1, g)
        k = b.order_keys()
        if ref is None:
            ref = k
        np.testing.assert_array_equal(k, ref)
        b.close()
