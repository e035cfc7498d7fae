"""CPU test of the host side of measure_ED: the per-point dicts built from the
observables kernel's outputs (site grids indexed [ix-1, iy-1], summaries
named after the fields of lgt_obs), on synthetic outputs."""
import numpy as np

from lgt_gb300 import _capi as C
from lgt_gb300 import ed


class _Shape:
    def __init__(self, nx, ny):
        self.nx, self.ny = nx, ny


def test_obs_fields_follow_the_struct():
    assert ed._OBS_FIELDS == tuple(name for name, _ in C.Obs._fields_)


def test_obs_dicts_layout():
    rng = np.random.default_rng(3)
    for nx, ny, K in ((4, 2, 64), (3, 4, 5), (2, 2, 1), (4, 1, 3)):
        ns, npl = nx * ny, (nx - 1) * (ny - 1)
        nf, e2 = rng.random(K * ns), rng.random(K * ns)
        pl = rng.random(max(K * npl, 1))
        summ = (C.Obs * K)()
        for k in range(K):
            for name, _ in C.Obs._fields_:
                setattr(summ[k], name, float(rng.random()))
        out = ed._obs_dicts(_Shape(nx, ny), K, nf, e2, pl, summ)
        assert len(out) == K
        for k, d in enumerate(out):
            assert list(d) == list(ed._OBS_FIELDS) + ["nf_grid", "E2_grid", "plaq_grid"]
            for name in ed._OBS_FIELDS:
                assert d[name] == getattr(summ[k], name)
            assert d["nf_grid"].shape == (nx, ny) and d["E2_grid"].shape == (nx, ny)
            assert d["plaq_grid"].shape == (nx - 1, ny - 1)
            for ix in range(nx):
                for iy in range(ny):
                    assert d["nf_grid"][ix, iy] == nf[k * ns + iy * nx + ix]
                    assert d["E2_grid"][ix, iy] == e2[k * ns + iy * nx + ix]
            for ix in range(nx - 1):
                for iy in range(ny - 1):
                    assert d["plaq_grid"][ix, iy] == pl[k * npl + iy * (nx - 1) + ix]


def test_coupling_points_broadcast():
    K, g, t, m = ed._as_points([0.5, 1.0, 2.0], 1.0, np.array([0.1]))
    assert K == 3 and g.tolist() == [0.5, 1.0, 2.0]
    assert t.tolist() == [1.0] * 3 and m.tolist() == [0.1] * 3
    assert all(a.dtype == np.float64 and a.flags.c_contiguous for a in (g, t, m))
    K, g, t, m = ed._as_points(0.8, 1.0, 0.3)
    assert K == 1 and (g[0], t[0], m[0]) == (0.8, 1.0, 0.3)
    K, g, t, m = ed._as_points(np.arange(4)[::2] + 1.0, [1, 1], 0.0)  # strided input
    assert g.tolist() == [1.0, 3.0] and g.flags.c_contiguous and t.dtype == np.float64
    import pytest
    with pytest.raises(ValueError):
        ed._as_points([1.0, 2.0], [1.0, 2.0, 3.0], 0.0)
