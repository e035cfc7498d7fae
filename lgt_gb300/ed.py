"""Exact diagonalisation of the U(1) lattice gauge theory on a GB300.

Host-side mirror of the ED entry points of NoaFeldman/LGT ``finite_ed.jl``
(same names, argument meaning and error behaviour), running on the CUDA
library ``liblgted.so`` through its C ABI (``include/lgt_ed.h``):

===========================  =============================================
reference (finite_ed.jl)     here
===========================  =============================================
build_basis      :125-162    :func:`build_basis` -> (states, key_dict)
_encode          :80-97      :func:`encode`
build_hamiltonian :252-322   :func:`build_hamiltonian` (matrix-free)
find_ground_state :333-341   :func:`find_ground_state`
ite_ground_state_ED :349-358 :func:`ite_ground_state_ED`
measure_ED       :369-393    :func:`measure_ED`
evolve_ED!       :405-431    :func:`evolve_ED`
===========================  =============================================

Beyond the reference, every Hamiltonian may carry K coupling points that
share one basis (pass arrays for g, t, m); the solvers then return K results
at once.  ``model="pjw"`` selects the plaquette + Jordan-Wigner Hamiltonian
of matter_gauge_entanglement_pjw.jl:82-147.  Arrays that mirror Julia
matrices are indexed [ix-1, iy-1].
"""
from __future__ import annotations

import ctypes
import weakref
from collections.abc import Mapping

import numpy as np

from . import _capi as C

_MODELS = {"ref": C.LGT_MODEL_REF, "jw": C.LGT_MODEL_JW, "plaq": C.LGT_MODEL_PLAQ,
           "pjw": C.LGT_MODEL_PJW}
_PREC = {"fp64": C.LGT_FP64, "fp32": C.LGT_FP32, "fp32_mixed": C.LGT_FP32_MIXED,
         "mixed": C.LGT_FP32_MIXED}
# lgt_tuning.hpsi_kernel codes (include/lgt_ed.h)
HPSI_KERNELS = {0: "rule", 1: "generic", 2: "fixed_vpl1", 3: "fixed_vpl2", 4: "fixed_wide",
                5: "table_vpl1", 6: "table_vpl2", 7: "table_wide", 8: "table_gather"}


def _p(a):
    """Data address of a host array for a ``c_void_p`` argument (the caller
    holds the array across the call)."""
    return a.ctypes.data if a is not None else None


# ---------------------------------------------------------------------------
# sectors
# ---------------------------------------------------------------------------

def staggered_charges(nx: int, ny: int) -> np.ndarray:
    """Staggered sector g = -1 on odd ix+iy, else 0 (mps_lgt.jl:472,
    finite_ed.jl:567-571)."""
    g = np.zeros((nx, ny), dtype=np.int32)
    for ix in range(1, nx + 1):
        for iy in range(1, ny + 1):
            if (ix + iy) % 2 == 1:
                g[ix - 1, iy - 1] = -1
    return g


def string_charges(nx: int, ny: int, iy_str: int | None = None) -> np.ndarray:
    """String-breaking sector g(1,iy_str) = +1, g(2,iy_str) = -2
    (finite_ed.jl:504-511, mps_lgt.jl:640-642)."""
    iy = ny // 2 if iy_str is None else iy_str
    g = np.zeros((nx, ny), dtype=np.int32)
    g[0, iy - 1] = 1
    g[1, iy - 1] = -2
    return g


def encode(n_f, e_R, e_U) -> int:
    """The reference's packed Int64 key ``_encode`` (finite_ed.jl:80-97):
    n_f bits (iy outer, ix inner), then 2-bit (e+1) fields of e_R and of
    e_U.  Returned as a signed 64-bit value (bit 63 may be set at 4x4)."""
    n_f = np.asarray(n_f)
    nx, ny = n_f.shape
    key, off = 0, 0
    for iy in range(ny):
        for ix in range(nx):
            key |= int(n_f[ix, iy]) << off
            off += 1
    e_R = np.asarray(e_R).reshape(nx - 1, ny) if nx > 1 else np.zeros((0, ny))
    for iy in range(ny):
        for ix in range(nx - 1):
            key |= int(e_R[ix, iy] + 1) << off
            off += 2
    e_U = np.asarray(e_U).reshape(nx, ny - 1) if ny > 1 else np.zeros((nx, 0))
    for iy in range(ny - 1):
        for ix in range(nx):
            key |= int(e_U[ix, iy] + 1) << off
            off += 2
    key &= (1 << 64) - 1
    return key - (1 << 64) if key >= (1 << 63) else key


# ---------------------------------------------------------------------------
# basis
# ---------------------------------------------------------------------------

class Basis:
    """GPU-resident Gauss-law basis, the ``states`` of build_basis.

    ``len(states)`` is the sector dimension; ``states[i]`` (0-based) gives the
    dict ``{"n_f", "e_R", "e_U"}`` of reference state i+1.  The basis itself
    lives on the device as sorted order keys."""

    def __init__(self, nx: int, ny: int, dg: int, g_charges, device: int = -1):
        L = C.load()
        self.nx, self.ny, self.dg = int(nx), int(ny), int(dg)
        g = np.asarray(g_charges, dtype=np.int32).reshape(nx, ny)
        self.g_charges = g.copy()
        gf = np.asfortranarray(g)
        h = ctypes.c_void_p()
        C.check(L.lgt_basis_create(nx, ny, dg, _p(gf), device, ctypes.byref(h)))
        self._h = h
        d = ctypes.c_int64()
        C.check(L.lgt_basis_dim(self._h, ctypes.byref(d)))
        self.dim = int(d.value)
        self._observers = {}
        self._hams = weakref.WeakSet()  # Hamiltonians made from this basis

    @property
    def handle(self):
        return self._h

    def __len__(self):
        return self.dim

    def close(self):
        for o in self._observers.values():
            o.close()
        self._observers = {}
        if getattr(self, "_h", None) and self._h.value:
            C.load().lgt_basis_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def order_keys(self, first: int = 0, count: int | None = None) -> np.ndarray:
        count = self.dim - first if count is None else count
        out = np.zeros(count, np.uint64)
        C.check(C.load().lgt_basis_keys(self._h, first, count, _p(out), None))
        return out

    def ref_keys(self, first: int = 0, count: int | None = None) -> np.ndarray:
        """_encode keys of the states (dg == 1), as Int64."""
        count = self.dim - first if count is None else count
        out = np.zeros(count, np.int64)
        C.check(C.load().lgt_basis_keys(self._h, first, count, None, _p(out)))
        return out

    def states(self, first: int = 0, count: int | None = None):
        """(n_f [n,nx,ny], e_R [n,nx-1,ny], e_U [n,nx,ny-1]) as int8."""
        count = self.dim - first if count is None else count
        nx, ny = self.nx, self.ny
        nf = np.zeros(count * nx * ny, np.int8)
        eR = np.zeros(max(count * (nx - 1) * ny, 1), np.int8)
        eU = np.zeros(max(count * nx * (ny - 1), 1), np.int8)
        C.check(C.load().lgt_basis_states(self._h, first, count, _p(nf), _p(eR), _p(eU)))

        def unflat(a, n, a1, a2):
            return a[: n * a1 * a2].reshape(n, a2, a1).transpose(0, 2, 1)
        return unflat(nf, count, nx, ny), unflat(eR, count, nx - 1, ny), unflat(eU, count, nx, ny - 1)

    def __getitem__(self, i):
        if i < 0:
            i += self.dim
        if not 0 <= i < self.dim:
            raise IndexError(i)
        nf, eR, eU = self.states(i, 1)
        return {"n_f": nf[0], "e_R": eR[0], "e_U": eU[0]}

    def lookup(self, ref_keys) -> np.ndarray:
        """key_dict values (1-based) of _encode keys, 0 where absent."""
        k = np.ascontiguousarray(np.asarray(ref_keys, dtype=np.int64).ravel())
        out = np.zeros(k.size, np.int64)
        C.check(C.load().lgt_basis_lookup(self._h, _p(k), k.size, _p(out)))
        return out

    def rank(self, order_keys) -> np.ndarray:
        """0-based indices of order keys, -1 where absent."""
        k = np.ascontiguousarray(np.asarray(order_keys, dtype=np.uint64).ravel())
        out = np.zeros(k.size, np.int64)
        C.check(C.load().lgt_basis_rank(self._h, _p(k), k.size, _p(out)))
        return out

    def index_of(self, n_f, e_R, e_U) -> int:
        """1-based index of a configuration, 0 when it is not in the basis."""
        return int(self.lookup([encode(n_f, e_R, e_U)])[0])

    def observer(self, K: int) -> "Hamiltonian":
        """A K-point operator on this basis used for measurements: any open
        Hamiltonian of K points made from it (the observables depend on the
        basis alone), else one of its own."""
        if K not in self._observers:
            for h in list(self._hams):
                if h.K == K and h.is_open():
                    return h
            one = np.ones(K)
            self._observers[K] = Hamiltonian(self, g=one, t=one, m=one, model="pjw")
        return self._observers[K]


class KeyDict(Mapping):
    """The ``key_dict`` of build_basis: _encode key -> 1-based index."""

    def __init__(self, basis: Basis):
        self.basis = basis

    def __getitem__(self, key):
        v = int(self.basis.lookup([key])[0])
        if v == 0:
            raise KeyError(key)
        return v

    def __contains__(self, key):
        return int(self.basis.lookup([key])[0]) != 0

    def __len__(self):
        return self.basis.dim

    def __iter__(self):
        return iter(int(k) for k in self.basis.ref_keys())


def build_basis(nx: int, ny: int, dg: int, g_charges, device: int = -1):
    """build_basis (finite_ed.jl:125-162): enumerate the Gauss-law sector of
    background charges ``g_charges`` [nx, ny] on the GPU.  Returns
    ``(states, key_dict)``.  An inconsistent sector raises ValueError, as the
    reference's @assert does (finite_ed.jl:127)."""
    b = Basis(nx, ny, dg, g_charges, device)
    return b, KeyDict(b)


# ---------------------------------------------------------------------------
# Hamiltonian
# ---------------------------------------------------------------------------

def _as_points(g, t, m):
    """(K, g[K], t[K], m[K]) as contiguous float64 arrays: each coupling is a
    scalar (or one value), repeated, or an array of the K points."""
    arrs = [np.atleast_1d(np.asarray(a, dtype=np.float64)) for a in (g, t, m)]
    K = max(a.size for a in arrs)
    out = []
    for a in arrs:
        if a.ndim == 1 and a.size == K:
            out.append(np.ascontiguousarray(a))
        elif a.size == 1:
            out.append(np.full(K, a.flat[0]))
        else:
            raise ValueError("couplings of %d and %d points cannot be combined" % (a.size, K))
    return (K, *out)


class Hamiltonian:
    """Matrix-free H on a basis for K coupling points (build_hamiltonian,
    finite_ed.jl:252-322; nothing of size nnz is stored)."""

    def __init__(self, basis: Basis, *, g, t, m, model="ref"):
        L = C.load()
        self.basis = basis
        self.K, self.g, self.t, self.m = _as_points(g, t, m)
        self.model = _MODELS[model] if isinstance(model, str) else int(model)
        h = ctypes.c_void_p()
        C.check(L.lgt_ham_create(basis.handle, self.K, _p(self.g), _p(self.t), _p(self.m),
                                 self.model, ctypes.byref(h)))
        basis._hams.add(self)
        self._h = h

    @property
    def handle(self):
        return self._h

    @property
    def shape(self):
        return (self.basis.dim, self.basis.dim)

    def is_open(self) -> bool:
        return bool(getattr(self, "_h", None) and self._h.value)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            C.load().lgt_ham_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_couplings(self, *, g=None, t=None, m=None):
        g = self.g if g is None else g
        t = self.t if t is None else t
        m = self.m if m is None else m
        K, g, t, m = _as_points(g, t, m)
        if K != self.K:
            raise ValueError("number of coupling points is fixed at %d" % self.K)
        C.check(C.load().lgt_ham_set_couplings(self._h, _p(g), _p(t), _p(m)))
        self.g, self.t, self.m = g, t, m

    def nnz(self) -> int:
        """nnz(H) as the reference counts it (finite_ed.jl:355)."""
        n = ctypes.c_int64()
        C.check(C.load().lgt_ham_nnz(self._h, ctypes.byref(n)))
        return int(n.value)

    def export_csr(self, k: int = 0):
        """(rowptr int64 [N+1], colidx int32 [nnz], values float64 [nnz]) of
        point k; equal to the colptr/rowval/nzval of the reference's CSC."""
        N = self.basis.dim
        nnz = self.nnz()
        rp = np.zeros(N + 1, np.int64)
        ci = np.zeros(max(nnz, 1), np.int32)
        va = np.zeros(max(nnz, 1), np.float64)
        C.check(C.load().lgt_ham_export_csr(self._h, k, _p(rp), _p(ci), _p(va)))
        return rp, ci[:nnz], va[:nnz]

    def to_scipy(self, k: int = 0):
        import scipy.sparse as sp
        rp, ci, va = self.export_csr(k)
        N = self.basis.dim
        return sp.csr_matrix((va, ci, rp), shape=(N, N))

    def _panel(self, x, dtype):
        """Host array (N,), (N,K) real or complex -> interleaved panel."""
        x = np.asarray(x)
        N, K = self.basis.dim, self.K
        cplx = np.iscomplexobj(x)
        if x.ndim == 1:
            x = x.reshape(N, 1)
        if x.shape != (N, K):
            raise ValueError("expected shape (%d,) or (%d, %d)" % (N, N, K))
        if cplx:
            p = np.empty((N, K, 2), dtype=dtype)
            p[..., 0] = x.real
            p[..., 1] = x.imag
            return np.ascontiguousarray(p), 2
        return np.ascontiguousarray(x, dtype=dtype), 1

    def matvec(self, x, precision="fp64", generic=False):
        """y = H x for host arrays: x of shape (N,) (K = 1) or (N, K), real or
        complex; precision "fp64" or "fp32".  ``generic`` forces the
        run-time-geometry kernel where a fixed-shape one exists."""
        prec = _PREC[precision]
        dtype = np.float64 if prec == C.LGT_FP64 else np.float32
        xin = np.asarray(x)
        px, nc = self._panel(xin, dtype)
        py = np.empty_like(px)
        flags = C.LGT_GENERIC_KERNELS if generic else 0
        C.check(C.load().lgt_matvec(self._h, _p(px), _p(py), nc, prec, flags))
        if nc == 2:
            y = py[..., 0] + 1j * py[..., 1]
        else:
            y = py
        return y.reshape(xin.shape)

    def row_order(self) -> np.ndarray:
        """The locality row order of the stored-table product (rows in
        breadth-first order of the hop graph): perm[n] is the basis index of
        row n of that order.  The Krylov drivers keep their vectors in it."""
        perm = np.zeros(self.basis.dim, np.int32)
        C.check(C.load().lgt_ham_row_order(self._h, _p(perm)))
        return perm

    def matvec_device(self, x_ptr: int, y_ptr: int, ncomp: int = 1, precision="fp64",
                      generic=False, row_order=False):
        """y = H x on device panels [N][K][ncomp] (raw device pointers);
        row_order: the panels are in the order of row_order()."""
        flags = C.LGT_DEVICE_PTRS | (C.LGT_GENERIC_KERNELS if generic else 0)
        if row_order:
            flags |= C.LGT_ROW_ORDER
        C.check(C.load().lgt_matvec(self._h, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr),
                                    ncomp, _PREC[precision], flags))

    def autotune(self, ncomp: int = 1, precision="fp64") -> dict:
        """Autotuner choice for this operator's Krylov panels (ncomp 1:
        ground states, 2: exponential steps); tunes on first use."""
        t = C.Tuning()
        C.check(C.load().lgt_autotune(self._h, int(ncomp), _PREC[precision], ctypes.byref(t)))
        return {"hpsi_kernel": HPSI_KERNELS.get(t.hpsi_kernel, str(t.hpsi_kernel)),
                "reduce_blocks": t.reduce_blocks, "hpsi_ms": t.hpsi_ms,
                "reduce_ms": t.reduce_ms, "measured": bool(t.measured)}

    def energy(self, psi) -> np.ndarray:
        """<psi|H|psi> / <psi|psi> per point, FP64."""
        px, nc = self._panel(np.asarray(psi), np.float64)
        e = np.zeros(self.K)
        C.check(C.load().lgt_energy(self._h, _p(px), nc, 0, _p(e)))
        return e


def build_hamiltonian(states: Basis, key_dict=None, nx=None, ny=None, dg=None, *, g, t, m,
                      model="ref") -> Hamiltonian:
    """build_hamiltonian (finite_ed.jl:252-322).  ``g``, ``t``, ``m`` may be
    arrays of K coupling points.  ``model``: "ref" (finite_ed.jl) or "pjw"
    (plaquette + Jordan-Wigner, matter_gauge_entanglement_pjw.jl:82-147)."""
    b = states
    for name, v, w in (("nx", nx, b.nx), ("ny", ny, b.ny), ("dg", dg, b.dg)):
        if v is not None and int(v) != w:
            raise ValueError("%s=%s does not match the basis (%s)" % (name, v, w))
    return Hamiltonian(b, g=g, t=t, m=m, model=model)


# ---------------------------------------------------------------------------
# solvers and observables
# ---------------------------------------------------------------------------

_SOLVERS = {"auto": C.LGT_SOLVER_AUTO, "panel": C.LGT_SOLVER_PANEL, "cta": C.LGT_SOLVER_CTA}


def _opts(for_exp, tol, krylovdim, maxiter, precision, seed, check_every, refine_steps,
          use_graph=True, start_given=False, reorth_passes=2, solver="auto"):
    o = C.defaults(for_exp)
    o.solver = _SOLVERS[solver]
    if tol is not None:
        o.tol = tol
    if krylovdim is not None:
        o.krylovdim = krylovdim
    if maxiter is not None:
        o.maxiter = maxiter
    o.precision = _PREC[precision]
    o.seed = seed
    if check_every is not None:
        o.check_every = check_every
    o.refine_steps = refine_steps
    o.use_graph = 1 if use_graph else 0
    o.start_given = 1 if start_given else 0
    o.reorth_passes = reorth_passes
    return o


def find_ground_state(H: Hamiltonian, *, tol=1e-10, krylovdim=50, maxiter=300, precision="fp64",
                      seed=0, v0=None, check_every=None, refine_steps=0, use_graph=True,
                      solver="auto", as_complex=True, return_info=False):
    """find_ground_state (finite_ed.jl:333-341): lowest eigenpair by Lanczos
    (full reorthogonalisation, restarts), on the GPU.  Defaults are the
    reference's eigsolve settings.  For K = 1 returns (E0: float, psi: [N]);
    for K > 1 (E0: [K], psi: [N, K]).  psi is complex128 (zero imaginary
    part, like the reference's ComplexF64 vector) unless as_complex=False.
    precision "fp32_mixed": FP32 H*psi and Krylov storage, FP64 dots,
    reorthogonalisation and tridiagonal solve; E0 is the FP64 Rayleigh
    quotient.  solver: "auto" (one CTA per point for sectors up to 8192
    states, else K-interleaved panels), "cta" or "panel".  Raises
    NotConverged like the reference's @assert (:339)."""
    N, K = H.basis.dim, H.K
    o = _opts(False, tol, krylovdim, maxiter, precision, seed, check_every, refine_steps,
              use_graph, v0 is not None, solver=solver)
    psi = np.empty((N, K), np.float64)  # written whole by the solver
    if v0 is not None:
        v = np.asarray(v0)
        psi[:] = np.real(v).reshape(N, K) if v.ndim == 1 else np.real(v)
    E0 = np.zeros(K)
    res = np.zeros(K)
    info = C.Info()
    C.check(C.load().lgt_ground_state(H.handle, ctypes.byref(o), _p(E0), _p(psi), _p(res), 0,
                                      ctypes.byref(info)))
    out_psi = psi.astype(np.complex128) if as_complex else psi
    if K == 1:
        E, P = float(E0[0]), out_psi[:, 0]
    else:
        E, P = E0, out_psi
    if return_info:
        return E, P, {"residual": res if K > 1 else float(res[0]), "matvecs": info.matvecs,
                      "restarts": info.restarts, "converged": info.converged,
                      "max_residual": info.max_residual, "seconds": info.seconds}
    return E, P


def find_ground_state_measured(H: Hamiltonian, *, tol=1e-10, krylovdim=50, maxiter=300,
                               precision="fp64", seed=0, check_every=None, refine_steps=0,
                               use_graph=True, solver="auto", as_complex=True):
    """find_ground_state then measure_ED of its state, the pair
    gs_benchmark.jl:116-125 runs per point, in one call
    (lgt_ground_state_observe: the observables are taken from the device
    copy of the state before the solve's one synchronisation).  Returns
    (E0, psi, obs), E0 and psi as find_ground_state returns them and obs as
    measure_ED(psi, ...) does: one dict for K = 1, else a list of K."""
    b = H.basis
    N, K = b.dim, H.K
    o = _opts(False, tol, krylovdim, maxiter, precision, seed, check_every, refine_steps,
              use_graph, False, solver=solver)
    psi = np.empty((N, K), np.float64)  # written whole by the solver
    E0 = np.zeros(K)
    info = C.Info()
    ns, npl = b.nx * b.ny, max((b.nx - 1) * (b.ny - 1), 0)
    nf = np.zeros(K * ns)
    e2 = np.zeros(K * ns)
    pl = np.zeros(max(K * npl, 1))
    summ = (C.Obs * K)()
    C.check(C.load().lgt_ground_state_observe(H.handle, ctypes.byref(o), _p(E0), _p(psi), None,
                                              0, ctypes.byref(info), _p(nf), _p(e2), _p(pl),
                                              summ))
    obs = _obs_dicts(b, K, nf, e2, pl, summ)
    out_psi = psi.astype(np.complex128) if as_complex else psi
    if K == 1:
        return float(E0[0]), out_psi[:, 0], obs[0]
    return E0, out_psi, obs


def find_ground_states(Hs, *, tol=1e-10, krylovdim=50, maxiter=300, precision="fp64", seed=0,
                       check_every=None, solver="auto", device_psi=None, return_info=False):
    """Ground states of several Hamiltonians (lattices, sectors, coupling
    grids) in one call: every (H, point) pair of a sector up to 8192 states
    runs in one persistent launch, one CTA each (uneven batch), larger
    sectors through the panel solver.  Returns a list of (E0 [K], psi
    [N, K]) per Hamiltonian (psi as float64 host arrays, or None when
    ``device_psi`` gives device panels: a list of device pointers)."""
    import torch  # device panels for the batch
    n = len(Hs)
    o = _opts(False, tol, krylovdim, maxiter, precision, seed, check_every, 0, True, False,
              solver=solver)
    E0s = [np.zeros(H.K) for H in Hs]
    res = [np.zeros(H.K) for H in Hs]
    if device_psi is None:
        panels = [torch.zeros((H.basis.dim, H.K), dtype=torch.float64,
                              device="cuda:%d" % _device_of(H)) for H in Hs]
        ptrs = [p.data_ptr() for p in panels]
    else:
        panels, ptrs = None, list(device_psi)
    arr_h = (ctypes.c_void_p * n)(*[H.handle.value for H in Hs])
    arr_e = (ctypes.c_void_p * n)(*[e.ctypes.data for e in E0s])
    arr_p = (ctypes.c_void_p * n)(*ptrs)
    arr_r = (ctypes.c_void_p * n)(*[r.ctypes.data for r in res])
    info = C.Info()
    C.check(C.load().lgt_ground_state_batch(n, arr_h, ctypes.byref(o), arr_e, arr_p, arr_r,
                                            C.LGT_DEVICE_PTRS, ctypes.byref(info)))
    out = [(E0s[i], panels[i].cpu().numpy() if panels is not None else None) for i in range(n)]
    if return_info:
        return out, {"residual": res, "matvecs": info.matvecs, "restarts": info.restarts,
                     "converged": info.converged, "max_residual": info.max_residual,
                     "seconds": info.seconds}
    return out


def _device_of(H):
    import torch
    return torch.cuda.current_device()


def ite_ground_state_ED(states, key_dict, nx, ny, dg, *, g, t, m, model="ref", **kw):
    """ite_ground_state_ED (finite_ed.jl:349-358): build H at (g, t, m) and
    return its ground state (E0, psi0)."""
    H = build_hamiltonian(states, key_dict, nx, ny, dg, g=g, t=t, m=m, model=model)
    try:
        return find_ground_state(H, **kw)
    finally:
        H.close()


_OBS_FIELDS = ("t", "nf_mean", "nf_even", "nf_odd", "E2_mean", "plaq_mean", "n_stag", "norm2")


def _obs_dicts(basis, K, nf, e2, pl, summ):
    """All K measurement dicts at once: grids as [nx, ny] views of one
    transposed array per observable (taken by iterating it), summaries
    through a numpy view of the lgt_obs array (no per-field ctypes access),
    each dict built as one display with the fields of lgt_obs in order."""
    nx, ny = basis.nx, basis.ny
    nf_g = list(nf.reshape(K, ny, nx).transpose(0, 2, 1).copy())
    e2_g = list(e2.reshape(K, ny, nx).transpose(0, 2, 1).copy())
    pnx, pny = max(nx - 1, 0), max(ny - 1, 0)
    pl_g = list(pl[:K * pnx * pny].reshape(K, pny, pnx).transpose(0, 2, 1).copy())
    sm = np.frombuffer(summ, dtype=np.float64).reshape(K, len(_OBS_FIELDS)).tolist()
    return [{"t": t, "nf_mean": n0, "nf_even": n1, "nf_odd": n2, "E2_mean": e, "plaq_mean": w,
             "n_stag": ns, "norm2": nn, "nf_grid": a, "E2_grid": b, "plaq_grid": c}
            for (t, n0, n1, n2, e, w, ns, nn), a, b, c in zip(sm, nf_g, e2_g, pl_g)]


def measure_ED(psi, states: Basis, nx=None, ny=None, dg=None, t_now: float = 0.0):
    """measure_ED (finite_ed.jl:369-393) on the GPU: site grids <n_f> and
    <E^2>, their means and sublattice means, plus the plaquette grid
    <W + W^dag>, its mean and the staggered density.  psi of shape (N,)
    gives one dict; (N, K) gives a list of K dicts."""
    b = states
    psi = np.asarray(psi)
    K = 1 if psi.ndim == 1 else psi.shape[1]
    obs = b.observer(K)
    px, nc = obs._panel(psi, np.float64)
    ns, npl = b.nx * b.ny, max((b.nx - 1) * (b.ny - 1), 0)
    nf = np.zeros(K * ns)
    e2 = np.zeros(K * ns)
    pl = np.zeros(max(K * npl, 1))
    summ = (C.Obs * K)()
    C.check(C.load().lgt_observe(obs.handle, _p(px), nc, C.LGT_FP64, 0, float(t_now), _p(nf),
                                 _p(e2), _p(pl), summ))
    out = _obs_dicts(b, K, nf, e2, pl, summ)
    return out[0] if psi.ndim == 1 else out


def evolve_ED(psi, H: Hamiltonian, states=None, nx=None, ny=None, dg=None, *, dt: float,
              n_steps: int, measure_every: int = 10, tol=1e-10, krylovdim=30, maxiter=100,
              precision="fp64", check_every=None, use_graph=True, return_state=False):
    """evolve_ED! (finite_ed.jl:405-431): n_steps Krylov steps
    psi <- exp(-i H dt) psi, renormalised after each, observables measured at
    every step (the reference measures every step and prints every
    ``measure_every``).  Returns the list of measurement dicts (t = step*dt,
    starting with t = 0), each with the site grids nf_grid and E2_grid
    (and plaq_grid) like measure_ED's; with return_state=True also the final state and
    the per-point norm drift.  As in the reference, the caller's psi is not
    modified.  For K > 1, psi is (N, K) and each entry of the list is a list
    of K dicts."""
    b = H.basis
    N, K = b.dim, H.K
    psi = np.asarray(psi)
    p = np.zeros((N, K, 2), np.float64)
    v = psi.reshape(N, K) if psi.ndim == 1 else psi
    p[..., 0] = np.real(v)
    p[..., 1] = np.imag(v)
    o = _opts(True, tol, krylovdim, maxiter, precision, 0, check_every, 0, use_graph)
    R = (n_steps + 1) * K
    obs = (C.Obs * R)()
    ns, npl = b.nx * b.ny, max((b.nx - 1) * (b.ny - 1), 0)
    nf = np.zeros(R * ns)
    e2 = np.zeros(R * ns)
    pl = np.zeros(max(R * npl, 1))
    drift = np.zeros(K)
    info = C.Info()
    C.check(C.load().lgt_expm_steps_grids(H.handle, ctypes.byref(o), float(dt), int(n_steps),
                                          _p(p), obs, _p(nf), _p(e2), _p(pl), _p(drift), 0,
                                          ctypes.byref(info)))
    recs = _obs_dicts(b, R, nf, e2, pl, obs)
    data = [recs[s * K] if K == 1 else recs[s * K:(s + 1) * K] for s in range(n_steps + 1)]
    if return_state:
        out = p[..., 0] + 1j * p[..., 1]
        return data, (out[:, 0] if psi.ndim == 1 else out), drift
    return data


def staggered_product_state(states: Basis) -> np.ndarray:
    """Strong-coupling product state: n_f = 1 on odd ix+iy, all E = 0
    (mps_lgt.jl:614-622), as a complex vector."""
    b = states
    nf = np.zeros((b.nx, b.ny), np.int8)
    for ix in range(1, b.nx + 1):
        for iy in range(1, b.ny + 1):
            if (ix + iy) % 2 == 1:
                nf[ix - 1, iy - 1] = 1
    i = b.index_of(nf, np.zeros((b.nx - 1, b.ny), np.int8), np.zeros((b.nx, b.ny - 1), np.int8))
    if i == 0:
        raise KeyError("staggered product state is not in this sector")
    v = np.zeros(b.dim, np.complex128)
    v[i - 1] = 1.0
    return v


def string_state(states: Basis) -> np.ndarray:
    """Quench-A initial state n_f(2,iy_str) = 1, e_R(1,iy_str) = +1, all
    else 0 (finite_ed.jl:519-532).  Raises like the reference's @assert
    (:530) when it is not in the basis."""
    b = states
    iy = b.ny // 2
    nf = np.zeros((b.nx, b.ny), np.int8)
    nf[1, iy - 1] = 1
    eR = np.zeros((b.nx - 1, b.ny), np.int8)
    eR[0, iy - 1] = 1
    i = b.index_of(nf, eR, np.zeros((b.nx, b.ny - 1), np.int8))
    if i == 0:
        raise KeyError("Initial state not found in basis!")
    v = np.zeros(b.dim, np.complex128)
    v[i - 1] = 1.0
    return v
