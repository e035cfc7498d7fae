"""CPU oracle for the exact-diagonalisation path of NoaFeldman/LGT.

TEST INFRASTRUCTURE ONLY.  This module is the checker the CUDA library is
compared with.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may import it; the product package
``lgt_gb300`` never does.

What it restates (reference file:line):

* ``build_basis``        finite_ed.jl:125-232 (C, ``lgt_oracle.c``), and a
  literal pure-Python copy of the same recursion for tiny lattices
  (``py_build_basis``) that cross-checks the C restatement;
* ``build_hamiltonian``  finite_ed.jl:252-322 (model "ref") and the
  plaquette + Jordan-Wigner term list matter_gauge_entanglement_pjw.jl:82-147
  on the column snake decoupling_U_soe.jl:41-54 (model "pjw");
* ``ground_state``       finite_ed.jl:333-341 (KrylovKit ``eigsolve``): dense
  ``eigh`` for small sectors, ARPACK ``eigsh`` otherwise;
* ``measure``            finite_ed.jl:369-393, plus the plaquette and
  staggered-density observables;
* ``evolve``             finite_ed.jl:405-431 (KrylovKit ``exponentiate``):
  exact propagation by eigendecomposition for small sectors,
  ``expm_multiply`` otherwise;
* sectors                mps_lgt.jl:472 (staggered), finite_ed.jl:504-511
  (string-breaking), and their product states mps_lgt.jl:614-622,
  finite_ed.jl:524-532.

Parity: the integer layer is pinned by the sector dimensions / nonzero
counts of the reference sectors and by the full-tensor-product construction
in ``oracle/fullspace.py``.  The Krylov layer is "parity unpinned" (Julia and
KrylovKit 0.10.2 are not available; no reference test stores eigenpairs).
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

MODEL_REF = 0
MODEL_PJW = 1
_MODELS = {"ref": MODEL_REF, "pjw": MODEL_PJW, MODEL_REF: MODEL_REF, MODEL_PJW: MODEL_PJW}

_lib = None


def lib():
    """Load (building if needed) the C restatement."""
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, i32, i64, u64, dbl = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64,
                                  ctypes.c_uint64, ctypes.c_double)
        L.orc_basis_new.restype = vp
        L.orc_basis_new.argtypes = [i32, i32, i32, vp]
        L.orc_basis_dim.restype = i64
        L.orc_basis_dim.argtypes = [vp]
        L.orc_basis_copy.restype = None
        L.orc_basis_copy.argtypes = [vp, vp, vp, vp, vp, vp]
        L.orc_basis_lookup.restype = i64
        L.orc_basis_lookup.argtypes = [vp, u64]
        L.orc_basis_free.restype = None
        L.orc_basis_free.argtypes = [vp]
        L.orc_ham_new.restype = vp
        L.orc_ham_new.argtypes = [vp, i32, dbl, dbl, dbl]
        L.orc_ham_rows.restype = vp
        L.orc_ham_rows.argtypes = [vp, i32, dbl, dbl, dbl, vp, i64]
        L.orc_ham_ntriplets.restype = i64
        L.orc_ham_ntriplets.argtypes = [vp]
        L.orc_ham_copy.restype = None
        L.orc_ham_copy.argtypes = [vp, vp, vp, vp]
        L.orc_ham_free.restype = None
        L.orc_ham_free.argtypes = [vp]
        L.orc_measure.restype = None
        L.orc_measure.argtypes = [vp, vp, vp, vp]
        L.orc_plaquette.restype = None
        L.orc_plaquette.argtypes = [vp, vp, vp, vp]
        L.orc_encode.restype = i64
        L.orc_encode.argtypes = [i32, i32, vp, vp, vp]
        L.orc_digit_bits.restype = i32
        L.orc_digit_bits.argtypes = [i32]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


# --------------------------------------------------------------------------
# Sectors and product states
# --------------------------------------------------------------------------

def staggered_charges(nx: int, ny: int) -> np.ndarray:
    """g = -1 on sites with odd ix+iy (1-based), else 0 (mps_lgt.jl:472,
    finite_ed.jl:567-571).  Indexed [ix-1, iy-1]."""
    g = np.zeros((nx, ny), dtype=np.int32)
    for ix in range(1, nx + 1):
        for iy in range(1, ny + 1):
            if (ix + iy) % 2 == 1:
                g[ix - 1, iy - 1] = -1
    return g


def string_charges(nx: int, ny: int) -> np.ndarray:
    """Quench-A sector: g(1,iy_str)=+1, g(2,iy_str)=-2, iy_str=div(ny,2)
    (finite_ed.jl:504-511)."""
    g = np.zeros((nx, ny), dtype=np.int32)
    iy = ny // 2
    g[0, iy - 1] = 1
    g[1, iy - 1] = -2
    return g


# --------------------------------------------------------------------------
# Basis
# --------------------------------------------------------------------------

@dataclass
class OracleBasis:
    nx: int
    ny: int
    dg: int
    g_charges: np.ndarray
    order_keys: np.ndarray  # uint64 [n]
    ref_keys: np.ndarray    # int64 [n] (_encode, dg == 1 only)
    nf: np.ndarray          # int8 [n, nx, ny]
    eR: np.ndarray          # int8 [n, nx-1, ny]
    eU: np.ndarray          # int8 [n, nx, ny-1]
    _h: int = 0

    @property
    def dim(self) -> int:
        return int(self.order_keys.shape[0])

    def __len__(self):
        return self.dim

    def index_of(self, nf, eR, eU) -> int:
        """key_dict lookup (0-based), -1 when absent (finite_ed.jl:527-531)."""
        L = lib()
        nf = np.asfortranarray(nf, dtype=np.int8)
        eR = np.asfortranarray(eR, dtype=np.int8)
        eU = np.asfortranarray(eU, dtype=np.int8)
        if self.dg == 1:
            k = L.orc_encode(self.nx, self.ny, _ptr(nf), _ptr(eR), _ptr(eU)) & (2**64 - 1)
        else:
            k = order_key(self.nx, self.ny, self.dg, nf, eU)
        return int(L.orc_basis_lookup(self._h, k))

    def __del__(self):
        if self._h and _lib is not None:
            _lib.orc_basis_free(self._h)
            self._h = 0


def _unflatten(a, n, nx, ny):
    """Per-state Julia column-major (nx x ny) blocks -> [n, nx, ny]."""
    if nx == 0 or ny == 0:
        return np.zeros((n, max(nx, 0), max(ny, 0)), dtype=np.int8)
    return a.reshape(n, ny, nx).transpose(0, 2, 1).copy()


def build_basis(nx: int, ny: int, dg: int, g_charges) -> OracleBasis:
    """build_basis (finite_ed.jl:125-162) through the C restatement."""
    L = lib()
    g = np.asfortranarray(np.asarray(g_charges, dtype=np.int32).reshape(nx, ny))
    h = L.orc_basis_new(nx, ny, dg, _ptr(g))
    if not h:
        raise ValueError("inconsistent sector or lattice beyond oracle limits")
    n = L.orc_basis_dim(h)
    ns, nr, nu = nx * ny, (nx - 1) * ny, nx * (ny - 1)
    ok = np.zeros(n, np.uint64)
    rk = np.zeros(n, np.int64)
    nf = np.zeros(n * ns, np.int8)
    eR = np.zeros(max(n * nr, 1), np.int8)
    eU = np.zeros(max(n * nu, 1), np.int8)
    L.orc_basis_copy(h, _ptr(ok), _ptr(rk), _ptr(nf), _ptr(eR), _ptr(eU))
    return OracleBasis(nx, ny, dg, g, ok, rk,
                       _unflatten(nf, n, nx, ny),
                       _unflatten(eR[: n * nr], n, nx - 1, ny),
                       _unflatten(eU[: n * nu], n, nx, ny - 1), h)


def digit_bits(dg: int) -> int:
    return int(lib().orc_digit_bits(dg))


def order_key(nx, ny, dg, nf, eU) -> int:
    """Order key of one configuration (see lgt_oracle.c:orc_order_key)."""
    w = digit_bits(dg)
    mask = 0
    for iy in range(ny):
        for ix in range(nx):
            mask |= int(nf[ix, iy]) << (iy * nx + ix)
    dig = 0
    for iy in range(ny - 1):
        for ix in range(nx):
            dig = (dig << w) | (int(eU[ix, iy]) + dg)
    return (mask << (w * nx * (ny - 1))) | dig


def py_build_basis(nx: int, ny: int, dg: int, g_charges, dedup: str = "encode"):
    """Literal pure-Python restatement of build_basis and its recursion
    (finite_ed.jl:125-232), for tiny lattices.  Returns the list of
    (n_f, e_R, e_U) int arrays in reference index order and the list of
    _encode keys (finite_ed.jl:80-97) as signed Int64 values.

    dedup="encode" keys the dictionary by _encode exactly as the reference
    does (finite_ed.jl:227-228); for dg > 1 its 2-bit fields collide and
    states are silently dropped.  dedup="config" keys it by the whole
    configuration, which is what the oracle and the GPU library define."""
    g = np.asarray(g_charges, dtype=np.int64).reshape(nx, ny)
    nft = -int(g.sum())
    assert 0 <= nft <= nx * ny, "Inconsistent sector"
    states, keys, key_dict = [], [], {}
    n_f = np.zeros((nx, ny), np.int64)
    e_R = np.zeros((max(nx - 1, 0), ny), np.int64)
    e_U = np.zeros((nx, max(ny - 1, 0)), np.int64)

    def encode(n_f, e_R, e_U):
        key, off = 0, 0
        for iy in range(ny):
            for ix in range(nx):
                key |= int(n_f[ix, iy]) << off
                off += 1
        for iy in range(ny):
            for ix in range(nx - 1):
                key |= int(e_R[ix, iy] + 1) << off
                off += 2
        for iy in range(ny - 1):
            for ix in range(nx):
                key |= int(e_U[ix, iy] + 1) << off
                off += 2
        key &= 2**64 - 1
        return key - 2**64 if key >= 2**63 else key

    def derive_and_check(q):
        for iy in range(ny):
            acc = 0
            for ix in range(nx):
                eu_now = int(e_U[ix, iy]) if iy < ny - 1 else 0
                eu_prev = int(e_U[ix, iy - 1]) if iy > 0 else 0
                acc += int(q[ix, iy]) - eu_now + eu_prev
                if ix < nx - 1:
                    if -dg <= acc <= dg:
                        e_R[ix, iy] = acc
                    else:
                        return
                elif acc != 0:
                    return
        k = encode(n_f, e_R, e_U)
        dk = k if dedup == "encode" else (n_f.tobytes(), e_R.tobytes(), e_U.tobytes())
        if dk not in key_dict:
            states.append((n_f.copy(), e_R.copy(), e_U.copy()))
            keys.append(k)
            key_dict[dk] = len(states) - 1

    def eU_row(q, S, iy):
        if iy == ny - 1:
            derive_and_check(q)
            return
        eU_inner(q, S, iy, 0, 0)

    def eU_inner(q, S, iy, ix, partial):
        if ix == nx - 1:
            last = S[iy] - partial
            if -dg <= last <= dg:
                e_U[nx - 1, iy] = last
                eU_row(q, S, iy + 1)
            return
        for v in range(-dg, dg + 1):
            e_U[ix, iy] = v
            eU_inner(q, S, iy, ix + 1, partial + v)

    for mask in range(2 ** (nx * ny)):
        if bin(mask).count("1") != nft:
            continue
        for iy in range(ny):
            for ix in range(nx):
                n_f[ix, iy] = (mask >> (iy * nx + ix)) & 1
        q = n_f + g
        R = [int(q[:, iy].sum()) for iy in range(ny)]
        S = list(np.cumsum(R))
        if S[ny - 1] != 0:
            continue
        eU_row(q, S, 0)
    return states, keys


# --------------------------------------------------------------------------
# Hamiltonian
# --------------------------------------------------------------------------

def build_hamiltonian(basis: OracleBasis, *, g: float, t: float, m: float, model="ref"):
    """Sparse H (scipy CSR, float64) in the basis: finite_ed.jl:252-322 for
    model "ref", matter_gauge_entanglement_pjw.jl:82-147 for model "pjw".
    The reference stores ComplexF64 with zero imaginary parts; H is real."""
    import scipy.sparse as sp
    L = lib()
    h = L.orc_ham_new(basis._h, _MODELS[model], float(g), float(t), float(m))
    if not h:
        raise RuntimeError("oracle Hamiltonian construction failed")
    try:
        n = L.orc_ham_ntriplets(h)
        I = np.zeros(n, np.int64)
        J = np.zeros(n, np.int64)
        V = np.zeros(n, np.float64)
        L.orc_ham_copy(h, _ptr(I), _ptr(J), _ptr(V))
    finally:
        L.orc_ham_free(h)
    N = basis.dim
    H = sp.coo_matrix((V, (I, J)), shape=(N, N)).tocsr()
    H.sum_duplicates()
    H.sort_indices()
    return H


def hamiltonian_rows(basis: OracleBasis, rows, *, g: float, t: float, m: float, model="ref"):
    """Rows ``rows`` (0-based) of the matrix of ``build_hamiltonian``
    without building the whole matrix (lgt_oracle.c:orc_ham_rows runs the
    reference's per-state loop body for each row's sources only).  Returns
    a scipy CSR matrix of shape (len(rows), N), duplicates summed as
    sparse() would (finite_ed.jl:321)."""
    import scipy.sparse as sp
    L = lib()
    rows = np.asarray(rows, dtype=np.int64)
    uniq, inv = np.unique(rows, return_inverse=True)
    h = L.orc_ham_rows(basis._h, _MODELS[model], float(g), float(t), float(m), _ptr(uniq),
                       int(uniq.size))
    if not h:
        raise RuntimeError("oracle row construction failed")
    try:
        n = L.orc_ham_ntriplets(h)
        I = np.zeros(n, np.int64)
        J = np.zeros(n, np.int64)
        V = np.zeros(n, np.float64)
        L.orc_ham_copy(h, _ptr(I), _ptr(J), _ptr(V))
    finally:
        L.orc_ham_free(h)
    H = sp.coo_matrix((V, (np.searchsorted(uniq, I), J)), shape=(uniq.size, basis.dim)).tocsr()
    H.sum_duplicates()
    H.sort_indices()
    return H[inv]


# --------------------------------------------------------------------------
# Ground state and time evolution
# --------------------------------------------------------------------------

def ground_state(H, *, tol: float = 1e-13, seed: int = 0, dense_max: int = 4000):
    """Lowest eigenpair (finite_ed.jl:333-341).  Dense ``eigh`` up to
    ``dense_max`` rows, ARPACK ``eigsh`` above.  The eigenvector is real and
    normalised; its sign is fixed so its largest-magnitude entry is
    positive."""
    N = H.shape[0]
    if N <= dense_max:
        w, v = np.linalg.eigh(H.toarray())
        E0, psi = float(w[0]), v[:, 0].copy()
    else:
        from scipy.sparse.linalg import eigsh
        rng = np.random.default_rng(seed)
        v0 = rng.standard_normal(N)
        w, v = eigsh(H, k=1, which="SA", tol=tol, v0=v0, ncv=min(50, N))
        E0, psi = float(w[0]), v[:, 0].copy()
    psi /= np.linalg.norm(psi)
    if psi[np.argmax(np.abs(psi))] < 0:
        psi = -psi
    return E0, psi


def spectrum_low(H, k: int = 2, dense_max: int = 4000):
    """Lowest k eigenvalues (gap diagnostics)."""
    N = H.shape[0]
    if N <= dense_max:
        return np.linalg.eigvalsh(H.toarray())[:k]
    from scipy.sparse.linalg import eigsh
    return np.sort(eigsh(H, k=k, which="SA", tol=1e-12, return_eigenvectors=False))


def evolve(psi0, H, basis: OracleBasis, *, dt: float, n_steps: int, dense_max: int = 3000):
    """evolve_ED! (finite_ed.jl:405-431): per step psi <- exp(-i H dt) psi,
    renormalise, measure.  Returns (psi_final, list of measurement dicts)."""
    psi = np.asarray(psi0, dtype=np.complex128).copy()
    data = [measure(psi, basis, 0.0)]
    N = H.shape[0]
    if N <= dense_max:
        w, V = np.linalg.eigh(H.toarray())
        ph = np.exp(-1j * dt * w)
        for step in range(1, n_steps + 1):
            psi = V @ (ph * (V.T @ psi))
            psi /= np.linalg.norm(psi)
            data.append(measure(psi, basis, step * dt))
    else:
        from scipy.sparse.linalg import expm_multiply
        A = (-1j * dt) * H.astype(np.complex128)
        for step in range(1, n_steps + 1):
            psi = expm_multiply(A, psi)
            psi /= np.linalg.norm(psi)
            data.append(measure(psi, basis, step * dt))
    return psi, data


# --------------------------------------------------------------------------
# Observables
# --------------------------------------------------------------------------

def measure(psi, basis: OracleBasis, t_now: float = 0.0) -> dict:
    """measure_ED (finite_ed.jl:369-393) plus the plaquette and staggered
    density: nf_grid, E2_grid [nx, ny]; nf_mean, nf_even, nf_odd, E2_mean;
    plaq_grid [(nx-1), (ny-1)] = <W_p + W_p^dag>, plaq_mean; n_stag =
    (1/N_s) sum (-1)^(ix+iy) <n_f>."""
    L = lib()
    psi = np.asarray(psi)
    prob = np.ascontiguousarray(np.abs(psi) ** 2, dtype=np.float64)
    nx, ny = basis.nx, basis.ny
    nf = np.zeros(nx * ny)
    e2 = np.zeros(nx * ny)
    L.orc_measure(basis._h, _ptr(prob), _ptr(nf), _ptr(e2))
    re = np.ascontiguousarray(psi.real, dtype=np.float64)
    im = np.ascontiguousarray(psi.imag, dtype=np.float64) if np.iscomplexobj(psi) else None
    npl = max((nx - 1) * (ny - 1), 0)
    pl = np.zeros(max(npl, 1))
    if npl:
        L.orc_plaquette(basis._h, _ptr(re), _ptr(im), _ptr(pl))
    nf_grid = nf.reshape(ny, nx).T
    E2_grid = e2.reshape(ny, nx).T
    even = [(ix, iy) for ix in range(1, nx + 1) for iy in range(1, ny + 1) if (ix + iy) % 2 == 0]
    odd = [(ix, iy) for ix in range(1, nx + 1) for iy in range(1, ny + 1) if (ix + iy) % 2 == 1]
    nf_even = float(np.mean([nf_grid[ix - 1, iy - 1] for ix, iy in even])) if even else float("nan")
    nf_odd = float(np.mean([nf_grid[ix - 1, iy - 1] for ix, iy in odd])) if odd else float("nan")
    stag = np.array([[1.0 if (ix + iy) % 2 == 0 else -1.0 for iy in range(1, ny + 1)]
                     for ix in range(1, nx + 1)])
    plaq_grid = pl[:npl].reshape(max(ny - 1, 0), max(nx - 1, 0)).T
    return dict(t=t_now, nf_mean=float(nf_grid.mean()), nf_even=nf_even, nf_odd=nf_odd,
                E2_mean=float(E2_grid.mean()), nf_grid=nf_grid, E2_grid=E2_grid,
                plaq_grid=plaq_grid,
                plaq_mean=float(plaq_grid.mean()) if npl else 0.0,
                n_stag=float((stag * nf_grid).mean()))


def staggered_product_index(basis: OracleBasis) -> int:
    """Index of the strong-coupling product state: n_f = 1 on odd ix+iy,
    all E = 0 (mps_lgt.jl:614-622)."""
    nx, ny = basis.nx, basis.ny
    nf = np.zeros((nx, ny), np.int8)
    for ix in range(1, nx + 1):
        for iy in range(1, ny + 1):
            if (ix + iy) % 2 == 1:
                nf[ix - 1, iy - 1] = 1
    return basis.index_of(nf, np.zeros((nx - 1, ny), np.int8), np.zeros((nx, ny - 1), np.int8))


def string_state_index(basis: OracleBasis) -> int:
    """Index of the quench-A initial state: n_f(2,iy_str) = 1,
    e_R(1,iy_str) = +1, all else 0 (finite_ed.jl:519-532)."""
    nx, ny = basis.nx, basis.ny
    iy = ny // 2
    nf = np.zeros((nx, ny), np.int8)
    nf[1, iy - 1] = 1
    eR = np.zeros((nx - 1, ny), np.int8)
    eR[0, iy - 1] = 1
    return basis.index_of(nf, eR, np.zeros((nx, ny - 1), np.int8))
