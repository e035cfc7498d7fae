"""Full tensor-product construction of the LGT Hamiltonian (test infrastructure).

TEST INFRASTRUCTURE ONLY.  An independent second restatement of the model,
built the way the reference's MPS/MPO code builds it -- as a sum of products
of local node operators -- rather than by the sector recursion of
finite_ed.jl.  Projecting it onto the oracle's sector basis must reproduce the
oracle's sector Hamiltonian exactly; this pins the oracle's conventions
(operator matrices, kron order, Jordan-Wigner strings, plaquette orientation)
to the reference's own operator definitions:

* local operators     u1_lgt_hamiltonian.jl:111-163 (op_E, op_U_gauge,
                      op_Udag_gauge, op_c, op_cdag, op_nf, op_parity_f)
* node embedding      u1_lgt_hamiltonian.jl:605-646 (site_dims, site_idx,
                      embed_f_site / embed_R_site / embed_U_site)
* on-site term        u1_lgt_hamiltonian.jl:658-677 (H_onsite_site)
* model "ref" terms   mps_lgt.jl:83-116 (lgt_terms, "matching finite_ed.jl")
* model "pjw" terms   matter_gauge_entanglement_pjw.jl:82-147
                      (lgt_terms_plaqjw_cs) on the column snake
                      decoupling_U_soe.jl:41-54
* Gauss penalty       mps_lgt.jl:465-513 (gauss_penalty_terms), used by the
                      reference's dense self-tests selftest_mps_lgt
                      (mps_lgt.jl:680-713) and selftest_plaqjw
                      (matter_gauge_entanglement_pjw.jl:263-292).

Only for lattices whose full Hilbert space is small (2x2: 1296, 3x2/2x3:
139968 states).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

D_F = 2  # spinless fermion (u1_lgt_hamiltonian.jl:79)


def gauge_dim(dg):
    return 2 * dg + 1


def op_E(dg):
    return np.diag(np.arange(-dg, dg + 1).astype(float))


def op_U(dg):
    """U|e> = |e+1>, zero at e = dg (u1_lgt_hamiltonian.jl:124-131)."""
    gd = gauge_dim(dg)
    U = np.zeros((gd, gd))
    for e in range(-dg, dg):
        U[e + 1 + dg, e + dg] = 1.0
    return U


def op_c():
    """c|1> = |0> (u1_lgt_hamiltonian.jl:139-144)."""
    c = np.zeros((D_F, D_F))
    c[0, 1] = 1.0
    return c


def op_nf():
    n = np.zeros((D_F, D_F))
    n[1, 1] = 1.0
    return n


def op_parity():
    return np.diag([1.0, -1.0])


def site_dims(ix, iy, nx, ny, dg):
    gd = gauge_dim(dg)
    dR = gd if ix < nx else 1
    dU = gd if iy < ny else 1
    return D_F * dR * dU, dR, dU


def site_idx(nf, eR, eU, dR, dU, dg):
    """0-based local index of |nf, eR, eU> (u1_lgt_hamiltonian.jl:614-618)."""
    iR = 0 if dR == 1 else eR + dg
    iU = 0 if dU == 1 else eU + dg
    return nf * dR * dU + iR * dU + iU


def embed_f(O, dR, dU):
    return np.kron(np.kron(O, np.eye(dR)), np.eye(dU))


def embed_R(O, dU):
    return np.kron(np.kron(np.eye(D_F), O), np.eye(dU))


def embed_U(O, dR):
    return np.kron(np.kron(np.eye(D_F), np.eye(dR)), O)


def onsite(ix, iy, nx, ny, dg, g, m):
    """H_onsite_site (u1_lgt_hamiltonian.jl:658-677)."""
    d, dR, dU = site_dims(ix, iy, nx, ny, dg)
    H = np.zeros((d, d))
    E2 = op_E(dg) @ op_E(dg)
    if ix < nx:
        H += (g * g / 2) * embed_R(E2, dU)
    if iy < ny:
        H += (g * g / 2) * embed_U(E2, dR)
    stag = 1 if (ix + iy) % 2 == 0 else -1
    H += m * stag * embed_f(op_nf(), dR, dU)
    return 0.5 * (H + H.T)


def column_snake(nx, ny):
    chain = []
    for ix in range(1, nx + 1):
        ys = range(1, ny + 1) if ix % 2 == 1 else range(ny, 0, -1)
        for iy in ys:
            chain.append((ix, iy))
    return chain


def terms(nx, ny, dg, *, g, t, m, model):
    """List of (coef, {site: local matrix}) exactly as lgt_terms /
    lgt_terms_plaqjw_cs build them."""
    chain = column_snake(nx, ny)
    pos = {s: p for p, s in enumerate(chain)}
    T = []
    for iy in range(1, ny + 1):
        for ix in range(1, nx + 1):
            T.append((1.0, {(ix, iy): onsite(ix, iy, nx, ny, dg, g, m)}))
    U = op_U(dg)
    cdag = op_c().T

    def add(coef, a, opa, b, opb):
        d = {a: opa, b: opb}
        if model == "pjw":
            lo, hi = sorted((pos[a], pos[b]))
            for p in range(lo + 1, hi):
                s = chain[p]
                _, dR, dU = site_dims(*s, nx, ny, dg)
                d[s] = embed_f(op_parity(), dR, dU)
        T.append((coef, d))

    for iy in range(1, ny + 1):
        for ix in range(1, nx):
            _, dRR, dUR = site_dims(ix + 1, iy, nx, ny, dg)
            _, _, dUL = site_dims(ix, iy, nx, ny, dg)
            AL = np.kron(np.kron(cdag, U), np.eye(dUL))
            BR = embed_f(op_c(), dRR, dUR)
            add(-t, (ix, iy), AL, (ix + 1, iy), BR)
            add(-t, (ix, iy), AL.T.copy(), (ix + 1, iy), BR.T.copy())
    for iy in range(1, ny):
        for ix in range(1, nx + 1):
            _, dRU, dUU = site_dims(ix, iy + 1, nx, ny, dg)
            _, dRD, _ = site_dims(ix, iy, nx, ny, dg)
            AD = np.kron(np.kron(cdag, np.eye(dRD)), U)
            BU = embed_f(op_c(), dRU, dUU)
            add(-t, (ix, iy), AD, (ix, iy + 1), BU)
            add(-t, (ix, iy), AD.T.copy(), (ix, iy + 1), BU.T.copy())
    if model == "pjw":
        invg2 = 1.0 / (2.0 * g * g)
        Ud = U.T.copy()
        for iy in range(1, ny):
            for ix in range(1, nx):
                A, B, C = (ix, iy), (ix + 1, iy), (ix, iy + 1)
                _, dAR, dAU = site_dims(*A, nx, ny, dg)
                _, dBR, _ = site_dims(*B, nx, ny, dg)
                _, _, dCU = site_dims(*C, nx, ny, dg)
                opA = embed_R(Ud, dAU) @ embed_U(U, dAR)
                opB = embed_U(Ud, dBR)
                opC = embed_R(U, dCU)
                T.append((-invg2, {A: opA, B: opB, C: opC}))
                T.append((-invg2, {A: opA.T.copy(), B: opB.T.copy(), C: opC.T.copy()}))
    return T


def site_order(nx, ny):
    """Site order of the full tensor product (any fixed order works; the
    fermion signs are carried by the explicit parity strings)."""
    return column_snake(nx, ny)


def hamiltonian(nx, ny, dg, *, g, t, m, model):
    """Full-space H as scipy CSR, sites in ``site_order``; the first site is
    the slowest index (kron convention of Julia and numpy alike)."""
    order = site_order(nx, ny)
    dims = [site_dims(ix, iy, nx, ny, dg)[0] for ix, iy in order]
    N = int(np.prod(dims))
    H = sp.csr_matrix((N, N))
    for coef, ops in terms(nx, ny, dg, g=g, t=t, m=m, model=model):
        M = sp.identity(1, format="csr")
        for s, d in zip(order, dims):
            M = sp.kron(M, sp.csr_matrix(ops[s]) if s in ops else sp.identity(d, format="csr"),
                        format="csr")
        H = H + coef * M
    return H.tocsr()


def gauss_penalty_diag(nx, ny, dg, g_charges, lam):
    """Diagonal of lam * sum_i (G_i - g_i)^2 with G_i = E_R(i) - E_R(i-x)
    + E_U(i) - E_U(i-y) - n_f(i) (finite_ed.jl:13-15, mps_lgt.jl:465-513)."""
    order = site_order(nx, ny)
    dims = [site_dims(ix, iy, nx, ny, dg) for ix, iy in order]
    N = int(np.prod([d[0] for d in dims]))
    idx = np.arange(N)
    # decode every local configuration
    nf, eR, eU = {}, {}, {}
    rem = idx.copy()
    for (ix, iy), (d, dR, dU) in reversed(list(zip(order, dims))):
        loc = rem % d
        rem //= d
        nf[(ix, iy)] = loc // (dR * dU)
        eR[(ix, iy)] = (loc // dU) % dR - (dg if dR > 1 else 0)
        eU[(ix, iy)] = loc % dU - (dg if dU > 1 else 0)
    pen = np.zeros(N)
    for iy in range(1, ny + 1):
        for ix in range(1, nx + 1):
            G = eR[(ix, iy)] + eU[(ix, iy)] - nf[(ix, iy)]
            if ix > 1:
                G = G - eR[(ix - 1, iy)]
            if iy > 1:
                G = G - eU[(ix, iy - 1)]
            pen += (G - int(g_charges[ix - 1, iy - 1])) ** 2
    return lam * pen


def sector_indices(basis):
    """Full-space index of every oracle basis state."""
    nx, ny, dg = basis.nx, basis.ny, basis.dg
    order = site_order(nx, ny)
    out = np.zeros(basis.dim, dtype=np.int64)
    for k in range(basis.dim):
        full = 0
        for ix, iy in order:
            d, dR, dU = site_dims(ix, iy, nx, ny, dg)
            er = int(basis.eR[k, ix - 1, iy - 1]) if ix < nx else 0
            eu = int(basis.eU[k, ix - 1, iy - 1]) if iy < ny else 0
            full = full * d + site_idx(int(basis.nf[k, ix - 1, iy - 1]), er, eu, dR, dU, dg)
        out[k] = full
    return out
