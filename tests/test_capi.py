"""CPU tests of the C ABI boundary: the library builds for sm_103a, loads,
exports every symbol include/lgt_ed.h declares, and its argument checks and
error codes behave without a GPU (no compute call is made here)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "lgt_ed.h")).read()
    return sorted(set(re.findall(r"LGT_API[^;{]*?\b(lgt_[a-z_0-9]+)\s*\(", src, re.S)))


def test_header_lists_the_python_binding():
    from lgt_gb300 import _capi
    assert header_symbols() == sorted(_capi.EXPORTS)


def test_hpsi_kernel_names_agree_across_bindings():
    """lgt_tuning.hpsi_kernel codes 0..8: the Python and Julia name lists
    cover the codes the header documents, in the same order."""
    import lgt_gb300 as lgt
    hdr = open(os.path.join(ROOT, "include", "lgt_ed.h")).read()
    doc = hdr[hdr.index("int32_t hpsi_kernel;"):hdr.index("int32_t reduce_blocks;")]
    assert "0 built-in rule" in doc and "5, 6, 7" in doc and "8 the stored table" in doc
    assert sorted(lgt.HPSI_KERNELS) == list(range(9))
    jl = open(os.path.join(ROOT, "lgt_gb300", "julia", "LGTED.jl")).read()
    names = re.search(r"HPSI_KERNELS = \(([^)]*)\)", jl, re.S).group(1)
    assert re.findall(r'"([a-z_0-9]+)"', names) == [lgt.HPSI_KERNELS[i] for i in range(9)]


def test_library_exports_every_declared_symbol():
    from lgt_gb300 import _capi
    path = _capi.library_path()
    _capi.load()
    lib = ctypes.CDLL(path)
    for name in header_symbols():
        assert hasattr(lib, name), name


def test_library_is_sm_103a_only():
    from lgt_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_defaults_are_the_reference_settings():
    from lgt_gb300 import _capi as C
    o = C.defaults(False)
    assert (o.krylovdim, o.maxiter, o.tol) == (50, 300, 1e-10)   # finite_ed.jl:336-338
    o = C.defaults(True)
    assert (o.krylovdim, o.maxiter, o.tol) == (30, 100, 1e-10)   # finite_ed.jl:417-419


def _create(nx, ny, dg, g):
    from lgt_gb300 import _capi as C
    lib = C.load()
    h = ctypes.c_void_p()
    gf = np.asfortranarray(np.asarray(g, np.int32).reshape(max(nx, 1), max(ny, 1)))
    code = lib.lgt_basis_create(nx, ny, dg, gf.ctypes.data_as(ctypes.c_void_p), -1,
                                ctypes.byref(h))
    return code, lib.lgt_last_error().decode()


def test_inconsistent_sector_is_a_status_not_an_abort():
    from lgt_gb300 import _capi as C
    g = np.zeros((3, 2), np.int32)
    g[0, 0] = 2  # N_f = -2  (finite_ed.jl:127 @assert)
    code, msg = _create(3, 2, 1, g)
    assert code == C.LGT_ERR_SECTOR and "Inconsistent sector" in msg
    g[0, 0] = -7  # N_f = 7 > 6 sites
    assert _create(3, 2, 1, g)[0] == C.LGT_ERR_SECTOR


def test_key_width_and_range_checks():
    from lgt_gb300 import _capi as C
    assert _create(6, 6, 1, np.zeros((6, 6)))[0] == C.LGT_ERR_KEYWIDTH   # 36 sites
    assert _create(5, 5, 1, np.zeros((5, 5)))[0] == C.LGT_ERR_KEYWIDTH   # 25 + 2*20 > 64 bits
    assert _create(3, 3, 9, np.zeros((3, 3)))[0] == C.LGT_ERR_ARG        # dg out of range
    assert _create(0, 3, 1, np.zeros((1, 3)))[0] == C.LGT_ERR_ARG


def test_null_arguments():
    from lgt_gb300 import _capi as C
    lib = C.load()
    assert lib.lgt_basis_dim(None, None) == C.LGT_ERR_ARG
    assert lib.lgt_ham_create(None, 1, None, None, None, 0, None) == C.LGT_ERR_ARG
    assert lib.lgt_matvec(None, None, None, 1, 0, 0) == C.LGT_ERR_ARG
    assert lib.lgt_launch_count(None) == C.LGT_ERR_ARG
    n = ctypes.c_uint64()
    assert lib.lgt_launch_count(ctypes.byref(n)) == C.LGT_OK
    assert b"sm_103a" in lib.lgt_version()


def test_python_encode_matches_oracle(oracle):
    import lgt_gb300 as L
    b = oracle.build_basis(4, 3, 1, oracle.staggered_charges(4, 3))
    for i in range(0, b.dim, 997):
        assert L.encode(b.nf[i], b.eR[i], b.eU[i]) == int(b.ref_keys[i])


def test_sector_helpers_match_oracle(oracle):
    import lgt_gb300 as L
    for nx, ny in [(3, 2), (4, 4), (3, 4)]:
        assert np.array_equal(L.staggered_charges(nx, ny), oracle.staggered_charges(nx, ny))
        assert np.array_equal(L.string_charges(nx, ny), oracle.string_charges(nx, ny))


def test_basis_outlives_its_hamiltonians_any_destroy_order():
    """Destroying the basis before a Hamiltonian made from it is allowed (the
    basis is reference-counted in the library); needs no GPU to check the
    symbol, the order itself is exercised by the GPU tests' garbage
    collection."""
    from lgt_gb300 import _capi as C
    lib = C.load(build_if_missing=False)
    assert hasattr(lib, "lgt_basis_destroy") and hasattr(lib, "lgt_ham_destroy")


def _split_top(s):
    """Split at commas outside (), {} and []."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({[":
            depth += 1
        elif ch in ")}]":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur.strip())
    return out


def _header_arity():
    src = open(os.path.join(ROOT, "include", "lgt_ed.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    ar = {}
    for m in re.finditer(r"LGT_API[^;{]*?\b(lgt_[a-z_0-9]+)\s*\(([^;]*?)\)\s*;", src, re.S):
        params = m.group(2).strip()
        ar[m.group(1)] = 0 if params in ("", "void") else len(_split_top(params))
    return ar


def test_julia_shim_calls_match_the_header():
    """Every ccall of the Julia shim names a declared entry point and passes
    as many arguments as the header's prototype takes (the shim cannot run
    here: no Julia)."""
    jl = open(os.path.join(ROOT, "lgt_gb300", "julia", "LGTED.jl")).read()
    ar = _header_arity()
    calls = []
    for m in re.finditer(r"ccall\(\(:(lgt_[a-z_0-9]+), libpath\),", jl):
        # return type, then the argument-type tuple up to its matching paren
        rest = jl[m.end():]
        i = rest.index(",") + 1
        while rest[i] in " \n":
            i += 1
        assert rest[i] == "(", m.group(1)
        depth, j = 0, i
        while True:
            depth += {"(": 1, ")": -1}.get(rest[j], 0)
            if depth == 0:
                break
            j += 1
        calls.append((m.group(1), rest[i + 1:j]))
    assert len(calls) >= 10
    for name, types in calls:
        assert name in ar, name
        t = types.replace("\n", " ").strip()
        n = 0 if t == "" else len(_split_top(t))
        assert n == ar[name], (name, n, ar[name])
