"""CPU tests of the double-float arithmetic (lgt_gb300/csrc/lgt_dfloat.cuh)
that the FP32-mixed Krylov reductions use in place of FP64: the routines
themselves, compiled for the host from the same header, against exact
results (math.fsum of exactly represented products, Fractions).

Bars.  A dot of n terms: |error| <= 4 n 2^-48 sum |a_i b_i| (the bound of
renormalised double-word sums), and on random data within sqrt(n) 2^-46
sum |a_i b_i|.  A Gram-Schmidt update w - V h of FP32 data (J vectors),
rounded to FP32 as the mixed path stores it: its error is dominated by
that final rounding, so it is within 1.5 times the error of the same
update accumulated in FP64 (and within 0.51 FP32 ulp per entry plus
(J + 1)^2 2^-48 of the terms' sizes, the Dot2 bound), for well-conditioned
passes and for passes that cancel three digits (the largest cancellation a
pass is kept for; more triggers a second pass).
"""
import ctypes
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "native", "dfloat_harness.cpp")


@pytest.fixture(scope="module")
def dfh(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    so = str(tmp_path_factory.mktemp("dfh") / "libdfh.so")
    subprocess.run([cxx, "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC", "-o", so,
                    SRC], check=True)
    L = ctypes.CDLL(so)
    vp, i64 = ctypes.c_void_p, ctypes.c_int64
    L.dfh_dot.restype = ctypes.c_double
    L.dfh_dot.argtypes = [vp, vp, i64]
    L.dfh_dot2.restype = ctypes.c_double
    L.dfh_dot2.argtypes = [vp, vp, vp, i64]
    L.dfh_update.restype = ctypes.c_float
    L.dfh_update.argtypes = [ctypes.c_float, vp, vp, i64]
    return L


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _exact_dot(a, b):
    # products of two FP32 values are exact in FP64; fsum rounds their sum once
    return math.fsum((a.astype(np.float64) * b.astype(np.float64)).tolist())


@pytest.mark.parametrize("n", [1, 7, 100, 1000, 20000])
@pytest.mark.parametrize("kind", ["random", "cancelling", "wide"])
def test_dot_error_bounds(dfh, n, kind):
    rng = np.random.default_rng(n + len(kind))
    a = rng.standard_normal(n).astype(np.float32)
    b = rng.standard_normal(n).astype(np.float32)
    if kind == "cancelling":  # second half cancels the first up to FP32 rounding
        h = n // 2
        a[h:2 * h] = a[:h]
        b[h:2 * h] = -b[:h] * np.float32(1 + 2**-20)
    elif kind == "wide":  # magnitudes over 2^-40 .. 2^40
        a *= np.float32(2.0) ** rng.integers(-20, 20, n).astype(np.float32)
        b *= np.float32(2.0) ** rng.integers(-20, 20, n).astype(np.float32)
    exact = _exact_dot(a, b)
    mag = float(np.sum(np.abs(a.astype(np.float64) * b.astype(np.float64))))
    got = dfh.dfh_dot(_p(a), _p(b), n)
    assert abs(got - exact) <= 4 * n * 2.0**-48 * mag + abs(exact) * 2.0**-52
    if kind == "random":
        assert abs(got - exact) <= math.sqrt(n) * 2.0**-46 * mag


def test_dot_against_double_float_residual(dfh):
    """The per-CTA kernels dot FP32 basis entries with a residual held as
    a double-float pair hi + lo."""
    rng = np.random.default_rng(3)
    n = 5000
    a = rng.standard_normal(n).astype(np.float32)
    w = rng.standard_normal(n)
    bh = w.astype(np.float32)
    bl = (w - bh.astype(np.float64)).astype(np.float32)
    exact = math.fsum((a.astype(np.float64) *
                       (bh.astype(np.float64) + bl.astype(np.float64))).tolist())
    mag = float(np.sum(np.abs(a.astype(np.float64) * w)))
    got = dfh.dfh_dot2(_p(a), _p(bh), _p(bl), n)
    assert abs(got - exact) <= 4 * n * 2.0**-48 * mag


@pytest.mark.parametrize("J", [1, 2, 5, 15, 50])
@pytest.mark.parametrize("cancel", [1.0, 1e-3])
def test_update_rounds_like_fp64(dfh, J, cancel):
    """One Gram-Schmidt pass w_new = w - V (V^T w) over n entries with an
    orthonormal FP32 basis V of J vectors; w has a share `cancel` outside
    span(V).  Entry by entry the double-float update (as k_update_df) is
    compared with the exact value and with the FP64 update, both rounded
    to FP32."""
    from fractions import Fraction
    rng = np.random.default_rng(J)
    n = 64
    Q, _ = np.linalg.qr(rng.standard_normal((n, J)))
    V = Q.astype(np.float32)
    w64 = V.astype(np.float64) @ rng.standard_normal(J)
    w64 = w64 / np.linalg.norm(w64) + cancel * rng.standard_normal(n) / math.sqrt(n)
    w = w64.astype(np.float32)
    h = V.astype(np.float64).T @ w.astype(np.float64)
    got = np.zeros(n, np.float32)
    ref64 = np.zeros(n, np.float32)
    exact = np.zeros(n)
    for r in range(n):
        vr = np.ascontiguousarray(V[r])
        got[r] = dfh.dfh_update(float(w[r]), _p(h), _p(vr), J)
        ex = Fraction(float(w[r])) - sum(Fraction(float(hi)) * Fraction(float(vi))
                                         for hi, vi in zip(h, vr))
        exact[r] = float(ex)
        acc = float(w[r])
        for hi, vi in zip(h.tolist(), vr.astype(np.float64).tolist()):
            acc -= hi * vi
        ref64[r] = np.float32(acc)
    terms = np.abs(w.astype(np.float64)) + np.abs(V.astype(np.float64)) @ np.abs(h)
    err = np.abs(got.astype(np.float64) - exact)
    ulp = np.spacing(np.abs(exact.astype(np.float32))).astype(np.float64)
    bound = (J + 1) ** 2 * 2.0**-48  # Dot2: FP32 rounding of the result + (J u)^2 of the terms
    assert np.all(err <= 0.51 * ulp + bound * terms)
    err64 = np.abs(ref64.astype(np.float64) - exact)
    assert np.linalg.norm(err) <= 1.5 * np.linalg.norm(err64) + bound * np.linalg.norm(terms)
