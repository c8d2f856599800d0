"""The FP64 transport's table-driven logarithm, sin/cos(pi U) and
cos/sin(2 pi U) of its uniforms U = (w + 1/2) 2^-32 (mcd_device.cuh: ln_word,
sincospi_word, cossin2pi_word), run on
the GPU through a test kernel (tests/special_check.cu, compiled here), against
the host: at 40 significant digits (Python's decimal) on 4000 words including
the edge words and every breakpoint, and against numpy's libm on 2e6 seeded
words.  What a trajectory needs is absolute accuracy: a step's error enters
the position as that error times the mean free path."""
import ctypes as C
import decimal
import os
import subprocess

import numpy as np
import pytest

from mcd import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def special(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("special") / "special.so")
    cmd = [build.nvcc(), "-shared", "-o", so, os.path.join(HERE, "special_check.cu"),
           "-I", build.CSRC, "-I", os.path.join(ROOT, "include"),
           "-Xcompiler", "-fPIC"] + build.ARCH + build.COMMON
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    lib = C.CDLL(so)
    lib.special_eval.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
    lib.special_eval.restype = C.c_int
    lib.rcp_eval.argtypes = [C.c_void_p, C.c_int64, C.c_void_p]
    lib.rcp_eval.restype = C.c_int

    def run(words):
        w = np.ascontiguousarray(words, dtype=np.uint32)
        out = np.empty((w.size, 5), dtype=np.float64)
        assert lib.special_eval(w.ctypes.data, w.size, out.ctypes.data) == 0
        assert not np.isnan(out).any(), "the adjoint's sin/cos of the same uniform differs"
        return out

    def rcp(d):
        d = np.ascontiguousarray(d, dtype=np.float64)
        out = np.empty_like(d)
        assert lib.rcp_eval(d.ctypes.data, d.size, out.ctypes.data) == 0
        return out
    run.rcp = rcp
    return run


def uniforms(w):
    return (w.astype(np.float64) + 0.5) * 2.0 ** -32          # exact


def edge_words():
    j = np.arange(256, dtype=np.uint64) << 24
    e = [0, 1, 2, 3, 0xFF, 0x100, 0xFFFFFF, 0x7FFFFFFF, 0x80000000, 0xFFFFFFFE, 0xFFFFFFFF]
    return np.unique(np.concatenate([j, np.maximum(j, 1) - 1, j + 0xFFFFFF, np.array(e, np.uint64)])).astype(np.uint32)


def decimal_ref(words):
    ctx = decimal.Context(prec=40)
    pi = decimal.Decimal("3.141592653589793238462643383279502884197169")
    def sincos(x):
        x2 = ctx.multiply(x, x)
        s, c, ts, tc = decimal.Decimal(0), decimal.Decimal(0), x, decimal.Decimal(1)
        for n in range(60):
            s, c = ctx.add(s, ts), ctx.add(c, tc)
            ts = ctx.divide(ctx.multiply(-ts, x2), (2 * n + 2) * (2 * n + 3))
            tc = ctx.divide(ctx.multiply(-tc, x2), (2 * n + 1) * (2 * n + 2))
        return s, c

    out = np.empty((len(words), 5))
    for k, w in enumerate(words):
        U = (decimal.Decimal(int(w)) + decimal.Decimal("0.5")) / decimal.Decimal(2 ** 32)
        s, c = sincos(ctx.multiply(pi, U))
        s2, c2 = sincos(ctx.multiply(pi, ctx.multiply(2, U) - 1))       # 2 pi U = pi + pi (2U - 1)
        out[k] = (float(U.ln(ctx)), float(s), float(c), float(-c2), float(-s2))
    return out


def test_against_forty_digits(special):
    rng = np.random.default_rng(5)
    words = np.concatenate([edge_words(), rng.integers(0, 2 ** 32, 4000 - edge_words().size, dtype=np.uint64)
                            .astype(np.uint32)])
    got, ref = special(words), decimal_ref(words)
    lnU = ref[:, 0]
    err_ln = np.abs(got[:, 0] - lnU)
    # absolute 2.5e-16 (|ln U| < 1), relative 2.5e-16 above
    assert np.all(err_ln <= 2.5e-16 * np.maximum(1.0, np.abs(lnU))), err_ln.max()
    assert np.abs(got[:, 1:] - ref[:, 1:]).max() <= 2e-16


def test_against_libm_on_two_million_words(special):
    rng = np.random.default_rng(6)
    words = rng.integers(0, 2 ** 32, 2_000_000, dtype=np.uint64).astype(np.uint32)
    got, U = special(words), uniforms(words)
    lnU = np.log(U)
    assert np.all(np.abs(got[:, 0] - lnU) <= 5e-16 * np.maximum(1.0, np.abs(lnU)))
    # numpy's sin(pi * U) carries the rounding of pi * U (up to 2.2e-16 times
    # the slope) besides its own
    assert np.abs(got[:, 1] - np.sin(np.pi * U)).max() <= 1e-15
    assert np.abs(got[:, 2] - np.cos(np.pi * U)).max() <= 1e-15
    assert np.abs(got[:, 3] - np.cos(2 * np.pi * U)).max() <= 2e-15
    assert np.abs(got[:, 4] - np.sin(2 * np.pi * U)).max() <= 2e-15


def test_reciprocal_within_two_ulp(special):
    """rcp_pos (the Rutherford angle's 1/(E (1 - U) + a0)): the hardware
    approximation and two third-order Newton-Raphson steps, within two ulp
    of the IEEE quotient over 1e-3 .. 1e7 (log-uniform, 1e6 values) and at
    every power of two in that range and its neighbours."""
    rng = np.random.default_rng(7)
    d = np.exp(rng.uniform(np.log(1e-3), np.log(1e7), 1_000_000))
    p2 = 2.0 ** np.arange(-9, 24)
    d = np.concatenate([d, p2, np.nextafter(p2, 0.0), np.nextafter(p2, np.inf)])
    got, want = special.rcp(d), 1.0 / d
    ulp = np.spacing(want)
    assert np.all(np.abs(got - want) <= 2 * ulp), np.max(np.abs(got - want) / ulp)
