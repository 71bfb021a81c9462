"""Double-float arithmetic used by the FP64-accurate device kernels, checked on
the host against exact rational arithmetic (the same code runs on the device)."""
import ctypes as C
from fractions import Fraction as Fr

import numpy as np
import pytest


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _values(n=600, seed=3):
    rng = np.random.default_rng(seed)
    # df64 keeps ~48 bits while both halves are normal binary32 numbers:
    # 2^-100 <= |x| <= 2^120 (finite-element entries live far inside this range)
    a = rng.standard_normal(n) * np.exp(rng.uniform(-30, 30, n))
    a[:8] = [0.0, 1.0, -1.0, 1 / 3, 2.0 ** -60, 1e-25, -7.25, 1 - 2.0 ** -40]
    return a


OPS = {0: (lambda x, y: Fr(x), 2.0 ** -48, "value"),
       1: (lambda x, y: Fr(x) + Fr(y), 2.0 ** -46, "sum"),
       2: (lambda x, y: Fr(x) * Fr(y), 2.0 ** -46, "value"),
       3: (lambda x, y: 1 / Fr(x), 2.0 ** -45.5, "value"),
       4: (lambda x, y: Fr(x) - Fr(y), 2.0 ** -46, "sum")}


@pytest.mark.parametrize("op", sorted(OPS))
def test_df64_ops_error_bounds(fgpu_lib, op):
    a, b = _values(), _values(seed=4)
    out = np.zeros_like(a)
    assert fgpu_lib.fgpu_host_df64_ops(op, len(a), _p(a), _p(b), _p(out)) == 0
    f, bound, kind = OPS[op]
    for x, y, o in zip(a, b, out):
        if op == 3 and x == 0:
            continue
        ex = f(x, y)
        if ex != 0 and not (Fr(2) ** -100 <= abs(ex) <= Fr(2) ** 120):
            continue                      # result outside the df64 range
        scale = abs(Fr(x)) + abs(Fr(y)) if kind == "sum" else abs(ex)
        if scale == 0:
            assert o == 0
            continue
        assert abs(Fr(o) - ex) <= bound * scale, (op, x, y, o)


def test_df64_roundtrip_exact_for_binary32_values(fgpu_lib):
    a = np.array([1.5, -3.0, 0.1, 1e-20, 2.0 ** 100], dtype=np.float32).astype(np.float64)
    out = np.zeros_like(a)
    fgpu_lib.fgpu_host_df64_ops(0, len(a), _p(a), None, _p(out))
    assert np.array_equal(out, a)
