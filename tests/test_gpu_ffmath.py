"""Float-float arithmetic (ffmath.cuh) against FP64 on inputs that float-float
represents exactly: relative error of a few 2^-48 for the arithmetic and
sqrt, a few 2^-48 of the argument's size for exp (its reduction) and cos
(absolute, near its zeros).  GRAND's ΔE is evaluated in this arithmetic; its
own tests compare the energies with the FP64 oracle."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
N = 20000
FNS = {"exp": 0, "cos": 1, "sqrt": 2, "rcp": 3, "mul": 4, "div": 5, "add": 6, "rsqrt": 7}


def _ff_inputs(rng, h):
    """h + l with l a float below half an ulp of h: exact in float-float."""
    h = np.asarray(h, np.float32)
    ulp = np.spacing(np.abs(h)).astype(np.float64)
    lo = (rng.uniform(-0.5, 0.5, h.shape) * ulp).astype(np.float32)
    return h.astype(np.float64) + lo.astype(np.float64)


def _run(gpu_lib, fn, x):
    lib = gpu_lib.load()
    lib.bromoc_gpu_ff_check.argtypes = [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    out = np.zeros_like(x)
    rc = lib.bromoc_gpu_ff_check(FNS[fn], len(x), x.ctypes.data, out.ctypes.data)
    assert rc == 0
    return out


def test_exp(gpu_lib):
    """Full precision for results above 2^-102; below, the low part is a
    float subnormal (relative error up to 2^-24 near 2^-126)."""
    x = _ff_inputs(np.random.default_rng(1), np.random.default_rng(2).uniform(-70, 86, N))
    y = _run(gpu_lib, "exp", x)
    rel = np.abs(y / np.exp(x) - 1.0)
    assert (rel <= 8e-15 * (1.0 + np.abs(x))).all(), rel.max()
    x = _ff_inputs(np.random.default_rng(7), np.random.default_rng(8).uniform(-87, -70, 2000))
    assert (np.abs(_run(gpu_lib, "exp", x) / np.exp(x) - 1.0) <= 2.0 ** -23).all()


def test_cos(gpu_lib):
    x = _ff_inputs(np.random.default_rng(3), np.random.default_rng(4).uniform(-300, 300, N))
    y = _run(gpu_lib, "cos", x)
    err = np.abs(y - np.cos(x))
    assert (err <= 8e-15 * (1.0 + np.abs(x))).all(), err.max()


@pytest.mark.parametrize("fn", ["sqrt", "rcp", "rsqrt"])
def test_sqrt_rcp(gpu_lib, fn):
    rng = np.random.default_rng(5)
    h = 10.0 ** rng.uniform(-6, 6, N)
    if fn == "rcp":
        h *= rng.choice([-1.0, 1.0], N)
    x = _ff_inputs(rng, h)
    y = _run(gpu_lib, fn, x)
    want = {"sqrt": np.sqrt, "rcp": lambda v: 1.0 / v, "rsqrt": lambda v: 1.0 / np.sqrt(v)}[fn](x)
    rel = np.abs(y / want - 1.0)
    assert (rel <= 2e-14).all(), rel.max()


@pytest.mark.parametrize("fn", ["mul", "div", "add"])
def test_arithmetic(gpu_lib, fn):
    rng = np.random.default_rng(6)
    x = _ff_inputs(rng, rng.choice([-1.0, 1.0], N) * 10.0 ** rng.uniform(-4, 4, N))
    y = _run(gpu_lib, fn, x)
    a, b = x, np.roll(x, -1)
    if fn == "add":
        assert (np.abs(y - (a + b)) <= 2e-14 * (np.abs(a) + np.abs(b))).all()
    else:
        want = a * b if fn == "mul" else a / b
        rel = np.abs(y / want - 1.0)
        assert (rel <= 2e-14).all(), rel.max()
