"""The library's table-driven FP64 routines (fp64_math.cuh), evaluated on the
device through pbsm3d_math_eval beside the CUDA functions they replace, and
both measured against an extended-precision host value (numpy longdouble:
80-bit on x86-64, IEEE quad on aarch64).

Bounds, in units in the last place of the correctly rounded result:
- exp_t (Tang 1989, 256-point table): 1.5 ulp on |x| < 700;
- log_t (Tang 1990, 256-point table): 4.5e-16 absolute where |log x| < 1
  and 2 ulp where |log x| >= 1 (the assembly uses it as an exp argument or
  far from x = 1, where an absolute bound is what matters);
- rcp_t (hardware estimate + two Newton-Raphson steps): 1 ulp;
- div_t (Markstein's residual correction): 1 ulp;
- pow_t = exp_t(y log_t(x)) for x in [1e-4, 1e4], |y| <= 2 (the assembly's
  exponents are 1.36, 1.75, 1.8, -0.258, 0.3333333): 2 + 4 |y ln x| ulp.
  The product y log x carries an absolute error of about an ulp of itself
  (log_t's error times |y|, and its own rounding), which exp turns into a
  relative error of the result that grows with |y ln x|: 40 ulp measured
  at |y ln x| near 18, under 20 ulp at the assembly's arguments (u_z^1.36
  with u_z <= 30 m/s gives |y ln x| < 4.7);
- f32_rn (round-to-nearest-even on the integer pipe): bit-identical to the
  hardware FP64 -> FP32 conversion, halfway cases included.
Outside the fast ranges (zero, negative, subnormal, huge, Inf, NaN) each
routine returns the CUDA function's value bit for bit.
"""
import ctypes as C

import numpy as np
import pytest

from chm_gb300 import capi

pytestmark = pytest.mark.gpu

N = 1 << 20


def ev(lib, fn, a, b=None):
    torch = pytest.importorskip("torch")
    ta = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()
    tb = None if b is None else torch.from_numpy(np.ascontiguousarray(b, dtype=np.float64)).cuda()
    out = torch.empty_like(ta)
    torch.cuda.synchronize()
    rc = lib.pbsm3d_math_eval(fn, ta.numel(), C.c_void_p(ta.data_ptr()),
                              None if tb is None else C.c_void_p(tb.data_ptr()), C.c_void_p(out.data_ptr()))
    assert rc == capi.OK, lib.pbsm3d_last_error(None)
    return out.cpu().numpy()


def ulps(y, exact_ld):
    """|y - exact| in ulps of the double nearest to exact."""
    z = exact_ld.astype(np.float64)
    sp = np.spacing(np.abs(z)).astype(np.longdouble)
    return np.abs(y.astype(np.longdouble) - exact_ld) / sp


def same_bits(a, b):
    return np.array_equal(a.view(np.int64), b.view(np.int64)) or bool(
        np.all((a == b) | (np.isnan(a) & np.isnan(b))))


# the function codes of pbsm3d_math_eval (include/pbsm3d.h)
EXP, LOG, RCP, DIV, POW, F32, CEXP, CLOG, CRCP, CDIV, CPOW, CF32 = range(12)


@pytest.fixture(scope="module")
def rng():
    return np.random.default_rng(20261204)


def test_exp(cuda_lib, rng):
    x = np.concatenate([rng.uniform(-700, 700, N), rng.uniform(-1e-3, 1e-3, N // 4), rng.uniform(-30, 30, N // 4),
                        np.array([0.0, -0.0, 1e-300, -1e-300, 699.999, -699.999])])
    y = ev(cuda_lib, EXP, x)
    ref = np.exp(x.astype(np.longdouble))
    e = ulps(y, ref)
    ec = ulps(ev(cuda_lib, CEXP, x), ref)
    print(f"exp_t max {float(e.max()):.3f} ulp, CUDA exp {float(ec.max()):.3f} ulp")
    assert e.max() <= 1.5
    special = np.array([700.0, -700.0, 709.7, 710.0, -745.0, -746.0, np.inf, -np.inf, np.nan, 1e308])
    assert same_bits(ev(cuda_lib, EXP, special), ev(cuda_lib, CEXP, special))


def test_log(cuda_lib, rng):
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, N), 1.0 + rng.uniform(-1e-3, 1e-3, N // 4),
                        rng.uniform(0.5, 2.0, N // 4), np.array([1.0, 2.0, 0.5, np.finfo(float).tiny,
                                                                np.finfo(float).max])])
    y = ev(cuda_lib, LOG, x)
    ref = np.log(x.astype(np.longdouble))
    absd = np.abs(y.astype(np.longdouble) - ref)
    e = ulps(y, ref)
    far = np.abs(ref) >= 1
    yc = ev(cuda_lib, CLOG, x)
    print(f"log_t max abs {float(absd[~far].max()):.2e} where |log x| < 1, max {float(e[far].max()):.3f} ulp "
          f"where |log x| >= 1; CUDA log {float(ulps(yc, ref).max()):.3f} ulp")
    assert absd[~far].max() <= 4.5e-16
    assert e[far].max() <= 2.0
    special = np.array([0.0, -0.0, -1.0, 5e-324, 1e-310, np.inf, -np.inf, np.nan])
    assert same_bits(ev(cuda_lib, LOG, special), ev(cuda_lib, CLOG, special))


def test_rcp_and_div(cuda_lib, rng):
    x = rng.choice([-1.0, 1.0], N) * 10.0 ** rng.uniform(-300, 300, N)
    y = ev(cuda_lib, RCP, x)
    ref = 1 / x.astype(np.longdouble)
    e = ulps(y, ref)
    print(f"rcp_t max {float(e.max()):.3f} ulp")
    assert e.max() <= 1.0
    a = rng.choice([-1.0, 1.0], N) * 10.0 ** rng.uniform(-150, 150, N)
    b = rng.choice([-1.0, 1.0], N) * 10.0 ** rng.uniform(-150, 150, N)
    q = ev(cuda_lib, DIV, a, b)
    eq = ulps(q, a.astype(np.longdouble) / b.astype(np.longdouble))
    print(f"div_t max {float(eq.max()):.3f} ulp")
    assert eq.max() <= 1.0
    special = np.array([0.0, -0.0, 5e-324, 1e-305, 1e305, np.inf, -np.inf, np.nan, 2.0 ** -1001, 2.0 ** 1001])
    assert same_bits(ev(cuda_lib, RCP, special), ev(cuda_lib, CRCP, special))


def test_pow(cuda_lib, rng):
    x = 10.0 ** rng.uniform(-4, 4, N)
    yv = rng.uniform(-2, 2, N)
    yv[: 5 * 1024] = np.repeat([1.36, 1.75, 1.8, -0.258, 0.3333333], 1024)
    p = ev(cuda_lib, POW, x, yv)
    ref = np.power(x.astype(np.longdouble), yv.astype(np.longdouble))
    e = ulps(p, ref)
    ec = ulps(ev(cuda_lib, CPOW, x, yv), ref)
    ylx = np.abs(yv * np.log(x))
    print(f"pow_t max {float(e.max()):.3f} ulp ({float((e / (2 + 4 * ylx)).max()):.2f} of the bound), "
          f"CUDA pow {float(ec.max()):.3f} ulp")
    assert (e <= 2 + 4 * ylx).all()


def test_f32_rounding(cuda_lib, rng):
    f = (rng.uniform(-1, 1, N) * 2.0 ** rng.integers(-125, 127, N)).astype(np.float32)
    f = f[np.isfinite(f) & (np.abs(f) >= np.finfo(np.float32).tiny) & (np.abs(f) < np.finfo(np.float32).max)]
    nxt = np.nextafter(f, np.float32(np.inf))
    mid = (f.astype(np.float64) + nxt.astype(np.float64)) / 2  # exact halfway cases
    x = np.concatenate([rng.uniform(-1, 1, N) * 2.0 ** rng.integers(-126, 128, N), mid, np.nextafter(mid, 0),
                        np.nextafter(mid, np.inf), np.array([0.0, -0.0, 1e-40, -1e-45, 3.5e38, 3.4028235e38,
                                                              np.inf, -np.inf, np.nan])])
    assert same_bits(ev(cuda_lib, F32, x), ev(cuda_lib, CF32, x))


def test_fp64_rate_probe(cuda_lib):
    """pbsm3d_fp64_rate measures the FP64 FMA rate that bounds the FP64
    kernels; the bench's FP64 roofline divides by it.  It must land near the
    GPU's FP64 pipe rate: 2 FMA a clock per SM (1.26 TFLOP/s on 152 SMs at
    2.07 GHz), within what clock states allow."""
    torch = pytest.importorskip("torch")
    rate = C.c_double(0.0)
    assert cuda_lib.pbsm3d_fp64_rate(C.byref(rate)) == capi.OK, cuda_lib.pbsm3d_last_error(None)
    props = torch.cuda.get_device_properties(0)
    nominal = 2.0 * props.multi_processor_count * 2.07e9
    assert 0.3 * nominal < rate.value < 1.2 * nominal, (rate.value, nominal)
    assert cuda_lib.pbsm3d_fp64_rate(None) == capi.ERR_INVALID_ARG
