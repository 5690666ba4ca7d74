"""The float-float outer update of the register-resident outer step, emulated in NumPy FP32 arithmetic in the kernel's
order (csrc/outer_step.cu, FF branch of outer_step_reg_kernel), against the FP64 update of the reference's outer
iteration x_new = x + om_a r + om_1 (x - x_prev) (fastops.py:252-257).

The claims checked: the step om_a r + om_1 (x - x_prev) carries FP32 relative accuracy (the FP64 form computes it from
the same FP32 r, so that is the precision the update had before); the sum with x is kept to about 48 bits (two-sum),
so the state does not lose the low bits of x over the outer iterations; the first step a0 r is a float-float product;
and the planes stay normalised (hi = fl32(hi + lo))."""

import numpy as np

f32 = np.float32


def _fma(a, b, c):
    """fl32(a b + c) for FP32 a, b, c: the product is exact in FP64 (24 + 24 bits), one rounding of the sum."""
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def _split(v):
    hi = f32(v)
    return hi, f32(v - np.float64(hi))


def ff_update(x, xp, r, om_a, om_1):
    """One element: x, xp FP64 values held as float-float; r FP32; the kernel's sequence of FP32 operations."""
    xh, xl = _split(x)
    ph, pl = _split(xp)
    oah, oal = _split(om_a)
    o1h, o1l = _split(om_1)
    d = f32(f32(xh - ph) + f32(xl - pl))
    dl = _fma(oah, r, _fma(o1h, d, _fma(oal, r, f32(o1l * d))))
    sh = f32(xh + dl)
    bb = f32(sh - xh)
    lo = f32(f32(f32(xh - f32(sh - bb)) + f32(dl - bb)) + xl)
    hi = f32(sh + lo)
    return hi, f32(lo - f32(hi - sh))


def ff_first(r, a0):
    a0h, a0l = _split(a0)
    h = f32(a0h * r)
    l_ = f32(_fma(a0h, r, -h) + f32(a0l * r))
    hi = f32(h + l_)
    return hi, f32(l_ - f32(hi - h))


def test_float_float_update_accuracy():
    rng = np.random.default_rng(0)
    worst = 0.0
    for _ in range(4000):
        x = rng.standard_normal()
        step_scale = 10.0 ** rng.uniform(-8, 0)  # late outer iterations take small steps
        xp = x - step_scale * rng.standard_normal()
        r = f32(step_scale * rng.standard_normal())
        om_a, om_1 = rng.uniform(0.1, 2.0), rng.uniform(0.0, 0.9)
        exact = x + om_a * np.float64(r) + om_1 * (x - xp)
        hi, lo = ff_update(x, xp, r, om_a, om_1)
        got = np.float64(hi) + np.float64(lo)
        step = abs(om_a * np.float64(r)) + abs(om_1 * (x - xp))
        assert hi == f32(np.float64(hi) + np.float64(lo))  # normalised planes
        # the error: a few FP32 roundings of the step, plus the state's own rounding of about 2^-48 |x| (an FP32
        # state would add 2^-25 |x|, about 3e-8 relative, at every step)
        worst = max(worst, abs(got - exact) / (4 * 2.0 ** -24 * step + 2.0 ** -47 * abs(x)))
    assert worst <= 1.0


def test_float_float_first_step_and_many_iterations():
    rng = np.random.default_rng(1)
    for _ in range(500):
        r = f32(rng.standard_normal())
        a0 = rng.uniform(0.01, 1.0)
        hi, lo = ff_first(r, a0)
        assert abs(np.float64(hi) + np.float64(lo) - a0 * np.float64(r)) <= 2.0 ** -46 * abs(a0 * np.float64(r))
    # 40 outer steps with exact (FP32-representable) steps: an FP32 state would drift by up to 40 x 2^-25 |x|
    # relative; the float-float state keeps the exact sum of the steps
    x = 1.0
    xs = [1.0, 1.0]
    for k in range(40):
        r = f32(rng.uniform(-1e-3, 1e-3))
        hi, lo = ff_update(xs[-1], xs[-2], r, 1.0, 0.0)
        xs.append(np.float64(hi) + np.float64(lo))
        x = x + np.float64(r)
    assert abs(xs[-1] - x) < 2.0 ** -44
