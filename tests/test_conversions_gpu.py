"""The FP64 <-> FP32 conversions the kernels perform on the integer pipe
agree with the hardware conversions: round to nearest even into FP32 over
the whole FP32 normal range (ties, carries into the exponent, the overflow
boundary), Inf and NaN, and exact FP32 -> FP64; arguments below 2^-126 flush
to zero by design.  The Newton-Raphson reciprocal of the harmonic means stays
within two units in the last place of the IEEE 1/x, with the same class and
sign of result, over the whole FP64 range."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _values():
    rng = np.random.default_rng(7)
    parts = [
        rng.standard_normal(200000) * 10.0 ** rng.integers(-45, 45, 200000),
        rng.uniform(-1, 1, 100000),
        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, 3.4028234663852886e38,
                  3.4028235677973366e38, 3.40282357e38, 1e39, -1e39, 1.1754943508222875e-38,
                  1.1754942e-38, 1e-40, -1e-45, 5e-324, np.finfo(np.float64).max]),
    ]
    # exact ties and near-ties at the 29 dropped mantissa bits
    base = rng.uniform(1, 2, 50000).astype(np.float32).astype(np.float64)
    ulp = np.spacing(base.astype(np.float32)).astype(np.float64)
    parts += [base + ulp / 2, base - ulp / 2, base + ulp / 2 * (1 + 2.0 ** -40), (base + ulp / 2) * 2.0 ** 100,
              -(base + ulp / 2) * 2.0 ** -100]
    # every FP32 exponent, mantissa all ones (rounding carries into the exponent)
    e = np.arange(-126, 128, dtype=np.float64)
    parts.append((2.0 - 2.0 ** -24) * 2.0 ** e)
    parts.append((2.0 - 2.0 ** -23) * 2.0 ** e)
    return np.ascontiguousarray(np.concatenate(parts), dtype=np.float64)


def test_integer_pipe_conversions_match_hardware():
    from mizuho_edit_gb300 import capi
    L = capi.load()
    v = _values()
    bad = C.c_int64(-1)
    capi.check(L.wpf_check_conversions(v.ctypes.data_as(capi.DP), v.size, C.byref(bad)),
               "wpf_check_conversions")
    assert bad.value == 0


def test_newton_reciprocal_within_two_ulp():
    from mizuho_edit_gb300 import capi
    L = capi.load()
    rng = np.random.default_rng(11)
    e = rng.uniform(-1070.0, 1020.0, 400000)
    parts = [
        rng.choice([-1.0, 1.0], e.size) * rng.uniform(1.0, 2.0, e.size) * 2.0 ** np.floor(e),
        rng.uniform(1e-13, 1e-9, 100000),            # permeability sums of the harmonic means
        rng.uniform(1.0, 2.0, 100000),
        # both sides of the guard exponents 2^-1000 and 2^1000, and the specials
        np.ldexp(rng.uniform(1.0, 2.0, 2000), rng.integers(-1003, -997, 2000)),
        np.ldexp(rng.uniform(1.0, 2.0, 2000), rng.integers(997, 1003, 2000)),
        np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                  np.finfo(np.float64).max, -np.finfo(np.float64).max, 1.0, -1.0, 0.5, 3.0]),
    ]
    v = np.ascontiguousarray(np.concatenate(parts), dtype=np.float64)
    ulp = C.c_int64(-1)
    bad = C.c_int64(-1)
    capi.check(L.wpf_check_reciprocal(v.ctypes.data_as(capi.DP), v.size, C.byref(ulp), C.byref(bad)),
               "wpf_check_reciprocal")
    print(f"refined reciprocal: largest distance from the IEEE 1/x {ulp.value} ulp over {v.size} values")
    assert bad.value == 0
    assert 0 <= ulp.value <= 2


def test_fp64_rate():
    """The FP64 FMA throughput probe returns a rate in the range a GB300 can
    have (spec sheet ~1.25 TFLOP/s; the bound is loose on purpose), twice the
    same to 10 %."""
    import ctypes as C
    from mizuho_edit_gb300 import capi
    L = capi.load()
    a, b = C.c_double(), C.c_double()
    capi.check(L.wpf_measure_fp64_rate(C.byref(a)), "wpf_measure_fp64_rate")
    capi.check(L.wpf_measure_fp64_rate(C.byref(b)), "wpf_measure_fp64_rate")
    print(f"FP64 FMA rate: {a.value:.3f} and {b.value:.3f} TFLOP/s")
    assert 0.2 < a.value < 20.0
    assert abs(a.value - b.value) <= 0.1 * a.value
