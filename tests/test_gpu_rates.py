"""The FP64 throughput probe behind the bench's FP64 roofline: both forms
measured, positive and finite, and the update form (a rounded product and a
rounded difference) not slower than general three-operand FMAs."""
import ctypes as C
import math

import pytest

pytestmark = pytest.mark.gpu


def test_fp64_rates(gpu):
    from sympiler_gb300._lib import OK, lib
    u, f = C.c_double(), C.c_double()
    assert lib().gbsym_fp64_rates(C.byref(u), C.byref(f), None) == OK
    assert math.isfinite(u.value) and math.isfinite(f.value)
    assert 10.0 < f.value < 1e5 and 10.0 < u.value < 1e5
    assert u.value > 0.9 * f.value
    assert lib().gbsym_fp64_rates(None, C.byref(f), None) != OK
