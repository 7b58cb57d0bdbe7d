"""The FP64 throughput probe behind the bench's FP64 roofline: both DFMA
streams measured, positive and finite, and neither above the pipe's peak of
two DFMAs per SM per clock (the update stream must not outrun the FMA
stream by more than noise: a probe whose products the compiler hoisted out
of its loop would report about twice the FMA stream's rate)."""
import ctypes as C
import math

import pytest

pytestmark = pytest.mark.gpu


def test_fp64_rates(gpu):
    import torch
    from sympiler_gb300._lib import OK, lib
    u, f = C.c_double(), C.c_double()
    assert lib().gbsym_fp64_rates(C.byref(u), C.byref(f), None) == OK
    assert math.isfinite(u.value) and math.isfinite(f.value)
    assert 10.0 < f.value < 1e5 and 10.0 < u.value < 1e5
    assert u.value < 1.1 * f.value
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert f.value < 1.05 * 2 * sms * 2.2  # G op/s: 2 DFMA per SM per clock, clock < 2.2 GHz
    assert lib().gbsym_fp64_rates(None, C.byref(f), None) != OK
