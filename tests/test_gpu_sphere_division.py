"""The sphere-normal kernel divides four numerators by one denominator through the
denominator's correctly rounded reciprocal and one exact-remainder correction per
quotient (Markstein's theorem): every quotient must equal the correctly rounded
division -- over 2^32 pseudo-random pairs of all signs and exponents -64..63, and
over every positive dividend for divisors around the kernel's (patch norms of
~1e6-1e7 m, weights near 1) and near powers of two."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_shared_denominator_quotients_are_correctly_rounded(gpu):
    divisors = np.array([1.0, 3.0, 0.7, 6.4e6, 1234567.875, 1e-3, 1.0 - 2.0 ** -24, 1.0 + 2.0 ** -23, 5.0e7],
                        np.float32)
    bad, first = C.c_ulonglong(), C.c_ulonglong()
    gpu.check(gpu.lib().tp_sphere_division_self_test(1 << 32, 2024, divisors.ctypes.data_as(C.POINTER(C.c_float)),
                                                     len(divisors), C.byref(bad), C.byref(first)))
    assert bad.value == 0, "%d quotients differ (first index %d)" % (bad.value, first.value)
