"""The LDL^T solve's shared-reciprocal division against the IEEE division (needs a GPU).

The solve divides by each pivot through its reciprocal (rcp.approx refined by one Newton step)
and Markstein's fused-multiply-add correction, for operands in [2^-60, 2^61); parity with the
oracle needs the bits of the IEEE division. The reciprocal is compared with 1/d for every float of
that range, and the quotients on seeded operand pairs over the whole float range, over the
step's range, on divisors with all-ones or near-power-of-two mantissas and on solver-like values:
no result may differ in any bit.
"""
import ctypes as C

import pytest

from avbd_gb300 import _lib as L

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 0xA5BD])
def test_shared_reciprocal_division_is_the_ieee_division(seed):
    rcp, quo = C.c_int64(-1), C.c_int64(-1)
    L.check(L.lib().avbd_check_division(0, 1 << 30, seed, C.byref(rcp), C.byref(quo)))
    assert rcp.value == 0, f"{rcp.value} reciprocals differ from 1/d"
    assert quo.value == 0, f"{quo.value} quotients differ from the IEEE division"
