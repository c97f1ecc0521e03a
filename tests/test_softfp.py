"""The step kernel's binary64 division and square root run on the integer
pipes (fv2d_gb300/csrc/softfp.cuh).  They must return exactly the bits of the
hardware x / y and sqrt(x): checked here on the GPU for 2^29 generated operand
sets per operation (random significands, arbitrary bit patterns including
zeros, subnormals, infinities and NaNs, exact and near-tie quotients, perfect
squares +- 1 ulp, extreme exponents)."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("op", [0, 1])
def test_integer_pipe_arithmetic_matches_hardware(gpu_lib, op):
    import fv2d_gb300 as fv
    for seed in (1, 2):
        bad, ex = fv.selftest_arith(op, 1 << 28, seed)
        assert bad == 0, ("division" if op == 0 else "sqrt", ex)
