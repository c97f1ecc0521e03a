"""The step kernel's binary64 division, square root, comparisons, fmin / fmax
and power-of-two scalings run on the integer pipes (fv2d_gb300/csrc/softfp.cuh).
They must return exactly the bits of the hardware instructions: checked here
on the GPU for 2^29 generated operand sets per operation (random significands,
arbitrary bit patterns including zeros, subnormals, infinities and NaNs, exact
and near-tie quotients, perfect squares +- 1 ulp, significands next to a power
of two, extreme exponents, equal and opposite operand pairs)."""
import pytest

pytestmark = pytest.mark.gpu


NAMES = {0: "division", 1: "sqrt", 2: "comparisons", 3: "fmax/fmin", 4: "power-of-two scaling", 5: "multiplication"}


@pytest.mark.parametrize("op", sorted(NAMES))
def test_integer_pipe_arithmetic_matches_hardware(gpu_lib, op):
    import fv2d_gb300 as fv
    for seed in (1, 2):
        bad, ex = fv.selftest_arith(op, 1 << 28, seed)
        assert bad == 0, (NAMES[op], ex)
