"""The integer-pipe double division and square root (dev_fpint.cuh) used by the
SPH passes and the tree moments, against the compiler's correctly rounded
operators on the GPU, bit for bit (csg_check_div_sqrt): 2^26 seeded operand
pairs per seed over moderate and extreme exponents, arbitrary bit patterns
(zeros, subnormals, infinities, NaNs), exact quotients and ties, power-of-two
divisors, signed zeros and SPH-like operands. Bar: zero mismatches."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 0x5EED0000])
def test_division_and_sqrt_match_the_compiler_bit_for_bit(lib, seed):
    bad_div, bad_sqrt = lib.check_div_sqrt(1 << 26, seed)
    assert (bad_div, bad_sqrt) == (0, 0)
