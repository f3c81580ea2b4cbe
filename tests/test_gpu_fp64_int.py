"""The integer-pipe FP64 division, square root and exact scalings against the GPU's own IEEE operations.

The solvers' per-contact law work (Fischer-Burmeister residual, cone projection, De Saxce change of variable)
divides and takes square roots on the integer pipe; the iterates match the oracle bit for bit only if these
operations round exactly as IEEE prescribes. 2^26 generated operands per seed: random bit patterns,
exponents near 1, extreme mantissas, quotients and roots close to exact.
"""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [0, 0x5EED])
def test_integer_pipe_ops_match_hardware(seed):
    import bogus_gpu

    assert bogus_gpu.check_fp64_ops(1 << 26, seed) == (0, 0, 0)


def test_check_rejects_bad_arguments():
    import bogus_gpu

    with pytest.raises(bogus_gpu.BogusGpuError):
        bogus_gpu.check_fp64_ops(-1)
