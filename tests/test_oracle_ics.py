"""The oracle's seeded initial conditions equal the library's, byte for byte.

The CPU baseline and the reference arm of the benchmark draw their bodies
with orc_generate_ics so that they never load the product library; that is
only valid if both generators produce the same Body[] for every kind, count
and seed. Host code on both sides: runs without a GPU.
"""
import numpy as np
import pytest

from conftest import same_bytes


@pytest.mark.parametrize("kind", range(7))
@pytest.mark.parametrize("n,seed", [(0, 1), (1, 2), (2, 0), (1000, 0x5EED0000), (3001, 77)])
def test_oracle_ics_equal_library_ics(lib, orc, kind, n, seed):
    got = orc.generate_ics(kind, n, seed)
    want = lib.generate_ics(kind, n, seed)
    assert len(got) == len(want) == n
    assert same_bytes(got, want)


def test_oracle_ics_equal_library_ics_at_benchmark_size(lib, orc):
    # the 100k merger of the default benchmark line, and the 1M bulge + disk
    for kind, n in ((1, 100_000), (2, 1_000_000)):
        assert same_bytes(orc.generate_ics(kind, n, 0x5EED0000), lib.generate_ics(kind, n, 0x5EED0000))


def test_oracle_ics_reject_bad_arguments(orc):
    with pytest.raises(ValueError):
        orc.generate_ics(7, 10, 1)
    with pytest.raises(ValueError):
        orc.generate_ics(0, -1, 1)
