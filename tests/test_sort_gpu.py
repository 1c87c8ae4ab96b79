"""The tree build's key sort (csg_sort_keys) against a CPU sort of the same keys.

The build orders bodies by 63-bit octant keys with an LSD radix sort (8 bits a
pass, single-pass tiles with decoupled look-back). Bar: bit-exact keys and the
stable permutation of numpy's stable argsort, on both tile sizes (1024 keys
below 2M keys, 4096 from 2M), ragged tile ends, duplicates, constant keys and
partial key widths.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def check(lib, keys, bits=64):
    got, idx = lib.sort_keys(keys, bits)
    want = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(idx, want.astype(np.int32))
    np.testing.assert_array_equal(got, keys[want])


@pytest.mark.parametrize("n", [1, 2, 31, 1023, 1024, 1025, 4097, 100_003])
def test_random_keys(lib, n):
    rng = np.random.default_rng(n)
    check(lib, rng.integers(0, 2 ** 63, n, dtype=np.uint64) * np.uint64(2)
          + rng.integers(0, 2, n, dtype=np.uint64))


def test_large_tiles_with_duplicates(lib):
    """2.1M keys (4096-key tiles), heavy duplication: stability is visible."""
    rng = np.random.default_rng(7)
    check(lib, rng.integers(0, 5000, 2_100_000, dtype=np.uint64) << np.uint64(40))


def test_constant_and_reversed(lib):
    check(lib, np.full(70_000, 0xDEADBEEF, dtype=np.uint64))
    check(lib, np.arange(70_000, dtype=np.uint64)[::-1].copy() << np.uint64(17))


def test_partial_widths(lib):
    rng = np.random.default_rng(3)
    for bits in (1, 8, 12, 31):
        check(lib, rng.integers(0, 2 ** bits, 50_000, dtype=np.uint64), bits)


def test_octant_keys_of_a_merger(lib):
    """Keys with the structure of the build's octant keys: 63-bit, clustered."""
    rng = np.random.default_rng(11)
    c = rng.integers(0, 2 ** 40, 64, dtype=np.uint64) << np.uint64(23)
    k = c[rng.integers(0, 64, 300_000)] | rng.integers(0, 2 ** 23, 300_000, dtype=np.uint64)
    check(lib, k)


def test_empty_and_bad_arguments(lib):
    got, idx = lib.sort_keys(np.zeros(0, dtype=np.uint64))
    assert len(got) == 0 and len(idx) == 0
    with pytest.raises(lib.CudaError):
        lib.sort_keys(np.zeros(4, dtype=np.uint64), bits=0)
    # a refused call leaves nothing behind for the next call on this thread
    check(lib, np.arange(5, dtype=np.uint64)[::-1].copy())
    pool, size = lib.octree_build(lib.generate_ics(0, 200, 1))
    assert size > 0
