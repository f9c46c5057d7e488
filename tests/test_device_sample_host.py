"""The device scene sampler's generator on the CPU: the library's
Philox-4x32-10 (xpbi_philox4x32_10, the function its sampling kernel uses)
against the published known-answer vectors and the Python restatement in
oracle/philox.py. No GPU needed."""
import importlib

import numpy as np

from oracle import philox as P

# Known-answer vectors of Philox-4x32-10 (counter, key -> output) published
# with the generator by its authors.
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


def test_oracle_philox_matches_the_published_vectors():
    for c, k, want in KAT:
        assert tuple(P.philox4x32_10(c, k)) == want


def test_library_philox_matches_the_oracle(built_lib):
    ds = importlib.import_module("xpbi-webgpu_gb300.device_sample")
    for c, k, want in KAT:
        assert tuple(int(x) for x in ds.philox(c, k)) == want
    rng = np.random.default_rng(5)
    for _ in range(200):
        c = rng.integers(0, 2 ** 32, 4, dtype=np.uint64)
        k = rng.integers(0, 2 ** 32, 2, dtype=np.uint64)
        assert [int(x) for x in ds.philox(c, k)] == P.philox4x32_10(c, k)


def test_sampler_rejects_bad_shapes(xp, built_lib):
    ds = importlib.import_module("xpbi-webgpu_gb300.device_sample")
    import pytest
    inf, nan = float("inf"), float("nan")
    for bad in (dict(kind=7, mat_id=0), ds.sphere([0, 0, 0], -1.0, 0), ds.box([0, 0, 0], [-1, 1, 1], 0),
                ds.box([-inf, 0, 0], [-inf, 1, 1], 0), ds.box([0, 0, 0], [nan, 1, 1], 0),
                ds.sphere([inf, 0, 0], 0.1, 0), ds.sphere([0, nan, 0], 0.1, 0)):
        with pytest.raises(xp.XpbiError) as e:
            ds.sample_shapes([bad], 0.01)
        assert e.value.code == 1
