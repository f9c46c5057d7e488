"""The allocation-free cell sort (xpbi_sort_cells_noalloc) against the
substep's own sort: same cell starts and permutation, bit for bit, on two
calls in a row that share the library's fixed scratch array.

The file is named to be collected last, so the entry point also runs after
every other test has used the device."""
import ctypes as C
import importlib

import numpy as np
import pytest

MAX_N = 262144
MAX_CELLS = 1048576


def _abi():
    return importlib.import_module("xpbi-webgpu_gb300._abi")


def _grid(sim):
    pw, _ = sim.uniforms(0)
    origin = np.frombuffer(pw[0:3].tobytes(), np.float32).copy()
    cs = float(np.frombuffer(pw[3:4].tobytes(), np.float32)[0])
    dims = pw[4:7].astype(np.int32)
    return origin, cs, dims


def _call(pos_dev, n, origin, cs, dims, cell_start, sorted_idx, stream):
    abi = _abi()
    o = (C.c_float * 3)(*origin.tolist())
    d = (C.c_int32 * 3)(*dims.tolist())
    return abi.lib().xpbi_sort_cells_noalloc(C.c_void_p(pos_dev), n, o, C.c_float(cs), d,
                                             C.c_void_p(cell_start), C.c_void_p(sorted_idx),
                                             C.c_void_p(stream))


def _sorted_by_rule(pos, origin, cs, dims):
    """Cell order with descending index inside a cell, in f32 arithmetic."""
    cell = np.floor((pos[:, :3] - origin[None, :]) / np.float32(cs))
    cell = np.clip(cell, 0, (dims - 1)[None, :].astype(np.float32)).astype(np.int64)
    key = cell[:, 0] + cell[:, 1] * dims[0] + cell[:, 2] * dims[0] * dims[1]
    idx = np.arange(len(pos))
    return np.lexsort((-idx, key)).astype(np.uint32), key


def _two_calls(torch, inputs, grid):
    """Enqueue the entry point on each input back to back, then read all."""
    origin, cs, dims = grid
    cells = int(np.prod(dims.astype(np.int64)))
    stream = torch.cuda.current_stream().cuda_stream
    outs = []
    for pos in inputs:
        n = len(pos)
        p = torch.from_numpy(np.ascontiguousarray(pos, np.float32)).cuda()
        cs_out = torch.full((cells + 1,), 0xDEAD, dtype=torch.int32, device="cuda")
        si_out = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        rc = _call(p.data_ptr(), n, origin, cs, dims, cs_out.data_ptr(), si_out.data_ptr(), stream)
        assert rc == 0, _abi().lib().xpbi_last_error()
        assert _status(stream) == 0, _abi().lib().xpbi_last_error()  # no wait ran out
        outs.append((p, cs_out, si_out))
    torch.cuda.synchronize()
    return [(c.cpu().numpy().view(np.uint32), s.cpu().numpy().view(np.uint32)) for _, c, s in outs]


def _status(stream):
    return _abi().lib().xpbi_sort_cells_noalloc_status(C.c_void_p(stream))


@pytest.mark.gpu
def test_noalloc_sort_matches_substep_sort(xp, built_lib):
    torch = pytest.importorskip("torch")
    sc = xp.scenes.config_dam_breach(scale=0.25)  # 250,000 particles, 579,081 cells
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        sim.step(20, sc["iterations"], sc["hasWater"])
        grid = _grid(sim)
        inputs, expect = [], []
        for _ in range(2):
            inputs.append(sim.read_state()["pos"])
            sim.encode_substep(sc["iterations"], sc["hasWater"])
            st = sim.read_state()
            expect.append((st["cellTab"], st["sortedIdx"]))
    n = len(inputs[0])
    assert n <= MAX_N and len(expect[0][0]) <= MAX_CELLS
    assert not np.array_equal(inputs[0], inputs[1])
    got = _two_calls(torch, inputs, grid)
    for (cell_start, sorted_idx), (cell_tab, ref_idx) in zip(got, expect):
        C_ = len(cell_tab)
        assert np.array_equal(cell_start[:C_], cell_tab)
        assert cell_start[C_] == n
        assert np.array_equal(sorted_idx, ref_idx)


@pytest.mark.gpu
def test_noalloc_sort_crowded_cells(xp, built_lib):
    """Buckets past the shared-memory sort (9,000 members) and between the
    rank rule and it (300 members), against the substep and the sort rule."""
    torch = pytest.importorskip("torch")
    sc = xp.scenes.config_dam_breach(scale=0.05)
    rng = np.random.default_rng(7)
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        origin, cs, dims = grid = _grid(sim)
        pos = sim.read_state()["pos"].copy()
        corner = origin + cs * np.array([dims[0] // 2, 3, dims[2] // 2], np.float32)
        pos[:9000, :3] = corner + cs * rng.uniform(0.1, 0.9, (9000, 3)).astype(np.float32)
        pos[20000:20300, :3] = corner + cs * (np.array([2, 0, 0], np.float32)
                                              + rng.uniform(0.1, 0.9, (300, 3)).astype(np.float32))
        sim.write_state(0, pos=pos)
        sim.encode_substep(sc["iterations"], sc["hasWater"])
        st = sim.read_state()
    want, key = _sorted_by_rule(pos, origin, cs, dims)
    assert np.bincount(key).max() >= 9000
    got = _two_calls(torch, [pos, pos], grid)
    for cell_start, sorted_idx in got:
        assert np.array_equal(sorted_idx, st["sortedIdx"])
        assert np.array_equal(sorted_idx, want)
        assert np.array_equal(cell_start[:-1], st["cellTab"])


def test_noalloc_sort_rejects_out_of_range(xp, built_lib):
    """Argument checks return before any device work (no GPU needed)."""
    abi = _abi()
    origin = np.zeros(3, np.float32)
    dims = np.array([8, 8, 8], np.int32)
    fake = 1 << 20  # aligned, never dereferenced: every call below is rejected
    cases = [
        (fake, MAX_N + 1, dims, fake, fake),             # too many particles
        (fake, 0, dims, fake, fake),                     # nothing to sort
        (fake, 16, np.array([1024, 1024, 2], np.int32), fake, fake),  # too many cells
        # products that wrap a 64-bit (or 32-bit) count if formed before the check
        (fake, 16, np.array([1 << 22, 1 << 22, 1 << 20], np.int32), fake, fake),
        (fake, 16, np.array([2**31 - 1] * 3, np.int32), fake, fake),
        (fake, 16, np.array([1 << 16, 1 << 16, 1], np.int32), fake, fake),
        (fake, 16, np.array([0, 8, 8], np.int32), fake, fake),        # empty grid
        (fake + 4, 16, dims, fake, fake),                # misaligned positions
        (fake, 16, dims, fake + 4, fake),                # misaligned cell starts
        (0, 16, dims, fake, fake),                       # NULL
    ]
    for pos, n, d, cs_out, si_out in cases:
        rc = _call(pos, n, origin, 0.1, d, cs_out, si_out, 0)
        assert rc == abi.ERR_INVALID, (n, d)
        assert abi.lib().xpbi_last_error()
    assert _call(fake, 16, origin, 0.0, dims, fake, fake, 0) == abi.ERR_INVALID


@pytest.mark.gpu
def test_noalloc_expired_wait_is_reported(xp, built_lib):
    """A bounded look-back wait that runs out inside the fixed scratch array
    reaches the caller through xpbi_sort_cells_noalloc_status (not as a
    silently wrong permutation), the word is cleared, and the next sort runs
    as before. The wait is the scan's own helper on a descriptor nothing
    publishes, with a short limit: nothing faults or spins without one."""
    torch = pytest.importorskip("torch")
    abi = _abi()
    stream = torch.cuda.current_stream().cuda_stream
    sc = xp.scenes.config_dam_breach(scale=0.05)
    with xp.Simulation(sc) as sim:
        sim.write_params(xp.params_for(sc))
        grid = _grid(sim)
        sim.encode_substep(sc["iterations"], sc["hasWater"])
        st = sim.read_state()
    pos = st["pos"]
    assert abi.lib().xpbi_test_noalloc_wait_expiry(1000, C.c_void_p(stream)) == 0
    assert _status(stream) == abi.ERR_DEVICE
    assert b"look-back" in abi.lib().xpbi_last_error()
    assert _status(stream) == 0  # read and cleared
    want, _ = _sorted_by_rule(pos, *grid)
    (cell_start, sorted_idx), = _two_calls(torch, [pos], grid)
    assert np.array_equal(sorted_idx, want)
    assert cell_start[-1] == len(pos)
    for bad in (0, (1 << 20) + 1):
        assert abi.lib().xpbi_test_noalloc_wait_expiry(bad, C.c_void_p(stream)) == abi.ERR_INVALID
