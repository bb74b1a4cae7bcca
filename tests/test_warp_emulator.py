"""The host stand-in for Warp that generates tests/golden/warp_reference.npz (test infrastructure):
its launch, by-reference hash-grid query, FP32 arithmetic and wp.utils semantics."""

import importlib.util
from pathlib import Path

import numpy as np


def _emu():
    path = Path(__file__).resolve().parent / "golden" / "warp_emulator.py"
    spec = importlib.util.spec_from_file_location("warp_emulator_under_test", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_launch_converts_scalars_and_runs_every_thread():
    wp = _emu()

    @wp.kernel
    def k(out: wp.array(dtype=wp.float32), a: wp.float32, n: wp.int32):
        i = wp.tid()
        out[i] = a * wp.float32(i) + wp.float32(n)

    out = wp.zeros(5, dtype=wp.float32)
    wp.launch(k, dim=5, inputs=[out, 0.1, 3])
    expect = np.float32(0.1) * np.arange(5, dtype=np.float32) + np.float32(3)
    np.testing.assert_array_equal(out.numpy(), expect)
    assert out.numpy().dtype == np.float32

    @wp.kernel
    def k2(out: wp.array3d(dtype=wp.float32)):
        j, i = wp.tid()
        out[j, i, 0] = wp.float32(10 * j + i)

    o2 = wp.zeros((2, 3, 1), dtype=wp.float32)
    wp.launch(k2, dim=(2, 3), inputs=[o2])
    np.testing.assert_array_equal(o2.numpy()[..., 0], [[0, 1, 2], [10, 11, 12]])


def test_hash_grid_query_writes_its_index_argument_and_covers_the_radius():
    wp = _emu()
    rng = np.random.default_rng(0)
    pts = rng.uniform(-3, 3, size=(200, 3)).astype(np.float32)
    pts[:, 2] = 0
    arr = wp.array(pts, dtype=wp.vec3)
    grid = wp.HashGrid(128, 128, 1)
    grid.build(points=arr, radius=1.0)
    for q in rng.uniform(-3, 3, size=(20, 2)):
        p = np.array([q[0], q[1], 0], np.float32)
        query = wp.hash_grid_query(grid.id, p, 1.0)
        idx = wp.int32(0)
        seen = []
        while wp.hash_grid_query_next(query, idx):
            seen.append(int(idx))
        assert seen == sorted(seen)  # increasing point index
        d = np.array([wp.length(pts[i] - p) for i in range(len(pts))])
        assert set(np.flatnonzero(d <= 1.0)) <= set(seen)  # every point the kernel's test accepts


def test_int32_cells_behave_as_int32_and_float32_rounds_each_operation():
    wp = _emu()
    m = wp.int32(0)
    m = m | (wp.int32(1) << np.int32(3))
    assert int(m) == 8 and ((m >> 3) & wp.int32(1)) == wp.int32(1)
    k = wp.int32(0)
    k += 1
    assert k == 1
    a, b = np.float32(1e8), np.float32(1.0)
    assert wp.dot(np.array([a, b], np.float32), np.array([b, b], np.float32)) == np.float32(np.float32(a) + b)


def test_utils_sort_is_stable_and_runs_and_scan_match_numpy():
    wp = _emu()
    keys = wp.array(np.array([3, 1, 3, 2, 1, 3, 9, 9], np.int32), dtype=wp.int32)
    vals = wp.array(np.arange(8, dtype=np.int32), dtype=wp.int32)
    wp.utils.radix_sort_pairs(keys, vals, 6)
    np.testing.assert_array_equal(keys.numpy()[:6], [1, 1, 2, 3, 3, 3])
    np.testing.assert_array_equal(vals.numpy()[:6], [1, 4, 3, 0, 2, 5])
    rv, rl, rc = (wp.zeros(6, dtype=wp.int32) for _ in range(3))
    wp.utils.runlength_encode(keys, rv, rl, rc, value_count=6)
    assert int(rc.numpy()[0]) == 3
    np.testing.assert_array_equal(rv.numpy()[:3], [1, 2, 3])
    np.testing.assert_array_equal(rl.numpy()[:3], [2, 1, 3])
    off = wp.zeros(6, dtype=wp.int32)
    wp.utils.array_scan(rl, off, inclusive=False)
    np.testing.assert_array_equal(off.numpy()[:4], [0, 2, 3, 6])
