"""CPU: the per-block dump format of SolverTest's LocalScalar3D::Dump/Load
(file names, 5-int header, padded brick) and the restart from blocks with
half the cells per axis (injection, sf3d_copy_x2)."""
import os

import numpy as np
import pytest

from bcmtools_gb300.dump import dump_path, read_blocks, write_blocks


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_round_trip_and_file_layout(tmp_path, dtype):
    vc, n = 2, (8, 6, 4)
    shape = (3, n[2] + 2 * vc, n[1] + 2 * vc, n[0] + 2 * vc)
    a = np.random.default_rng(1).uniform(-1, 1, size=shape).astype(dtype)
    write_blocks(a, vc, str(tmp_path), "p", 42, rank=3)
    path = dump_path(str(tmp_path), "p", 3, 1, 42)
    assert os.path.basename(path) == "dump-p-00003-00001-0000000042.bin"
    raw = open(path, "rb").read()
    assert list(np.frombuffer(raw[:20], np.int32)) == [8, 6, 4, 2, 1]
    assert len(raw) == 20 + a[1].size * np.dtype(dtype).itemsize
    assert np.array_equal(np.frombuffer(raw[20:], dtype), a[1].ravel())
    b = read_blocks(shape, vc, str(tmp_path), "p", 42, rank=3, dtype=dtype)
    assert np.array_equal(a, b)


def test_restart_from_half_size_blocks_injects(tmp_path):
    vc = 1
    coarse = np.random.default_rng(2).uniform(size=(2, 4 + 2, 4 + 2, 4 + 2))
    write_blocks(coarse, vc, str(tmp_path), "x", 0)
    fine_shape = (2, 8 + 2, 8 + 2, 8 + 2)
    start = np.full(fine_shape, -7.0)
    got = read_blocks(fine_shape, vc, str(tmp_path), "x", 0, dtype=np.float64, out=start.copy())
    for b in range(2):
        for k in range(8):
            for j in range(8):
                for i in range(8):
                    assert got[b, k + 1, j + 1, i + 1] == coarse[b, k // 2 + 1, j // 2 + 1, i // 2 + 1]
    # ghosts are left as they were
    assert np.all(got[:, 0] == -7.0) and np.all(got[:, :, :, -1] == -7.0)


def test_mismatched_blocks_are_rejected(tmp_path):
    write_blocks(np.zeros((1, 7, 7, 7)), 1, str(tmp_path), "x", 0)
    with pytest.raises(ValueError):
        read_blocks((1, 9, 9, 9), 2, str(tmp_path), "x", 0, dtype=np.float64)
    with pytest.raises(ValueError):
        read_blocks((1, 8, 8, 8), 1, str(tmp_path), "x", 0, dtype=np.float64)
