"""PC2 streaming writer on the GPU: the file format of the reference's bake
(header bytes, float32 local positions per sample), samples equal to the
downloaded positions through the reference's float32 object-local transform,
written while the solver keeps stepping; an uncommitted close leaves no
file."""
import os

import numpy as np
import pytest

from xpbd_gb300 import pc2, scene
from xpbd_gb300.native import NativeXpbdBatch, NativeXpbdSolver

pytestmark = pytest.mark.gpu


def _matrix():
    c, s = np.cos(0.3), np.sin(0.3)
    m = np.eye(4, dtype=np.float32)
    m[:3, :3] = [[c, -s, 0], [s, c, 0], [0, 0, 1]]
    m[:3, 3] = [0.25, -0.5, 1.0]
    return m


@pytest.mark.parametrize("use_matrix", [False, True], ids=["world", "local"])
def test_pc2_matches_downloads(use_matrix, gpu_lib, tmp_path):
    sc = scene.plain_grid_scene(24, 8)
    solver = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    path = str(tmp_path / "cloth_xpbd.pc2")
    m = _matrix() if use_matrix else None
    w = pc2.Pc2Writer(solver, path, start_frame=5)
    expect = []
    for f in range(8):
        solver.step(10, 2, diagnostics=False, synchronize=False)
        w.write(m)
        expect.append(solver.download_positions().copy())
    assert w.close() == 8
    assert os.path.exists(path) and not os.path.exists(path + ".realtime.tmp")
    hdr, data = pc2.read_pc2(path)
    assert hdr == {"magic": b"POINTCACHE2\0", "version": 1, "vertex_count": 24 * 24, "start_frame": 5.0,
                   "sample_rate": 1.0, "samples": 8}
    for f, pos in enumerate(expect):
        if m is None:
            assert np.array_equal(data[f], pos)
        else:
            np.testing.assert_allclose(data[f], pc2.to_local(pos, m), rtol=0, atol=2e-6)


def test_pc2_batch_cloth_and_discard(gpu_lib, tmp_path):
    scs = scene.batched_scenes(3, seed=2, frames=3, side_range=(10, 20))
    batch = NativeXpbdBatch([(s.cloth, s.options, s.static_triangles) for s in scs])
    path = str(tmp_path / "b.pc2")
    w = pc2.Pc2Writer(batch, path, start_frame=1, cloth=2)
    for _ in range(3):
        batch.step(10, 2, diagnostics=False, synchronize=False)
        w.write()
    last = batch.download_cloth_positions(2).copy()
    assert w.close() == 3
    hdr, data = pc2.read_pc2(path)
    assert hdr["vertex_count"] == len(scs[2].cloth.positions_world) and hdr["samples"] == 3
    assert np.array_equal(data[-1], last)
    # an uncommitted writer removes its temporary file
    tmp = str(tmp_path / "x.pc2")
    w2 = pc2.Pc2Writer(batch, tmp, start_frame=0, cloth=0)
    w2.write()
    w2.close(commit=False)
    assert not os.path.exists(tmp) and not os.path.exists(tmp + ".realtime.tmp")
