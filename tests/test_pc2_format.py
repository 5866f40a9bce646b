"""PC2 reader against a file packed the way the reference's bake writes it
(session_manager.py:4624-4643)."""
import struct

import numpy as np

from xpbd_gb300 import pc2


def test_reader_and_transform(tmp_path):
    path = tmp_path / "c.pc2"
    world = np.random.default_rng(0).normal(size=(3, 5, 3)).astype(np.float32)
    m = np.eye(4, dtype=np.float32)
    m[:3, 3] = [1.0, 2.0, 3.0]
    with open(path, "wb") as f:
        f.write(struct.pack("<12siiffi", b"POINTCACHE2\0", 1, 5, 7.0, 1.0, 3))
        for s in world:
            f.write(np.ascontiguousarray(pc2.to_local(s, m), dtype="<f4").tobytes())
    hdr, data = pc2.read_pc2(str(path))
    assert hdr["magic"] == b"POINTCACHE2\0" and hdr["vertex_count"] == 5 and hdr["samples"] == 3
    assert hdr["start_frame"] == 7.0 and hdr["sample_rate"] == 1.0
    np.testing.assert_array_equal(data, world + np.float32([1.0, 2.0, 3.0]))
