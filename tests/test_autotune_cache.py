"""Host logic of the autotuner front end: cache keys, hits and misses, a
corrupt cache file, with a fake solver in place of the library."""
import json

from xpbd_gb300 import autotune


class FakeSolver:
    LAUNCH_SLOTS = ("vertex_block", "hash_block", "prim_lanes", "warp_block", "query_block", "group_lanes",
                    "group_block", "dynamic_block", "fast_ee_form", "fused_frame", "tri_lanes", "neighbor_lanes")

    def __init__(self, vertices=1000):
        self.info = {"cloths": 2, "vertices": vertices, "edges": 2900, "triangles": 1900, "fast": 1, "strict": 1,
                     "dynamic": 0, "sdf": 0}
        self.config = dict(zip(self.LAUNCH_SLOTS, (128, 256, 8, 256, 256, 8, 256, 128, 32, 1, 8, 2)))
        self.native_calls = 0

    def solver_info(self):
        return dict(self.info)

    def launch_config(self):
        return dict(self.config)

    def set_launch_config(self, cfg):
        self.config.update(cfg)

    def _autotune_native(self, substeps, iterations, rounds):
        self.native_calls += 1
        self.config["prim_lanes"] = 16
        self.config["vertex_block"] = 64
        return 9.5, 10.0


def test_miss_then_hit(tmp_path):
    path = str(tmp_path / "tune.json")
    s = FakeSolver()
    r = autotune.tune(s, 10, 2, path=path)
    assert not r["cached"] and s.native_calls == 1
    assert r["config"]["prim_lanes"] == 16 and r["tuned_ms"] == 9.5 and r["default_ms"] == 10.0
    s2 = FakeSolver()
    r2 = autotune.tune(s2, 10, 2, path=path)
    assert r2["cached"] and s2.native_calls == 0
    assert s2.config["prim_lanes"] == 16 and s2.config["vertex_block"] == 64


def test_key_depends_on_workload_and_schedule(tmp_path):
    path = str(tmp_path / "tune.json")
    autotune.tune(FakeSolver(), 10, 2, path=path)
    other = FakeSolver(vertices=2000)
    assert not autotune.tune(other, 10, 2, path=path)["cached"]
    assert not autotune.tune(FakeSolver(), 5, 2, path=path)["cached"]
    assert len(json.load(open(path))) == 3


def test_corrupt_cache_is_remeasured(tmp_path):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    s = FakeSolver()
    r = autotune.tune(s, 10, 2, path=str(path))
    assert not r["cached"] and s.native_calls == 1
    assert isinstance(json.load(open(path)), dict)


def test_no_cache_always_measures(tmp_path):
    path = str(tmp_path / "tune.json")
    s = FakeSolver()
    autotune.tune(s, 10, 2, path=path, use_cache=False)
    autotune.tune(s, 10, 2, path=path, use_cache=False)
    assert s.native_calls == 2


def test_cache_path_from_environment(monkeypatch, tmp_path):
    monkeypatch.setenv("XPBD_GB300_TUNE_CACHE", str(tmp_path / "x.json"))
    assert autotune.cache_path() == str(tmp_path / "x.json")
