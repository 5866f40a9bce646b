"""Parity with the reference solver itself, run on the same GPU.

The reference's own CUDA solver (native/src/ssbl_xpbd_cuda_abi41.cu, built
unchanged with its own flags by oracle/build_ref.py) and this repository's
library receive byte-identical ABI41 configs, meshes and pins through the
same ctypes mirror.

* Integer structures (the spec rule: bit-exact on identical input
  positions): per-vertex cells, per-bucket pre-clamp counts and member
  multisets of the vertex, triangle and edge hashes, and the per-vertex
  vertex-vertex neighbour sets, read from the reference through the test-only
  probe (oracle/ref_probe.cu) and from the product through
  xpbd_gb300_read_buffer.  The reference fills buckets in atomic arrival
  order (abi41.cu:4568-4574) and keeps the first 32 arrivals, so members are
  compared as multisets, and a bucket over 32 as a subset of ours.
* Positions: the reference is nondeterministic (its stretch pass reads
  positions while other threads add float corrections to them,
  abi41.cu:1952-1978), so four reference runs are taken and their spread
  (the largest difference between two of them) is the noise floor.  After
  one substep and one frame the product's largest vertex error is within
  1e-4 of the cloth extent.  Over ten frames without contact it is within
  the larger of that and four noise floors.  In contact phases single
  vertices of the reference's own runs part by more than the tolerance, so
  there the mean vertex error must stay within 1e-4, the 99th percentile
  within ten of the reference's 99th-percentile spreads, and the largest
  error below 50 tolerances (a guard against gross errors).  The product's
  stretch pass is a deterministic snapshot gather where the reference's
  threads read positions that others are updating, so in contact phases
  the product parts from the reference by more than the reference's runs
  part from one another: on the 16-cloth batch sample after ten frames the
  99th percentile measured up to 5.7 spreads per cloth, and the same
  cloth 2.6-5.4 spreads from one set of four reference runs to the next; in fast mode the
  cluster filter also keeps the first contact in candidate order (atomic
  arrival in the reference, increasing id here).

Set XPBD_PARITY_REPORT to a file name to have the measured figures written
there as JSON.
"""
import json
import os

import numpy as np
import pytest

import ref_solver as R

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not R.available(), reason="reference comparator not built (oracle/build_ref.py)")]

TOL = 1.0e-4  # of the cloth extent
REPORT: dict = {}


def _record(key, value):
    REPORT[key] = value
    path = os.environ.get("XPBD_PARITY_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(REPORT, f, indent=1, sort_keys=True)
    print(key, value)


def _product(sc, **kw):
    from xpbd_gb300 import native

    return native.NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles, key_division="reference", **kw)


# --------------------------------------------------------------- integers --

def _folded(sc, seed, gap):
    rng = np.random.default_rng(seed)
    p = sc.cloth.positions_world.copy()
    right = p[:, 0] > 0.0
    p[right, 0] = -p[right, 0] + 0.001
    p[right, 2] += gap
    p[:, :2] += rng.uniform(-2e-4, 2e-4, (len(p), 2)).astype(np.float32)
    return np.ascontiguousarray(p, np.float32)


def _positions_after(sc, frames):
    g = _product(sc)
    for _ in range(frames):
        g.step(sc.substeps, sc.iterations, diagnostics=False)
    p = g.download_positions().copy()
    g.close()
    return p


def _compare_structures(sc, pos):
    g = _product(sc)
    r = R.RefSolver.from_scene(sc)
    try:
        if pos is not None:
            g.update_positions(pos)
            r.set_state(pos)
        g.build_self_structures()
        r.build_self_structures()
        V = len(sc.cloth.positions_world)
        info, cells = r.hash_info()
        hi = g.hash_info()
        assert list(hi[:3]) == list(info[:3]), (hi, info)
        assert list(hi[3:6]) == list(info[3:6]), (hi, info)
        stats = {}
        # vertex hash: cells and buckets
        gc = g.read_buffer(3, np.int32, 4 * V).reshape(V, 4)[:, :3]
        rc = r.read(R.VERTEX_CELLS, np.int32, 3 * V).reshape(V, 3)
        assert np.array_equal(gc, rc), int((gc != rc).any(axis=1).sum())
        for kind, (cnt_id, slot_id, start_id, nb) in {
            "vertex": (R.VERTEX_BUCKET_COUNTS, R.VERTEX_BUCKET_SLOTS, 4, int(info[0])),
            "triangle": (R.TRI_BUCKET_COUNTS, R.TRI_BUCKET_SLOTS, 6, int(info[1])),
            "edge": (R.EDGE_BUCKET_COUNTS, R.EDGE_BUCKET_SLOTS, 8, int(info[2])),
        }.items():
            rcount = r.read(cnt_id, np.int32, nb)
            rslots = r.read(slot_id, np.int32, nb * R.SLOTS).reshape(nb, R.SLOTS)
            start = g.read_buffer(start_id, np.int32, nb + 1)
            ent = g.read_buffer(start_id + 1, np.int32, max(int(start[-1]), 1))
            assert np.array_equal(np.diff(start), rcount), kind
            full = over = 0
            for b in np.flatnonzero(rcount):
                mine = ent[start[b]:start[b + 1]]
                theirs = rslots[b, :min(rcount[b], R.SLOTS)]
                if rcount[b] <= R.SLOTS:
                    assert np.array_equal(np.sort(mine), np.sort(theirs)), (kind, b)
                    full += 1
                else:
                    assert np.isin(theirs, mine).all() and len(np.unique(theirs)) == len(theirs), (kind, b)
                    over += 1
            stats[kind] = {"occupied": int(full + over), "over_32": int(over), "max": int(rcount.max()),
                           "entries": int(rcount.sum())}
        # vertex-vertex neighbour sets
        rn = r.read(R.NEIGHBOR_COUNTS, np.uint32, V).astype(np.int64)
        rs = r.read(R.NEIGHBOR_SLOTS, np.uint32, V * 32).reshape(V, 32)
        pn = g.read_buffer(10, np.int32, V).astype(np.int64)
        ps = g.read_buffer(11, np.int32, V * 32).reshape(V, 32)
        assert np.array_equal(np.minimum(pn, 32), np.minimum(rn, 32))
        full = 0
        for i in np.flatnonzero(rn):
            if rn[i] < 32:
                assert set(rs[i, :rn[i]].tolist()) == set(ps[i, :pn[i]].tolist()), i
                full += 1
        stats["neighbors"] = {"vertices": int((rn > 0).sum()), "pairs": int(rn.sum()), "at_32": int((rn >= 32).sum()),
                              "compared": full}
        return stats
    finally:
        g.close()
        r.close()


@pytest.mark.parametrize("case", ["drop10k_rest", "drop10k_frame30", "drop10k_frame60", "folded64", "folded64_fast"])
def test_integer_structures_bit_exact(gpu_lib, case):
    from xpbd_gb300 import scene

    if case.startswith("drop10k"):
        sc = scene.drop_scene(100, 60)
        frames = 0 if case.endswith("rest") else int(case.split("frame")[1])
        pos = None if frames == 0 else _positions_after(sc, frames)
    else:
        sc = scene.drop_scene(64, 1, seed=7, self_mode=1 if case.endswith("fast") else 2)
        pos = _folded(sc, 3, 0.0012)
    stats = _compare_structures(sc, pos)
    _record(f"integers/{case}", stats)
    if case.startswith("folded"):
        assert stats["neighbors"]["compared"] > 1000  # the fold puts most vertices in contact


# -------------------------------------------------------------- positions --

def _scene(name):
    from xpbd_gb300 import scene

    return {
        "plain32": lambda: scene.plain_grid_scene(32, 10),
        "drop10k": lambda: scene.drop_scene(100, 30),
        "drop10k_fast": lambda: scene.drop_scene(100, 30, self_mode=1),
        "hard_stretch_0.4": lambda: scene.hardness_grid_scene(32, 0.4, 10),
        "hard_stretch_1.0": lambda: scene.hardness_grid_scene(32, 1.0, 10),
    }[name]()


def _run_ref(sc, frames, substeps):
    r = R.RefSolver.from_scene(sc)
    for _ in range(frames):
        r.step(substeps, sc.iterations, diagnostics=False, synchronize=True)
    p = r.download_positions()
    r.close()
    return p


def _horizons(sc):
    # one substep of the frame's schedule = a one-substep frame of dt / S
    return [("substep1", 1, 1, sc.options.dt / sc.substeps), ("frame1", 1, sc.substeps, sc.options.dt),
            ("frame10", 10, sc.substeps, sc.options.dt)]


REF_RUNS = 4


def _compare(mine, runs, extent):
    """The product's positions against several reference runs, in units of
    the cloth extent: the largest coordinate error against the nearest run,
    the reference's spread (largest coordinate difference between two of its
    runs), and per-vertex distances to the runs' median (mean, 99th
    percentile) beside the 99th percentile of the runs' own distances to it."""
    stack = np.stack(runs)
    center = np.median(stack, 0)
    d_mine = np.linalg.norm(mine - center, axis=1)
    d_runs = np.linalg.norm(stack - center[None], axis=2).max(0)
    return {"max_error": min(float(np.abs(mine - r).max()) for r in runs) / extent,
            "noise_floor": max(float(np.abs(runs[i] - runs[j]).max()) for i in range(len(runs))
                               for j in range(i + 1, len(runs))) / extent,
            "mean_error": float(d_mine.mean()) / extent,
            "p99_error": float(np.quantile(d_mine, 0.99)) / extent,
            "p99_noise": float(np.quantile(d_runs, 0.99)) / extent}


def _check(tag, r, contact):
    if tag in ("substep1", "frame1"):
        assert r["max_error"] <= TOL, (tag, r)
    elif not contact:
        assert r["max_error"] <= max(TOL, 4.0 * r["noise_floor"]), (tag, r)
    else:
        assert r["mean_error"] <= TOL, (tag, r)
        assert r["p99_error"] <= max(TOL, 10.0 * r["p99_noise"]), (tag, r)
        assert r["max_error"] <= 50.0 * TOL, (tag, r)


@pytest.mark.parametrize("name", ["plain32", "drop10k", "drop10k_fast", "hard_stretch_0.4", "hard_stretch_1.0"])
def test_positions_within_tolerance_of_reference(gpu_lib, name):
    horizons = _horizons(_scene(name))
    if name.startswith("drop10k"):
        horizons.append(("frame30", 30, 10, 1.0 / 60.0))
    for tag, frames, substeps, dt in horizons:
        sc = _scene(name)
        sc.options.dt = dt
        runs = [_run_ref(sc, frames, substeps) for _ in range(REF_RUNS)]
        g = _product(sc)
        for _ in range(frames):
            g.step(substeps, sc.iterations, diagnostics=False)
        p = g.download_positions().copy()
        g.close()
        assert np.isfinite(p).all()
        r = _compare(p, runs, sc.extent)
        r["max_displacement"] = float(np.abs(runs[0] - sc.cloth.positions_world).max()) / sc.extent
        _record(f"positions/{name}/{tag}", r)
        _check(tag, r, contact=tag == "frame30")


def test_batch_sample_within_tolerance_of_reference(gpu_lib):
    """Sixteen cloths of the uneven 256-cloth mix (every 16th: sizes,
    compliances, pins, fast and strict self collision) in one product batch,
    each against four runs of its own reference solver.  After one frame every
    cloth is within 1e-4 of its extent.  After ten frames the larger cloths
    are in contact with the sphere and with themselves, where single vertices
    of the reference's own runs already part by more than that: each cloth
    is held to the contact-phase rule (mean, 99th percentile against the
    reference's own spread, gross-error guard on the largest error).  In
    fast mode the cluster filter keeps the first contact per cluster in
    candidate order (abi41.cu:793-832); the reference's order is its atomic
    arrival order, ours increasing id, which is one more reason single
    vertices part once contacts decide."""
    from xpbd_gb300 import native, scene

    scs = scene.batched_scenes(256, seed=0, frames=10)[::16]
    for tag, frames in (("frame1", 1), ("frame10", 10)):
        batch = native.NativeXpbdBatch([(s.cloth, s.options, s.static_triangles) for s in scs], key_division="reference")
        for _ in range(frames):
            batch.step(scs[0].substeps, scs[0].iterations, diagnostics=False)
        allp = batch.download_positions().copy()
        batch.close()
        rows = []
        for k, s in enumerate(scs):
            runs = [_run_ref(s, frames, s.substeps) for _ in range(REF_RUNS)]
            v0, nv = batch.cloth_vertices(k)
            mine = allp[v0:v0 + nv]
            assert np.isfinite(mine).all()
            r = _compare(mine, runs, s.extent)
            r.update({"cloth": k * 16, "vertices": nv, "fast": bool(s.meta.get("fast"))})
            rows.append(r)
        _record(f"positions/batch16/{tag}", {"max_error": max(r["max_error"] for r in rows),
                                            "noise_floor": max(r["noise_floor"] for r in rows), "cloths": rows})
        for r in rows:
            _check(tag, r, contact=True)


def test_diagnostics_counters_against_reference(gpu_lib):
    """The integer diagnostics the ABI exposes (abi.h:70-207) after one frame of
    the folded cloth: the same contact work is found (candidate and contact
    counts within a few percent: positions differ at the noise level inside
    the frame) and no slot overflows in either solver."""
    from xpbd_gb300 import scene

    sc = scene.drop_scene(64, 1, seed=7)
    pos = _folded(sc, 3, 0.0012)
    g = _product(sc)
    r = R.RefSolver.from_scene(sc)
    g.update_positions(pos)
    r.solver.update_positions(pos)
    g.step(sc.substeps, sc.iterations, diagnostics=True)
    r.step(sc.substeps, sc.iterations, diagnostics=True)
    dg, dr = g.diagnostics(), r.diagnostics()
    g.close()
    r.close()
    keys = [k for k, v in dr.items() if isinstance(v, int) and ("contact" in k or "candidate" in k or "overflow" in k)]
    table = {k: (int(dg[k]), int(dr[k])) for k in keys}
    _record("diagnostics/folded64_frame1", table)
    assert keys
    for k, (mine, theirs) in table.items():
        if "overflow" in k:
            assert mine == theirs == 0, k
        else:
            assert abs(mine - theirs) <= max(0.05 * theirs, 16), (k, mine, theirs)
