"""Differentiable form: the library's rollout and hand-written adjoint.

* forward with equal compliances is bit-identical to the solver;
* forward with a per-constraint compliance field matches the float64
  reference rollout (oracle/xpbd_diff_reference.py) to 1e-4 m;
* the adjoint gradient matches the reference's autograd gradient and
  central finite differences of the GPU forward (h = 1e-3 relative);
* the torch.autograd.Function returns the adjoint's gradient."""
import numpy as np
import pytest
import torch

from xpbd_gb300 import scene
from xpbd_gb300.diff import DiffCloth, rollout
from xpbd_gb300.native import NativeXpbdSolver
from xpbd_diff_reference import Rollout

pytestmark = pytest.mark.gpu


def _fields(sc, center_s, center_b, seed):
    ks = scene.compliance_field(len(sc.cloth.edges), center_s, 1.0, seed)
    kb = scene.compliance_field(len(sc.cloth.bends), center_b, 1.0, seed + 1)
    return ks, kb


def test_forward_equals_solver(gpu_lib):
    sc = scene.diff_scene(16, 4)
    dc = DiffCloth(sc.cloth, sc.options)
    ks = torch.full((len(sc.cloth.edges),), sc.options.stretch_compliance, dtype=torch.float32, device="cuda")
    kb = torch.full((len(sc.cloth.bends),), sc.options.bend_compliance, dtype=torch.float32, device="cuda")
    solver = NativeXpbdSolver(sc.cloth, sc.options, sc.static_triangles)
    stepped = 0
    for frames in (1, 4):
        x = dc.rollout(ks, kb, frames, 10, 2).cpu().numpy()
        while stepped < frames:
            solver.step(10, 2, diagnostics=False, synchronize=True)
            stepped += 1
        assert np.array_equal(x, solver.download_positions()), frames


def _loss_setup(n=10, frames=5, cs=3e-3, cb=3e-3):
    sc = scene.diff_scene(n, frames, stretch=cs, bend=cb)
    ks, kb = _fields(sc, cs, cb, 3)
    kts, ktb = _fields(sc, cs, cb, 11)
    ref = Rollout(sc.cloth, sc.options)
    target = ref.run(torch.tensor(kts, dtype=torch.float64), torch.tensor(ktb, dtype=torch.float64), frames, 10, 2).detach()
    return sc, ks, kb, ref, target


def test_forward_matches_reference(gpu_lib):
    sc, ks, kb, ref, _ = _loss_setup()
    dc = DiffCloth(sc.cloth, sc.options)
    x = dc.rollout(torch.tensor(ks, device="cuda"), torch.tensor(kb, device="cuda"), sc.frames, 10, 2).cpu().numpy()
    xr = ref.run(torch.tensor(ks, dtype=torch.float64), torch.tensor(kb, dtype=torch.float64), sc.frames, 10, 2).numpy()
    assert np.abs(x - xr).max() <= 1e-4


def test_adjoint_matches_reference_autograd(gpu_lib):
    sc, ks, kb, ref, target = _loss_setup()
    dc = DiffCloth(sc.cloth, sc.options)
    ksd, kbd = torch.tensor(ks, device="cuda"), torch.tensor(kb, device="cuda")
    x = dc.rollout(ksd, kbd, sc.frames, 10, 2)
    g = 2.0 * (x.double() - target.cuda()).float()
    gs, gb = dc.backward(g)
    rs = torch.tensor(ks, dtype=torch.float64, requires_grad=True)
    rb = torch.tensor(kb, dtype=torch.float64, requires_grad=True)
    ((ref.run(rs, rb, sc.frames, 10, 2) - target) ** 2).sum().backward()
    for mine, theirs in ((gs.cpu().double(), rs.grad), (gb.cpu().double(), rb.grad)):
        rel = float(torch.linalg.norm(mine - theirs) / torch.linalg.norm(theirs))
        cos = float(torch.dot(mine, theirs) / (torch.linalg.norm(mine) * torch.linalg.norm(theirs)))
        assert rel < 2e-2 and cos > 0.999, (rel, cos)


def test_adjoint_matches_finite_differences(gpu_lib):
    """Central differences of the float32 GPU forward along 8 random
    directions (h = 1e-3 relative).  At this step the float32 rounding of a
    whole rollout is of the order of the signal, so the check is
    statistical: median relative error under 15 % and the finite
    differences correlated with the adjoint's predictions.  The exact
    single-parameter check is done in float64 on the reference rollout
    (tests/test_diff_reference.py), which the adjoint matches above."""
    sc = scene.diff_scene(16, 10, stretch=1e-3, bend=1e-3)
    ks = scene.compliance_field(len(sc.cloth.edges), 1e-3, 2.0, 3)
    kb = scene.compliance_field(len(sc.cloth.bends), 1e-3, 2.0, 4)
    kts = scene.compliance_field(len(sc.cloth.edges), 1e-3, 2.0, 11)
    ktb = scene.compliance_field(len(sc.cloth.bends), 1e-3, 2.0, 12)
    dc = DiffCloth(sc.cloth, sc.options)
    tgt = dc.rollout(torch.tensor(kts, device="cuda"), torch.tensor(ktb, device="cuda"), sc.frames, 10, 2).double()
    ksd, kbd = torch.tensor(ks, device="cuda"), torch.tensor(kb, device="cuda")

    def loss(a, b):
        return float(((dc.rollout(a, b, sc.frames, 10, 2).double() - tgt) ** 2).sum())

    x = dc.rollout(ksd, kbd, sc.frames, 10, 2)
    gs, gb = dc.backward((2.0 * (x.double() - tgt)).float())
    rng = np.random.default_rng(0)
    h = 1e-3
    fds, ans = [], []
    for _ in range(8):
        vs = torch.tensor(rng.standard_normal(len(ks)), dtype=torch.float32, device="cuda")
        vb = torch.tensor(rng.standard_normal(len(kb)), dtype=torch.float32, device="cuda")
        fds.append((loss(ksd * (1 + h * vs), kbd * (1 + h * vb)) - loss(ksd * (1 - h * vs), kbd * (1 - h * vb))) / (2 * h))
        ans.append(float((gs.double() * ksd.double() * vs.double()).sum() + (gb.double() * kbd.double() * vb.double()).sum()))
    fds, ans = np.array(fds), np.array(ans)
    rel = np.abs(fds - ans) / np.abs(ans)
    assert np.median(rel) < 0.15, (fds, ans)
    assert np.corrcoef(fds, ans)[0, 1] > 0.95, (fds, ans)


def test_autograd_function_and_checkpoint_recompute(gpu_lib):
    sc, ks, kb, _, target = _loss_setup(n=8, frames=3)
    dc = DiffCloth(sc.cloth, sc.options)
    ksd = torch.tensor(ks, device="cuda", requires_grad=True)
    kbd = torch.tensor(kb, device="cuda", requires_grad=True)
    tgt = target.float().cuda()
    out = rollout(ksd, kbd, dc, sc.frames)
    dc.rollout(ksd * 2, kbd * 2, sc.frames, 10, 2)  # another rollout in between: backward recomputes
    ((out - tgt) ** 2).sum().backward()
    x = dc.rollout(ksd.detach(), kbd.detach(), sc.frames, 10, 2)
    gs, gb = dc.backward(2.0 * (x - tgt))
    assert torch.allclose(ksd.grad, gs) and torch.allclose(kbd.grad, gb)


def test_cdiff_configuration_runs(gpu_lib):
    """64 x 64 cloth, 60 frames x 10 substeps, per-constraint compliance
    fields: forward and adjoint complete with finite gradients."""
    sc = scene.diff_scene(64, 60)
    ks, kb = _fields(sc, 1e-7, 1e-4, 0)
    kts, ktb = _fields(sc, 1e-7, 1e-4, 1)
    dc = DiffCloth(sc.cloth, sc.options)
    tgt = dc.rollout(torch.tensor(kts, device="cuda"), torch.tensor(ktb, device="cuda"), 60, 10, 2)
    ksd = torch.tensor(ks, device="cuda", requires_grad=True)
    kbd = torch.tensor(kb, device="cuda", requires_grad=True)
    loss = ((rollout(ksd, kbd, dc, 60) - tgt) ** 2).sum()
    loss.backward()
    assert torch.isfinite(ksd.grad).all() and torch.isfinite(kbd.grad).all()
    assert float(loss.detach()) > 0


# ---------------------------------------------------------------- Cdiff --
# The differentiable configuration itself: 64 x 64 cloth, 60 frames x 10
# substeps x 2 iterations, per-constraint compliance fields log-uniform
# within a decade of 1e-7 (stretch) and 1e-4 (bend), loss = squared distance
# of the final positions to the rollout of another seeded compliance field.

def _cdiff(frames=60):
    sc = scene.diff_scene(64, frames)
    ks, kb = _fields(sc, 1e-7, 1e-4, 0)
    kts, ktb = _fields(sc, 1e-7, 1e-4, 1)
    return sc, ks, kb, kts, ktb


def _report(key, value):
    import json
    import os

    path = os.environ.get("XPBD_DIFF_REPORT")
    if path:
        data = json.load(open(path)) if os.path.exists(path) else {}
        data[key] = value
        with open(path, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
    print(key, value)


def _fd_check(r, ks, kb, kts, ktb, frames, hs):
    """float64 central differences of the restated rollout against its
    autograd gradient: 64 seeded single compliances and 8 seeded directions
    at each relative step h, all perturbed rollouts in one batched float64
    rollout.  Returns, per h, the single-compliance errors over the largest
    single effect and the relative errors of the directions."""
    dev = "cuda"
    f64 = lambda a: torch.tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    target = r.run(f64(kts), f64(ktb), frames, 10, 2).detach()
    ksr, kbr = f64(ks).requires_grad_(), f64(kb).requires_grad_()
    loss0 = ((r.run(ksr, kbr, frames, 10, 2) - target) ** 2).sum()
    loss0.backward()
    gs, gb = ksr.grad.detach(), kbr.grad.detach()
    E, B = len(ks), len(kb)
    rng = np.random.default_rng(5)
    idx = rng.choice(E + B, 64, replace=False)
    S = torch.zeros(72, E, dtype=torch.float64, device=dev)
    Bm = torch.zeros(72, B, dtype=torch.float64, device=dev)
    for n, k in enumerate(idx):
        if k < E:
            S[n, k] = 1.0
        else:
            Bm[n, k - E] = 1.0
    S[64:] = f64(rng.standard_normal((8, E)))
    Bm[64:] = f64(rng.standard_normal((8, B)))
    base_s, base_b = f64(ks), f64(kb)
    an = ((gs * base_s * S).sum(-1) + (gb * base_b * Bm).sum(-1)).cpu().numpy()
    scale = float(np.abs(an[:64]).max())
    out = {"loss": float(loss0.detach()), "largest_single_effect": scale}
    for h in hs:
        with torch.no_grad():
            ps = torch.cat([base_s * (1 + h * S), base_s * (1 - h * S)])
            pb = torch.cat([base_b * (1 + h * Bm), base_b * (1 - h * Bm)])
            L = ((r.run(ps, pb, frames, 10, 2) - target) ** 2).sum((-1, -2)).cpu().numpy()
        fd = (L[:72] - L[72:]) / (2 * h)
        out[h] = {"single": np.abs(fd[:64] - an[:64]) / scale, "dirs": np.abs(fd[64:] - an[64:]) / np.abs(an[64:]),
                  "sign": bool((np.sign(fd[64:]) == np.sign(an[64:])).all())}
    return out


def test_cdiff_reference_gradient_matches_finite_differences(gpu_lib):
    """float64 central differences of the restated rollout at the Cdiff
    configuration against its autograd gradient (64 single compliances and 8
    directions).

    Over the 60 frames the cloth swings down from its two pinned corners and
    folds through the bottom of the swing; from about frame 45 on the
    rollout's sensitivity to its state grows by many orders of magnitude (the
    adjoint of the positions reaches ~1e17), so the loss has kinks at the
    scale of the configured step: a 1e-3 relative change of all compliances
    at once moves the step's clamps (stretch / bend correction caps, the
    velocity-feedback clamp) across their thresholds somewhere in the 600
    substeps.  Hence, at 60 frames: single compliances at the configured
    h = 1e-3 and directions at h = 1e-4 agree closely, directions at
    h = 1e-3 agree in sign and in the median; at 40 frames, before the fold,
    everything agrees closely at h = 1e-4."""
    sc, ks, kb, kts, ktb = _cdiff()
    r = Rollout(sc.cloth, sc.options, device="cuda")
    full = _fd_check(r, ks, kb, kts, ktb, 60, (1.0e-3, 1.0e-4))
    early = _fd_check(r, ks, kb, kts, ktb, 40, (1.0e-4,))
    rep = {}
    for name, res in (("60", full), ("40", early)):
        rep[name] = {"loss": res["loss"], "largest_single_effect": res["largest_single_effect"]}
        for h, v in res.items():
            if isinstance(v, dict):
                rep[name][f"h={h:g}"] = {"single_abs_err_over_scale_max": float(v["single"].max()),
                                         "single_abs_err_over_scale_median": float(np.median(v["single"])),
                                         "direction_rel_err": [float(x) for x in v["dirs"]]}
    _report("cdiff/float64_fd", rep)
    assert full[1.0e-3]["single"].max() <= 5e-3, rep
    assert full[1.0e-4]["dirs"].max() <= 5e-3, rep
    assert full[1.0e-3]["sign"] and np.median(full[1.0e-3]["dirs"]) <= 0.1, rep
    assert early[1.0e-4]["single"].max() <= 2e-3 and early[1.0e-4]["dirs"].max() <= 1e-4, rep


def _adjoint_along(dc, r, ks, kb, kts, ktb, frames, dtype):
    """The GPU's adjoint of one rollout against autograd of the restated
    rollout taken along the GPU rollout's own trajectory: for every frame,
    from the last back, the restatement re-runs that frame from the GPU's
    checkpoint (cast to `dtype`) and its vector-Jacobian product carries the
    adjoint of the state back and adds the compliance gradient."""
    dev = "cuda"
    target = dc.rollout(torch.tensor(kts, device=dev), torch.tensor(ktb, device=dev), frames, 10, 2).double()
    x = dc.rollout(torch.tensor(ks, device=dev), torch.tensor(kb, device=dev), frames, 10, 2)
    seed = 2.0 * (x.double() - target)
    gs, gb = dc.backward(seed.float())
    k1t = torch.tensor(ks, dtype=dtype, device=dev)
    k2t = torch.tensor(kb, dtype=dtype, device=dev)
    g1, g2 = torch.zeros_like(k1t), torch.zeros_like(k2t)
    lam = [seed.to(dtype), torch.zeros_like(seed, dtype=dtype), torch.zeros_like(seed, dtype=dtype)]
    for f in range(frames - 1, -1, -1):
        ck = dc.checkpoint(f)[..., :3].to(dtype)
        state = [ck[i].clone().requires_grad_() for i in range(3)]
        a1, a2 = k1t.clone().requires_grad_(), k2t.clone().requires_grad_()
        out = r.frame(*state, a1, a2, 10, 2)
        torch.autograd.backward(list(out), lam)
        g1 += a1.grad
        g2 += a2.grad
        lam = [t.grad if t.grad is not None else torch.zeros_like(t) for t in state]
    mine = torch.cat([gs.double(), gb.double()])
    theirs = torch.cat([g1, g2]).double()
    return {"rel_l2": float(torch.linalg.norm(mine - theirs) / torch.linalg.norm(theirs)),
            "cosine": float(torch.dot(mine, theirs) / (torch.linalg.norm(mine) * torch.linalg.norm(theirs))),
            "finite": bool(torch.isfinite(mine).all()), "norm": float(torch.linalg.norm(mine))}


def test_cdiff_adjoint_along_its_trajectory(gpu_lib):
    """The GPU's float32 adjoint at the Cdiff configuration against autograd
    of the restated rollout along the GPU rollout's own trajectory.

    Over all 60 frames it is compared with float32 autograd: both take the
    clamps' branches where the float32 step takes them.  Up to frame 40 it
    is also compared with float64 autograd from the upcast checkpoints.  Past
    the fold (about frame 45) the adjoint of the state grows to ~1e17, and a
    float64 re-run of a frame from a float32 checkpoint switches some clamps
    differently from the float32 step; its vector-Jacobian product then
    belongs to another branch of the piecewise-smooth step, and the two
    gradients part whatever the adjoint does, so that comparison stops at 40
    frames."""
    sc, ks, kb, kts, ktb = _cdiff()
    dc = DiffCloth(sc.cloth, sc.options)
    r32 = Rollout(sc.cloth, sc.options, dtype=torch.float32, device="cuda")
    r64 = Rollout(sc.cloth, sc.options, device="cuda")
    full32 = _adjoint_along(dc, r32, ks, kb, kts, ktb, 60, torch.float32)
    early64 = _adjoint_along(dc, r64, ks, kb, kts, ktb, 40, torch.float64)
    _report("cdiff/adjoint_along_trajectory", {"float32_60_frames": full32, "float64_40_frames": early64})
    assert full32["finite"] and early64["finite"]
    assert full32["rel_l2"] < 1e-2 and full32["cosine"] > 0.9999, full32
    assert early64["rel_l2"] < 2e-3 and early64["cosine"] > 0.99999, early64
