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
