"""The float64 reference rollout used to check the adjoint is itself checked
here: its autograd gradient against central finite differences (CPU)."""
import numpy as np
import torch

from xpbd_gb300 import scene
from xpbd_diff_reference import Rollout


def test_reference_autograd_matches_finite_differences():
    sc = scene.diff_scene(6, 6, stretch=3e-3, bend=3e-3)
    r = Rollout(sc.cloth, sc.options)
    ks = torch.tensor(scene.compliance_field(len(sc.cloth.edges), 3e-3, 1.0, 1), dtype=torch.float64, requires_grad=True)
    kb = torch.tensor(scene.compliance_field(len(sc.cloth.bends), 3e-3, 1.0, 2), dtype=torch.float64, requires_grad=True)
    target = r.run(ks.detach() * 1.3, kb.detach() * 0.7, 6, 4, 2).detach()

    def loss(a, b):
        return ((r.run(a, b, 6, 4, 2) - target) ** 2).sum()

    L = loss(ks, kb)
    L.backward()
    rng = np.random.default_rng(0)
    for _ in range(4):
        vs = torch.tensor(rng.standard_normal(len(ks)))
        vb = torch.tensor(rng.standard_normal(len(kb)))
        h = 1e-4
        with torch.no_grad():
            lp = loss(ks * (1 + h * vs), kb * (1 + h * vb))
            lm = loss(ks * (1 - h * vs), kb * (1 - h * vb))
        fd = float(lp - lm) / (2 * h)
        an = float((ks.grad * ks.detach() * vs).sum() + (kb.grad * kb.detach() * vb).sum())
        assert abs(fd - an) <= 1e-4 * max(abs(fd), abs(an)) + 1e-14, (fd, an)


def test_reference_single_parameter_finite_differences():
    """64 random single compliances and 8 random directions, central
    differences at h = 1e-3 relative, float64."""
    sc = scene.diff_scene(8, 4, stretch=1e-3, bend=1e-3)
    r = Rollout(sc.cloth, sc.options)
    ks0 = scene.compliance_field(len(sc.cloth.edges), 1e-3, 2.0, 3)
    kb0 = scene.compliance_field(len(sc.cloth.bends), 1e-3, 2.0, 4)
    ks = torch.tensor(ks0, dtype=torch.float64, requires_grad=True)
    kb = torch.tensor(kb0, dtype=torch.float64, requires_grad=True)
    target = r.run(torch.tensor(scene.compliance_field(len(ks0), 1e-3, 2.0, 11), dtype=torch.float64),
                   torch.tensor(scene.compliance_field(len(kb0), 1e-3, 2.0, 12), dtype=torch.float64), 4, 10, 2).detach()

    def loss(a, b):
        return float(((r.run(a, b, 4, 10, 2) - target) ** 2).sum())

    L = ((r.run(ks, kb, 4, 10, 2) - target) ** 2).sum()
    L.backward()
    h = 1e-3
    rng = np.random.default_rng(1)
    base_s, base_b = ks.detach(), kb.detach()
    # floor: parameters with a negligible effect are compared against the
    # largest single-parameter effect
    scale = float(max((ks.grad * base_s).abs().max(), (kb.grad * base_b).abs().max()))
    for idx in rng.choice(len(ks0) + len(kb0), 64, replace=False):
        a, b = base_s.clone(), base_b.clone()
        a2, b2 = base_s.clone(), base_b.clone()
        if idx < len(ks0):
            a[idx] *= 1 + h
            a2[idx] *= 1 - h
            an = float(ks.grad[idx] * base_s[idx])
        else:
            j = idx - len(ks0)
            b[j] *= 1 + h
            b2[j] *= 1 - h
            an = float(kb.grad[j] * base_b[j])
        fd = (loss(a, b) - loss(a2, b2)) / (2 * h)
        assert abs(fd - an) <= 1e-2 * abs(an) + 1e-3 * scale, (idx, fd, an, scale)
    for _ in range(8):
        vs, vb = torch.tensor(rng.standard_normal(len(ks0))), torch.tensor(rng.standard_normal(len(kb0)))
        fd = (loss(base_s * (1 + h * vs), base_b * (1 + h * vb)) - loss(base_s * (1 - h * vs), base_b * (1 - h * vb))) / (2 * h)
        an = float((ks.grad * base_s * vs).sum() + (kb.grad * base_b * vb).sum())
        # a direction moves every compliance, so caps and clamps near their
        # thresholds switch within the step: a looser bound
        assert abs(fd - an) <= 3e-2 * abs(an) + 1e-3 * scale, (fd, an, scale)
