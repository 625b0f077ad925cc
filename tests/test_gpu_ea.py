"""Fixed-step emission-absorption march and its adjoint on the GPU.

Tolerances: forward images within 1e-5 relative (plus 1e-6 absolute for
near-zero channels) of the oracle; the FP32 adjoint within 1e-3 relative
(norm over the checked entries) of central finite differences of the FP64
GPU march (eps = 1e-3) and of the oracle's FP64 gradient.
"""
import numpy as np
import pytest

from barney_gb300 import _native as N
from barney_gb300 import scenes
from barney_gb300.ea import EAProblem
import oracle

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-6


def small_problem(dims=48, nviews=6, size=48):
    gt = scenes.ea_scene(dims)
    views = scenes.fibonacci_views(nviews, 2.5, size)
    step = 0.5 / (dims - 1)
    return gt, views, step


def test_forward_matches_oracle(cuda):
    gt, views, step = small_problem()
    p = EAProblem(gt, views, step)
    img = p.render().cpu().numpy().reshape(-1, 4)
    o = oracle.Oracle(gt)
    ref32 = o.ea_render(views, step)
    ref64 = o.ea_render(views, step, use_double=True)
    np.testing.assert_allclose(img, ref32, rtol=RTOL, atol=ATOL)
    # FP32 against FP64: rounding of sample positions, trilinear weights and
    # steep TF segments; measured max ~3e-4 relative on 0.2% of channels
    np.testing.assert_allclose(img, ref64, rtol=1e-3, atol=1e-5)
    assert img[:, 3].max() > 0.5


def test_forward_f64_matches_oracle(cuda):
    gt, views, step = small_problem(nviews=3)
    p = EAProblem(gt, views, step)
    img = p.render_f64().cpu().numpy().reshape(-1, 4)
    ref64 = oracle.Oracle(gt).ea_render(views, step, use_double=True)
    np.testing.assert_allclose(img, ref64, rtol=1e-6, atol=1e-7)


def test_constant_density_beer_lambert(cuda):
    """Known answer: a constant field maps to constant (rgb, sigma); a pixel
    whose march takes n steps gives A = 1-exp(-n sigma dt), C = rgb*A."""
    vol = np.full((16, 16, 16), 0.5, np.float32)
    tf = np.tile(np.array([[0.2, 0.6, 0.9, 0.4]], np.float32), (4, 1))
    s = scenes.Scene(scalars=vol, tf=tf, base_density=3.0)
    views = [dict(pos=(0.0, 0.0, 2.5), dir=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0), fovy=20.0, width=8, height=8)]
    step = 0.01
    img = EAProblem(s, views, step).render().cpu().numpy().reshape(8, 8, 4)
    # central pixels: the ray runs along -z through the whole box (t0=2, t1=3)
    sigma = 0.4 * 3.0
    t0, t1 = 2.0, 3.0
    n = sum(1 for i in range(200) if t0 + (i + 0.5) * step < t1)
    a = 1 - np.exp(-n * sigma * step)
    c = img[3, 3]
    np.testing.assert_allclose(c[3], a, rtol=2e-5)
    np.testing.assert_allclose(c[:3], np.array([0.2, 0.6, 0.9]) * a, rtol=2e-5)


@pytest.mark.parametrize("tf_kind", ["ramp", "two_peaks"])
def test_adjoint_matches_oracle_and_finite_differences(cuda, tf_kind):
    """The two-peak TF has knots (slope changes) inside the data range, where a
    central difference averages two one-sided slopes; the finite-difference
    check therefore runs on the knot-free ramp TF, and both TFs are checked
    against the oracle's FP64 gradient."""
    import torch
    gt, views, step = small_problem(dims=40, nviews=4, size=40)
    if tf_kind == "ramp":
        gt.tf = scenes.tf_ramp(256, 0.9)
    p_gt = EAProblem(gt, views, step)
    target = p_gt.render()
    start = scenes.Scene(scalars=np.full_like(gt.scalars, 0.3) + 0.2 * gt.scalars, tf=gt.tf,
                         base_density=gt.base_density)
    p = EAProblem(start, views, step)
    img = p.render()
    gimg = 2.0 * (img - target)  # dL/dI of L = sum (I - target)^2
    gv, gt_tf = p.backward(img, gimg)
    gv, gt_tf = gv.cpu().numpy().astype(np.float64), gt_tf.cpu().numpy().astype(np.float64)
    # FP64 oracle gradient
    o = oracle.Oracle(start)
    ov, ot = o.ea_backward(views, step, gimg.cpu().numpy().reshape(-1, 4))
    ov = ov.reshape(-1)
    sel = np.flatnonzero(np.abs(ov) > 1e-3 * np.abs(ov).max())
    assert np.linalg.norm(gv.reshape(-1)[sel] - ov[sel]) <= 1e-3 * np.linalg.norm(ov[sel])
    assert np.linalg.norm(gt_tf - ot) <= 1e-3 * np.linalg.norm(ot)
    if tf_kind != "ramp":
        return
    # central finite differences of the FP64 march, eps = 1e-3
    rng = np.random.default_rng(44)
    tgt64 = target.double()

    def loss(pp):
        return float(((pp.render_f64() - tgt64) ** 2).sum().item())

    def fd_of(make, base, eps=1e-3):
        hi, lo = np.float32(base + eps), np.float32(base - eps)
        return (loss(make(float(hi))) - loss(make(float(lo)))) / (float(hi) - float(lo))

    vox = rng.choice(sel, size=16, replace=False)
    base = start.scalars.reshape(-1)
    fd = np.array([fd_of(lambda x, v=v: p.with_voxel(int(v), x), float(base[v])) for v in vox])
    an = gv.reshape(-1)[vox]
    assert np.linalg.norm(fd - an) <= 1e-3 * np.linalg.norm(fd) + 1e-6, (fd, an)
    tsel = np.flatnonzero(np.abs(ot.reshape(-1)) > 1e-3 * np.abs(ot).max())
    ent = rng.choice(tsel, size=min(16, tsel.size), replace=False)
    tfb = start.tf.reshape(-1)
    fd = np.array([fd_of(lambda x, e=e: p.with_tf_entry(int(e), x), float(tfb[e])) for e in ent])
    an = gt_tf.reshape(-1)[ent]
    assert np.linalg.norm(fd - an) <= 1e-3 * np.linalg.norm(fd) + 1e-6, (fd, an)


def test_autograd_function(cuda):
    import torch
    from barney_gb300.ea import ea_render_autograd
    gt, views, step = small_problem(dims=32, nviews=2, size=32)
    p = EAProblem(gt, views, step)
    vox = p.scalars.clone().requires_grad_(True)
    tf = p.tf.clone().requires_grad_(True)
    img = ea_render_autograd(vox, tf, p)
    w = torch.rand_like(img)
    (img * w).sum().backward()
    gv, gtf = p.backward(img.detach(), w)
    # the adjoint's atomics sum in no fixed order: equal up to FP32 reassociation
    torch.testing.assert_close(vox.grad.reshape(-1), gv.reshape(-1), rtol=1e-4, atol=1e-6)
    torch.testing.assert_close(tf.grad.reshape(-1), gtf.reshape(-1), rtol=1e-4, atol=1e-5)
