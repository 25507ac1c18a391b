"""Photometric corner refinement (gpu): forward residual, hand-written adjoint
and Gauss-Newton, through the C ABI.

Checks: the FP32 forward against an FP64 torch restatement of the same
residual; the adjoint's dL/dcorners and dL/dimage against FP64 autograd of
that restatement and against FP64 central finite differences (step 1e-3 px);
a torch.autograd.Function over the C ABI (test harness only); Gauss-Newton
reducing the corner error of perturbed detections.
"""
import numpy as np
import pytest

import bdcudatag
import scenes
from helpers import corner_error, matches

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

S = 8  # samples per cell side


def detected_quads(frame_indices, max_quads):
    """Detected quads of 1280x800 refinement frames matched to ground truth:
    (frames uint8 [F,H,W], corners [n,8], truth [n,8], templates [n,C,C] (C=10),
    image_index [n]); tag36h11 only so every template has 10 cells."""
    frames, corners, truth, templates, index = [], [], [], [], []
    det = bdcudatag.Detector(0, 1280, 800)
    for fi in frame_indices:
        img, tags = scenes.render_scene(scenes.REFINE_1280, fi, 1280, 800)
        n, d = det.detect(img)
        for k in range(n):
            for t in tags:
                if t.family == 0 and t.id == d["id"][k] and matches(d["corners"][k], t.corners):
                    corners.append(d["corners"][k].astype(np.float32))
                    truth.append(t.corners.reshape(8))
                    templates.append(bdcudatag.tag_template(0, int(t.id)))
                    index.append(len(frames))
        frames.append(img)
        if len(corners) >= max_quads:
            break
    n = min(len(corners), max_quads)
    return (np.stack(frames), np.stack(corners[:n]), np.stack(truth[:n]),
            np.stack(templates[:n]), np.array(index[:n], np.int32))


def ref_forward(images64, corners64, templates, image_index, levels64):
    """FP64 restatement of the residual (same sample grid, homography closed
    form and bilinear rule as the kernel)."""
    n = corners64.shape[0]
    F, H, W = images64.shape
    C = templates.shape[-1]
    dim = C - 2
    x0, y0, x1, y1, x2, y2, x3, y3 = corners64.unbind(1)
    dx1, dx2, dx3 = x1 - x2, x3 - x2, x0 - x1 + x2 - x3
    dy1, dy2, dy3 = y1 - y2, y3 - y2, y0 - y1 + y2 - y3
    det = dx1 * dy2 - dx2 * dy1
    g = (dx3 * dy2 - dx2 * dy3) / det
    k = (dx1 * dy3 - dx3 * dy1) / det
    h = [x1 - x0 + g * x1, x3 - x0 + k * x3, x0, y1 - y0 + g * y1, y3 - y0 + k * y3, y0, g, k]
    s = torch.arange(C * C * S * S, device=corners64.device)
    cell, sub = s // (S * S), s % (S * S)
    cy, cx, sy, sx = cell // C, cell % C, sub // S, sub % S
    u = ((cx - 1).double() + (sx.double() + 0.5) / S) / dim
    v = ((cy - 1).double() + (sy.double() + 0.5) / S) / dim
    hh = [t[:, None] for t in h]
    den = hh[6] * u + hh[7] * v + 1.0
    X = (hh[0] * u + hh[1] * v + hh[2]) / den
    Y = (hh[3] * u + hh[4] * v + hh[5]) / den
    inside = (den > 1e-6) & (X >= 0) & (Y >= 0) & (X < W - 1) & (Y < H - 1)
    Xc = torch.where(inside, X, torch.zeros_like(X))
    Yc = torch.where(inside, Y, torch.zeros_like(Y))
    ix, iy = Xc.detach().floor().long(), Yc.detach().floor().long()
    fx, fy = Xc - ix, Yc - iy
    flat = images64.reshape(-1)
    base = image_index.long()[:, None] * (H * W) + iy * W + ix
    a, b = flat[base], flat[base + 1]
    c, d = flat[base + W], flat[base + W + 1]
    val = (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy
    t = templates.reshape(n, C * C).double()[:, cell]
    lo, hi = levels64[:, :1], levels64[:, 1:]
    r = torch.where(inside, val - (lo + (hi - lo) * t), torch.zeros_like(val))
    return r, 0.5 * (r * r).sum(1)


def kernel_args(images, corners, templates, index, levels):
    return bdcudatag.refine_args(images, corners, templates, index, levels, samples_per_cell=S)


class RefineResidual(torch.autograd.Function):
    """Residuals through bd_refine_forward; gradients through the hand-written
    adjoint bd_refine_backward (test harness only)."""

    @staticmethod
    def forward(ctx, corners, images_f, images_u8, templates, index, levels):
        n = corners.shape[0]
        C = templates.shape[-1]
        res = torch.empty((n, C * C * S * S), device="cuda", dtype=torch.float32)
        args = kernel_args(images_u8, corners.detach().contiguous(), templates, index, levels)
        rc = bdcudatag.lib().bd_refine_forward(args, res.data_ptr(), None, None)
        assert rc == 0, bdcudatag.last_error()
        ctx.save_for_backward(corners.detach().contiguous())
        ctx.extra = (images_u8, templates, index, levels, images_f.shape)
        return res

    @staticmethod
    def backward(ctx, grad_res):
        (corners,) = ctx.saved_tensors
        images_u8, templates, index, levels, shape = ctx.extra
        gc = torch.zeros_like(corners)
        gi = torch.zeros(shape, device="cuda", dtype=torch.float32)
        args = kernel_args(images_u8, corners, templates, index, levels)
        rc = bdcudatag.lib().bd_refine_backward(args, grad_res.contiguous().data_ptr(), gc.data_ptr(),
                                                gi.data_ptr(), None)
        assert rc == 0, bdcudatag.last_error()
        return gc, gi, None, None, None, None


@pytest.fixture(scope="module")
def quads():
    frames, corners, truth, templates, index = detected_quads(range(4), 12)
    rng = np.random.default_rng(44)
    perturbed = corners + rng.uniform(-1.5, 1.5, corners.shape).astype(np.float32)
    levels = np.tile(np.array([[35.0, 215.0]], np.float32), (len(corners), 1))
    return frames, perturbed, truth, templates, index, levels


def to_cuda(frames, corners, templates, index, levels):
    return (torch.from_numpy(frames).cuda(), torch.from_numpy(corners).cuda(),
            torch.from_numpy(templates).cuda(), torch.from_numpy(index).cuda(),
            torch.from_numpy(levels).cuda())


def test_forward_matches_fp64(quads):
    frames, corners, _, templates, index, levels = quads
    im, co, te, ix, lv = to_cuda(frames, corners, templates, index, levels)
    n = co.shape[0]
    res = torch.empty((n, 100 * S * S), device="cuda")
    loss = torch.empty(n, device="cuda")
    assert bdcudatag.lib().bd_refine_forward(kernel_args(im, co, te, ix, lv), res.data_ptr(),
                                             loss.data_ptr(), None) == 0
    r64, l64 = ref_forward(im.double(), co.double(), te, ix, lv.double())
    torch.cuda.synchronize()
    assert torch.allclose(loss.double(), l64, rtol=1e-4, atol=1e-3)
    # FP32 sample positions carry ~1e-4 px of rounding near x ~ 1000; on an
    # edge of 255 DN/px that is ~0.03 DN of residual.
    diff = (res.double() - r64).abs()
    assert diff.max().item() < 0.1 and diff.mean().item() < 2e-3


def test_adjoint_matches_fp64_autograd_and_finite_differences(quads):
    frames, corners, _, templates, index, levels = quads
    im, co, te, ix, lv = to_cuda(frames, corners, templates, index, levels)
    # Reference gradient: FP64 autograd of the restatement, upstream dL/dr = r.
    c64 = co.double().requires_grad_(True)
    i64 = im.double().requires_grad_(True)
    r64, l64 = ref_forward(i64, c64, te, ix, lv.double())
    l64.sum().backward()
    # Kernel adjoint with the same upstream gradient (its own residuals).
    n = co.shape[0]
    res = torch.empty((n, 100 * S * S), device="cuda")
    args = kernel_args(im, co, te, ix, lv)
    assert bdcudatag.lib().bd_refine_forward(args, res.data_ptr(), None, None) == 0
    gc = torch.zeros_like(co)
    gi = torch.zeros(im.shape, device="cuda", dtype=torch.float32)
    assert bdcudatag.lib().bd_refine_backward(args, res.data_ptr(), gc.data_ptr(), gi.data_ptr(), None) == 0
    torch.cuda.synchronize()
    ref_c = c64.grad
    assert (gc.double() - ref_c).norm() / ref_c.norm() < 1e-3
    per_quad = (gc.double() - ref_c).norm(dim=1) / ref_c.norm(dim=1).clamp_min(1.0)
    assert per_quad.max() < 5e-3
    ref_i = i64.grad
    assert (gi.double() - ref_i).norm() / ref_i.norm() < 1e-3
    # FP64 central differences of the restatement, step 1e-3 px.
    eps = 1e-3
    fd = torch.zeros_like(ref_c)
    with torch.no_grad():
        for j in range(8):
            d = torch.zeros_like(c64)
            d[:, j] = eps
            lp = ref_forward(im.double(), c64 + d, te, ix, lv.double())[1]
            lm = ref_forward(im.double(), c64 - d, te, ix, lv.double())[1]
            fd[:, j] = (lp - lm) / (2 * eps)
    assert (fd - ref_c).norm() / ref_c.norm() < 2e-2
    assert (fd - gc.double()).norm() / fd.norm() < 2e-2


def test_autograd_function(quads):
    frames, corners, _, templates, index, levels = quads
    im, co, te, ix, lv = to_cuda(frames, corners, templates, index, levels)
    corners_t = co.clone().requires_grad_(True)
    images_f = im.float().requires_grad_(True)
    res = RefineResidual.apply(corners_t, images_f, im, te, ix, lv)
    (0.5 * (res * res).sum()).backward()
    c64 = co.double().requires_grad_(True)
    i64 = im.double().requires_grad_(True)
    ref_forward(i64, c64, te, ix, lv.double())[1].sum().backward()
    assert (corners_t.grad.double() - c64.grad).norm() / c64.grad.norm() < 1e-3
    assert (images_f.grad.double() - i64.grad).norm() / i64.grad.norm() < 1e-3


def test_gauss_newton_reduces_corner_error():
    frames, corners, truth, templates, index = detected_quads(range(8), 40)
    rng = np.random.default_rng(7)
    start = corners + rng.uniform(-1.5, 1.5, corners.shape).astype(np.float32)
    im = torch.from_numpy(frames).cuda()
    co = torch.from_numpy(start.copy()).cuda()
    te = torch.from_numpy(templates).cuda()
    ix = torch.from_numpy(index).cuda()
    loss = torch.empty(co.shape[0], device="cuda")
    args = bdcudatag.refine_args(im, co, te, ix, None, samples_per_cell=S)
    assert bdcudatag.lib().bd_refine_gauss_newton(args, co.data_ptr(), 5, loss.data_ptr(), None) == 0
    after = co.cpu().numpy()
    before = np.array([corner_error(s, t) for s, t in zip(start, truth)])
    after_e = np.array([corner_error(a, t) for a, t in zip(after, truth)])
    assert np.median(before) > 0.5
    assert np.median(after_e) < 0.2 and np.median(after_e) < np.median(before) / 3, (before, after_e)
    assert np.mean(after_e < before) > 0.9
