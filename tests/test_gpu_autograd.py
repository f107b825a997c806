"""Multi-plane SATs, box filters and their autograd backward on the GPU.

Plane stacks are integer-exact against the oracle plane by plane.  Box means
and gradients are floating point (f32 through an f32 SAT) and are compared
with float64 torch references with the tolerances written below:

  box means        |m - m64| <= 4 * eps32 * max|S64| / area + 1e-7
  gradients        |g - g64| <= 1e-4 * max(1, max|g64|)
  central FD       |g - fd|  <= 1e-4 * max(1, max|fd|)   (FP64 loss, h = 1e-3)
"""
import numpy as np
import pytest
import torch

import sat_gb300
from sat_gb300 import autograd as AG
from sat_gb300 import api
from tests.util import bits, to_dev, to_np

pytestmark = pytest.mark.gpu

EPS32 = float(np.finfo(np.float32).eps)


def sat64(x: torch.Tensor) -> torch.Tensor:
    return x.double().cumsum(-1).cumsum(-2)


def box_means64(x: torch.Tensor, radii) -> torch.Tensor:
    """Clipped box means in float64 by the four-corner rule on a zero-padded
    SAT (differentiable, for reference gradients)."""
    H, W = x.shape[-2:]
    S = torch.nn.functional.pad(sat64(x), (1, 0, 1, 0))  # S[y+1, x+1] = SAT(y, x)
    ys = torch.arange(H, device=x.device)
    xs = torch.arange(W, device=x.device)
    outs = []
    for r in radii:
        ya, yb = (ys - r).clamp(min=0), (ys + r).clamp(max=H - 1)
        xa, xb = (xs - r).clamp(min=0), (xs + r).clamp(max=W - 1)
        s = (S[..., yb + 1, :][..., xb + 1] - S[..., ya, :][..., xb + 1]
             - S[..., yb + 1, :][..., xa] + S[..., ya, :][..., xa])
        area = ((yb - ya + 1).double()[:, None] * (xb - xa + 1).double()[None, :])
        outs.append(s / area)
    return torch.stack(outs, dim=-3)


def test_planes_integer_exact(cuda, oracle):
    n, c, h, w = 2, 3, 131, 277
    a = oracle.gen("u8", 11, (n * c * h, w)).reshape(n, c, h, w)
    x = to_dev(a)
    out = to_np(sat_gb300.sat(x, torch.uint32))
    for i in range(n):
        for j in range(c):
            ref = oracle.sat_serial(a[i, j], np.uint32)
            assert np.array_equal(bits(out[i, j]), bits(ref)), (i, j)


def test_planes_pitched_and_reverse(cuda, oracle):
    """Planes whose rows are a slice of wider rows (pitch > width), forward
    and reverse, f32 -> f32 and u8 -> u32."""
    p, h, w, pitch = 5, 97, 200, 256
    a = oracle.gen("u8", 12, (p * h, w)).reshape(p, h, w)
    base = torch.zeros((p, h, pitch), dtype=torch.uint8, device=cuda)
    base[..., :w] = to_dev(a)
    x = base[..., :w]
    for rev in (False, True):
        out = to_np(sat_gb300.sat(x, torch.uint32, reverse=rev))
        for i in range(p):
            ref = oracle.sat_reverse(a[i], np.uint32) if rev else oracle.sat_serial(a[i], np.uint32)
            assert np.array_equal(bits(out[i]), bits(ref)), (i, rev)
    af = oracle.gen("f32n", 13, (p * h, w)).astype(np.float32).reshape(p, h, w)
    outf = to_np(sat_gb300.sat(to_dev(af), torch.float32))
    for i in range(p):
        ref = oracle.sat_fp64(af[i])
        den = oracle.sat_fp64(af[i], absval=True)
        assert np.max(np.abs(outf[i] - ref) / np.maximum(den, 1e-30)) <= 1e-5


@pytest.mark.parametrize("mode", ["plain", "compensated"])
def test_planes_float_modes(cuda, oracle, mode):
    """Stacks through the default kernels of each accumulator: f64 outputs
    (warp-specialized tiles) and compensated f32 (register tiles)."""
    p, h, w = 6, 77, 301
    a = oracle.gen("f32n", 15, (p * h, w)).astype(np.float32).reshape(p, h, w)
    if mode == "plain":
        out = to_np(sat_gb300.sat(to_dev(a), torch.float64))
        tol = 1e-13
    else:
        out = to_np(sat_gb300.sat(to_dev(a), torch.float32, mode="compensated"))
        tol = 2e-7
    for i in range(p):
        ref = oracle.sat_fp64(a[i])
        den = oracle.sat_fp64(a[i], absval=True)
        assert np.max(np.abs(out[i].astype(np.float64) - ref) / np.maximum(den, 1e-30)) <= tol, i


def test_planes_many_small(cuda, oracle):
    """More planes than tiles per plane: 300 planes of 40 x 70."""
    a = oracle.gen("u8", 14, (300 * 40, 70)).reshape(300, 40, 70)
    out = to_np(sat_gb300.sat(to_dev(a), torch.uint32))
    for i in (0, 1, 150, 299):
        assert np.array_equal(bits(out[i]), bits(oracle.sat_serial(a[i], np.uint32))), i


@pytest.mark.parametrize("shape", [(1, 1, 37, 53), (2, 3, 64, 64), (1, 2, 5, 300)])
def test_box_means_forward(cuda, shape):
    g = torch.Generator(device="cpu").manual_seed(21)
    x = torch.randn(shape, generator=g, dtype=torch.float32).to(cuda)
    radii = (0, 1, 3, 40)  # 40 exceeds every side: the whole image
    m = AG.box_filter_means(x, radii)
    ref = box_means64(x, radii)
    H, W = shape[-2:]
    smax = float(sat64(x.abs()).max())
    for k, r in enumerate(radii):
        area_min = (min(r, H - 1) + 1) * (min(r, W - 1) + 1)
        tol = 4 * EPS32 * smax / area_min + 1e-7
        err = float((m[..., k, :, :].double() - ref[..., k, :, :]).abs().max())
        assert err <= tol, (r, err, tol)


def _four_corner64(S: torch.Tensor, radii):
    """Box means in float64 from the given SAT S (..., H, W) by the four-corner
    rule, and per element the magnitudes |A| + |B| of its two row-segment
    differences A = S(yb,xb) - S(yb,xa-1), B = S(ya-1,xb) - S(ya-1,xa-1)."""
    H, W = S.shape[-2:]
    P = torch.nn.functional.pad(S.double(), (1, 0, 1, 0))
    ys = torch.arange(H, device=S.device)
    xs = torch.arange(W, device=S.device)
    means, mags = [], []
    for r in radii:
        ya, yb = (ys - r).clamp(min=0), (ys + r).clamp(max=H - 1)
        xa, xb = (xs - r).clamp(min=0), (xs + r).clamp(max=W - 1)
        A = P[..., yb + 1, :][..., xb + 1] - P[..., yb + 1, :][..., xa]
        B = P[..., ya, :][..., xb + 1] - P[..., ya, :][..., xa]
        area = ((yb - ya + 1).double()[:, None] * (xb - xa + 1).double()[None, :])
        means.append((A - B) / area)
        mags.append((A.abs() + B.abs()) / area)
    return torch.stack(means, dim=-3), torch.stack(mags, dim=-3)


@pytest.mark.parametrize("shape", [(2, 3, 256, 256), (1, 1, 1024, 1024)])
def test_box_means_forward_interior_blocks(cuda, shape):
    """Sizes where most blocks of the forward kernel are interior (every
    output of the 32 x 64 block has the whole window of the largest radius and
    the row and column before it), so the branch-free path is what is checked.
    Each mean is compared with the four-corner rule evaluated in float64 on the
    kernel's own f32 SAT: the kernel does two f32 subtractions of corner
    values, one of the differences and a multiply by the f32 1/area^2, so
    |m - m64| <= 2 eps32 (|A| + |B|) / area + 4 eps32 |m64| per element.  The
    means are also checked end to end against float64 from x with the file's
    tolerance."""
    g = torch.Generator(device="cpu").manual_seed(31)
    x = torch.randn(shape, generator=g, dtype=torch.float32).to(cuda)
    radii = (3, 7, 15)
    S = sat_gb300.sat(x, torch.float32)
    m = api.box_means_from_sat(S, radii)
    m64, mag = _four_corner64(S, radii)
    err = (m.double() - m64).abs()
    bound = 2 * EPS32 * mag + 4 * EPS32 * m64.abs() + 1e-30
    assert bool((err <= bound).all()), float((err / bound).max())
    # the interior fraction really is the bulk: blocks of 32 columns x 64 rows
    H, W = shape[-2:]
    rmax = max(radii)
    bx = [x0 for x0 in range(0, W, 32) if x0 - rmax - 1 >= 0 and x0 + 31 + rmax <= W - 1]
    by = [y0 for y0 in range(0, H, 64) if y0 - rmax - 1 >= 0 and y0 + 63 + rmax <= H - 1]
    frac = len(bx) * len(by) / ((-(-W // 32)) * (-(-H // 64)))
    assert frac >= (0.8 if H >= 1024 else 0.35), frac  # 420 of 512 blocks at 1024^2, 12 of 32 at 256^2
    ref = box_means64(x, radii)
    smax = float(sat64(x.abs()).max())
    for k, r in enumerate(radii):
        tol = 4 * EPS32 * smax / (r + 1) ** 2 + 1e-7
        assert float((m[..., k, :, :].double() - ref[..., k, :, :]).abs().max()) <= tol, r


def test_box_means_huge_radius_is_the_whole_image(cuda):
    """A radius far beyond the image (up to INT_MAX) filters like radius
    max(H, W) - 1, whose window already covers the whole image."""
    x = torch.rand((2, 33, 70), device=cuda)
    S = sat_gb300.sat(x, torch.float32)
    m = api.box_means_from_sat(S, (69, 1 << 20, 2**31 - 1))
    full = x.double().mean(dim=(-2, -1))[:, None, None, None].expand(2, 3, 33, 70)
    assert torch.allclose(m.double(), full, atol=1e-5)
    assert torch.equal(m[:, 0], m[:, 1]) and torch.equal(m[:, 0], m[:, 2])


def test_box_means_single_radius_matches_full_sum(cuda):
    x = torch.rand((3, 17, 29), device=cuda)
    m = AG.box_filter_means(x, (100,))
    full = x.double().mean(dim=(-2, -1))
    assert torch.allclose(m[:, 0].double(), full[:, None, None].expand(3, 17, 29), atol=1e-6)


def _grads(x, radii, wts):
    xg = x.clone().requires_grad_(True)
    loss = (AG.box_filter_means(xg, radii) * wts).sum()
    loss.backward()
    x64 = x.double().clone().requires_grad_(True)
    loss64 = (box_means64(x64, radii) * wts.double()).sum()
    loss64.backward()
    return xg.grad, x64.grad


@pytest.mark.parametrize("shape", [(2, 3, 64, 64), (1, 1, 33, 150), (1, 1, 1, 9)])
def test_box_grad_vs_float64_cumsum(cuda, shape):
    g = torch.Generator(device="cpu").manual_seed(22)
    x = torch.randn(shape, generator=g).to(cuda)
    radii = (3, 7, 15)
    wts = torch.randn(shape[:-2] + (3,) + shape[-2:], generator=g).to(cuda)
    gx, g64 = _grads(x, radii, wts)
    tol = 1e-4 * max(1.0, float(g64.abs().max()))
    assert float((gx.double() - g64).abs().max()) <= tol


@pytest.mark.parametrize("shape,radii", [
    ((1, 2, 200, 333), (2, 9, 32)),   # interior blocks next to border blocks, ragged block edges
    ((1, 1, 130, 170), (33,)),        # a radius whose window spans most of the image: no interior block
    ((1, 1, 97, 131), (0, 1, 32, 70)),  # radius 0, and a radius wider than the image on one side
])
def test_box_grad_tiles_and_large_radii(cuda, shape, radii):
    g = torch.Generator(device="cpu").manual_seed(25)
    x = torch.randn(shape, generator=g).to(cuda)
    wts = torch.randn(shape[:-2] + (len(radii),) + shape[-2:], generator=g).to(cuda)
    gx, g64 = _grads(x, radii, wts)
    tol = 1e-4 * max(1.0, float(g64.abs().max()))
    assert float((gx.double() - g64).abs().max()) <= tol


def test_box_grad_central_fd(cuda):
    """64 x 64 crops: the kernel gradient against FP64 central differences
    (h = 1e-3) of the FP64 loss at 24 random pixels."""
    g = torch.Generator(device="cpu").manual_seed(23)
    x = torch.randn((1, 3, 64, 64), generator=g).to(cuda)
    radii = (3, 7, 15)
    wts = torch.randn((1, 3, 3, 64, 64), generator=g).to(cuda)
    xg = x.clone().requires_grad_(True)
    (AG.box_filter_means(xg, radii) * wts).sum().backward()
    grad = xg.grad.double()
    x64 = x.double()
    h = 1e-3
    rng = np.random.default_rng(23)
    pts = [(int(rng.integers(3)), int(rng.integers(64)), int(rng.integers(64))) for _ in range(20)]
    pts += [(0, 0, 0), (1, 63, 63), (2, 0, 63), (0, 63, 0)]
    fds, ours = [], []
    for c, i, j in pts:
        e = torch.zeros_like(x64)
        e[0, c, i, j] = h
        lp = float((box_means64(x64 + e, radii) * wts.double()).sum())
        lm = float((box_means64(x64 - e, radii) * wts.double()).sum())
        fds.append((lp - lm) / (2 * h))
        ours.append(float(grad[0, c, i, j]))
    fds, ours = np.array(fds), np.array(ours)
    assert np.max(np.abs(fds - ours)) <= 1e-4 * max(1.0, np.max(np.abs(fds)))


def test_sat_function_grad(cuda):
    g = torch.Generator(device="cpu").manual_seed(24)
    x = torch.randn((2, 45, 71), generator=g).to(cuda)
    w = torch.randn((2, 45, 71), generator=g).to(cuda)
    xg = x.clone().requires_grad_(True)
    (AG.sat(xg) * w).sum().backward()
    x64 = x.double().clone().requires_grad_(True)
    (sat64(x64) * w.double()).sum().backward()
    assert float((xg.grad.double() - x64.grad).abs().max()) <= 1e-4 * float(x64.grad.abs().max())


def test_box_layer_module(cuda):
    layer = AG.BoxFilter((1, 2))
    x = torch.randn((2, 8, 8), device=cuda, requires_grad=True)
    y = layer(x)
    assert y.shape == (2, 2, 8, 8)
    y.sum().backward()
    assert x.grad is not None and x.grad.shape == x.shape


def test_box_filter_rejects_bad_args(cuda):
    x = torch.randn((4, 4), device=cuda)
    s = api.sat(x)
    with pytest.raises(sat_gb300.SatError):
        api.box_means_from_sat(s, ())
    with pytest.raises(sat_gb300.SatError):
        api.box_means_from_sat(s, (1, 2, 3, 4, 5))
    with pytest.raises(sat_gb300.SatError):
        api.box_means_from_sat(s, (-1,))
    with pytest.raises(sat_gb300.SatError):
        api.box_means_from_sat(s.double(), (1,))


@pytest.mark.parametrize("shape,radii", [((2, 3, 256, 256), (3, 7, 15)), ((1, 2, 200, 333), (2, 9, 32)),
                                         ((1, 1, 97, 131), (0, 1, 32, 70)), ((3, 1, 1, 9), (1,)),
                                         ((2, 1, 1, 1), (0, 3)), ((1, 2, 300, 1), (4,)),
                                         ((1, 1, 129, 257), (1, 128))])
def test_grad_x_matches_separate_calls(cuda, shape, radii):
    """satgb_box_filter_bwd_x (adjoint gather into the output, reverse SAT in
    place) against the separate calls (adjoint into a dL/dSAT tensor, then the
    reverse SAT into a new tensor): to 1e-5 of the largest gradient, and both
    to the float64 autograd gradient."""
    g = torch.Generator(device="cpu").manual_seed(27)
    wts = torch.randn(shape[:-2] + (len(radii),) + shape[-2:], generator=g).to(cuda)
    gx = api.box_means_grad_x(wts, radii)
    two = sat_gb300.sat(api.box_means_adjoint(wts, radii), torch.float32, reverse=True)
    scale = max(1.0, float(two.abs().max()))
    assert float((gx - two).abs().max()) <= 1e-5 * scale
    x = torch.randn(shape, generator=g).to(cuda)
    x64 = x.double().clone().requires_grad_(True)
    (box_means64(x64, radii) * wts.double()).sum().backward()
    assert float((gx.double() - x64.grad).abs().max()) <= 1e-4 * max(1.0, float(x64.grad.abs().max()))


def test_grad_x_pitched_planes(cuda):
    """Gradient planes and the output as strided views (row pitch > width)."""
    g = torch.Generator(device="cpu").manual_seed(28)
    base = torch.randn((2, 2, 70, 96), generator=g).to(cuda)
    wts = base[..., :90]
    out_base = torch.full((2, 70, 100), float("nan"), device=cuda)
    out = out_base[..., :90]
    api.box_means_grad_x(wts, (2, 5), out=out)
    ref = sat_gb300.sat(api.box_means_adjoint(wts.contiguous(), (2, 5)), torch.float32, reverse=True)
    assert float((out - ref).abs().max()) <= 1e-5 * max(1.0, float(ref.abs().max()))
    assert bool(torch.isnan(out_base[..., 90:]).all())  # the row padding is never written
