"""Sphere-traced depth maps and fitting the fractal's parameters to one.

render(): cg_trace_depth -- every pixel's ray marched on the estimator (the
          march of ShapeMesh::get_focii, src/mesh/mod.rs:229-241), hit when
          DE < 1e-4 x pixel footprint.
DepthRender: the render as a torch.autograd.Function of (power, rotation);
          its backward is cg_trace_backward_capped, the implicit-surface
          gradient dt/dtheta = -(dDE/dtheta) / (grad_x DE . d) at each hit,
          evaluated by the adjoint kernel, without the pixels whose
          derivative exceeds `cap`.
fit():    Adam on per-pixel L1 depth loss over pixels hit in both maps, plus
          (surface_weight > 0) the mean |DE| of the current shape at the
          target's own surface points, the term that carries the pixels the
          mask drops; the learning rate cosine-annealed from `lr`.

Why the cap: the estimator iterates a chaotic map, so at a small share of
points the exact derivative of the f32 DE with respect to the parameters is
enormous (the 99.9th percentile of |dt/dtheta| on the 256 x 256 map is
~200, of |dDE/dtheta| at the target's surface points up to 10^6, against
medians of 0.9 and 0.2).  Those points change by a finite, small amount over
any step an optimiser takes, but their derivatives swamp the sum: the raw
gradient of the depth loss points away from its finite difference (cosine
-0.4 averaged over six parameter points), and the surface term's is 10^5
times too large.  Leaving out the pixels above cap 2 (a tenth) and the
surface points above 1 gives cosines of 0.95 and 0.99 with the finite
differences, at the right scale for the surface term.
"""
import ctypes as C
import math

from . import _ffi
from ._ffi import check, load


def _torch():
    import torch
    return torch


def camera(width=1024, height=1024, distance=2.5, fov_deg=60.0):
    """Camera at `distance` on +z looking at the origin, y up."""
    c = _ffi.CgCamera()
    for k, v in enumerate((0.0, 0.0, distance)):
        c.eye[k] = v
    for k in range(3):
        c.target[k] = 0.0
    for k, v in enumerate((0.0, 1.0, 0.0)):
        c.up[k] = v
    c.fov_y = math.radians(fov_deg)
    c.width = width
    c.height = height
    return c


def _shape(power, rot, max_iters, bailout):
    s = _ffi.CgShape()
    s.kind = _ffi.CG_SHAPE_MANDELBULB_POLAR
    s.power = int(round(float(power)))
    s.power_f = float(power)
    s.max_iters = int(max_iters)
    s.bailout = float(bailout)
    for k in range(3):
        s.rot[k] = float(rot[k])
    return s


def render(power, rot, cam, max_steps=256, eps_scale=1e-4, max_iters=15, bailout=2.5,
           out=None, fast=False):
    """(height, width) CUDA depth map; -1 where the ray misses.  fast=True
    marches with the fast polar estimator (branch-free arctangent, SFU
    powers and sin/cos): same hits to within the march's tolerance."""
    torch = _torch()
    if out is None:
        out = torch.empty((cam.height, cam.width), dtype=torch.float32, device="cuda")
    shape = _shape(power, rot, max_iters, bailout)
    numerics = _ffi.CG_NUMERICS_FAST if fast else _ffi.CG_NUMERICS_EXACT
    check(load().cg_trace_depth(C.byref(shape), C.byref(cam), max_steps, eps_scale, numerics,
                                C.c_void_p(out.data_ptr()),
                                C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return out


def _make_render_fn():
    torch = _torch()

    class DepthRender(torch.autograd.Function):
        @staticmethod
        def forward(ctx, power, rot, cam, max_steps, eps_scale, max_iters, bailout, fast, cap):
            p = float(power)
            r = [float(v) for v in rot.detach().cpu()]
            depth = render(p, r, cam, max_steps, eps_scale, max_iters, bailout, fast=fast)
            ctx.save_for_backward(depth)
            ctx.shape = _shape(p, r, max_iters, bailout)
            ctx.cam = cam
            ctx.cap = float(cap)
            ctx.param_devices = (power.device if torch.is_tensor(power) else None,
                                 rot.device if torch.is_tensor(rot) else None)
            return depth

        @staticmethod
        def backward(ctx, grad_depth):
            (depth,) = ctx.saved_tensors
            g = grad_depth.detach().contiguous().float()
            params = torch.empty(4, dtype=torch.float32, device=depth.device)
            check(load().cg_trace_backward_capped(
                C.byref(ctx.shape), C.byref(ctx.cam), C.c_void_p(depth.data_ptr()),
                C.c_void_p(g.data_ptr()), ctx.cap, C.c_void_p(params.data_ptr()),
                C.c_void_p(torch.cuda.current_stream().cuda_stream)))
            pdev, rdev = ctx.param_devices
            return (params[0].to(pdev), params[1:4].to(rdev), None, None, None, None, None,
                    None, None)

    return DepthRender


_RENDER = None


def depth_render(power, rot, cam, max_steps=256, eps_scale=1e-4, max_iters=15, bailout=2.5,
                 fast=False, cap=0.0):
    """The depth map as a differentiable function of (power, rot); the
    backward leaves out pixels with |dt/dtheta_k| > cap (0: none)."""
    global _RENDER
    if _RENDER is None:
        _RENDER = _make_render_fn()
    return _RENDER.apply(power, rot, cam, max_steps, eps_scale, max_iters, bailout, fast, cap)


def l1_loss(depth, target):
    """Mean |depth - target| over pixels hit in both maps."""
    mask = (depth > 0) & (target > 0)
    n = mask.sum().clamp(min=1)
    return ((depth - target).abs() * mask).sum() / n


def pixel_rays(cam):
    """(height, width, 3) CUDA tensor of unit ray directions, formed as
    cg_trace_depth forms them (the camera basis in double, then f32)."""
    torch = _torch()
    eye = [cam.eye[k] for k in range(3)]
    f = [cam.target[k] - eye[k] for k in range(3)]
    fl = math.sqrt(sum(v * v for v in f))
    f = [v / fl for v in f]
    up = [cam.up[k] for k in range(3)]
    r = [f[1] * up[2] - f[2] * up[1], f[2] * up[0] - f[0] * up[2], f[0] * up[1] - f[1] * up[0]]
    rl = math.sqrt(sum(v * v for v in r))
    r = [v / rl for v in r]
    u = [r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]]
    th = math.tan(0.5 * cam.fov_y)
    aspect = cam.width / cam.height
    px = (torch.arange(cam.width, device="cuda", dtype=torch.float32) + 0.5) / cam.width
    py = (torch.arange(cam.height, device="cuda", dtype=torch.float32) + 0.5) / cam.height
    uu = ((px * 2.0 - 1.0) * th * aspect)[None, :, None]
    vv = ((1.0 - py * 2.0) * th)[:, None, None]
    F = torch.tensor(f, device="cuda", dtype=torch.float32)
    Rt = torch.tensor(r, device="cuda", dtype=torch.float32)
    U = torch.tensor(u, device="cuda", dtype=torch.float32)
    d = F + uu * Rt + vv * U
    return d / d.norm(dim=-1, keepdim=True)


def surface_points(target, cam):
    """(n, 3) CUDA tensor: the hit points eye + t d of the target's pixels."""
    torch = _torch()
    d = pixel_rays(cam)
    hit = target > 0
    eye = torch.tensor([cam.eye[k] for k in range(3)], device="cuda", dtype=torch.float32)
    return (eye + target[hit][:, None] * d[hit]).contiguous()


def _make_surface_fn():
    torch = _torch()

    class SurfaceL1(torch.autograd.Function):
        """mean |DE(p_i; power, rot)| and its gradient from one adjoint pass
        per point (cg_de_grad), without the points whose |dDE/dtheta_k|
        exceeds cap."""

        @staticmethod
        def forward(ctx, power, rot, points, max_iters, bailout, cap):
            from .autograd import de_grad
            g = de_grad(points, float(power), [float(v) for v in rot.detach().cpu()], max_iters,
                        bailout)
            ok = torch.isfinite(g).all(dim=1)
            n = ok.sum().clamp(min=1)
            de = g[:, 0]
            loss = de[ok].abs().sum() / n
            J = g[:, 4:8]
            keep = ok & (J.abs().max(dim=1).values <= cap) if cap > 0 else ok
            grad = (torch.sign(de[keep])[:, None] * J[keep]).sum(dim=0) / n
            ctx.save_for_backward(grad)
            ctx.devs = (power.device if torch.is_tensor(power) else None,
                        rot.device if torch.is_tensor(rot) else None)
            return loss

        @staticmethod
        def backward(ctx, gout):
            (grad,) = ctx.saved_tensors
            pdev, rdev = ctx.devs
            return ((gout * grad[0]).to(pdev), (gout * grad[1:4]).to(rdev), None, None, None,
                    None)

    return SurfaceL1


_SURFACE = None


def surface_loss(power, rot, points, max_iters=15, bailout=2.5, cap=1.0):
    """Mean |DE| of the shape (power, rot) at `points`: zero when its surface
    passes through them, and it counts every target pixel, also those the
    current render misses.  Differentiable in power and rot; the gradient
    leaves out points with |dDE/dtheta_k| > cap (0: none)."""
    global _SURFACE
    if _SURFACE is None:
        _SURFACE = _make_surface_fn()
    return _SURFACE.apply(power, rot, points, max_iters, bailout, cap)


def fit(target, cam, power0=8.0, rot0=(0.0, 0.0, 0.0), steps=300, lr=1e-2, max_steps=256,
        eps_scale=1e-4, callback=None, fast=False, surface_weight=1.0, cap=2.0,
        surface_cap=1.0, anneal=True):
    """Adam on (power, rotation); returns (power, rot, losses), the depth L1
    loss of each step.  fast=True marches with the fast estimator; the
    gradient is exact either way.  The objective is the depth L1 loss (its
    backward without pixels above `cap`) plus surface_weight times
    surface_loss at the target's surface points (without points above
    surface_cap); with anneal the learning rate falls from lr to 0 on a
    cosine over the steps.  surface_weight=0, cap=0, anneal=False is plain
    Adam on the masked depth loss."""
    torch = _torch()
    power = torch.tensor(float(power0), requires_grad=True)
    rot = torch.tensor([float(v) for v in rot0], requires_grad=True)
    opt = torch.optim.Adam([power, rot], lr=lr)
    sched = (torch.optim.lr_scheduler.CosineAnnealingLR(opt, T_max=steps) if anneal else None)
    pts = surface_points(target, cam) if surface_weight > 0 else None
    losses = []
    for it in range(steps):
        opt.zero_grad()
        depth = depth_render(power, rot, cam, max_steps, eps_scale, fast=fast, cap=cap)
        loss = l1_loss(depth, target)
        total = loss
        if pts is not None:
            total = loss + surface_weight * surface_loss(power, rot, pts, cap=surface_cap)
        total.backward()
        opt.step()
        if sched is not None:
            sched.step()
        losses.append(float(loss.detach()))
        if callback:
            callback(it, float(power.detach()), rot.detach().tolist(), losses[-1])
    return float(power.detach()), rot.detach().tolist(), losses
