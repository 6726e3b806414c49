"""Sphere-traced depth maps and fitting the fractal's parameters to one.

render(): cg_trace_depth -- every pixel's ray marched on the estimator (the
          march of ShapeMesh::get_focii, src/mesh/mod.rs:229-241), hit when
          DE < 1e-4 x pixel footprint.
DepthRender: the render as a torch.autograd.Function of (power, rotation);
          its backward is cg_trace_backward, the implicit-surface gradient
          dt/dtheta = -(dDE/dtheta) / (grad_x DE . d) at each hit, evaluated
          by the adjoint kernel.
fit():    Adam on per-pixel L1 depth loss over pixels hit in both maps.
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
        def forward(ctx, power, rot, cam, max_steps, eps_scale, max_iters, bailout, fast):
            p = float(power)
            r = [float(v) for v in rot.detach().cpu()]
            depth = render(p, r, cam, max_steps, eps_scale, max_iters, bailout, fast=fast)
            ctx.save_for_backward(depth)
            ctx.shape = _shape(p, r, max_iters, bailout)
            ctx.cam = cam
            ctx.param_devices = (power.device if torch.is_tensor(power) else None,
                                 rot.device if torch.is_tensor(rot) else None)
            return depth

        @staticmethod
        def backward(ctx, grad_depth):
            (depth,) = ctx.saved_tensors
            g = grad_depth.detach().contiguous().float()
            params = torch.empty(4, dtype=torch.float32, device=depth.device)
            check(load().cg_trace_backward(C.byref(ctx.shape), C.byref(ctx.cam),
                                           C.c_void_p(depth.data_ptr()), C.c_void_p(g.data_ptr()),
                                           C.c_void_p(params.data_ptr()),
                                           C.c_void_p(torch.cuda.current_stream().cuda_stream)))
            pdev, rdev = ctx.param_devices
            return (params[0].to(pdev), params[1:4].to(rdev), None, None, None, None, None,
                    None)

    return DepthRender


_RENDER = None


def depth_render(power, rot, cam, max_steps=256, eps_scale=1e-4, max_iters=15, bailout=2.5,
                 fast=False):
    global _RENDER
    if _RENDER is None:
        _RENDER = _make_render_fn()
    return _RENDER.apply(power, rot, cam, max_steps, eps_scale, max_iters, bailout, fast)


def l1_loss(depth, target):
    """Mean |depth - target| over pixels hit in both maps."""
    mask = (depth > 0) & (target > 0)
    n = mask.sum().clamp(min=1)
    return ((depth - target).abs() * mask).sum() / n


def fit(target, cam, power0=8.0, rot0=(0.0, 0.0, 0.0), steps=300, lr=1e-2, max_steps=256,
        eps_scale=1e-4, callback=None, fast=False):
    """Adam on (power, rotation); returns (power, rot, losses).  fast=True
    marches with the fast estimator; the gradient is exact either way."""
    torch = _torch()
    power = torch.tensor(float(power0), requires_grad=True)
    rot = torch.tensor([float(v) for v in rot0], requires_grad=True)
    opt = torch.optim.Adam([power, rot], lr=lr)
    losses = []
    for it in range(steps):
        opt.zero_grad()
        depth = depth_render(power, rot, cam, max_steps, eps_scale, fast=fast)
        loss = l1_loss(depth, target)
        loss.backward()
        opt.step()
        losses.append(float(loss.detach()))
        if callback:
            callback(it, float(power.detach()), rot.detach().tolist(), losses[-1])
    return float(power.detach()), rot.detach().tolist(), losses
