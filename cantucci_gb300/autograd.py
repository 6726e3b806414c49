"""The distance estimator as a torch.autograd.Function.

forward:  cg_min_distance_from (the polar-form estimator, f32).
backward: cg_de_backward -- the hand-written adjoint kernel, which recomputes
          the iterates from checkpoints instead of saving them -- giving
          dL/dpoints and dL/d(power, euler angles).

    power = torch.tensor(8.0, requires_grad=True)
    rot = torch.zeros(3, requires_grad=True)
    d = mandelbulb_de(points, power, rot, max_iters=15, bailout=2.5)
    d.sum().backward()
"""
import ctypes as C

from . import _ffi
from ._ffi import check, load


def _torch():
    import torch
    return torch


def _shape(power: float, rot, max_iters: int, bailout: float) -> _ffi.CgShape:
    s = _ffi.CgShape()
    s.kind = _ffi.CG_SHAPE_MANDELBULB_POLAR
    s.power = int(round(power))
    s.power_f = float(power)
    s.max_iters = int(max_iters)
    s.bailout = float(bailout)
    for k in range(3):
        s.rot[k] = float(rot[k])
    return s


def _make_function():
    torch = _torch()

    class MandelbulbDE(torch.autograd.Function):
        @staticmethod
        def forward(ctx, points, power, rot, max_iters, bailout):
            pts = points.detach().contiguous().float()
            shape = _shape(float(power), [float(r) for r in rot.detach().cpu()], max_iters,
                           bailout)
            out = torch.empty(pts.shape[0], dtype=torch.float32, device=pts.device)
            stream = torch.cuda.current_stream(pts.device)
            check(load().cg_min_distance_from(C.byref(shape), C.c_void_p(pts.data_ptr()),
                                              pts.shape[0], C.c_void_p(out.data_ptr()),
                                              _ffi.CG_NUMERICS_EXACT,
                                              C.c_void_p(stream.cuda_stream)))
            ctx.save_for_backward(pts)  # the points only; no iterates
            ctx.shape = shape
            ctx.param_devices = (power.device if torch.is_tensor(power) else None,
                                 rot.device if torch.is_tensor(rot) else None)
            return out

        @staticmethod
        def backward(ctx, grad_out):
            (pts,) = ctx.saved_tensors
            g = grad_out.detach().contiguous().float()
            gp = torch.empty_like(pts) if ctx.needs_input_grad[0] else None
            params = torch.empty(4, dtype=torch.float32, device=pts.device)
            stream = torch.cuda.current_stream(pts.device)
            check(load().cg_de_backward(C.byref(ctx.shape), C.c_void_p(pts.data_ptr()),
                                        C.c_void_p(g.data_ptr()), pts.shape[0],
                                        C.c_void_p(gp.data_ptr()) if gp is not None else None,
                                        C.c_void_p(params.data_ptr()),
                                        C.c_void_p(stream.cuda_stream)))
            pdev, rdev = ctx.param_devices
            gpow = params[0].to(pdev) if ctx.needs_input_grad[1] else None
            grot = params[1:4].to(rdev) if ctx.needs_input_grad[2] else None
            return gp, gpow, grot, None, None

    return MandelbulbDE


_FN = None


def mandelbulb_de(points, power, rot, max_iters: int = 15, bailout: float = 2.5):
    """DE of (n, 3) CUDA points for a polar Mandelbulb with tensor parameters
    `power` (scalar) and `rot` (3 Euler angles), differentiable in all three."""
    global _FN
    if _FN is None:
        _FN = _make_function()
    return _FN.apply(points, power, rot, max_iters, bailout)


def de_grad(points, power: float, rot=(0.0, 0.0, 0.0), max_iters: int = 15,
            bailout: float = 2.5, mode: str = "adjoint", with_power: bool = True,
            fast: bool = False):
    """(n, 8) CUDA tensor: DE, dDE/dp (3), dDE/dpower, dDE/d(euler) (3).

    mode "adjoint": reverse mode with checkpoint recompute (cg_de_grad).
    mode "tangent": forward mode, one pass (cg_de_grad_tangent); with
    with_power=False it skips the power direction (column 4 is 0), which is
    all a normal needs; fast=True iterates with the fast polar estimator's
    arithmetic."""
    if fast and mode != "tangent":
        raise ValueError("fast numerics are for mode 'tangent'")
    torch = _torch()
    pts = points.contiguous().float()
    out = torch.empty((pts.shape[0], 8), dtype=torch.float32, device=pts.device)
    shape = _shape(power, rot, max_iters, bailout)
    stream = C.c_void_p(torch.cuda.current_stream(pts.device).cuda_stream)
    if mode == "adjoint":
        check(load().cg_de_grad(C.byref(shape), C.c_void_p(pts.data_ptr()), pts.shape[0],
                                C.c_void_p(out.data_ptr()), stream))
    elif mode == "tangent":
        flags = (1 if with_power else 0) | (2 if fast else 0)
        check(load().cg_de_grad_tangent(C.byref(shape), C.c_void_p(pts.data_ptr()),
                                        pts.shape[0], flags, C.c_void_p(out.data_ptr()), stream))
    else:
        raise ValueError("mode is 'adjoint' or 'tangent'")
    return out


def spatial_grad(points, shape):
    """(n, 4) CUDA tensor: DE and dDE/dp of any shape, one forward-mode pass
    per point (cg_de_spatial_grad)."""
    torch = _torch()
    pts = points.contiguous().float()
    out = torch.empty((pts.shape[0], 4), dtype=torch.float32, device=pts.device)
    check(load().cg_de_spatial_grad(C.byref(shape._cshape()), C.c_void_p(pts.data_ptr()),
                                    pts.shape[0], C.c_void_p(out.data_ptr()),
                                    C.c_void_p(torch.cuda.current_stream(pts.device).cuda_stream)))
    return out


def fd_grad(points, shape, h: float):
    """(n, 3) central-difference gradient with six estimator calls per point."""
    torch = _torch()
    pts = points.contiguous().float()
    out = torch.empty((pts.shape[0], 3), dtype=torch.float32, device=pts.device)
    check(load().cg_fd_grad(C.byref(shape._cshape()), C.c_void_p(pts.data_ptr()), pts.shape[0],
                            float(h), C.c_void_p(out.data_ptr()),
                            C.c_void_p(torch.cuda.current_stream(pts.device).cuda_stream)))
    return out
