"""Full-waveform-inversion face: the velocity -> seismogram map as a
torch.autograd.Function whose backward is the GPU library's exact discrete
adjoint (st_shot_gradient), and the L2 misfit + gradient of a set of shots
(st_fwi_gradient). Velocities are torch CUDA tensors (nx, ny, nz), z fastest.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import call
from .wave import WaveEquationSolver, _shot_c


def set_velocity_device(solver: WaveEquationSolver, vel: torch.Tensor):
    """Sets the model from a CUDA tensor. Inside solver.on_stream(torch's
    current stream) the copy is ordered on that stream; otherwise the current
    stream is synchronised first so the tensor is complete."""
    v = vel.detach().to(device="cuda", dtype=torch.float32).contiguous()
    cur = torch.cuda.current_stream()
    if solver.stream_ptr() != cur.cuda_stream:
        cur.synchronize()
    call("st_solver_set_velocity_device", solver.handle, v.data_ptr())
    if solver.stream_ptr() != cur.cuda_stream:
        torch.cuda.ExternalStream(solver.stream_ptr()).synchronize()


def _ckpt(checkpoint):
    """checkpoint: None (store every step) or (segment_steps, max_slots)."""
    if checkpoint is None:
        return None
    seg, slots = checkpoint
    return int(seg), int(slots)


def shot_gradient(solver, src, wavelet, nt, rec, adj_src, grad_v, snap_kind=_lib.ST_SNAP_FP32, checkpoint=None):
    """grad_v += d<F(v), adj_src>/dv for one shot (device tensors). With
    checkpoint=(segment_steps, max_slots) the forward history is recomputed
    from FP32 checkpoints instead of stored for every step."""
    shot, _keep = _shot_c(src, wavelet, nt, rec)
    ck = _ckpt(checkpoint)
    if ck is None:
        return call("st_shot_gradient", solver.handle, C.byref(shot), adj_src.data_ptr(), int(snap_kind),
                    grad_v.data_ptr())
    st = _lib.CheckpointStatsC()
    call("st_shot_gradient_checkpointed", solver.handle, C.byref(shot), adj_src.data_ptr(), int(snap_kind), ck[0],
         ck[1], grad_v.data_ptr(), C.byref(st))
    return {k: getattr(st, k) for k, _ in _lib.CheckpointStatsC._fields_}


def fwi_gradient(solver, src, wavelet, nt, rec, d_obs, grad_v=None, snap_kind=_lib.ST_SNAP_FP32, residual=None,
                 checkpoint=None):
    """L2 misfit 1/2 sum (F(v) - d_obs)^2 of one shot (FP64) and, when grad_v is
    given, grad_v += its gradient (checkpoint as in shot_gradient)."""
    shot, _keep = _shot_c(src, wavelet, nt, rec)
    m = C.c_double(0.0)
    gv = grad_v.data_ptr() if grad_v is not None else None
    rs = residual.data_ptr() if residual is not None else None
    ck = _ckpt(checkpoint)
    if ck is None:
        call("st_fwi_gradient", solver.handle, C.byref(shot), d_obs.data_ptr(), int(snap_kind), gv, C.byref(m), rs)
    else:
        call("st_fwi_gradient_checkpointed", solver.handle, C.byref(shot), d_obs.data_ptr(), int(snap_kind), ck[0],
             ck[1], gv, C.byref(m), rs, None)
    return m.value


class SeismicModeling(torch.autograd.Function):
    """d = F(v): seismograms [n_shots, nt, nrec] of every shot for velocity v.
    backward: the exact adjoint of the discrete forward map (fused GPU
    kernel), forward snapshots recomputed and stored with snap_kind. Both run
    on torch's current stream (the solver is switched to it for the call), so
    they are ordered with the surrounding torch work without a device sync."""

    @staticmethod
    def forward(ctx, vel, solver, shots, nt, snap_kind, checkpoint=None):
        from .wave import shot_forward
        nrec = shots[0].rec.count
        with solver.on_stream(torch.cuda.current_stream()):
            set_velocity_device(solver, vel)
            out = torch.zeros((len(shots), nt, nrec), device="cuda", dtype=torch.float32)
            for i, sh in enumerate(shots):
                shot_forward(solver, sh.src, sh.wavelet, nt, sh.rec, seis=out[i])
        ctx.save_for_backward(vel)
        ctx.solver, ctx.shots, ctx.nt, ctx.snap_kind, ctx.checkpoint = solver, shots, nt, snap_kind, checkpoint
        return out.to(vel.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (vel,) = ctx.saved_tensors
        solver = ctx.solver
        with solver.on_stream(torch.cuda.current_stream()):
            set_velocity_device(solver, vel)
            g = torch.zeros(vel.shape, device="cuda", dtype=torch.float32)
            go = grad_out.to(dtype=torch.float32).contiguous()
            for i, sh in enumerate(ctx.shots):
                shot_gradient(solver, sh.src, sh.wavelet, ctx.nt, sh.rec, go[i].contiguous(), g, ctx.snap_kind,
                              checkpoint=ctx.checkpoint)
        return g.to(vel.dtype), None, None, None, None, None


def modeling(vel: torch.Tensor, solver: WaveEquationSolver, shots, nt: int, snap_kind=_lib.ST_SNAP_FP32,
             checkpoint=None):
    """Differentiable seismograms; checkpoint=(segment_steps, max_slots)
    recomputes the forward history in backward instead of storing it."""
    return SeismicModeling.apply(vel, solver, shots, nt, snap_kind, checkpoint)
