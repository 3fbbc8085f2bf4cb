"""Gradient harness for differentiable stepping (torch.autograd wrapper of the C ABI).

The product is the C entry points of include/box2d/gpu.h (b2World_BeginTape,
b2World_StepBatch, b2World_StepBackwardBatch).  This module wraps them in a
torch.autograd.Function for the drop-boxes workload: W independent worlds, each with
boxes of half-extent 0.5 dropped from given heights onto the static ground, initial
velocities v0 and one friction coefficient per world (set on the ground and on every
box, so the mixed friction sqrt(mu * mu) equals mu).  The forward pass records the
steps and returns the final box positions; the backward pass runs the hand-written
adjoint and returns dL/dv0 and dL/dmu.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .capi import Backend, WorldId, bind_batch_api, bind_gpu_api, world_array

STATE = 6  # per body: p.x p.y angle v.x v.y w


def bind_adjoint_api(lib: C.CDLL) -> None:
    lib.b2World_BeginTape.argtypes = [WorldId, C.c_int]
    lib.b2World_BeginTape.restype = None
    lib.b2World_GetTapeSteps.argtypes = [WorldId]
    lib.b2World_GetTapeSteps.restype = C.c_int
    lib.b2World_StepBackward.argtypes = [WorldId, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.b2World_StepBackward.restype = C.c_int
    lib.b2World_StepBackwardBatch.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.b2World_StepBackwardBatch.restype = C.c_int
    lib.b2World_GetBackwardCheck.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.b2World_GetBackwardCheck.restype = None


class DropBoxes:
    """W drop-boxes worlds stepped together on the GPU library."""

    def __init__(self, backend: Backend, heights: np.ndarray, steps: int = 120, substeps: int = 4, dt: float = 1.0 / 60.0,
                 kinds: np.ndarray | None = None):
        self.b = backend
        self.heights = np.ascontiguousarray(heights, np.float32)
        # per world and body: 0 box, 1 circle, 2 capsule (all boxes when None)
        self.kinds = None if kinds is None else np.ascontiguousarray(kinds, np.int32)
        self.worlds_n, self.boxes = self.heights.shape
        self.steps, self.substeps, self.dt = steps, substeps, dt
        self.bodies = self.boxes + 1  # ground is body 0
        self.shapes = self.boxes + 1
        bind_gpu_api(backend.lib)
        bind_batch_api(backend.lib)
        bind_adjoint_api(backend.lib)
        self.worlds = []
        self.last_status = 0

    def create(self, v0: np.ndarray, mu: np.ndarray, record: bool = True) -> None:
        """Builds the worlds (recording the next `steps` steps when `record`)."""
        self.destroy()
        L = self.b.lib
        for w in range(self.worlds_n):
            world = self.b.drop_boxes(self.heights[w], v0[w, :, 0], v0[w, :, 1], float(mu[w]),
                                      None if self.kinds is None else self.kinds[w])
            if record:
                L.b2World_BeginTape(world, self.steps)
            self.worlds.append(world)
        self.ids = world_array(self.worlds)

    def step_all(self) -> None:
        """Steps every world `steps` times, all worlds per batched call."""
        L = self.b.lib
        for _ in range(self.steps):
            L.b2World_StepBatch(self.ids, len(self.worlds), self.dt, self.substeps)

    def run(self, v0: np.ndarray, mu: np.ndarray, record: bool = True) -> np.ndarray:
        """Builds the worlds, steps them and returns final box positions [W, boxes, 2]."""
        self.create(v0, mu, record)
        self.step_all()
        return self.positions()

    def positions(self) -> np.ndarray:
        L = self.b.lib
        out = np.zeros((self.worlds_n, self.boxes, 2), np.float32)
        buf = np.zeros(7 * self.bodies, np.float32)
        for w, world in enumerate(self.worlds):
            L.b2World_GetBodyStates(world, buf.ctypes.data, self.bodies)
            out[w] = buf.reshape(self.bodies, 7)[1:, 0:2]
        return out

    def backward(self, grad_p: np.ndarray):
        """dL/dv0 [W, boxes, 2] and dL/dmu [W] for dL/dp_final = grad_p."""
        L = self.b.lib
        n = len(self.worlds)
        gf = np.zeros((n, self.bodies, STATE), np.float32)
        gf[:, 1:, 0:2] = grad_p
        gi = np.zeros_like(gf)
        gmu = np.zeros((n, self.shapes), np.float32)
        rc = L.b2World_StepBackwardBatch(world_array(self.worlds), n, self.bodies, self.shapes, gf.ctypes.data, gi.ctypes.data,
                                         gmu.ctypes.data)
        self.last_status = rc
        if rc != 0:
            raise RuntimeError(f"b2World_StepBackwardBatch failed: {rc}")
        return gi[:, 1:, 3:5].copy(), gmu.sum(1)

    def destroy(self):
        for w in self.worlds:
            self.b.destroy(w)
        self.worlds = []


class DropBoxesStep(torch.autograd.Function):
    """p_final = f(v0, mu) through `steps` recorded steps; gradients by the adjoint."""

    @staticmethod
    def forward(ctx, v0: torch.Tensor, mu: torch.Tensor, sim: DropBoxes):
        p = sim.run(v0.detach().cpu().numpy(), mu.detach().cpu().numpy(), record=True)
        ctx.sim = sim
        return torch.from_numpy(p)

    @staticmethod
    def backward(ctx, grad_p: torch.Tensor):
        gv0, gmu = ctx.sim.backward(grad_p.detach().cpu().numpy().astype(np.float32))
        return torch.from_numpy(gv0), torch.from_numpy(gmu.astype(np.float32)), None


def drop_boxes_loss(sim: DropBoxes, v0: torch.Tensor, mu: torch.Tensor) -> torch.Tensor:
    """Sum of squared final box positions over all worlds."""
    p = DropBoxesStep.apply(v0, mu, sim)
    return (p.double() ** 2).sum()
