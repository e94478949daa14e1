"""Density grid over a Gaussian field (C ABI ``arap_grid_*``).

Mirrors the reference's grid set-up (getOverallAABB, getGridSamples,
UpdateContainingRelationship, GetAdaLpfRatio; GaussianView.cpp:3601-4149,
4670-4751) and the host contract of its density sampler (forward3d_grid,
GaussianView.cpp:4222-4249).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import GridInfo, check
from .deform import _f32, _p, _s

LPF_PARAMETER = 0.2  # GaussianView.hpp:482


class Grid:
    """Cell binning of one Gaussian field; owns the CSR on the device."""

    def __init__(self, pos, rot, scale, opacity, grid_num, padding=1):
        lib = _lib.load()
        self.pos, self.rot, self.scale, self.opacity = _f32(pos), _f32(rot), _f32(scale), _f32(opacity)
        self.N = self.pos.shape[0]
        info = GridInfo()
        h = C.c_void_p()
        check("arap_grid_build", lib.arap_grid_build(
            C.byref(h), self.N, _p(self.pos), _p(self.rot), _p(self.scale), _p(self.opacity),
            int(grid_num), int(padding), C.byref(info), _s()))
        self._h = h
        self.info = info
        self.grid_num = int(grid_num)
        self.n_valid = int(info.n_valid)
        self.n_pairs = int(info.n_pairs)
        self.step = float(info.step)
        self.min_xyz = tuple(info.min_xyz)
        self.max_xyz = tuple(info.max_xyz)
        self.sample_pos = torch.empty((self.n_valid * 64, 3), dtype=torch.float32, device="cuda")
        check("arap_grid_samples", lib.arap_grid_samples(h, _p(self.sample_pos), _s()))
        # low_pass_filter_param = (step/4)^2 * lpf_parameter (GaussianView.cpp:3879-3881)
        self.lpf_param = (self.step / 4.0) ** 2 * LPF_PARAMETER

    def status(self) -> int:
        """Read and clear the grid's device status word (synchronises)."""
        return _lib.load().arap_grid_status(self._h, _s())

    def arrays(self):
        """(cell_offsets [g^3+1], cell_lists [n_pairs], valid_cells [n_valid]) as int32 tensor copies."""
        off, lst, val = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check("arap_grid_arrays", _lib.load().arap_grid_arrays(self._h, C.byref(off), C.byref(lst), C.byref(val)))
        g3 = self.grid_num ** 3
        return (_wrap_i32(off.value, g3 + 1), _wrap_i32(lst.value, self.n_pairs),
                _wrap_i32(val.value, self.n_valid))

    def center_order(self, pos=None):
        """Stable cell order of the Gaussian centres (int64 permutation)."""
        pos = self.pos if pos is None else _f32(pos)
        out = torch.empty((pos.shape[0],), dtype=torch.int32, device="cuda")
        check("arap_grid_center_order", _lib.load().arap_grid_center_order(
            self._h, pos.shape[0], _p(pos), _p(out), _s()))
        return out.long()

    def ada_lpf(self, samples=None, lpf=LPF_PARAMETER):
        samples = self.sample_pos if samples is None else _f32(samples)
        out = torch.empty((self.n_valid, 9), dtype=torch.float32, device="cuda")
        check("arap_grid_ada_lpf", _lib.load().arap_grid_ada_lpf(self._h, _p(samples), float(lpf), _p(out), _s()))
        return out

    def density(self, shs, samples=None, ada=None, lpf_param=None):
        samples = self.sample_pos if samples is None else _f32(samples)
        lpf_param = self.lpf_param if lpf_param is None else lpf_param
        S = self.n_valid * 64
        sigma = torch.empty((S,), dtype=torch.float32, device="cuda")
        feat = torch.empty((S, 48), dtype=torch.float32, device="cuda")
        check("arap_grid_density", _lib.load().arap_grid_density(
            self._h, _p(self.pos), _p(self.rot), _p(self.scale), _p(self.opacity), _p(_f32(shs)), _p(samples),
            _p(ada) if ada is not None else None, float(lpf_param), _p(sigma), _p(feat), _s()))
        return sigma, feat

    def stage2_loss_grad(self, params, aim_sigma, aim_feature, samples=None, ada=None, lpf_param=None,
                         cell_active=None, feature_weight=1.0, with_loss=True):
        """The Stage-II L1 loss and its gradient (arap_stage2_loss_grad).

        ``params``: dict of raw attributes ``pos`` [N,3], ``rot`` [N,4],
        ``log_scale`` [N,3], ``logit_opacity`` [N], ``shs`` [N,48] of the
        Gaussians this grid was built over.  Returns ((shape loss, feature
        loss) or None, dict of gradients shaped as ``params``)."""
        samples = self.sample_pos if samples is None else _f32(samples)
        lpf_param = self.lpf_param if lpf_param is None else lpf_param
        p = {k: _f32(params[k]) for k in ("pos", "rot", "log_scale", "logit_opacity", "shs")}
        grads = {k: torch.empty_like(v) for k, v in p.items()}
        act = None
        if cell_active is not None:
            act = torch.as_tensor(cell_active, device="cuda").to(torch.uint8).contiguous()
        loss = (C.c_double * 2)() if with_loss else None
        check("arap_stage2_loss_grad", _lib.load().arap_stage2_loss_grad(
            self._h, _p(p["pos"]), _p(p["rot"]), _p(p["log_scale"]), _p(p["logit_opacity"]), _p(p["shs"]),
            _p(samples), _p(ada) if ada is not None else None, float(lpf_param), _p(_f32(aim_sigma)),
            _p(_f32(aim_feature)), _p(act) if act is not None else None, float(feature_weight),
            _p(grads["pos"]), _p(grads["rot"]), _p(grads["log_scale"]), _p(grads["logit_opacity"]),
            _p(grads["shs"]), C.cast(loss, C.POINTER(C.c_double)) if loss is not None else None, _s()))
        return ((loss[0], loss[1]) if loss is not None else None), grads

    def stage2_cell_flags(self, aim_opacity=None, converged=None):
        """(empty [n_valid] uint8 or None, converged [n_valid] uint8 or None):
        JudgeEmptyGrid from the samples' aim opacities and ExpandOpRange of
        ``converged`` (arap_stage2_cell_flags)."""
        empty = None
        if aim_opacity is not None:
            aim_opacity = _f32(aim_opacity)
            empty = torch.empty((self.n_valid,), dtype=torch.uint8, device="cuda")
        conv = None
        if converged is not None:
            conv = torch.as_tensor(converged, device="cuda").to(torch.uint8).contiguous().clone()
        check("arap_stage2_cell_flags", _lib.load().arap_stage2_cell_flags(
            self._h, _p(aim_opacity) if aim_opacity is not None else None,
            _p(empty) if empty is not None else None, _p(conv) if conv is not None else None, _s()))
        return empty, conv

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().arap_grid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DevView:
    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (int(ptr or 0), False),
                                         "version": 3}


def _wrap_i32(ptr, n):
    """Copy n int32 from a library-owned device pointer into a new tensor."""
    if n == 0:
        return torch.empty((0,), dtype=torch.int32, device="cuda")
    return torch.as_tensor(_DevView(ptr, n), device="cuda").clone()


def build_grid(pos, rot, scale, opacity, grid_num, padding=1):
    return Grid(pos, rot, scale, opacity, grid_num, padding)


# Learning rates for opacity, SH, mean, quaternion, log-scale (GaussianView.hpp:418).
STAGE2_LEARNING_RATES = (0.0, 0.002, 0.005, 0.1, 0.0001)


class Stage2Adam:
    """Adam moments of the raw attributes of N Gaussians (arap_stage2_adam)."""

    def __init__(self, N, lr=STAGE2_LEARNING_RATES):
        self.N = int(N)
        self.lr = (C.c_float * 5)(*[float(v) for v in lr])
        self.m = torch.zeros((self.N, 59), dtype=torch.float32, device="cuda")
        self.v = torch.zeros((self.N, 59), dtype=torch.float32, device="cuda")
        self.step = 0

    def update(self, params, grads, moved=None):
        """One step; ``params`` (float32 CUDA tensors, contiguous) is updated in place."""
        self.step += 1
        mv = None
        if moved is not None:
            mv = torch.as_tensor(moved, device="cuda").to(torch.uint8).contiguous()
        for k in ("pos", "rot", "log_scale", "logit_opacity", "shs"):
            t = params[k]
            if t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous():
                raise ValueError("Stage2Adam.update: %s must be a contiguous float32 CUDA tensor" % k)
        check("arap_stage2_adam", _lib.load().arap_stage2_adam(
            self.N, self.step, C.cast(self.lr, C.c_void_p), _p(mv) if mv is not None else None,
            _p(params["logit_opacity"]), _p(params["shs"]), _p(params["pos"]), _p(params["rot"]),
            _p(params["log_scale"]), _p(grads["logit_opacity"]), _p(grads["shs"]), _p(grads["pos"]),
            _p(grads["rot"]), _p(grads["log_scale"]), _p(self.m), _p(self.v), _s()))


def stage2_align(grid, params, aim_sigma, aim_feature, steps=101, moved=None, lr=STAGE2_LEARNING_RATES,
                 feature_weight=1.0, ada=None, lpf_param=None, cell_active=None):
    """The Stage-II loop (GPUOptimize, GaussianView.cpp:4363-4486, run
    ``_optimize_steps`` = 101 times, GaussianView.hpp:420): loss and gradient,
    then an Adam step of the moved Gaussians, ``steps`` times.  ``params`` is
    updated in place; returns the (shape, feature) loss before each step."""
    opt = Stage2Adam(params["pos"].shape[0], lr)
    losses = []
    for _ in range(int(steps)):
        loss, grads = grid.stage2_loss_grad(params, aim_sigma, aim_feature, ada=ada, lpf_param=lpf_param,
                                            cell_active=cell_active, feature_weight=feature_weight)
        losses.append(loss)
        opt.update(params, grads, moved=moved)
    return losses
