"""GB300 twin of ``tensorf/tensor_vm.py``.

``TensorVM`` keeps the reference's API (``initialize``, ``interpolate``, ``grid_dim``,
``channel_dim``) but stores its three vector-matrix pairs channel-last on the device
(lines ``[3][G][C]``, planes ``[3][G][G][C]``) and evaluates them with the sm_103a
kernels behind ``tvm_vm_features_fwd`` / ``tvm_vm_features_bwd``.
"""
from __future__ import annotations

from typing import Optional

import torch

from . import _lib
from ._util import ptr, require_cuda, stream_handle

_DTYPE_CODE = {torch.float32: _lib.TVM_F32, torch.bfloat16: _lib.TVM_BF16}


def field_struct(lines: torch.Tensor, planes: torch.Tensor) -> _lib.VmField:
    g = planes.shape[1]
    c = planes.shape[-1]
    if lines.shape != (3, g, c) or planes.shape != (3, g, g, c):
        raise ValueError(f"bad field shapes {tuple(lines.shape)} / {tuple(planes.shape)}")
    if lines.dtype != planes.dtype or lines.dtype not in _DTYPE_CODE:
        raise TypeError("lines/planes must both be float32 or bfloat16")
    return _lib.VmField(grid_dim=g, channels=c, dtype=_DTYPE_CODE[lines.dtype], _pad=0,
                        lines=ptr(lines, name="lines"), planes=ptr(planes, name="planes"))


class _Interpolate(torch.autograd.Function):
    """Autograd twin of TensorVM.interpolate (tensor_vm.py:42-89). Gradients flow to
    the FP32 lines/planes (not to the coordinates: floor has no gradient and the
    reference's callers never differentiate through sample positions)."""

    @staticmethod
    def forward(ctx, coords, lines, planes):
        n = coords.shape[1]
        out = torch.empty((3 * planes.shape[-1], n), dtype=torch.float32, device=coords.device)
        f = field_struct(lines, planes)
        _lib.call("tvm_vm_features_fwd", ctypes_ref(f), ptr(coords, torch.float32, "coords"), n,
                  ptr(out), stream_handle())
        ctx.save_for_backward(coords, lines, planes)
        return out

    @staticmethod
    def backward(ctx, gout):
        coords, lines, planes = ctx.saved_tensors
        gl = torch.zeros(lines.shape, dtype=torch.float32, device=lines.device)
        gp = torch.zeros(planes.shape, dtype=torch.float32, device=planes.device)
        f = field_struct(lines, planes)
        _lib.call("tvm_vm_features_bwd", ctypes_ref(f), ptr(coords), coords.shape[1],
                  ptr(gout.contiguous()), ptr(gl), ptr(gp), stream_handle())
        return None, gl.to(lines.dtype), gp.to(planes.dtype)


def ctypes_ref(s):
    import ctypes
    return ctypes.byref(s)


class TensorVM:
    """Three vector-matrix pairs stacked on axis 0 (tensor_vm.py:14-40), channel-last."""

    def __init__(self, lines: torch.Tensor, planes: torch.Tensor):
        self.lines = lines
        self.planes = planes

    @staticmethod
    def initialize(grid_dim: int, per_axis_channel_dim: int, generator: Optional[torch.Generator] = None,
                   dtype=torch.float32, device="cuda", stddev: float = 0.1) -> "TensorVM":
        """N(0, stddev^2) init (training.py:44, tensor_vm.py:116-138)."""
        require_cuda()
        g, c = grid_dim, per_axis_channel_dim
        lines = (torch.randn((3, g, c), generator=generator) * stddev).to(device=device, dtype=dtype)
        planes = (torch.randn((3, g, g, c), generator=generator) * stddev).to(device=device, dtype=dtype)
        return TensorVM(lines, planes)

    @staticmethod
    def from_reference(vector: torch.Tensor, matrix: torch.Tensor, dtype=torch.float32) -> "TensorVM":
        """From the reference's channel-first stacked arrays vector (3, C, G) and
        matrix (3, C, G, G) (tensor_vm.py:129-138)."""
        require_cuda()
        vector = vector.to(device="cuda", dtype=torch.float32).contiguous()
        matrix = matrix.to(device="cuda", dtype=torch.float32).contiguous()
        c, g = vector.shape[1], vector.shape[2]
        lines = torch.empty((3, g, c), dtype=dtype, device="cuda")
        planes = torch.empty((3, g, g, c), dtype=dtype, device="cuda")
        _lib.call("tvm_vm_to_channel_last", g, c, ptr(vector), ptr(matrix), _DTYPE_CODE[dtype], ptr(lines),
                  ptr(planes), stream_handle())
        return TensorVM(lines, planes)

    def to_reference(self):
        """Back to channel-first (vector (3, C, G), matrix (3, C, G, G)), float32."""
        return (self.lines.float().permute(0, 2, 1).contiguous(),
                self.planes.float().permute(0, 3, 1, 2).contiguous())

    def interpolate(self, ijk: torch.Tensor) -> torch.Tensor:
        """(3, *) in [-1, 1] -> (3C, *) (tensor_vm.py:42-89)."""
        batch = ijk.shape[1:]
        assert ijk.shape[0] == 3
        coords = ijk.reshape(3, -1).to(torch.float32).contiguous()
        out = _Interpolate.apply(coords, self.lines, self.planes)
        return out.reshape((out.shape[0],) + tuple(batch))

    def resize(self, grid_dim: int) -> "TensorVM":
        """TensorVM.resize (tensor_vm.py:91-100): every pair resampled to grid_dim like
        resize_with_aligned_corners (linear, antialias, aligned corners). float32."""
        src_l = self.lines.float().contiguous()
        src_p = self.planes.float().contiguous()
        c = src_l.shape[-1]
        lines = torch.empty((3, grid_dim, c), dtype=torch.float32, device=src_l.device)
        planes = torch.empty((3, grid_dim, grid_dim, c), dtype=torch.float32, device=src_l.device)
        _lib.call("tvm_resize_field", self.grid_dim(), grid_dim, c, ptr(src_l), ptr(src_p), ptr(lines), ptr(planes),
                  stream_handle())
        return TensorVM(lines, planes)

    def grid_dim(self) -> int:
        return int(self.planes.shape[1])

    def channel_dim(self) -> int:
        return int(self.planes.shape[-1]) * 3
