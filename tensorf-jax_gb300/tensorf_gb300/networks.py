"""GB300 twin of ``tensorf/networks.py``: the appearance ``FeatureMlp``.

Hyper-parameters and the flax parameter tree (``Dense_0`` .. ``Dense_3``, kernels
``(in, out)``, and ``Embed_0`` when camera embeddings are on) are the reference's
(networks.py:38-121). The weights live in the flat parameter buffer of
``render.LearnableParams``; ``apply`` runs ``tvm_mlp_fwd`` (and ``tvm_mlp_bwd`` under
autograd).
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, Optional

import torch

from . import _lib
from ._util import ptr, stream_handle, workspace


@dataclasses.dataclass(frozen=True)
class FeatureMlp:
    feature_squash_dim: int = 27
    units: int = 128
    feature_n_freqs: int = 6
    viewdir_n_freqs: int = 6
    num_cameras: Optional[int] = None  # set to enable FiLM camera embeddings (networks.py:103-111)

    def __post_init__(self):
        if self.num_cameras is not None and (self.num_cameras < 1 or self.units % 2):
            raise ValueError("camera embeddings need num_cameras >= 1 and an even number of units")

    def encoded_dim(self) -> int:
        """networks.py:77-82."""
        return (self.feature_squash_dim + 3 + 2 * self.feature_n_freqs * self.feature_squash_dim
                + 2 * self.viewdir_n_freqs * 3)

    def init_params(self, feat_dim: int, generator: Optional[torch.Generator] = None) -> Dict[str, Dict[str, torch.Tensor]]:
        """Flax-layout parameters (CPU float32): lecun_normal for Dense_0 / Dense_3,
        kaiming_normal for Dense_1 / Dense_2 (networks.py:9-10), biases zero. Flax
        samples truncated normals; a plain normal with the same variance is used."""
        def normal(fan_in, fan_out, var):
            return torch.randn((fan_in, fan_out), generator=generator) * math.sqrt(var / fan_in)
        u = self.units
        return {
            "Dense_0": {"kernel": normal(feat_dim, self.feature_squash_dim, 1.0)},
            "Dense_1": {"kernel": normal(self.encoded_dim(), u, 2.0), "bias": torch.zeros(u)},
            "Dense_2": {"kernel": normal(u, u, 2.0), "bias": torch.zeros(u)},
            "Dense_3": {"kernel": normal(u, 3, 1.0), "bias": torch.zeros(3)},
            # nn.Embed's default init: variance 1 / num_cameras (fan-in along axis 0).
            **({"Embed_0": {"embedding": torch.randn((self.num_cameras, u), generator=generator)
                            * math.sqrt(1.0 / self.num_cameras)}} if self.num_cameras else {}),
        }

    def apply(self, learnable_params, features: torch.Tensor, viewdirs: torch.Tensor,
              camera_indices: Optional[torch.Tensor] = None) -> torch.Tensor:
        """rgb = FeatureMlp(features (*, 3C), viewdirs (*, 3), camera_indices (*,))
        (networks.py:45-121); camera_indices is needed when num_cameras is set."""
        batch = features.shape[:-1]
        f = features.reshape(-1, features.shape[-1]).to(torch.float32).contiguous()
        d = viewdirs.reshape(-1, 3).to(torch.float32).contiguous()
        if self.num_cameras is not None:
            if camera_indices is None:
                raise ValueError("a FeatureMlp with camera embeddings needs camera_indices")
            cams = camera_indices.reshape(-1).to(device=f.device, dtype=torch.int32).contiguous()
        else:
            cams = None
        out = _MlpFn.apply(f, d, learnable_params.params, learnable_params, cams)
        return out.reshape(tuple(batch) + (3,))


class _MlpFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, features, viewdirs, params, lp, cams):
        n = features.shape[0]
        md = lp.model_desc()
        ws = workspace(_lib.load().tvm_mlp_workspace_size(ctypes_byref(md), n), features.device)
        rgb = torch.empty((n, 3), dtype=torch.float32, device=features.device)
        _lib.call("tvm_mlp_fwd", ctypes_byref(md), ptr(params), ptr(features), ptr(viewdirs), ptr(cams), n,
                  ptr(rgb), ptr(ws), ws.numel(), stream_handle())
        ctx.save_for_backward(features, viewdirs, params)
        ctx.lp = lp
        ctx.cams = cams
        return rgb

    @staticmethod
    def backward(ctx, grad_rgb):
        features, viewdirs, params = ctx.saved_tensors
        lp = ctx.lp
        n = features.shape[0]
        md = lp.model_desc()
        ws = workspace(_lib.load().tvm_mlp_workspace_size(ctypes_byref(md), n), features.device)
        gfeat = torch.empty_like(features)
        gparams = torch.zeros_like(params)
        _lib.call("tvm_mlp_bwd", ctypes_byref(md), ptr(params), ptr(features), ptr(viewdirs), ptr(ctx.cams), n,
                  ptr(grad_rgb.contiguous()), ptr(gfeat), ptr(gparams), ptr(ws), ws.numel(), stream_handle())
        return gfeat, None, gparams, None, None


def ctypes_byref(s):
    import ctypes
    return ctypes.byref(s)
