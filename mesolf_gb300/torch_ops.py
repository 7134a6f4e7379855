"""PyTorch operator registrations for the projector and the RL solve (``import
mesolf_gb300.torch_ops`` registers them):

* ``torch.ops.mesolf.conv_vec(bitmap, kernels)`` -- the MEX projector
  (``src/cuda/mex_lfm_convolution_vec.cu``), CUDA tensors in MATLAB index order;
* ``torch.ops.mesolf.rl_solve(lfimg, H, Ht, max_iter, precision)`` -- the RL solve
  (``recon_theory_phase_space_LFM_with_filter.m``), returns the (Xr, Xc, Z) volume;
* ``torch.ops.mesolf.rl_solve_batch(lfimgs, H, Ht, z0, nz, max_iter, precision)`` --
  independent patches of one PSF in one batched tensor-core solve.

Each call goes through libmesolf_lf.so (no CPU path); the fake (meta) implementations give
the output shapes so the ops can be traced.  Results are returned contiguous in the index
order of the inputs.
"""
from __future__ import annotations

from typing import List

import torch

from . import api

__all__ = ["conv_vec", "rl_solve", "rl_solve_batch"]


@torch.library.custom_op("mesolf::conv_vec", mutates_args=())
def conv_vec(bitmap: torch.Tensor, kernels: torch.Tensor) -> torch.Tensor:
    return api.mex_lfm_convolution_vec(bitmap, kernels).contiguous()


@conv_vec.register_fake
def _conv_vec_fake(bitmap, kernels):
    return torch.empty(bitmap.shape, dtype=torch.float32, device=bitmap.device)


@torch.library.custom_op("mesolf::rl_solve", mutates_args=())
def rl_solve(lfimg: torch.Tensor, H: torch.Tensor, Ht: torch.Tensor, max_iter: int,
             precision: str = "fp32") -> torch.Tensor:
    psf = api.PhaseSpacePSF(H, Ht)
    try:
        s = api.RLSolver(psf, tuple(lfimg.shape))
        try:
            return s.run(lfimg, max_iter, precision=precision, want_stats=False).contiguous()
        finally:
            s.close()
    finally:
        psf.close()


@rl_solve.register_fake
def _rl_solve_fake(lfimg, H, Ht, max_iter, precision="fp32"):
    return torch.empty((lfimg.shape[0], lfimg.shape[1], H.shape[4]), dtype=torch.float32, device=lfimg.device)


@torch.library.custom_op("mesolf::rl_solve_batch", mutates_args=())
def rl_solve_batch(lfimgs: List[torch.Tensor], H: torch.Tensor, Ht: torch.Tensor, z0: List[int], nz: List[int],
                   max_iter: int, precision: str = "bf16x2") -> List[torch.Tensor]:
    psf = api.PhaseSpacePSF(H, Ht)
    try:
        b = api.BatchSolver(psf, [tuple(x.shape) for x in lfimgs], list(zip(z0, nz)))
        try:
            return [o.contiguous() for o in b.run(list(lfimgs), max_iter, precision=precision, want_stats=False)]
        finally:
            b.close()
    finally:
        psf.close()


@rl_solve_batch.register_fake
def _rl_solve_batch_fake(lfimgs, H, Ht, z0, nz, max_iter, precision="bf16x2"):
    return [torch.empty((x.shape[0], x.shape[1], k), dtype=torch.float32, device=x.device)
            for x, k in zip(lfimgs, nz)]
