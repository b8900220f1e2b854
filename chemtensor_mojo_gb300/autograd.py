"""Energy gradient of an MPS through torch.autograd (thin binding over ct_energy_grad).

``mps_energy(mpo, sites)`` returns E = <psi|H|psi> / <psi|psi> as a 0-d tensor;
its backward calls the hand-written adjoint of the environment chain in
libctdmrg (the right-environment sweep with checkpointed left environments),
giving dE/dA_i for every site tensor, canonical or not.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import torch

from . import _lib
from .dense_tensor import get_context
from .mps_state import MatrixProductOperator


def energy_and_gradient(mpo: MatrixProductOperator, sites: Sequence[torch.Tensor], checkpoint_every: int = 0,
                        ctx=None, prec: str = "fp64"):
    """-> (E, [dE/dA_i]) for CUDA float64 site tensors of shape [Dl, d, Dr].  prec "tf32x3" runs
    the environment chain and the one-site effective Hamiltonians on the tensor cores."""
    ctx = ctx or get_context()
    N = len(sites)
    if mpo.num_sites() != N:
        raise ValueError("MPS and MPO must have the same number of sites")
    d = int(sites[0].shape[1])
    bd = [int(sites[0].shape[0])] + [int(s.shape[2]) for s in sites]
    for i, s in enumerate(sites):
        if s.dim() != 3 or s.dtype != torch.float64 or not s.is_cuda:
            raise TypeError("site tensors must be CUDA float64 [Dl, d, Dr]")
        if i > 0 and s.shape[0] != sites[i - 1].shape[2]:
            raise ValueError(f"Bond mismatch between sites {i - 1} and {i}")
    sites_c = [s.contiguous() for s in sites]
    grads = [torch.empty_like(s) for s in sites_c]
    mpo_pp, k1 = _lib.ptr_array([s.tensor.storage.data_ptr() for s in mpo.sites])
    mps_pp, k2 = _lib.ptr_array([s.data_ptr() for s in sites_c])
    g_pp, k3 = _lib.ptr_array([g.data_ptr() for g in grads])
    E = C.c_double()
    ctx.call("ct_energy_grad", _lib.PRECISIONS[prec], N, d, _lib.i64_array(mpo.bond_dims), mpo_pp, _lib.i64_array(bd),
             mps_pp, g_pp, int(checkpoint_every), C.byref(E))
    return E.value, grads


class _MPSEnergy(torch.autograd.Function):
    @staticmethod
    def forward(fctx, mpo, checkpoint_every, prec, *sites):
        E, grads = energy_and_gradient(mpo, sites, checkpoint_every, prec=prec)
        fctx.save_for_backward(*grads)
        return torch.tensor(E, dtype=torch.float64, device=sites[0].device)

    @staticmethod
    def backward(fctx, grad_out):
        grads = fctx.saved_tensors
        return (None, None, None) + tuple(grad_out * g for g in grads)


def mps_energy(mpo: MatrixProductOperator, sites: Sequence[torch.Tensor], checkpoint_every: int = 0,
               prec: str = "fp64") -> torch.Tensor:
    """E = <psi|H|psi>/<psi|psi>, differentiable in every site tensor."""
    return _MPSEnergy.apply(mpo, int(checkpoint_every), prec, *sites)
