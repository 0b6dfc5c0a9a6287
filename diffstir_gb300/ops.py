"""Batched 3x3 SVD and SVD backward on the GPU (dstir_svd3, dstir_svd3_backward).

These are the per-particle SVD kernels of the path exposed on their own: the
reference's svd kernel (ti.svd of F_tmp, simulation_functions.py:55-58) and its
hand-written backward_svd / svd_grad (:61-93).
"""

import ctypes

import torch

from ._lib import check, lib


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _f(t, shape):
    return t.to(device='cuda', dtype=torch.float32).reshape(shape).contiguous()


def svd3(A):
    """A [n,3,3] -> U [n,3,3], S [n,3], V [n,3,3] with A = U diag(S) V^T."""
    A = _f(A, (-1, 3, 3))
    n = A.shape[0]
    U = torch.empty_like(A)
    V = torch.empty_like(A)
    S = torch.empty((n, 3), device=A.device)
    check(lib().dstir_svd3(_p(A), _p(U), _p(S), _p(V), n, _s()), None, 'dstir_svd3')
    return U, S, V


def svd3_backward(gU, gS, gV, U, S, V):
    """dL/dA from dL/dU, dL/dS (diagonal), dL/dV; FP64 in the 1/(s_j^2-s_i^2) terms."""
    U = _f(U, (-1, 3, 3))
    n = U.shape[0]
    gU, gV, V = _f(gU, (n, 3, 3)), _f(gV, (n, 3, 3)), _f(V, (n, 3, 3))
    gS, S = _f(gS, (n, 3)), _f(S, (n, 3))
    gA = torch.empty_like(U)
    check(lib().dstir_svd3_backward(_p(gU), _p(gS), _p(gV), _p(U), _p(S), _p(V), _p(gA), n, _s()), None,
          'dstir_svd3_backward')
    return gA
