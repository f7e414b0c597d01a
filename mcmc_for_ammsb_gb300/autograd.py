"""torch.autograd binding of the minibatch edge log-likelihood and its
hand-written adjoint kernels (ammsb_edge_loglik_* in include/ammsb_gpu.h).

    L = sum_q log p(y_q | pi_a = phi_src[a_q] / sum(phi_src[a_q]),
                         pi_b = pi_nbr[b_q], beta(theta))

with p the normaliser prob_sum of update_beta (mcmc_sampler_stochastic.cc
:212-240), summed over sampled pairs; cal_edge_likelihood (learner.h:100-139)
is the same probability less eps * (1 - sum_k pi_ak pi_bk) for a link.  Its
gradient in phi_src is the update_phi gradient of the reference
(mcmc_sampler_stochastic.cc:274-296, neighbour pi fixed), in theta the
update_beta gradient (cc:212-240): the SGRLD drift.  The gradient in pi_nbr
is the same expression's derivative in the neighbour row.

Tensors must be CUDA tensors of one dtype (float32 or float64); there is no
CPU path.  The backward recomputes every per-pair K-vector from the rows and
keeps only p_q and the row sums from the forward.
"""
import ctypes

import torch
from torch.autograd.function import once_differentiable

from . import _native

_DTYPES = {torch.float32: _native.REAL_F32, torch.float64: _native.REAL_F64}


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None and t.numel() else ctypes.c_void_p(0)


def _stream(device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _check_status(ws, device):
    flags = ctypes.c_int32(0)
    _native.check(_native.lib().ammsb_edge_loglik_status(_ptr(ws), _stream(device),
                                                        ctypes.byref(flags)))
    if flags.value & 1:
        raise IndexError("edge log-likelihood: a pair index is out of range")
    if flags.value & 2:
        raise ValueError("edge log-likelihood: a phi row sum or a probability is not positive")


class EdgeLogLikelihood(torch.autograd.Function):
    """Inputs: phi_src (n_src x K), pi_nbr (n_nbr x K), theta (K x 2), and the
    pair arrays grouped by source (src_ptr int64 [n_src + 1], pair_nbr int32,
    pair_y uint8) and by neighbour (pair_src int32, nbr_ptr int64 [n_nbr + 1],
    nbr_pairs int32), all on one CUDA device.  Use edge_log_likelihood()
    to build the groupings from plain pair lists."""

    @staticmethod
    def forward(ctx, phi_src, pi_nbr, theta, src_ptr, pair_nbr, pair_y, pair_src, nbr_ptr,
                nbr_pairs, epsilon):
        dtype = phi_src.dtype
        if dtype not in _DTYPES:
            raise TypeError("phi_src must be float32 or float64")
        for name, t in (("phi_src", phi_src), ("pi_nbr", pi_nbr), ("theta", theta)):
            if not t.is_cuda:
                raise RuntimeError("%s is not a CUDA tensor: the edge log-likelihood runs on "
                                   "the GPU only" % name)
            if t.dtype != dtype:
                raise TypeError("phi_src, pi_nbr and theta must share one dtype")
        n_src, K = phi_src.shape
        n_nbr = pi_nbr.shape[0]
        if pi_nbr.shape[1] != K or tuple(theta.shape) != (K, 2):
            raise ValueError("shapes: phi_src (n_src, K), pi_nbr (n_nbr, K), theta (K, 2)")
        phi_src = phi_src.contiguous()
        pi_nbr = pi_nbr.contiguous()
        theta = theta.contiguous()
        n_pairs = pair_nbr.shape[0]
        L = _native.lib()
        code = _DTYPES[dtype]
        ws_bytes = L.ammsb_edge_loglik_workspace_size(code, K, n_src, n_pairs)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device=phi_src.device)
        loss = torch.empty((), dtype=dtype, device=phi_src.device)
        dev = phi_src.device
        _native.check(L.ammsb_edge_loglik_forward(
            code, K, _ptr(phi_src), K, _ptr(pi_nbr), K, n_nbr, _ptr(theta), float(epsilon),
            _ptr(src_ptr), n_src, _ptr(pair_nbr), _ptr(pair_y), n_pairs, _ptr(loss), _ptr(ws),
            _stream(dev)))
        _check_status(ws, dev)
        ctx.save_for_backward(phi_src, pi_nbr, theta, src_ptr, pair_nbr, pair_y, pair_src,
                              nbr_ptr, nbr_pairs, ws)
        ctx.epsilon = float(epsilon)
        return loss

    @staticmethod
    @once_differentiable
    def backward(ctx, grad_loss):
        (phi_src, pi_nbr, theta, src_ptr, pair_nbr, pair_y, pair_src, nbr_ptr, nbr_pairs,
         ws) = ctx.saved_tensors
        dtype = phi_src.dtype
        n_src, K = phi_src.shape
        n_nbr = pi_nbr.shape[0]
        n_pairs = pair_nbr.shape[0]
        gl = grad_loss.detach().to(dtype=dtype).contiguous()
        gphi = torch.empty_like(phi_src)
        gtheta = torch.empty_like(theta)
        want_nbr = ctx.needs_input_grad[1]
        gpin = torch.empty_like(pi_nbr) if want_nbr else None
        dev = phi_src.device
        _native.check(_native.lib().ammsb_edge_loglik_backward(
            _DTYPES[dtype], K, _ptr(phi_src), K, _ptr(pi_nbr), K, n_nbr, _ptr(theta), ctx.epsilon,
            _ptr(src_ptr), n_src, _ptr(pair_nbr), _ptr(pair_y), n_pairs, _ptr(pair_src),
            _ptr(nbr_ptr), _ptr(nbr_pairs), _ptr(gl),
            _ptr(gphi) if n_src else ctypes.c_void_p(0),
            (_ptr(gpin) if n_nbr else ctypes.c_void_p(0)) if want_nbr else None,
            _ptr(gtheta), _ptr(ws), _stream(dev)))
        if want_nbr and n_nbr == 0:
            gpin = torch.zeros_like(pi_nbr)
        _check_status(ws, dev)
        return (gphi if ctx.needs_input_grad[0] else None, gpin,
                gtheta if ctx.needs_input_grad[2] else None,
                None, None, None, None, None, None, None)


def group_pairs(src, nbr, y, n_src, n_nbr):
    """Groups a pair list (src, nbr, y: 1-D CUDA tensors) by source and by
    neighbour: returns (src_ptr, pair_nbr, pair_y, pair_src, nbr_ptr,
    nbr_pairs) in the layout EdgeLogLikelihood takes."""
    dev = src.device
    src = src.to(torch.int64)
    nbr = nbr.to(torch.int64)
    order = torch.sort(src, stable=True).indices
    pair_src = src[order]
    pair_nbr = nbr[order]
    pair_y = y[order].to(torch.uint8).contiguous()
    src_ptr = torch.zeros(n_src + 1, dtype=torch.int64, device=dev)
    src_ptr[1:] = torch.cumsum(torch.bincount(pair_src, minlength=n_src)[:n_src], 0)
    by_nbr = torch.sort(pair_nbr, stable=True).indices
    nbr_ptr = torch.zeros(n_nbr + 1, dtype=torch.int64, device=dev)
    nbr_ptr[1:] = torch.cumsum(torch.bincount(pair_nbr, minlength=n_nbr)[:n_nbr], 0)
    return (src_ptr, pair_nbr.to(torch.int32).contiguous(), pair_y,
            pair_src.to(torch.int32).contiguous(), nbr_ptr, by_nbr.to(torch.int32).contiguous())


def edge_log_likelihood(phi_src, pi_nbr, theta, src, nbr, y, epsilon):
    """Sum over pairs q of log p(y[q] | phi_src[src[q]], pi_nbr[nbr[q]],
    theta): differentiable in phi_src, pi_nbr and theta through the
    hand-written adjoint kernels."""
    if not (src.is_cuda and nbr.is_cuda and y.is_cuda):
        raise RuntimeError("pair arrays must be CUDA tensors: the edge log-likelihood runs on "
                           "the GPU only")
    n_src, n_nbr = phi_src.shape[0], pi_nbr.shape[0]
    if src.numel():
        lo = torch.stack([src.min(), nbr.min()]).cpu()
        hi = torch.stack([src.max(), nbr.max()]).cpu()
        if int(lo.min()) < 0 or int(hi[0]) >= n_src or int(hi[1]) >= n_nbr:
            raise IndexError("pair indices out of range")
    groups = group_pairs(src, nbr, y, n_src, n_nbr)
    return EdgeLogLikelihood.apply(phi_src, pi_nbr, theta, *groups, epsilon)
