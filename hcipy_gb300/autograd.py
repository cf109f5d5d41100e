"""Adjoint (reverse-mode) forms of the device operators, as ``torch.autograd.Function``s.

The reference has no gradients; HCIPy users differentiate wavefront-control losses by finite differences or
hand-written adjoints.  Here every operator on the path has its exact adjoint on the device, so a loss built
from DeformableMirror -> LyotCoronagraph -> FraunhoferPropagator -> intensity differentiates with
``loss.backward()``.  Convention (torch's): for a real loss L and a complex tensor z, z.grad = dL/d(conj z)
times 2, so a linear map y = A x back-propagates g -> A^H g.

* ``mft_apply``: one matrix Fourier transform with a scalar factor; its adjoint is the conjugate-transposed
  transform (the HX_ADJOINT direction of the plan for a forward transform, the forward direction for an
  inverse transform on uniformly weighted grids).
* ``phase_apply``: e exp(i c s) for a real screen s (DM surfaces, atmospheric phase).
* ``influence_apply``: the DM surface from actuator commands, adjoint = the transposed sparse product.
* ``LyotFunction``: the fused Lyot coronagraph; it is linear in E, so its adjoint needs no stored
  intermediates: E^* = S^* g - P^H[(1 - M)^* (P^-1)^H (S^* g)], two fused MFT calls.
"""
import numpy as np
import torch

from . import _lib
from . import kernels


def _conj(a):
    return complex(a).conjugate()


class _MftFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, ft, direction, alpha):
        ctx.ft = ft
        ctx.direction = direction
        ctx.alpha = alpha
        ctx.in_dtype = x.dtype
        if direction == _lib.HX_FORWARD:
            src, dst = ft.input_grid, ft.output_grid
        else:
            src, dst = ft.output_grid, ft.input_grid
        return ft._run(x, src, dst, direction, alpha).data

    @staticmethod
    def backward(ctx, g):
        ft, d, a = ctx.ft, ctx.direction, ctx.alpha
        g = g.contiguous()
        if d == _lib.HX_FORWARD:
            res = ft._run(g, ft.output_grid, ft.input_grid, _lib.HX_ADJOINT, _conj(a))
        elif d == _lib.HX_ADJOINT:
            res = ft._run(g, ft.input_grid, ft.output_grid, _lib.HX_FORWARD, _conj(a))
        else:
            if ft._win is not None or ft._wout is not None:
                raise NotImplementedError('the adjoint of an inverse MFT needs uniformly weighted grids')
            res = ft._run(g, ft.input_grid, ft.output_grid, _lib.HX_FORWARD, _conj(a))
        return res.data.to(ctx.in_dtype), None, None, None


def mft_apply(ft, x, direction, alpha):
    """alpha * (MFT in ``direction``)(x), differentiable in x."""
    return _MftFunction.apply(x, ft, direction, complex(alpha))


class _LinearFunction(torch.autograd.Function):
    """y = op(x) for a linear operator with a known adjoint: the gradient of x is adjoint(gradient of y)."""

    @staticmethod
    def forward(ctx, x, op, adjoint):
        ctx.adjoint = adjoint
        ctx.in_dtype = x.dtype
        return op(x)

    @staticmethod
    def backward(ctx, g):
        return ctx.adjoint(g.contiguous()).to(ctx.in_dtype), None, None


def linear_apply(x, op, adjoint):
    """op(x), differentiable in x through ``adjoint`` (callables on device tensors)."""
    return _LinearFunction.apply(x, op, adjoint)


class _PhaseFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, e, s, scale):
        ctx.save_for_backward(e, s)
        ctx.scale = scale
        return kernels.apply_phase(e, s, scale)

    @staticmethod
    def backward(ctx, g):
        e, s = ctx.saved_tensors
        need_e, need_s = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        g_e, g_s = kernels.apply_phase_grad(e, s, ctx.scale, g, need_e=need_e, need_s=need_s)
        if g_s is not None:
            g_s = g_s.to(s.dtype)
        return g_e, g_s, None


def phase_apply(e, s, scale):
    """e * exp(i scale s), differentiable in e and s."""
    return _PhaseFunction.apply(e, s, float(scale))


class _InfluenceFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coeffs, basis):
        ctx.basis = basis
        ctx.dtype = coeffs.dtype
        return basis.apply(coeffs)

    @staticmethod
    def backward(ctx, g):
        return ctx.basis.apply_transpose(g).to(ctx.dtype), None


def influence_apply(basis, coeffs):
    """Surface sum_a M[:, a] coeffs[..., a] of a ``kernels.SparseBasis``, differentiable in coeffs."""
    return _InfluenceFunction.apply(coeffs, basis)


class LyotFunction(torch.autograd.Function):
    """LyotCoronagraph.forward on a field E (..., n_pupil) with its adjoint (see the module docstring)."""

    @staticmethod
    def forward(ctx, e, coronagraph, inst):
        ctx.coronagraph = coronagraph
        ctx.inst = inst
        ctx.in_dtype = e.dtype
        return coronagraph._lyot_tensor(e, inst)

    @staticmethod
    def backward(ctx, g):
        lyot, inst = ctx.coronagraph, ctx.inst
        ft = inst.fourier_transform
        if ft._win is not None or ft._wout is not None:
            raise NotImplementedError('the Lyot adjoint needs uniformly weighted grids')
        g = g.contiguous()
        a_fwd = complex(ft._w_in_scalar) * inst.norm_factor
        a_bwd = complex(ft._w_out_scalar / (2 * np.pi)**ft.ndim) / inst.norm_factor
        one_minus, stop = lyot._fused_masks(torch.complex64 if ft.precision == 'split' else g.dtype)
        u = g if stop is None else g * stop.conj().to(g.dtype)
        if ft.precision == 'split':
            # u - P^H[(1 - M)^* (P^-1)^H u] is the Lyot chain itself with the conjugated mask and alphas and no
            # stop (P^H and P^-1 share their matrices on uniform grids): one hx_lyot_execute, whose row pass forms
            # the difference and writes the input's dtype
            m_conj = one_minus.conj().resolve_conj().contiguous()
            res = lyot._lyot_call(u, inst, m_conj, None, _conj(a_bwd), _conj(a_fwd), ctx.in_dtype)
            return res, None, None
        # v = (1 - M)^* . (P^-1)^H u  : forward-direction transform, mask fused in the epilogue
        v = ft._run(u, ft.input_grid, ft.output_grid, _lib.HX_FORWARD, _conj(a_bwd), epilogue=_lib.HX_EPI_MUL,
                    mask=one_minus.conj()).data
        # E^* = u - P^H v  : adjoint-direction transform with the subtraction fused into the last GEMM's epilogue
        res = ft._run(v, ft.output_grid, ft.input_grid, _lib.HX_ADJOINT, _conj(a_fwd), epilogue=_lib.HX_EPI_BABINET,
                      src=u).data
        return res.to(ctx.in_dtype), None, None


class _IntensitySumFunction(torch.autograd.Function):
    """Weighted intensity sums per field; the backward pass is one kernel, 2 g w E."""

    @staticmethod
    def forward(ctx, e, w):
        ctx.save_for_backward(e)
        ctx.w = w
        return kernels.intensity_sums(e, w)

    @staticmethod
    def backward(ctx, g):
        e, = ctx.saved_tensors
        return kernels.intensity_sums_grad(e, ctx.w, g), None


def intensity_sum_apply(e, w):
    return _IntensitySumFunction.apply(e, w)
