"""Dark-hole contrast on the device.

The reference forms intensities with numexpr (hcipy/optics/wavefront.py:113-143) and averages them over a
region of interest in numpy (hcipy/metrics/contrast.py:37-75).  Here the weighted sum of |E|^2 over the region
is one fused reduction straight from the electric field, in compensated float-float arithmetic (deterministic
order), and differentiable: the loss of a dark-hole optimisation.
"""
import torch

from .field import Field, as_tensor


def intensity_sum(field, weights=None):
    """sum_p w[p] |E[..., p]|^2 per field (``weights``: a real weight or region mask per point, default 1).

    ``field`` is a complex Field or tensor with optional leading batch dimensions; returns a float64 tensor of
    the batch shape (0-d for one field), differentiable in the field.
    """
    e = field.data if isinstance(field, Field) else field
    e = e if isinstance(e, torch.Tensor) and e.is_cuda else as_tensor(e)
    if e.is_complex() and e.is_conj():
        e = e.resolve_conj()
    if torch.is_grad_enabled() and e.requires_grad:
        from .autograd import intensity_sum_apply
        return intensity_sum_apply(e, weights)
    from .kernels import intensity_sums
    return intensity_sums(e.detach(), weights)


def mean_intensity_in_roi(field, mask):
    """Mean |E|^2 over the points where ``mask`` is nonzero (the reference's get_mean_intensity_in_roi,
    contrast.py:37-52, taken from the field instead of an intensity image)."""
    m = mask.data if isinstance(mask, Field) else mask
    m = as_tensor(torch.as_tensor(m) if not isinstance(m, torch.Tensor) else m).reshape(-1)
    count = int((m != 0).sum())
    if count == 0:
        raise ValueError('the region of interest is empty')
    return intensity_sum(field, (m != 0).to(torch.float32)) / count
