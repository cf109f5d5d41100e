"""Broadband imaging: one pupil field (or a batch of them) to many wavelengths, each on its own focal grid.

The reference propagates one wavelength per call and, for focal grids that follow the diffraction scale
(num_airy proportional to lambda0 / lambda), rebuilds a propagator per wavelength (its instance cache keys on the
wavelength, hcipy/optics/optical_element.py:261-790).  Here every wavelength keeps its matrix Fourier transform
plan on the device, a call runs all of them back to back on one stream, and ``capture`` records the whole call
(every wavelength's transforms and the optional atmosphere/DM phase ahead of them) as a CUDA graph, so a frame
replays with one graph launch instead of a few dozen kernel launches from Python.
"""
import numpy as np
import torch

from .field import Field, as_tensor, make_focal_grid
from .optics import Wavefront
from .propagation import FraunhoferPropagator


def diffraction_scaled_focal_grids(q, num_airy, wavelengths, reference_wavelength):
    """Per-wavelength focal grids make_focal_grid(q, num_airy * lambda0 / lambda) in lambda0/D units: the same
    sampling, a radius that shrinks with lambda, so the grids have uneven sizes (2 q num_airy lambda0/lambda
    samples across: 284^2 to 232^2 for q=4, num_airy=32 over 0.9-1.1 lambda0)."""
    return [make_focal_grid(q, num_airy * reference_wavelength / wl) for wl in wavelengths]


class BroadbandImager(object):
    """Images at each wavelength of ``wavelengths`` through a perfect lens.

    ``forward(e)`` takes a pupil field tensor (..., npix) (or a Field/Wavefront) and returns a list of complex
    image tensors, one per wavelength, each (..., n_focal(lambda)).  ``pre`` is an optional callable
    ``pre(wavefront) -> wavefront`` applied per wavelength before the lens (an atmosphere, a DM).
    """

    def __init__(self, pupil_grid, wavelengths, focal_grids, focal_length=1, precision='fp32', pre=None):
        if len(focal_grids) != len(wavelengths):
            raise ValueError('one focal grid per wavelength is needed')
        self.pupil_grid = pupil_grid
        self.wavelengths = [float(w) for w in wavelengths]
        self.focal_grids = list(focal_grids)
        self.pre = pre
        self.props = [FraunhoferPropagator(pupil_grid, g, focal_length=focal_length, precision=precision)
                      for g in self.focal_grids]
        self._graph = None

    def forward(self, e):
        t = as_tensor(e.electric_field if isinstance(e, Wavefront) else e)
        out = []
        for wl, prop in zip(self.wavelengths, self.props):
            wf = Wavefront(Field(t, self.pupil_grid), wl)
            if self.pre is not None:
                wf = self.pre(wf)
            out.append(prop.forward(wf).electric_field.data)
        return out

    __call__ = forward

    def capture(self, example):
        """Record ``forward`` for inputs shaped like ``example`` in a CUDA graph; ``replay`` then runs it.

        A warm-up call first creates every plan and workspace (plan creation synchronizes and may not be
        captured)."""
        t = as_tensor(example.electric_field if isinstance(example, Wavefront) else example)
        self._static_in = t.clone()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(2):
                self.forward(self._static_in)
        torch.cuda.current_stream().wait_stream(side)
        self._graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self._graph):
            self._static_out = self.forward(self._static_in)
        return self

    def replay(self, e):
        """Copy ``e`` into the captured input, replay the graph, return the captured outputs (valid until the
        next replay)."""
        if self._graph is None:
            raise RuntimeError('capture() first')
        t = as_tensor(e.electric_field if isinstance(e, Wavefront) else e)
        self._static_in.copy_(t)
        self._graph.replay()
        return self._static_out
