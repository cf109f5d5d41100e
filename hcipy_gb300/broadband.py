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

    The wavelengths' transforms are independent (each has its own plan), and one of them fills only a fraction of
    the GPU (a 1024^2 -> 256^2 transform is a few dozen output tiles), so ``forward`` runs ``pre`` for every
    wavelength in order on the calling stream and hands each wavelength's transform to one of ``streams`` side
    streams: transforms of different wavelengths overlap, and inside a captured graph they become parallel
    branches.  ``streams=1`` runs everything on the calling stream.  With more than one stream the transforms'
    split GEMMs use the throughput tile policy (no K split: the other wavelengths fill the GPU).
    """

    def __init__(self, pupil_grid, wavelengths, focal_grids, focal_length=1, precision='fp32', pre=None,
                 streams=8):
        if len(focal_grids) != len(wavelengths):
            raise ValueError('one focal grid per wavelength is needed')
        self.pupil_grid = pupil_grid
        self.wavelengths = [float(w) for w in wavelengths]
        self.focal_grids = list(focal_grids)
        self.pre = pre
        self.num_streams = max(1, min(int(streams), len(self.focal_grids)))
        schedule = 'throughput' if self.num_streams > 1 else 'latency'
        self.props = [FraunhoferPropagator(pupil_grid, g, focal_length=focal_length, precision=precision,
                                           schedule=schedule) for g in self.focal_grids]
        self._streams = None
        self._graph = None

    def _side_streams(self):
        if self._streams is None:
            self._streams = [torch.cuda.Stream() for _ in range(self.num_streams)]
        return self._streams

    def _phase_screen(self):
        """The screen of ``pre`` when it is a pure phase element (an atmosphere without scintillation), else None:
        the split transforms then apply its phase while slicing their input (``forward_phase_screen``)."""
        pre = self.pre
        owner = getattr(pre, '__self__', None)  # a bound ``forward`` of an element counts as the element
        if owner is not None and getattr(pre, '__func__', None) is getattr(type(owner), 'forward', None):
            pre = owner
        hook = getattr(pre, '_pure_phase_screen', None)
        return hook() if hook is not None else None

    def _one(self, t, wl, prop, screen):
        """(image, field kept alive or None) of one wavelength."""
        if screen is not None:
            img = prop.forward_phase_screen(t, screen, 1.0 / wl, wl)
            if img is not None:
                return img, None
        wf = Wavefront(Field(t, self.pupil_grid), wl)
        if self.pre is not None:
            wf = self.pre(wf)
        return prop.forward(wf).electric_field.data, wf.electric_field.data

    def forward(self, e, concurrent=True):
        t = as_tensor(e.electric_field if isinstance(e, Wavefront) else e)
        screen = self._phase_screen()
        if not concurrent or self.num_streams == 1:
            return [self._one(t, wl, prop, screen)[0] for wl, prop in zip(self.wavelengths, self.props)]
        main = torch.cuda.current_stream()
        streams = self._side_streams()
        capturing = torch.cuda.is_current_stream_capturing()
        out = []
        # Each wavelength's field stays referenced until every side stream has joined: freed earlier, its memory
        # could go to the next wavelength's field on the calling stream while a side stream still reads it
        # (record_stream guards that outside a capture; inside one only the reference does).
        fields = []
        for i, (wl, prop) in enumerate(zip(self.wavelengths, self.props)):
            fused = screen is not None and prop.phase_screen_fusable(t, screen, wl)
            wf = None
            if not fused:
                wf = Wavefront(Field(t, self.pupil_grid), wl)
                if self.pre is not None:
                    wf = self.pre(wf)  # in order on the calling stream: ``pre`` may keep state
                fields.append(wf.electric_field.data)
            side = streams[i % len(streams)]
            side.wait_stream(main)
            with torch.cuda.stream(side):
                if fused:
                    img = prop.forward_phase_screen(t, screen, 1.0 / wl, wl)
                else:
                    img = prop.forward(wf).electric_field.data
            if not capturing:
                # the field was made on the calling stream and is read on ``side``; the image is made on
                # ``side`` and handed back: tell the allocator about both uses
                if wf is not None:
                    wf.electric_field.data.record_stream(side)
                img.record_stream(main)
            out.append(img)
        for side in streams:
            main.wait_stream(side)
        del fields
        return out

    __call__ = forward


    def capture(self, example):
        """Record ``forward`` for inputs shaped like ``example`` in a CUDA graph; ``replay`` then runs it.

        Warm-up calls first create every plan and workspace (plan creation synchronizes and may not be
        captured); the first runs the wavelengths one after the other, so that the split-GEMM autotuner, when it
        is on, times its candidates on an otherwise idle GPU."""
        t = as_tensor(example.electric_field if isinstance(example, Wavefront) else example)
        self._static_in = t.clone()
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            self.forward(self._static_in, concurrent=False)
            self.forward(self._static_in)
        torch.cuda.current_stream().wait_stream(side)
        from ._lib import launch_count
        self._graph = torch.cuda.CUDAGraph()
        before = launch_count()
        with torch.cuda.graph(self._graph):
            self._static_out = self.forward(self._static_in)
        self.graph_kernels = launch_count() - before  # library kernels recorded in the graph
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
