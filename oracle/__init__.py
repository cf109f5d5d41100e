"""CPU oracle for the HCIPy diffraction path -- TEST INFRASTRUCTURE ONLY.

This package restates, in plain numpy (float64 / complex128), the reference
algorithms of the path that the CUDA library implements: the matrix Fourier
transform, the zero-padded FFT, the chirp-Z / zoom FFT, the Fourier filter and
angular-spectrum transfer function, the Lyot-coronagraph Babinet chain, the
multi-scale, vortex and vector-vortex coronagraphs with the Stokes parameters
of a polarised wavefront, the pyramid wavefront-sensor optics (plain and
modulated), the deformable-mirror phase and the infinite-atmospheric-layer
extrusion with its quintic sub-pixel shift.  Each function cites the reference file and lines it
follows (paths are relative to the HCIPy source tree).

Parity status: pinned.  ``tests/test_oracle_golden.py`` checks every function
here against golden vectors produced by running the HCIPy reference itself
(``tests/golden/make_golden.py``).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package, and only as the checker or the timed CPU
baseline.  The library in ``hcipy_gb300`` never imports it and has no CPU path.
"""
from . import grids, fourier, optics, atmosphere  # noqa: F401
