"""hcipy_gb300: the HCIPy diffraction hot path on one GB300 GPU (sm_103a).

Drop-in classes with the reference signatures; fields live on the device and
every operator runs hand-written CUDA kernels from ``lib/libhcipy_gb300.so``
through the C ABI of ``include/hcipy_gb300.h``.  There is no CPU path.
"""
from .field import (Field, CartesianGrid, RegularCoords, SeparatedCoords, UnstructuredCoords, make_uniform_grid,
                    make_pupil_grid, make_focal_grid, make_focal_grid_from_pupil_grid)
from .fourier import (FourierTransform, ComputationalComplexity, MatrixFourierTransform, make_fourier_transform,
                      make_fft_grid, get_fft_parameters, is_fft_grid)
from .optics import (Wavefront, OpticalElement, AgnosticOpticalElement, EmptyOpticalElement, OpticalSystem,
                     Apodizer, PhaseApodizer, SurfaceApodizer, make_agnostic_forward, make_agnostic_backward)
from .propagation import FraunhoferPropagator, AngularSpectrumPropagator, FresnelPropagator
from .fft import FastFourierTransform, ChirpZTransform, ZoomFastFourierTransform, FourierFilter
from .wavefront_sensing import PyramidWavefrontSensorOptics, ModulatedPyramidWavefrontSensorOptics
from .graphs import CapturedCall
from .coronagraphy import LyotCoronagraph, MultiScaleCoronagraph, VortexCoronagraph, VectorVortexCoronagraph
from .deformable_mirror import (ModeBasis, DeformableMirror, TipTiltMirror, make_actuator_positions,
                                make_gaussian_influence_functions, find_illuminated_actuators)
from .atmosphere import (AtmosphericLayer, InfiniteAtmosphericLayer, MultiLayerAtmosphere,
                         Cn_squared_from_fried_parameter, fried_parameter_from_Cn_squared, subpixel_shift,
                         power_spectral_density_von_karman, SpectralNoiseFactoryMultiscale)
from .broadband import BroadbandImager, diffraction_scaled_focal_grids
from .efc import SVD, inverse_tikhonov, inverse_truncated, inverse_truncated_modal, poke_jacobian, efc_step, run_efc
from .metrics import intensity_sum, mean_intensity_in_roi
from .io import (read_fits, write_fits, read_grid, write_grid, read_field, write_field, read_mode_basis,
                 write_mode_basis)
from ._lib import HXError, launch_count, autotune

__all__ = [
    'Field', 'CartesianGrid', 'RegularCoords', 'SeparatedCoords', 'UnstructuredCoords', 'make_uniform_grid',
    'make_pupil_grid', 'make_focal_grid', 'make_focal_grid_from_pupil_grid',
    'FourierTransform', 'ComputationalComplexity', 'MatrixFourierTransform', 'make_fourier_transform',
    'make_fft_grid', 'get_fft_parameters', 'is_fft_grid',
    'Wavefront', 'OpticalElement', 'AgnosticOpticalElement', 'EmptyOpticalElement', 'OpticalSystem', 'Apodizer',
    'PhaseApodizer',
    'make_agnostic_forward', 'make_agnostic_backward',
    'FraunhoferPropagator', 'AngularSpectrumPropagator', 'FresnelPropagator', 'LyotCoronagraph',
    'MultiScaleCoronagraph', 'VortexCoronagraph', 'VectorVortexCoronagraph', 'PyramidWavefrontSensorOptics',
    'ModulatedPyramidWavefrontSensorOptics', 'SurfaceApodizer', 'TipTiltMirror',
    'CapturedCall', 'HXError',
    'launch_count',
    'FastFourierTransform', 'ChirpZTransform', 'ZoomFastFourierTransform', 'FourierFilter',
    'ModeBasis', 'DeformableMirror', 'make_actuator_positions', 'make_gaussian_influence_functions',
    'find_illuminated_actuators', 'AtmosphericLayer', 'InfiniteAtmosphericLayer', 'MultiLayerAtmosphere',
    'Cn_squared_from_fried_parameter', 'fried_parameter_from_Cn_squared', 'subpixel_shift',
    'power_spectral_density_von_karman', 'SpectralNoiseFactoryMultiscale',
    'BroadbandImager', 'diffraction_scaled_focal_grids', 'autotune',
    'SVD', 'inverse_tikhonov', 'inverse_truncated', 'inverse_truncated_modal', 'poke_jacobian', 'efc_step',
    'run_efc', 'read_fits', 'write_fits', 'read_grid', 'write_grid', 'read_field', 'write_field',
    'read_mode_basis', 'write_mode_basis', 'intensity_sum', 'mean_intensity_in_roi',
]
