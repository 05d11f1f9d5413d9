"""catana_gb300 -- GB300-native (sm_103a) spherical Fourier-Bessel decomposition.

Drop-in for the decomposition path of CatAna's Python package (python/catana/
__init__.py): ``PointContainer``, ``PixelizedPointContainer``, ``Point``,
``sfb_decomposition`` (raw and HEALPix overloads), ``KClkk`` and
``besseltools.SphericalBesselZeros`` keep the reference's names, arguments and
errors.  The compute runs in libcatana_gpu.so (hand-written CUDA for sm_103a behind
the C ABI in include/catana_gpu.h); there is no CPU fallback.
"""
from . import _lib  # noqa: F401  (raises ImportError when the library is missing)
from . import besseltools, io
from .basictypes import FunctionInterpolator, PixelizedPointContainer, Point, PointContainer
from .decomposition import (KClkk, SFBAccumulator, compute_kln, ingest, sfb_decomposition,
                            sfb_decomposition_batched, sfb_decomposition_healpix, sfb_reverse)

__all__ = ["Point", "PointContainer", "FunctionInterpolator", "PixelizedPointContainer", "KClkk", "sfb_decomposition",
           "sfb_decomposition_healpix", "sfb_decomposition_batched", "SFBAccumulator", "sfb_reverse", "ingest", "compute_kln",
           "besseltools", "io"]
__version__ = "0.1.0"
