"""GB300-native detector-error-model compiler with GreenPeas' Python surface.

    import greenpeas_gb300 as gp
    driver = gp.get_driver(circuit)                  # circuit: stim.Circuit or stim text
    dem = driver.compile_detector_error_model(circuit)

See ``error_analysis`` (the compile path and its batched form), ``autograd``
(noise-rate gradients), ``serving`` (continuous batching of compile
requests), ``codes`` and ``workloads`` (circuit generators) and ``dem`` (the
DEM type returned when stim is not installed).
"""

from ._native import GpcError
from .autograd import NoiseRateDEM
from .codes import BBCode, SurfaceCode
from .dem import DetectorErrorModel
from .error_analysis import CorrelationLevel, Driver, Lowerer, Tape, get_driver, tune_cache_clear

__all__ = ["BBCode", "CorrelationLevel", "DetectorErrorModel", "Driver", "GpcError", "Lowerer", "NoiseRateDEM", "SurfaceCode",
           "Tape", "get_driver", "tune_cache_clear"]
