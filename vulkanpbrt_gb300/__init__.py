"""vulkanpbrt_gb300: GB300-native (sm_103a) per-frame path of VulkanPBRT.

The native library (csrc/, C ABI in include/vulkanpbrt_gb300.h) holds the
path tracer, accumulator and BMFR/BFR denoisers; this package mirrors the
reference's render-module classes over that ABI.
"""
from ._abi import PbrtError, declared_symbols, lib  # noqa: F401
from .render_modules import (  # noqa: F401
    BFR,
    BFRBlender,
    BMFR,
    AccumulationBuffer,
    Accumulator,
    CameraMatrices,
    Commands,
    GBuffer,
    IlluminationBuffer,
    IlluminationBufferDemodulated,
    IlluminationBufferDemodulatedFloat,
    IlluminationBufferFinal,
    IlluminationBufferFinalDemodulated,
    IlluminationBufferFinalFloat,
    Image,
    PushConstants,
    Taa,
    format_convert,
)

from .pipeline import PBRTPipeline, SceneHandle  # noqa: F401,E402
from . import nn  # noqa: F401,E402  (registers the neural-denoiser operators)
from .neural import NeuralDenoiser  # noqa: F401,E402
from .batch import Batch  # noqa: F401,E402
from .denoiser_utils import DenoisingBlockSize, DenoisingType, add_denoiser_to_commands  # noqa: F401,E402

__version__ = "0.1.0"
