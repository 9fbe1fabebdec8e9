"""Denoiser selection (source/util/DenoiserUtils.cpp:9-131) and its enums
(source/renderModules/PipelineStructs.hpp:15-30).

`add_denoiser_to_commands` builds the denoiser the reference builds for a
(type, block size) pair, records its dispatches into `commands` and returns
the final image (the reference's `final_descriptor_image` out-parameter).

Differences from the reference, each deliberate:
* BMFR with X8X16X32 blends with the accumulated illumination's images 0 and
  1 (average, average of squares), as the BFR branch does; the reference
  passes images 1 and 2 (DenoiserUtils.cpp:107-108), and the accumulated
  IlluminationBufferDemodulated has only two images.
* Block size X64 and type SVG, for which the reference records nothing and
  leaves the final image unset (DenoiserUtils.cpp:125-127, and no X64 case
  in its switches), raise NotImplementedError.
"""
from __future__ import annotations

import enum
from typing import Optional

from .render_modules import (BFR, BMFR, AccumulationBuffer, BFRBlender, Commands, GBuffer, IlluminationBuffer, Image,
                             PushConstants)


class DenoisingType(enum.IntEnum):
    NONE = 0
    BMFR = 1
    BFR = 2
    SVG = 3


class DenoisingBlockSize(enum.IntEnum):
    X8 = 0
    X16 = 1
    X32 = 2
    X64 = 3
    X8X16X32 = 4


_SIZES = {DenoisingBlockSize.X8: 8, DenoisingBlockSize.X16: 16, DenoisingBlockSize.X32: 32}


def _make(denoising_type, bs, width, height, g_buffer, illumination_buffer, accumulation_buffer):
    if denoising_type == DenoisingType.BFR:
        return BFR(width, height, bs, bs, g_buffer, illumination_buffer, accumulation_buffer)
    # BMFR(width, height, 8, 8, ..., 64) for the 8x8 blocks (DenoiserUtils.cpp:79, 106)
    return BMFR(width, height, bs, bs, g_buffer, illumination_buffer, accumulation_buffer, 64 if bs == 8 else 256)


def add_denoiser_to_commands(denoising_type: DenoisingType, denoising_size: DenoisingBlockSize, commands: Commands,
                             compile, width: int, height: int, compute_constants: PushConstants, g_buffer: GBuffer,
                             illumination_buffer: IlluminationBuffer,
                             accumulation_buffer: AccumulationBuffer) -> Optional[Image]:
    """Returns the denoiser's final image (None for DenoisingType.NONE, as
    the reference leaves it unset). `compile` is the reference's compile
    traversal: images are allocated at construction here, so it is unused."""
    denoising_type = DenoisingType(denoising_type)
    denoising_size = DenoisingBlockSize(denoising_size)
    if denoising_type == DenoisingType.NONE:
        return None
    if denoising_type == DenoisingType.SVG:
        raise NotImplementedError("DenoisingType.SVG: the reference has no implementation either")
    if denoising_size == DenoisingBlockSize.X64:
        raise NotImplementedError("DenoisingBlockSize.X64: the reference builds no denoiser for it")
    if denoising_size != DenoisingBlockSize.X8X16X32:
        d = _make(denoising_type, _SIZES[denoising_size], width, height, g_buffer, illumination_buffer,
                  accumulation_buffer)
        d.compile(compile)
        d.update_image_layouts(compile)
        d.add_dispatch_to_command_graph(commands, compute_constants)
        return d.get_final_descriptor_image()
    ds = [_make(denoising_type, bs, width, height, g_buffer, illumination_buffer, accumulation_buffer)
          for bs in (8, 16, 32)]
    ims = illumination_buffer.illumination_images
    blender = BFRBlender(width, height, ims[0], ims[1], *(d.get_final_descriptor_image() for d in ds))
    for d in ds:
        d.compile(compile)
        d.update_image_layouts(compile)
    blender.compile(compile)
    blender.update_image_layouts(compile)
    for d in ds:
        d.add_dispatch_to_command_graph(commands, compute_constants)
    blender.add_dispatch_to_command_graph(commands)
    return blender.get_final_descriptor_image()
