"""NeuralDenoiser: the kernel-predicting U-Net as a render module beside BMFR
and BFR (same construction from a G-buffer and an illumination buffer, same
dispatch / final-image interface), over the pbrt_neural_* C ABI. No
reference counterpart: the reference's denoisers are BMFR and BFR
(source/renderModules/denoisers/)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import _abi
from ._abi import PbrtImage, check, lib, stream_handle
from .render_modules import BMFR, Commands, GBuffer, Handle, IlluminationBuffer, Image

H = C.c_void_p
_abi.add_signatures({
    "pbrt_neural_param_count": (C.c_int32, [C.POINTER(C.c_int64)]),
    "pbrt_neural_create": (C.c_int32, [C.c_uint32, C.c_uint32, H, H, H, H, C.c_int64, C.POINTER(H)]),
    "pbrt_neural_set_params": (C.c_int32, [H, H, C.c_int64]),
    "pbrt_neural_set_fallback": (C.c_int32, [H, H, C.c_float, C.c_int32]),
    "pbrt_neural_set_gate_model": (C.c_int32, [H, C.POINTER(C.c_float), C.c_int32]),
    "pbrt_neural_dispatch": (C.c_int32, [H, H]),
    "pbrt_neural_dispatch_direct": (C.c_int32, [H, H]),
    "pbrt_neural_final_image": (C.c_int32, [H, C.POINTER(PbrtImage)]),
    "pbrt_neural_images": (C.c_int32, [H, C.POINTER(PbrtImage), C.POINTER(PbrtImage)]),
    "pbrt_neural_fallback_tiles": (C.c_int32, [H, H, C.POINTER(C.c_uint32)]),
    "pbrt_neural_fallback_mask": (C.c_int32, [H, C.POINTER(PbrtImage)]),
    "pbrt_neural_calibrate": (C.c_int32, [H, H]),
    "pbrt_neural_set_precision": (C.c_int32, [H, C.c_int32]),
    "pbrt_neural_fp8_layers": (C.c_int32, [H, C.POINTER(C.c_int32), C.c_int32]),
    "pbrt_neural_set_fp8_layers": (C.c_int32, [H, C.POINTER(C.c_int32), C.c_int32]),
    "pbrt_neural_autotune": (C.c_int32, [H, H]),
    "pbrt_neural_conv_kernels": (C.c_int32, [H, C.POINTER(C.c_int32), C.c_int32]),
    "pbrt_neural_set_conv_kernels": (C.c_int32, [H, C.POINTER(C.c_int32), C.c_int32]),
})

WEIGHTS = Path(__file__).resolve().parent / "weights" / "kpunet.npz"
GATE = Path(__file__).resolve().parent / "weights" / "gate.json"


def gate_coefficients(path=None) -> np.ndarray:
    """The learned tile gate's 4 x 9 coefficients (default: the packaged fit)."""
    import json

    d = json.loads(Path(path or GATE).read_text())
    return np.asarray(d["coef"], np.float32)


def param_count() -> int:
    n = C.c_int64()
    check(lib().pbrt_neural_param_count(C.byref(n)))
    return n.value


def load_params(weights=None) -> np.ndarray:
    """FP32 parameter vector from an .npz written by KPUNet.save (default:
    the trained weights shipped with the package) or an array."""
    if weights is None:
        weights = WEIGHTS
    if isinstance(weights, (str, Path)):
        with np.load(weights) as d:
            weights = d["params"]
    p = np.ascontiguousarray(np.asarray(weights, dtype=np.float32))
    if p.size != param_count():
        raise ValueError(f"NeuralDenoiser: {p.size} parameters, the network has {param_count()}")
    return p


class NeuralDenoiser(Handle):
    """Denoises the demodulated illumination of `illu_buffer` (one sample, or
    the Accumulator's output with `acc_buffer` giving the sample counts) with
    the G-buffer's albedo, normal and depth. With `fallback` (a BMFR over the
    same frame, dispatched first), the learned gate shows per tile the blend
    of the network's and BMFR's outputs it predicts best (gate_model
    "default": the packaged coefficients; or 36 numbers); with gate_model
    None, tiles whose mean predicted error exceeds `threshold` show BMFR's
    final image."""

    def __init__(self, width: int, height: int, g_buffer: GBuffer, illu_buffer: IlluminationBuffer, weights=None,
                 fallback: BMFR | None = None, threshold: float = 0.5, tile: int = 32, acc_buffer=None,
                 gate_model="default"):
        p = load_params(weights)
        h = C.c_void_p()
        check(lib().pbrt_neural_create(width, height, g_buffer.ptr, illu_buffer.ptr,
                                       acc_buffer.ptr if acc_buffer is not None else None, p.ctypes.data_as(H),
                                       p.size, C.byref(h)))
        super().__init__(h)
        self._inputs = (g_buffer, illu_buffer, acc_buffer)
        self.width, self.height = width, height
        d, v, f = PbrtImage(), PbrtImage(), PbrtImage()
        check(lib().pbrt_neural_images(h, C.byref(d), C.byref(v)))
        check(lib().pbrt_neural_final_image(h, C.byref(f)))
        self.denoised, self.variance, self._final = Image(d, self), Image(v, self), Image(f, self)
        self._fallback = None
        self.gate_coef = None
        self.set_fallback(fallback, threshold, tile)
        if fallback is not None and gate_model is not None:
            self.set_gate_model(gate_coefficients() if isinstance(gate_model, str) else gate_model)

    def set_gate_model(self, coef) -> None:
        """Learned tile gate (4 x 9 coefficients; see pbrt_nn_gate_model) or None for the threshold rule."""
        if coef is None:
            check(lib().pbrt_neural_set_gate_model(self.ptr, None, 0))
            self.gate_coef = None
            return
        c = np.ascontiguousarray(np.asarray(coef, np.float32))
        check(lib().pbrt_neural_set_gate_model(self.ptr, c.ctypes.data_as(C.POINTER(C.c_float)), c.size))
        self.gate_coef = c

    def set_params(self, weights) -> None:
        p = load_params(weights)
        check(lib().pbrt_neural_set_params(self.ptr, p.ctypes.data_as(H), p.size))

    def set_fallback(self, fallback: BMFR | None, threshold: float = 0.5, tile: int = 32) -> None:
        check(lib().pbrt_neural_set_fallback(self.ptr, fallback.ptr if fallback is not None else None, threshold,
                                             tile))
        self._fallback = fallback
        self.threshold, self.tile = threshold, tile
        m = PbrtImage()
        check(lib().pbrt_neural_fallback_mask(self.ptr, C.byref(m)))
        self.fallback_mask = Image(m, self) if m.data else None

    def calibrate(self, stream=None) -> None:
        """FP8 scales from one BF16 pass over the current inputs, then each layer timed in BF16 and FP8
        (fp8_layers: where FP8 is faster)."""
        check(lib().pbrt_neural_calibrate(self.ptr, stream_handle(stream)))

    def set_precision(self, bits: int) -> None:
        """16: BF16 convolutions; 8: FP8 e4m3 for the layers fp8_layers marks (after calibrate)."""
        check(lib().pbrt_neural_set_precision(self.ptr, bits))

    def fp8_layers(self) -> list:
        """Per convolution (kpunet's layer order): True where the FP8 mode runs it in e4m3."""
        m = (C.c_int32 * 18)()
        check(lib().pbrt_neural_fp8_layers(self.ptr, m, 18))
        return [bool(v) for v in m]

    def set_fp8_layers(self, mask) -> None:
        """Fix the FP8 mode's per-layer precision (the first convolution stays BF16)."""
        m = (C.c_int32 * 18)(*[1 if v else 0 for v in mask])
        check(lib().pbrt_neural_set_fp8_layers(self.ptr, m, 18))

    KINDS = ("mma", "umma", "umma_planes")

    def autotune(self, stream=None) -> list:
        """Times the mma.sync and tcgen05 kernels (the latter with the first input's halo as swizzled
        pixel rows and as 8-channel planes) for every convolution on the current inputs; keeps the fastest."""
        check(lib().pbrt_neural_autotune(self.ptr, stream_handle(stream)))
        return self.conv_kernels()

    def conv_kernels(self) -> list:
        """Per-layer convolution kernel: "mma", "umma" (tcgen05) or "umma_planes" (tcgen05, the first
        input's halo as 8-channel planes; the same bits as "umma")."""
        k = (C.c_int32 * 18)()
        check(lib().pbrt_neural_conv_kernels(self.ptr, k, 18))
        return [self.KINDS[v] for v in k]

    def set_conv_kernels(self, kinds) -> None:
        k = (C.c_int32 * 18)(*[self.KINDS.index(x) for x in kinds])
        check(lib().pbrt_neural_set_conv_kernels(self.ptr, k, 18))

    def dispatch(self, push_constants=None, stream=None, graph: bool = True) -> None:
        fn = lib().pbrt_neural_dispatch if graph else lib().pbrt_neural_dispatch_direct
        check(fn(self.ptr, stream_handle(stream)))

    def add_dispatch_to_command_graph(self, commands: Commands, push_constants=None) -> None:
        commands.add(lambda s: self.dispatch(push_constants, s))

    def get_final_descriptor_image(self) -> Image:
        return self._final

    def fallback_tiles(self, stream=None) -> int:
        n = C.c_uint32()
        check(lib().pbrt_neural_fallback_tiles(self.ptr, stream_handle(stream), C.byref(n)))
        return n.value
