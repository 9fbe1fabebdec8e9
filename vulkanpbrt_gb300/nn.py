"""Neural-denoiser operators over the C ABI (BF16 tensor-core convolutions and
the FP32 helpers around them). Tensors are torch CUDA tensors used as plain
device buffers in NHWC layout; every operator runs this library's kernels on
the current torch stream and raises PbrtError on a rejected call."""
from __future__ import annotations

import ctypes as C

from . import _abi
from ._abi import check, lib

H = C.c_void_p
i32, i64, f32 = C.c_int32, C.c_int64, C.c_float
_abi.add_signatures({
    "pbrt_nn_conv3x3": (i32, [H, i32, H, i32, H, H, H, H, i32, i32, i32, i32, i32, H]),
    "pbrt_nn_conv3x3_wgrad": (i32, [H, H, i32, H, i32, H, i32, i32, i32, i32, H]),
    "pbrt_nn_conv3x3_fp8": (i32, [H, i32, H, i32, H, H, H, H, H, i32, i32, i32, i32, i32, H]),
    "pbrt_nn_quantize_weights_fp8": (i32, [H, H, i32, i32, H, H, H]),
    "pbrt_nn_channel_amax": (i32, [H, i64, i32, H, H]),
    "pbrt_nn_conv3x3_umma": (i32, [H, i32, H, i32, H, H, H, i32, i32, i32, i32, i32, H]),
    "pbrt_nn_conv3x3_umma_pooled": (i32, [H, i32, H, H, H, H, i32, i32, i32, i32, i32, H]),
    "pbrt_nn_conv3x3_umma_f32": (i32, [H, i32, H, H, H, i32, i32, i32, i32, i32, H]),
    "pbrt_nn_conv3x3_wgrad_umma": (i32, [H, H, i32, H, i32, H, i32, i32, i32, i32, H]),
    "pbrt_nn_conv3x3_fp8_umma": (i32, [H, i32, H, i32, H, H, H, H, H, H, i32, i32, i32, i32, i32, H]),
    "pbrt_nn_umma_status": (i32, [H, C.POINTER(C.c_uint32)]),
    "pbrt_nn_flip_weights": (i32, [H, H, i32, i32, H]),
    "pbrt_nn_features": (i32, [H, i32, H, H, H, H, i32, i32, i32, i32, i32, H, H, H]),
    "pbrt_nn_avgpool2": (i32, [H, H, i32, i32, i32, i32, i32, H]),
    "pbrt_nn_avgpool2_bwd_add": (i32, [H, H, i32, i32, i32, i32, H]),
    "pbrt_nn_relu_bwd": (i32, [H, H, H, H, i64, i32, H]),
    "pbrt_nn_split_upsum": (i32, [H, i32, i32, i32, i32, i32, H, H, H]),
    "pbrt_nn_kp_head": (i32, [H, H, H, H, H, H, H, H, H, H, i32, i32, i32, i32, i32, H]),
    "pbrt_nn_kp_head_bwd": (i32, [H, H, H, H, H, H, H, H, i32, i32, i32, i32, i32, H, H, H, H, H, H, H]),
    "pbrt_nn_relmse_loss": (i32, [H, H, H, H, i32, i32, i32, i32, i32, f32, H, H, H, H]),
    "pbrt_nn_adam": (i32, [H, H, H, H, H, i64, f32, f32, f32, f32, i32, f32, H]),
    "pbrt_nn_gate": (i32, [H, i32, i32, i32, f32, i32, H, H, H]),
    "pbrt_nn_gate_model": (i32, [H, H, i32, i32, i32, i32, H, H, H, H, H, i32, H, H, H, H, H, H, H, H, H]),
    "pbrt_nn_compose": (i32, [H, i32, i32, i32, H, H, i32, H, H, H, H]),
})

RELU, ACCUMULATE, KSTEP, NO_WIDE = 1, 2, 4, 8


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def conv3x3(x1, w, bias=None, x2=None, relu=False, out=None, out32=None, accumulate=False, store_bf16=True,
            kernel="halo"):
    """y = relu?(conv3x3(concat(x1, up2(x2))) + bias). x1 [N,H,W,C1] bf16, x2 [N,H/2,W/2,C2] bf16,
    w [Cout, 9, C1+C2] bf16, bias [Cout] f32. Returns the BF16 output [N,H,W,Cout] (None when
    store_bf16 is False: only out32 is written, added to when accumulate is set). kernel: "halo"
    (input halo staged once per channel chunk; 16 x 16 tiles for Cout <= 48), "halo4x2" (8 x 16 tiles
    only) or "kstep" (pipelined per tap and 16 channels)."""
    import torch

    n, h, wd, c1 = x1.shape
    c2 = 0 if x2 is None else x2.shape[3]
    cout = w.shape[0]
    if out is None and store_bf16:
        out = torch.empty((n, h, wd, cout), dtype=torch.bfloat16, device=x1.device)
    flags = (RELU if relu else 0) | (ACCUMULATE if accumulate else 0) | (KSTEP if kernel == "kstep" else 0) | \
        (NO_WIDE if kernel == "halo4x2" else 0)
    check(lib().pbrt_nn_conv3x3(_ptr(x1), c1, _ptr(x2), c2, _ptr(w), _ptr(bias), _ptr(out if store_bf16 else None),
                                _ptr(out32), n, h, wd, cout, flags, _stream()))
    return out if store_bf16 else None


def conv3x3_fp8(x1, w8, wscale, inv_xscale, bias=None, x2=None, relu=False, out=None, kernel="auto",
                pooled=False, box=True):
    """FP8 (e4m3) forward: w8 [Cout, 9, Cin] uint8 e4m3 with per-output-channel scales wscale [Cout] (activation
    scales folded in), inv_xscale [Cin] quantises the BF16 input on load. Returns BF16 [N,H,W,Cout].
    kernel: "auto" (tcgen05 where it applies), "mma" (the mma.sync kernel) or "umma" (tcgen05 only: raises
    PbrtError where it does not apply). pooled=True (tcgen05, single input) also returns the 2x2 average
    pooling of the output, from the epilogue. box=False: the tcgen05 form gathers the upsampled second input with
    cp.async instead of loading its half-resolution box by TMA."""
    import torch

    n, h, wd, c1 = x1.shape
    c2 = 0 if x2 is None else x2.shape[3]
    cout = w8.shape[0]
    if out is None:
        out = torch.empty((n, h, wd, cout), dtype=torch.bfloat16, device=x1.device)
    flags = (RELU if relu else 0) | (0 if box else 16)
    if kernel == "umma" or pooled:
        pool = torch.empty((n, h // 2, wd // 2, cout), dtype=torch.bfloat16, device=x1.device) if pooled else None
        check(lib().pbrt_nn_conv3x3_fp8_umma(_ptr(x1), c1, _ptr(x2), c2, _ptr(w8), _ptr(wscale), _ptr(inv_xscale),
                                             _ptr(bias), _ptr(out), _ptr(pool), n, h, wd, cout, flags, _stream()))
        return (out, pool) if pooled else out
    flags |= 8 if kernel == "mma" else 0
    check(lib().pbrt_nn_conv3x3_fp8(_ptr(x1), c1, _ptr(x2), c2, _ptr(w8), _ptr(wscale), _ptr(inv_xscale), _ptr(bias),
                                    _ptr(out), n, h, wd, cout, flags, _stream()))
    return out


def quantize_weights_fp8(w32, xscale, w8=None, wscale=None):
    """w32 [Cout, 9, Cin] f32, xscale [Cin] -> (w8 uint8 e4m3, wscale [Cout])."""
    import torch

    cout, _, cin = w32.shape
    if w8 is None:
        w8 = torch.empty((cout, 9, cin), dtype=torch.uint8, device=w32.device)
    if wscale is None:
        wscale = torch.empty(cout, dtype=torch.float32, device=w32.device)
    check(lib().pbrt_nn_quantize_weights_fp8(_ptr(w32), _ptr(xscale), cout, cin, _ptr(w8), _ptr(wscale), _stream()))
    return w8, wscale


def channel_amax(x, amax):
    c = x.shape[-1]
    check(lib().pbrt_nn_channel_amax(_ptr(x), x.numel() // c, c, _ptr(amax), _stream()))
    return amax


def conv3x3_umma(x1, w, bias=None, x2=None, relu=False, out=None, persistent=True, tma=True, specialised=True,
                 box=True, swizzle=True):
    """tcgen05 forward (BF16 out): as conv3x3, Cout in {16, ..., 128}. persistent=False forces the
    per-tile kernel (the persistent one is used when the weights and two input halos fit in shared memory);
    tma=False gathers the persistent kernel's input halo with cp.async instead of a TMA load; specialised=False
    uses the single-role persistent kernel instead of the warp-specialised one; box=False gathers the upsampled
    second input with cp.async instead of loading its half-resolution box by TMA; swizzle=False loads the
    first input's halo as 8-channel planes instead of swizzled whole-pixel rows (the default for a single
    input of 16 or 32 channels and Cout 32 or 48)."""
    import torch

    n, h, wd, c1 = x1.shape
    c2 = 0 if x2 is None else x2.shape[3]
    cout = w.shape[0]
    if out is None:
        out = torch.empty((n, h, wd, cout), dtype=torch.bfloat16, device=x1.device)
    flags = (RELU if relu else 0) | (0 if persistent else 2) | (0 if tma else 4) | (0 if specialised else 8) | \
        (0 if box else 16) | (0 if swizzle else 32)
    check(lib().pbrt_nn_conv3x3_umma(_ptr(x1), c1, _ptr(x2), c2, _ptr(w), _ptr(bias), _ptr(out), n, h, wd, cout,
                                     flags, _stream()))
    return out


def conv3x3_umma_pooled(x1, w, bias=None, relu=False, swizzle=True):
    """conv3x3_umma of a single input that also returns the 2x2 average pooling of its output
    (the same bits as avgpool2 of it), from the warp-specialised kernel's epilogue."""
    import torch

    n, h, wd, c1 = x1.shape
    cout = w.shape[0]
    out = torch.empty((n, h, wd, cout), dtype=torch.bfloat16, device=x1.device)
    pooled = torch.empty((n, h // 2, wd // 2, cout), dtype=torch.bfloat16, device=x1.device)
    check(lib().pbrt_nn_conv3x3_umma_pooled(_ptr(x1), c1, _ptr(w), _ptr(bias), _ptr(out), _ptr(pooled), n, h, wd,
                                            cout, (RELU if relu else 0) | (0 if swizzle else 32), _stream()))
    return out, pooled


def conv3x3_umma_f32(x1, w, out32, bias=None, relu=False, tma=True):
    """tcgen05 convolution of one input into the FP32 tensor out32 [N,H,W,Cout] (any Cout that is a
    multiple of 16, in slices): the backward-data pass with flip_weights' weights."""
    n, h, wd, c1 = x1.shape
    cout = w.shape[0]
    flags = (RELU if relu else 0) | (0 if tma else 4)
    check(lib().pbrt_nn_conv3x3_umma_f32(_ptr(x1), c1, _ptr(w), _ptr(bias), _ptr(out32), n, h, wd, cout, flags,
                                         _stream()))
    return out32


def umma_status() -> int:
    """Error flags of the tcgen05 kernels since the last call (0 = none); synchronises."""
    f = C.c_uint32()
    check(lib().pbrt_nn_umma_status(_stream(), C.byref(f)))
    return f.value


def conv3x3_wgrad(dy, x1, dw, x2=None, kernel="mma"):
    """dw [Cout, 9, Cin] f32 += dY^T . im2col(concat(x1, up2(x2))); kernel "mma" (mma.sync) or "umma" (tcgen05)."""
    n, h, wd, c1 = x1.shape
    c2 = 0 if x2 is None else x2.shape[3]
    fn = lib().pbrt_nn_conv3x3_wgrad_umma if kernel == "umma" else lib().pbrt_nn_conv3x3_wgrad
    check(fn(_ptr(dy), _ptr(x1), c1, _ptr(x2), c2, _ptr(dw), n, h, wd, dy.shape[3], _stream()))
    return dw


def flip_weights(w, out=None):
    """[Cout, 9, Cin] -> [Cin, 9, Cout] with the taps reversed (backward-data weights)."""
    import torch

    cout, _, cin = w.shape
    if out is None:
        out = torch.empty((cin, 9, cout), dtype=w.dtype, device=w.device)
    check(lib().pbrt_nn_flip_weights(_ptr(w), _ptr(out), cout, cin, _stream()))
    return out


def features(illum, albedo, normal, depth, feat, rad, spp=None):
    """illum [N,h,w,4] f32|f16, albedo [N,h,w,4] u8, normal [N,h,w,2] f32, depth [N,h,w] f32, spp [N,h,w] u8
    (accumulator steps of 1/256, optional) -> feat [N,PH,PW,16] bf16 and rad [N,PH,PW,3] f32 (padded, edges
    replicated, clamped to [0, 10])."""
    import torch

    n, h, w = illum.shape[:3]
    ph, pw = feat.shape[1:3]
    check(lib().pbrt_nn_features(_ptr(illum), int(illum.dtype == torch.float16), _ptr(albedo), _ptr(normal),
                                 _ptr(depth), _ptr(spp), w, h, pw, ph, n, _ptr(feat), _ptr(rad), _stream()))


def avgpool2(x, out):
    import torch

    n, h, w, c = x.shape
    check(lib().pbrt_nn_avgpool2(_ptr(x), _ptr(out), int(x.dtype == torch.float32), n, h, w, c, _stream()))
    return out


def avgpool2_bwd_add(dy, dx):
    n, h, w, c = dx.shape
    check(lib().pbrt_nn_avgpool2_bwd_add(_ptr(dy), _ptr(dx), n, h, w, c, _stream()))


def relu_bwd(dy, y, out, db=None):
    c = y.shape[-1]
    check(lib().pbrt_nn_relu_bwd(_ptr(dy), _ptr(y), _ptr(out), _ptr(db), y.numel() // c, c, _stream()))
    return out


def split_upsum(dcat, c1, dx1, dx2):
    n, h, w, c = dcat.shape
    check(lib().pbrt_nn_split_upsum(_ptr(dcat), c1, c - c1, n, h, w, _ptr(dx1), _ptr(dx2), _stream()))


def kp_head(F, Wh, bh, R, out, coarse=None, kw=None, filt=None, alpha=None, var=None):
    n, h, w, c = F.shape
    check(lib().pbrt_nn_kp_head(_ptr(F), _ptr(Wh), _ptr(bh), _ptr(R), _ptr(coarse), _ptr(out), _ptr(kw), _ptr(filt),
                                _ptr(alpha), _ptr(var), n, h, w, c, Wh.shape[0], _stream()))
    return out


def kp_head_bwd(F, Wh, bh, R, kw, filt, dout, dF, dWh, dbh, coarse=None, alpha=None, dvar=None, dcoarse=None):
    n, h, w, c = F.shape
    check(lib().pbrt_nn_kp_head_bwd(_ptr(F), _ptr(Wh), _ptr(bh), _ptr(R), _ptr(coarse), _ptr(kw), _ptr(filt),
                                    _ptr(alpha), n, h, w, c, Wh.shape[0], _ptr(dout), _ptr(dvar), _ptr(dF), _ptr(dWh),
                                    _ptr(dbh), _ptr(dcoarse), _stream()))


def relmse_loss(out, target, albedo, dout, loss, var=None, dvar=None, var_weight=0.1):
    """out [N,PH,PW,3] f32 (padded), target [N,h,w,3] f32, albedo [N,h,w,4] u8; loss [2] f32 (+=)."""
    n, ph, pw = out.shape[:3]
    h, w = target.shape[1:3]
    check(lib().pbrt_nn_relmse_loss(_ptr(out), _ptr(target), _ptr(albedo), _ptr(var), n, ph, pw, h, w, var_weight,
                                    _ptr(dout), _ptr(dvar), _ptr(loss), _stream()))


def adam(w, g, m, v, step, lr=1e-4, b1=0.9, b2=0.999, eps=1e-8, w_bf16=None, grad_scale=1.0):
    check(lib().pbrt_nn_adam(_ptr(w), _ptr(g), _ptr(m), _ptr(v), _ptr(w_bf16), w.numel(), lr, b1, b2, eps, step,
                             grad_scale, _stream()))


def gate(var, w, h, threshold, tile, mask, count):
    """mask [tiles] u8 = mean(exp(var)) over each tile x tile block of the w x h image > threshold."""
    check(lib().pbrt_nn_gate(_ptr(var), var.shape[-1], w, h, threshold, tile, _ptr(mask), _ptr(count), _stream()))


def compose(out, albedo, final_bgra, mask=None, tile=32, fallback=None, denoised=None):
    """out [PH,PW,3] f32 -> final_bgra [h,w,4] u8; masked tiles copy fallback."""
    pw = out.shape[-2]
    h, w = final_bgra.shape[:2]
    check(lib().pbrt_nn_compose(_ptr(out), pw, w, h, _ptr(albedo), _ptr(mask), tile, _ptr(fallback),
                                _ptr(final_bgra), _ptr(denoised), _stream()))
