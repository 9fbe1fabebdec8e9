"""The FP64 re-solve of ill-conditioned BMFR blocks (no reference
counterpart; the reference keeps bmfrFit.comp's FP32 Householder solution,
shaders/bmfrFit.comp:27-86).

With fp64_resolve on, the fused FP32 kernel records every block whose
R-factor diagonal ratio max|R_ii| / min|R_ii| exceeds the condition limit,
and bmfr_fp64_kernel recomputes those blocks' quantised, noise-regularised
features and solves the least-squares fit in FP64. Checked here:

* on a frame with one normal everywhere and one depth on its left half, the
  largest ratio and the flagged-block count agree with the default limit of
  1e6 -- the fit's 1e-4 noise term (bmfrGeneral.comp:103-117) keeps the
  ratio of features in [0, 1] far below it;
* with the limit lowered so that every block is re-solved, the weights of
  every block equal numpy's float64 least-squares solution on the same
  R16F-quantised features (the oracle's bmfrPre) plus the same noise, to
  FP32 rounding -- and are closer to it than the FP32 fit on the flat wall;
* the re-solved blocks' denoised output is finite.
"""
import ctypes as C

import numpy as np
import pytest

from denoise_cases import get, inputs, put

pytestmark = pytest.mark.gpu

BW = 32


def _flat_wall(W, H, seed=23):
    """Synthetic G-buffer with one normal everywhere (theta = phi = 0, whose
    decode is exact on the GPU and the CPU, so both build bit-identical
    features) and one depth on the left half (a flat wall facing the camera)."""
    s = inputs(W, H, seed=seed, frame=0)
    s["normal"][...] = 0.0
    s["depth"][:, : W // 2] = 4.0
    return s


def _noise_table(oracle, frame):
    """The fit's per-row noise 2e-4 * (hash - 0.5) for the 10 feature columns, rows r = lx * BW + ly."""
    P = BW * BW
    rnd = oracle.lib().oracle_bmfr_random
    h = [[rnd(C.c_uint32((r + cc * P * P + frame * 13 * P * P) & 0xFFFFFFFF)) for r in range(P)] for cc in range(10)]
    return np.float32(2e-4) * (np.asarray(h, np.float32) - np.float32(0.5))


def _lstsq_weights(oracle, s, cam, W, H, frame):
    """float64 least squares of every block: [gh, gw, 10, 3]."""
    from vulkanpbrt_gb300.camera import col_major

    feats = oracle.bmfr_pre(BW, frame, 0, col_major(cam.inv_view), col_major(cam.inv_proj), s["depth"], s["normal"],
                            s["noisy16"])
    noise = _noise_table(oracle, frame)
    gw, gh = W // BW + 2, H // BW + 2
    out = np.zeros((gh, gw, 10, 3))
    for gy in range(gh):
        for gx in range(gw):
            blk = feats[:, gy * BW:(gy + 1) * BW, gx * BW:(gx + 1) * BW].astype(np.float32)  # [13, ly, lx]
            cols = blk.transpose(0, 2, 1).reshape(13, -1)  # row r = lx * BW + ly
            A = (cols[:10] + noise).astype(np.float64).T
            B = cols[10:].astype(np.float64).T
            out[gy, gx] = np.linalg.lstsq(A, B, rcond=None)[0]
    return out


def _weights(bm, gh, gw):
    w = get(bm.weights).reshape(30, gh, gw)  # layer i * 3 + channel
    return w.reshape(10, 3, gh, gw).transpose(2, 3, 0, 1).astype(np.float64)


def test_fp64_resolve_matches_float64_least_squares(cuda, oracle):
    import vulkanpbrt_gb300 as vp

    W, H, frame = 320, 192, 0
    s = _flat_wall(W, H)
    cam = s["camera"]
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulated(W, H)
    acc = vp.AccumulationBuffer(W, H)
    for img, key in ((g.depth, "depth"), (g.normal, "normal"), (g.albedo, "albedo"), (acc.motion, "motion"),
                     (acc.spp, "spp")):
        put(img, s[key])
    put(illu.illumination_images[0], s["noisy16"])
    pc = vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view,
                          frame_number=frame)
    gw, gh = W // BW + 2, H // BW + 2
    ref = _lstsq_weights(oracle, s, cam, W, H, frame)

    # FP32 fit alone (the reference's solution)
    bm32 = vp.BMFR(W, H, BW, BW, g, illu, acc, 256)
    bm32.dispatch(pc)
    w32 = _weights(bm32, gh, gw)

    # default limit: the ratio stays far below 1e6, nothing is re-solved
    bm = vp.BMFR(W, H, BW, BW, g, illu, acc, 256, fp64_resolve=True)
    bm.dispatch(pc)
    n, ratio = bm.condition_stats()
    print(f"default limit 1e6: {n} blocks re-solved, largest R-diagonal ratio {ratio:.4g}")
    assert np.isfinite(ratio) and 1.0 <= ratio < 1e6 and n == 0
    assert bm.fp64_block_count() == 0
    np.testing.assert_array_equal(_weights(bm, gh, gw), w32)

    # limit 1: every block goes to the FP64 solver
    bm.set_condition_limit(1.0)
    bm.dispatch(pc)
    n, ratio2 = bm.condition_stats()
    assert n == gw * gh and ratio2 == ratio
    w64 = _weights(bm, gh, gw)
    scale = np.abs(ref).max(axis=(2, 3), keepdims=True) + 1e-6
    err64 = (np.abs(w64 - ref) / scale).max(axis=(2, 3))
    err32 = (np.abs(w32 - ref) / scale).max(axis=(2, 3))
    wall = np.zeros((gh, gw), bool)
    wall[1:-1, 1: (W // 2) // BW] = True  # blocks whose pixels all lie on the flat wall
    print(f"weights vs float64 lstsq (relative to each block's largest weight): FP64 re-solve worst "
          f"{err64.max():.3g}; FP32 fit worst {err32.max():.3g}, on the flat wall {err32[wall].max():.3g}")
    assert err64.max() < 1e-5
    assert err32[wall].max() > 10 * err64[wall].max()
    den = get(bm.denoised)[1]
    assert np.isfinite(den.astype(np.float32)).all()


def test_condition_limit_rejects_bad_values(cuda):
    import vulkanpbrt_gb300 as vp

    W, H = 128, 96
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulated(W, H)
    acc = vp.AccumulationBuffer(W, H)
    bm = vp.BMFR(W, H, BW, BW, g, illu, acc, 256)
    for bad in (0.5, float("inf"), float("nan")):
        with pytest.raises(vp.PbrtError, match="condition limit"):
            bm.set_condition_limit(bad)
    with pytest.raises(vp.PbrtError, match="fp64_resolve"):
        bm.condition_stats()
