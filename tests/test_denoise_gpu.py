"""CUDA accumulator / BMFR / BFR against the CPU oracle on the same seeded inputs.

Tolerances: BMFR and BFR outputs (RGBA16F) within 1e-3 relative (+1e-4
absolute floor near zero) on >= 99.9% of pixels -- the remaining pixels are
those where an FP32 rounding difference flips a reduction result across a
half-precision rounding boundary or a sign() in BFR's L1 mode; the final
BGRA8 image within 1 LSB. Accumulator: motion / illumination within 1e-3
relative, spp bit-exact.
"""
import numpy as np
import pytest

from denoise_cases import close_fraction, get, inputs, put, stats

pytestmark = pytest.mark.gpu


def _setup(vp, s, W, H, bw, kind, fk=256, position_type=0):
    g = vp.GBuffer(W, H)
    put(g.depth, s["depth"])
    put(g.normal, s["normal"])
    put(g.albedo, s["albedo"])
    illu = vp.IlluminationBufferDemodulated(W, H)
    put(illu.illumination_images[0], s["noisy16"])
    acc = vp.AccumulationBuffer(W, H)
    put(acc.motion, s["motion"])
    put(acc.spp, s["spp"])
    if kind == "bmfr":
        d = vp.BMFR(W, H, bw, bw, g, illu, acc, fk, position_type=position_type)
    else:
        d = vp.BFR(W, H, bw, bw, g, illu, acc)
    return g, illu, acc, d


def _pc(vp, cam, frame):
    return vp.PushConstants(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view, frame_number=frame)


# 8x8 and 16x16 blocks fit 10 features to 64 / 256 rows; some blocks are ill
# conditioned enough that a 1-ulp sinf/cosf difference in the normal decode,
# flipping one R16F-quantised feature, moves the output by a few percent.
# 32x32 blocks (the reference's default) meet the bar on every pixel.
MIN_FRACTION = {32: 0.999, 16: 0.998, 8: 0.998}


@pytest.mark.parametrize("bw,fk,position_type", [(32, 256, 0), (16, 256, 0), (8, 64, 0), (32, 256, 2), (32, 256, 1)])
def test_bmfr_matches_oracle(cuda, oracle, bw, fk, position_type):
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.camera import col_major

    W, H = 320, 180
    den_ref = np.zeros((2, H, W, 4), np.float16)
    for frame in (0, 1):
        s = inputs(W, H, seed=11, frame=frame)
        if frame == 0:
            g, illu, acc, bm = _setup(vp, s, W, H, bw, "bmfr", fk, position_type)
        else:
            put(acc.motion, s["motion"])
            put(acc.spp, s["spp"])
            put(illu.illumination_images[0], s["noisy16"])
        cam = s["camera"]
        bm.dispatch(_pc(vp, cam, frame))
        feats, w_ref, fin_ref = oracle.bmfr(bw, fk, frame, position_type, col_major(cam.inv_view),
                                            col_major(cam.inv_proj), s["depth"], s["normal"], s["albedo"],
                                            s["noisy16"], s["motion"], s["spp"], den_ref)
        den = get(bm.denoised)
        fin = get(bm.get_final_descriptor_image())
        layer = (frame & 1) ^ 1
        frac = stats(f"bmfr bw={bw} pt={position_type} frame={frame} denoised", den[layer], den_ref[layer])
        assert frac >= MIN_FRACTION[bw]
        lsb = np.abs(fin.astype(int) - fin_ref.astype(int))
        print(f"  final: max |diff| {lsb.max()} LSB, >1 LSB on {(lsb > 1).mean() * 100:.4f}%")
        assert (lsb <= 1).mean() >= 0.999
        w = get(bm.weights)[..., 0]
        assert np.isfinite(w).mean() > 0.99


@pytest.mark.parametrize("bw,fk", [(32, 256), (16, 256), (8, 64)])
def test_bmfr_fit_is_bit_exact_when_inputs_agree(cuda, oracle, bw, fk):
    """With normals whose decode is exact on both sides (theta = phi = 0) the
    fit sees bit-identical features: weights and denoised output must then be
    bit-identical to the oracle (same summation order, same rounding)."""
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.camera import col_major

    W, H = 256, 160
    den_ref = np.zeros((2, H, W, 4), np.float16)
    for frame in (0, 1):
        s = inputs(W, H, seed=7, frame=frame)
        s["normal"] = np.zeros_like(s["normal"])
        if frame == 0:
            g, illu, acc, bm = _setup(vp, s, W, H, bw, "bmfr", fk)
        else:
            put(acc.motion, s["motion"])
            put(acc.spp, s["spp"])
            put(illu.illumination_images[0], s["noisy16"])
            put(g.normal, s["normal"])
        cam = s["camera"]
        bm.dispatch(_pc(vp, cam, frame))
        _, w_ref, fin_ref = oracle.bmfr(bw, fk, frame, 0, col_major(cam.inv_view), col_major(cam.inv_proj),
                                        s["depth"], s["normal"], s["albedo"], s["noisy16"], s["motion"], s["spp"],
                                        den_ref)
        w = get(bm.weights)[..., 0]
        assert np.array_equal(w, w_ref, equal_nan=True), f"weights differ in {(w != w_ref).sum()} entries"
        den = get(bm.denoised)
        assert np.array_equal(den.view(np.uint16), den_ref.view(np.uint16))
        fin = get(bm.get_final_descriptor_image())
        assert np.abs(fin.astype(int) - fin_ref.astype(int)).max() <= 1


@pytest.mark.parametrize("bw", [16, 8, 32])
def test_bfr_matches_oracle(cuda, oracle, bw):
    import vulkanpbrt_gb300 as vp

    W, H = 256, 144
    den_ref = np.zeros((2, H, W, 4), np.float16)
    for frame in (0, 1):
        s = inputs(W, H, seed=21, frame=frame)
        if frame == 0:
            g, illu, acc, bf = _setup(vp, s, W, H, bw, "bfr")
        else:
            put(acc.motion, s["motion"])
            put(acc.spp, s["spp"])
            put(illu.illumination_images[0], s["noisy16"])
        bf.dispatch(_pc(vp, s["camera"], frame))
        fin_ref = oracle.bfr(bw, bw, frame, s["depth"], s["normal"], s["albedo"], s["motion"], s["spp"], s["noisy16"],
                             den_ref)
        den = get(bf.denoised)
        fin = get(bf.get_final_descriptor_image())
        layer = (frame & 1) ^ 1
        frac = stats(f"bfr bw={bw} frame={frame} denoised", den[layer], den_ref[layer])
        assert frac >= 0.999
        lsb = np.abs(fin.astype(int) - fin_ref.astype(int))
        print(f"  final: max |diff| {lsb.max()} LSB")
        assert (lsb <= 1).mean() >= 0.999


def test_accumulator_matches_oracle(cuda, oracle):
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.camera import Camera, col_major

    W, H = 320, 180
    s = inputs(W, H, seed=31)
    cam0 = s["camera"]
    cam1 = Camera((0.05, -2.95, 1.02), (0.0, 0.0, 1.0), aspect=W / H)
    g = vp.GBuffer(W, H)
    src = vp.IlluminationBufferDemodulatedFloat(W, H)
    accu = vp.Accumulator(g, src, separate_matrices=True)
    ab = accu.accumulation_buffer
    cmds = vp.Commands()
    accu.add_dispatch_to_command_graph(cmds)
    ab.copy_to_back_images(cmds, g, accu.accumulated_illumination)
    prev_depth = np.zeros((H, W), np.float32)
    prev_spp = np.zeros((H, W), np.uint8)
    prev_out = np.zeros((H, W, 4), np.float16)
    for frame, cam in enumerate([cam0, cam1, cam1]):
        depth = s["depth"] * (1.0 + 0.002 * frame)
        noisy = s["noisy"] * (1 + frame)
        put(g.depth, depth.astype(np.float32))
        put(g.normal, s["normal"])
        put(src.illumination_images[0], noisy)
        prev = [cam0, cam0, cam1][frame]
        accu.set_camera_matrices(frame, vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj),
                                 vp.CameraMatrices(prev.view, prev.inv_view))
        cmds.submit()
        motion = get(ab.motion)
        spp = get(ab.spp)[..., 0]
        illum = get(accu.accumulated_illumination.illumination_images[0])
        prev_origin = np.linalg.inv(prev.view.astype(np.float64))[:3, 3].tolist() + [1.0]
        m_ref, spp_ref, il_ref = oracle.accumulate(frame, 1, col_major(cam.inv_proj), col_major(cam.inv_view),
                                                   col_major(prev.view), prev_origin, noisy, depth.astype(np.float32),
                                                   prev_depth, prev_spp, prev_out)
        agree = (spp == spp_ref).mean()
        print(f"accumulate frame {frame}: spp agree {agree * 100:.4f}%, reprojected {(m_ref[..., 0] >= 0).mean() * 100:.1f}%")
        assert agree >= 0.999
        assert close_fraction(motion, m_ref)[0] >= 0.999
        assert close_fraction(illum, il_ref)[0] >= 0.999
        prev_depth, prev_spp, prev_out = depth.astype(np.float32), spp_ref, il_ref


def test_invalid_configurations_are_rejected(cuda):
    import vulkanpbrt_gb300 as vp

    g = vp.GBuffer(64, 64)
    illu = vp.IlluminationBufferDemodulated(64, 64)
    acc = vp.AccumulationBuffer(64, 64)
    with pytest.raises(vp.PbrtError, match="smaller than the mirror padding"):
        vp.BMFR(64, 64, 32, 32, g, illu, acc)
    with pytest.raises(vp.PbrtError, match="work size"):
        vp.BMFR(64, 64, 24, 24, g, illu, acc)
    final = vp.IlluminationBufferFinal(64, 64)
    with pytest.raises(vp.PbrtError, match="Demodulated"):
        vp.BFR(64, 64, 16, 16, g, final, acc)
