"""Offline replay (source/io/RenderIO.cpp, VulkanPBRT.cpp:211-243, 568-605)
on the GPU: frames traced here are downloaded through the OfflineGBuffer /
OfflineIllumination staging commands, exported as OpenEXR with their camera
matrices, imported again and uploaded into fresh buffers; the replayed
accumulate + BMFR frames then match the live ones (bit-exact inputs except
the normals, which the file stores as cartesian vectors)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _camera(sc, f, W, H):
    from vulkanpbrt_gb300.camera import Camera

    eye = np.asarray(sc.camera_eye, np.float64) + np.array([0.05 * f, 0.0, 0.02 * f])
    return Camera(tuple(eye), sc.camera_center, aspect=W / H)


def test_replay_round_trip(cuda, tmp_path):
    import torch

    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300 import render_io as R
    from vulkanpbrt_gb300 import scene as S

    W, H, F = 128, 80, 3
    sc = S.cornell_spheres(seed=3)
    sh = vp.SceneHandle(sc)
    g = vp.GBuffer(W, H)
    illu = vp.IlluminationBufferDemodulatedFloat(W, H)
    pipe = vp.PBRTPipeline(sh, g, illu, True, max_recursion_depth=4, min_recursion_depth=4)
    pc = vp.PushConstants()
    g_stager, i_stager = R.OfflineGBuffer(), R.OfflineIllumination()
    dl = vp.Commands()
    g_stager.download_from_g_buffer_command(g, dl)
    i_stager.download_from_illumination_buffer_command(illu, dl)
    gbufs = [R.OfflineGBuffer() for _ in range(F)]
    illus = [R.OfflineIllumination() for _ in range(F)]
    mats = []
    for f in range(F):
        cam = _camera(sc, f, W, H)
        pc.set(view_inverse=cam.inv_view, proj_inverse=cam.inv_proj, prev_view=cam.view, frame_number=f)
        pipe.trace(pc)
        dl.submit()
        g_stager.transfer_staging_data_to(gbufs[f])
        i_stager.transfer_staging_data_to(illus[f])
        mats.append(vp.CameraMatrices(cam.view, cam.inv_view, cam.proj, cam.inv_proj))
    assert np.array_equal(gbufs[F - 1].depth, g.depth.tensor().cpu().numpy()[..., 0])
    assert np.array_equal(illus[F - 1].noisy, illu.illumination_images[0].tensor().cpu().numpy())
    pat = {k: str(tmp_path / f"{k}_%d.exr") for k in ("position", "depth", "normal", "material", "albedo", "illu")}
    R.GBufferIO.export_g_buffer(pat["position"], pat["depth"], pat["normal"], pat["material"], pat["albedo"], F, gbufs,
                                mats)
    R.IlluminationBufferIO.export_illumination(pat["illu"], F, illus)
    R.MatrixIO.export_matrices(str(tmp_path / "m.json"), mats)
    mats2 = R.MatrixIO.import_matrices(str(tmp_path / "m.json"))
    gb2 = R.GBufferIO.import_g_buffer_depth(pat["depth"], pat["normal"], pat["material"], pat["albedo"], F)
    gbp = R.GBufferIO.import_g_buffer_position(pat["position"], pat["normal"], pat["material"], pat["albedo"], mats2, F)
    il2 = R.IlluminationBufferIO.import_illumination(pat["illu"], F)
    for f in range(F):
        assert np.array_equal(gb2[f].depth, gbufs[f].depth)
        assert np.array_equal(gb2[f].albedo, gbufs[f].albedo)
        assert np.abs(gb2[f].normal - gbufs[f].normal)[..., 0].max() < 2e-3
        assert np.array_equal(il2[f].noisy, illus[f].noisy)
        hit = gbufs[f].depth < 100
        rel = np.abs(gbp[f].depth - gbufs[f].depth)[hit] / gbufs[f].depth[hit]
        assert rel.max() < 1e-4
    # replay: upload into fresh buffers, accumulate + BMFR; the same on the live frames
    def run(frames_g, frames_i, mats_):
        g_ = vp.GBuffer(W, H)
        il_ = R.illumination_buffer_for(frames_i[0].noisy, W, H)
        gs, is_ = R.OfflineGBuffer(), R.OfflineIllumination()
        up = vp.Commands()
        gs.upload_to_g_buffer_command(g_, up)
        is_.upload_to_illumination_buffer_command(il_, up)
        accu = vp.Accumulator(g_, il_, separate_matrices=True)
        ai, ab = accu.accumulated_illumination, accu.accumulation_buffer
        bm = vp.BMFR(W, H, 32, 32, g_, ai, ab, 256)
        pcs = vp.PushConstants()
        for f in range(F):
            gs.transfer_staging_data_from(frames_g[f])
            is_.transfer_staging_data_from(frames_i[f])
            up.submit()
            accu.set_camera_matrices(f, mats_[f], mats_[f - 1 if f else f])
            vp.lib().pbrt_accumulator_dispatch(accu.ptr, None)
            pcs.set(view_inverse=mats_[f].inv_view, proj_inverse=mats_[f].inv_proj, prev_view=mats_[f].view,
                    frame_number=f)
            bm.dispatch(pcs)
            vp.lib().pbrt_accumulation_buffer_copy_to_back_images(ab.ptr, g_.ptr, ai.ptr, None)
        torch.cuda.synchronize()
        assert np.array_equal(g_.depth.tensor().cpu().numpy()[..., 0], frames_g[F - 1].depth)
        return bm.get_final_descriptor_image().tensor().cpu().numpy().astype(int)

    live = run(gbufs, illus, mats)
    replay = run(gb2, il2, mats2)
    diff = np.abs(live - replay)[..., :3]
    assert (diff > 2).mean() < 0.01 and diff.mean() < 0.1, (diff.max(), diff.mean())
    assert live[..., :3].mean() > 1
