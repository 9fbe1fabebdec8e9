"""The CPU oracle against the known-answer vectors and analytic cases (no GPU)."""
import json

import numpy as np
import pytest

from conftest import ROOT

KAT = json.loads((ROOT / "tests" / "golden" / "kat_integer.json").read_text())


def test_golden_file_is_current():
    """The committed vectors equal what the generator produces."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", ROOT / "tests" / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    assert [mg.bmfr_random(a) for a in KAT["bmfr_random"]["in"]] == KAT["bmfr_random"]["out"]
    assert [mg.wang_hash(a) for a in KAT["wang_hash"]["in"]] == KAT["wang_hash"]["out"]


def test_bmfr_random_kat(oracle):
    got = [oracle.lib().oracle_bmfr_random(a) for a in KAT["bmfr_random"]["in"]]
    assert np.array_equal(np.float32(got), np.float32(KAT["bmfr_random"]["out"]))


def test_half_conversion_kat(oracle):
    for f, bits in zip(KAT["f32_to_f16_bits"]["in"], KAT["f32_to_f16_bits"]["out"]):
        assert oracle.lib().oracle_f2h(f) == bits, f


def test_half_conversion_matches_numpy_exhaustively_on_random_floats(oracle):
    rng = np.random.default_rng(7)
    vals = np.concatenate([rng.normal(0, 1, 2000), rng.normal(0, 1e4, 2000), rng.uniform(-1e-4, 1e-4, 2000),
                           np.array([np.inf, -np.inf])]).astype(np.float32)
    with np.errstate(over="ignore"):
        want = vals.astype(np.float16).view(np.uint16)
    got = np.array([oracle.lib().oracle_f2h(float(v)) for v in vals], np.uint16)
    assert np.array_equal(got, want)
    # and back
    back = np.array([oracle.lib().oracle_h2f(int(b)) for b in want], np.float32)
    assert np.array_equal(back, want.view(np.float16).astype(np.float32))


def test_mirror_kat(oracle):
    for (x, s), want in zip(KAT["mirror"]["in"], KAT["mirror"]["out"]):
        assert oracle.lib().oracle_mirror(x, s) == want


def _gbuffer(W, H, seed=0):
    from vulkanpbrt_gb300 import synthetic

    return synthetic.gbuffer_scene(W, H, seed=seed)


def test_bmfr_fit_matches_float64_least_squares(oracle):
    """bmfrFit's Householder solve against numpy lstsq on the same noised, quantised features."""
    from vulkanpbrt_gb300.camera import col_major

    W, H, bw = 96, 96, 32
    s = _gbuffer(W, H, seed=3)
    cam = s["camera"]
    feats = oracle.bmfr_pre(bw, 0, 0, col_major(cam.inv_view), col_major(cam.inv_proj), s["depth"], s["normal"],
                            s["noisy"].astype(np.float16))
    weights = oracle.bmfr_fit(W, H, bw, 256, 0, feats)
    gw, gh = W // bw + 2, H // bw + 2
    P = bw * bw
    for gy in range(gh):
        for gx in range(gw):
            A = np.zeros((P, 13))
            for r in range(P):
                px, py = r // bw + gx * bw, r % bw + gy * bw
                A[r] = feats[:, py, px].astype(np.float64)
                for c in range(10):
                    h = (r + c * P * P) & 0xFFFFFFFF
                    A[r, c] = np.float32(np.float32(A[r, c]) + np.float32(2e-4) * (np.float32(oracle.lib().oracle_bmfr_random(h)) - np.float32(0.5)))
            ws, *_ = np.linalg.lstsq(A[:, :10], A[:, 10:], rcond=None)
            got = weights[:, gy, gx].reshape(10, 3)
            fit64 = A[:, :10] @ ws
            fit32 = A[:, :10] @ got.astype(np.float64)
            scale = np.abs(fit64).max() + 1e-3
            assert np.abs(fit32 - fit64).max() / scale < 2e-3, (gx, gy)


def test_bmfr_weights_exact_for_linear_signal(oracle):
    """A noisy colour that is an exact linear function of the features is reproduced by the fit."""
    from vulkanpbrt_gb300.camera import col_major

    W, H, bw = 80, 80, 16
    s = _gbuffer(W, H, seed=5)
    cam = s["camera"]
    depth = s["depth"].copy()
    depth[depth > 1e3] = 50.0  # keep the sky out of this analytic case
    n = s["normal"]
    # colour = 0.3 + 0.2 * n.z (n decoded), an exact member of the feature span
    nz = np.cos(n[..., 0])
    col = (0.3 + 0.2 * nz).astype(np.float32)
    noisy = np.stack([col, col, col, np.ones_like(col)], -1).astype(np.float16)
    feats = oracle.bmfr_pre(bw, 0, 0, col_major(cam.inv_view), col_major(cam.inv_proj), depth, n, noisy)
    weights = oracle.bmfr_fit(W, H, bw, 256, 0, feats)
    den = np.zeros((2, H, W, 4), np.float16)
    motion = np.full((H, W, 2), -1, np.float16)
    spp = np.ones((H, W), np.uint8)
    oracle.bmfr_post(bw, 0, 0, col_major(cam.inv_view), col_major(cam.inv_proj), depth, n, s["albedo"], motion, spp,
                     weights, den)
    out = den[1, ..., 0].astype(np.float32)
    assert np.abs(out - col).max() < 5e-3


def test_accumulator_static_camera_reprojects_to_pixel_centres(oracle):
    from vulkanpbrt_gb300.camera import col_major

    W, H = 64, 48
    s = _gbuffer(W, H, seed=2)
    cam = s["camera"]
    # Fronto-parallel plane 10 units ahead: ray length varies slowly, so the
    # shader's half-pixel uv drift (scale W/(W-.5)) stays inside its 1% test.
    ys, xs = np.mgrid[0:H, 0:W]
    clip = np.stack([(xs + .5) / W * 2 - 1, (ys + .5) / H * 2 - 1, np.ones_like(xs * 1.0), np.ones_like(xs * 1.0)], -1)
    dv = clip @ np.linalg.inv(cam.proj64).T
    dv = dv[..., :3] / np.linalg.norm(dv[..., :3], axis=-1, keepdims=True)
    depth = (10.0 / -dv[..., 2]).astype(np.float32)
    prev_origin = np.linalg.inv(cam.view64)[:3, 3].tolist() + [1.0]
    zeros16 = np.zeros((H, W, 4), np.float16)
    m0, spp0, il0 = oracle.accumulate(0, 1, col_major(cam.inv_proj), col_major(cam.inv_view), col_major(cam.view),
                                      prev_origin, s["noisy"], depth, depth, np.zeros((H, W), np.uint8), zeros16)
    assert (m0 == -1).all()
    assert (spp0 == 1).all()  # 1/256 stored in R8_UNORM rounds to 1/255
    m1, spp1, il1 = oracle.accumulate(1, 1, col_major(cam.inv_proj), col_major(cam.inv_view), col_major(cam.view),
                                      prev_origin, s["noisy"] * 3, depth, depth, spp0, il0)
    u = (xs + 0.5) / W
    ok = m1[..., 0] >= 0
    assert ok.mean() > 0.95
    # The shader's uv scale W/(W-.5) maps pixel centres slightly off centre.
    want = ((u * 2 - 1) + 1) * 0.5 * (W / (W - 0.5))
    assert np.abs(m1[..., 0].astype(np.float32)[ok] - want[ok]).max() < 2e-3
    assert (spp1[ok] == 2).all()
