"""BFRBlender on the CPU: the oracle's restatement of shaders/bfrBlender.comp
against an independent float32 restatement written here (scalar numpy
float32, the shader's operation order), on analytic cases whose blend weight
is known in closed form, and the host-side rules of add_denoiser_to_commands
(source/util/DenoiserUtils.cpp) that need no GPU."""
import numpy as np
import pytest

f32 = np.float32


def _blend_py(avg, avg_sq, den8, den16, den32, radius):
    H, W = den8.shape[:2]
    k = f32(1.0) / f32(3.0)
    out = np.zeros((H, W, 4), np.uint8)

    def lum(c):
        c = c.astype(np.float32)
        return (c[0] * k + c[1] * k) + c[2] * k

    def mix(x, y, a):
        return x * (f32(1) - a) + y * a

    def mix3(a, b, c, t):
        t = np.fmin(t / f32(1), f32(1))
        af = np.fmax(f32(1) - t / f32(0.5), f32(0))
        bf = t / f32(0.5) if t < f32(0.5) else f32(1) - (t - f32(0.5)) / (f32(1) - f32(0.5))
        cf = (f32(1) - af) - bf
        return (af * a + bf * b) + cf * c

    for y in range(H):
        for x in range(W):
            sq = av = f32(0)
            count = 0
            for dy in range(-radius, radius + 1):
                for dx in range(-radius, radius + 1):
                    sx, sy = x + dx, y + dy
                    cur = lum(avg[sy, sx, :3]) if 0 <= sx < W and 0 <= sy < H else f32(0)
                    count += 1
                    w = f32(1) / f32(count)
                    sq = mix(sq, cur * cur, w)
                    av = mix(av, cur, w)
            av = mix(av, lum(avg[y, x, :3]), f32(0.5))
            sq = mix(sq, lum(avg_sq[y, x, :3]), f32(0.5))
            with np.errstate(invalid="ignore"):
                sd = np.sqrt(sq - av * av)
            for c in range(3):
                v = mix3(f32(den32[y, x, c]) / f32(255), f32(den16[y, x, c]) / f32(255),
                         f32(den8[y, x, c]) / f32(255), sd)
                out[y, x, c] = int(np.floor(min(max(v, f32(0)), f32(1)) * f32(255) + f32(0.5)))
            out[y, x, 3] = 255
    return out


def _dens(rng, H, W):
    return [rng.integers(0, 256, (H, W, 4), dtype=np.uint8) for _ in range(3)]


@pytest.mark.parametrize("dtype,radius", [(np.float16, 2), (np.float32, 1), (np.float16, 0)])
def test_oracle_matches_python_restatement(oracle, dtype, radius):
    rng = np.random.default_rng(7)
    H, W = 9, 13
    avg = (rng.random((H, W, 4)) ** 3 * 2).astype(dtype)
    avg_sq = (avg.astype(np.float32) ** 2 * rng.uniform(0.5, 3.0, (H, W, 1))).astype(dtype)
    d8, d16, d32 = _dens(rng, H, W)
    got = oracle.bfr_blend(avg, avg_sq, d8, d16, d32, radius=radius, threads=2)
    want = _blend_py(avg, avg_sq, d8, d16, d32, radius)
    assert np.array_equal(got, want)


def test_blend_weights_closed_form(oracle):
    """Zero average and average square: deviation 0 -> the 32x32 result.
    Average-square luminance 0.5: sq = 0.25, deviation 0.5 -> the 16x16
    result. A luminance field alternating 0 / 6: deviation >= 1 -> 8x8."""
    rng = np.random.default_rng(1)
    H, W = 8, 10
    d8, d16, d32 = _dens(rng, H, W)
    z = np.zeros((H, W, 4), np.float16)
    out = oracle.bfr_blend(z, z, d8, d16, d32, radius=2)
    assert np.array_equal(out[..., :3], d32[..., :3]) and (out[..., 3] == 255).all()
    half = np.full((H, W, 4), 0.5, np.float16)
    out = oracle.bfr_blend(z, half, d8, d16, d32, radius=2)
    assert np.array_equal(out[..., :3], d16[..., :3])
    alt = np.zeros((H, W, 4), np.float32)
    alt[::2, ::2, :3] = 6.0
    alt[1::2, 1::2, :3] = 6.0
    big = np.full((H, W, 4), 100.0, np.float32)
    out = oracle.bfr_blend(alt, big, d8, d16, d32, radius=1)
    assert np.array_equal(out[..., :3], d8[..., :3])


def test_denoiser_utils_rejects_what_the_reference_leaves_unset(native_lib):
    import vulkanpbrt_gb300 as vp
    from vulkanpbrt_gb300.denoiser_utils import DenoisingBlockSize as S, DenoisingType as T

    args = (vp.Commands(), None, 64, 32, vp.PushConstants(), None, None, None)
    assert vp.add_denoiser_to_commands(T.NONE, S.X32, *args) is None
    with pytest.raises(NotImplementedError):
        vp.add_denoiser_to_commands(T.SVG, S.X32, *args)
    with pytest.raises(NotImplementedError):
        vp.add_denoiser_to_commands(T.BMFR, S.X64, *args)
    assert [int(t) for t in T] == [0, 1, 2, 3] and [int(s) for s in S] == [0, 1, 2, 3, 4]
