// Device restatement of the reference's shading math: random.glsl, camera.glsl,
// color.glsl, brdf.glsl, sampling.glsl, lighting.glsl, geometry.glsl and
// ptClosesthit.rchit / ptAlphaHit.rahit / ptMiss.rmiss.
#pragma once
#include "scene.cuh"

namespace pbrt {

// ptConstants.glsl:4-11
constexpr float kPI = 3.14159265359f;
constexpr float kRecipPI = 0.31830988618f;
constexpr float kEpsilon = 1e-6f;
constexpr float kMinRoughness = 0.04f;
constexpr float kMaxRadiance = 1e1f;
constexpr float kMinTermination = 0.05f;

// ---------------------------------------------------------------------------
// random.glsl:9-96 -- 3 Tausworthe + 1 LCG generator, wangHash seeding.
struct Rng {
  uint32_t x, y, z, w;
};
PBRT_HD uint32_t taus_step(uint32_t z, int s1, int s2, int s3, uint32_t m) {
  uint32_t b = (((z << s1) ^ z) >> s2);
  return (((z & m) << s3) ^ b);
}
PBRT_HD uint32_t wang_hash(uint32_t seed) {
  seed = (seed ^ 61u) ^ (seed >> 16);
  seed *= 9u;
  seed = seed ^ (seed >> 4);
  seed *= 0x27d4eb2du;
  seed = seed ^ (seed >> 15);
  return seed;
}
PBRT_D float rng_next(Rng& e) {
  e.x = taus_step(e.x, 13, 19, 12, 4294967294u);
  e.y = taus_step(e.y, 2, 25, 4, 4294967288u);
  e.z = taus_step(e.z, 3, 11, 17, 4294967280u);
  e.w = 1664525u * e.w + 1013904223u;
  return __fmul_rn(2.3283064365387e-10f, __uint2float_rn(e.x ^ e.y ^ e.z ^ e.w));
}
PBRT_D Rng rng_init(uint32_t x, uint32_t y, uint32_t frame) {
  Rng r;
  r.x = wang_hash(x);
  r.y = wang_hash(y);
  r.z = wang_hash(frame);
  r.w = wang_hash((x + y) * frame);
  return r;
}

// ---------------------------------------------------------------------------
// color.glsl
PBRT_D float luminance(float3 c) { return dot(c, f3(0.2126f, 0.7152f, 0.0722f)); }
// normalize() of the shading code: the hardware reciprocal square root
// (2 ulp) instead of three correctly rounded divisions; ray generation, the
// surface normal (stored in the G-buffer as angles) and the denoisers keep
// the exact form. The BRDF, sampling and tangent-frame divisions below use
// the hardware reciprocal too (__fdividef); GLSL's own x / y is 2.5 ulp.
PBRT_D float3 nrmz(float3 a) { return a * rsqrtf(dot(a, a)); }
// pow(c, 2.2) with the hardware exp2 / log2 (c >= 0: filtered texel values;
// relative error ~1e-6, GLSL's own pow precision is exp2(y * log2(x))'s)
PBRT_D float3 srgb_to_linear(float3 c) { return f3(__powf(c.x, 2.2f), __powf(c.y, 2.2f), __powf(c.z, 2.2f)); }
PBRT_D float pow5(float x) {  // pow(x, 5.0)
  const float x2 = x * x;
  return x2 * x2 * x;
}
PBRT_D float3 linear_to_srgb(float3 c) {
  const float g = 1.0f / 2.2f;
  return f3(powf(c.x, g), powf(c.y, g), powf(c.z, g));
}
PBRT_D float convert_metallic(float3 diffuse, float3 specular, float max_specular) {
  float pd = sqrtf(0.299f * diffuse.x * diffuse.x + 0.587f * diffuse.y * diffuse.y + 0.114f * diffuse.z * diffuse.z);
  float ps = sqrtf(0.299f * specular.x * specular.x + 0.587f * specular.y * specular.y + 0.114f * specular.z * specular.z);
  if (ps < kMinRoughness) return 0.f;
  float a = kMinRoughness;
  float b = __fdividef(pd * (1.0f - max_specular), 1.0f - kMinRoughness) + ps - 2.0f * kMinRoughness;
  float c = kMinRoughness - ps;
  float D = fmaxf(b * b - 4.0f * a * c, 0.0f);
  return clampf(__fdividef(-b + sqrtf(D), 2.0f * a), 0.0f, 1.0f);
}

// ---------------------------------------------------------------------------
// Surface description (ptStructures.glsl:30-44).
struct SurfaceInfo {
  float perceptual_roughness, metalness, alpha_roughness;
  int illum;
  float3 r0, r90, diffuse, specular, emissive, transmissive, normal;
  float3 basis0, basis1, basis2;  // mat3 columns: T, B, N
  float ior;
};
PBRT_D float3 basis_mul(const SurfaceInfo& s, float3 v) { return s.basis0 * v.x + s.basis1 * v.y + s.basis2 * v.z; }

// brdf.glsl:61-164
PBRT_D float specular_sample_weight(const SurfaceInfo& s) {
  float wd = mixf(luminance(s.diffuse), 0.f, s.metalness);
  float ws = luminance(s.specular);
  return fminf(1.f, __fdividef(ws, wd + wd));
}
PBRT_D float pdf_brdf(const SurfaceInfo& s, float3 v, float3 l, float3 h) {
  float pdf_d = kRecipPI * dot(l, s.normal);
  float a2 = s.alpha_roughness * s.alpha_roughness;
  float nh = dot(h, s.normal);
  float q = nh * nh * (a2 - 1.0f) + 1.0f;
  float pdf_s = __fdividef(a2, kPI * (q * q));
  pdf_s *= nh;
  return mixf(pdf_d, pdf_s, specular_sample_weight(s));
}
PBRT_D float3 brdf_eval(float3 v, float3 l, float3 h, const SurfaceInfo& s) {
  float3 n = s.normal;
  float NdotL = clampf(dot(n, l), 0.001f, 1.0f);
  float NdotV = clampf(fabsf(dot(n, v)), 0.001f, 1.0f);
  float NdotH = clampf(dot(n, h), 0.f, 1.0f);
  float VdotH = clampf(dot(v, h), 0.f, 1.0f);
  // specularReflection (brdf.glsl:88-92)
  float3 F = s.r0 + (s.r90 - s.r90 * s.r0) * exp2f((-5.55473f * VdotH - 6.98316f) * VdotH);
  // geometricOcclusion (brdf.glsl:104-112)
  float r = s.alpha_roughness * s.alpha_roughness;
  float aL = __fdividef(2.0f * NdotL, NdotL + sqrtf(r + (1.0f - r) * (NdotL * NdotL)));
  float aV = __fdividef(2.0f * NdotV, NdotV + sqrtf(r + (1.0f - r) * (NdotV * NdotV)));
  float G = aL * aV;
  // microfacetDistribution (brdf.glsl:125-130)
  float f = (NdotH * r - NdotH) * NdotH + 1.0f;
  float D = __fdividef(r, kPI * f * f);
  // BRDF_Diffuse_Disney (brdf.glsl:61-69)
  float fd90 = 0.5f + 2.0f * s.perceptual_roughness * VdotH * VdotH;
  float dim = 0.9f;  // min over (1 - 0.1) per channel
  float dis = ((1.0f + (fd90 - 1.0f) * pow5(1.0f - NdotL)) * (1.0f + (fd90 - 1.0f) * pow5(1.0f - NdotV))) *
              kRecipPI * dim;
  float3 diffuse_c = (f3(1.f) - F) * (s.diffuse * dis);
  float3 spec = F * (G * D * __fdividef(1.0f, 4.0f * NdotL * NdotV));
  if (dot(n, l) <= 0.f) spec = f3(0.f);
  return diffuse_c + spec;
}

// sampling.glsl:11-27
PBRT_D float3 sample_ggx(float rx, float ry, float alpha2) {
  float phi = 2.f * kPI * rx;
  float cos_h = sqrtf(__fdividef(1.0f - ry, 1.0f + (alpha2 - 1.0f) * ry));
  float sin_h = sqrtf(1.0f - cos_h * cos_h);
  float sp, cp;
  __sincosf(phi, &sp, &cp);  // phi in [0, 2 pi): the hardware sine / cosine
  return f3(sin_h * cp, sin_h * sp, cos_h);
}
PBRT_D float3 sample_hemisphere(float rx, float ry) {
  float t = 2.f * kPI * ry;
  float sr = sqrtf(rx);
  float st, ct;
  __sincosf(t, &st, &ct);
  float dx = sr * ct, dy = sr * st;
  return f3(dx, dy, sqrtf(fmaxf(0.f, 1.0f - dx * dx - dy * dy)));
}

// sampleBRDF (sampling.glsl:29-78). The engine is taken by value in the
// shader: the caller's stream does not advance.
PBRT_D float3 sample_brdf(const SurfaceInfo& s, Rng re, float3 v, float3& l, float& pdf) {
  float ux = rng_next(re), uy = rng_next(re), uz = rng_next(re);
  float sw = specular_sample_weight(s);
  float3 b2 = s.basis2;
  bool entering = dot(v, s.normal) >= 0.f;
  if (s.illum == 7 && !entering) b2 = -b2;
  float3 h;
  if (uz < sw) {
    h = sample_ggx(ux, uy, s.alpha_roughness * s.alpha_roughness);
    h = s.basis0 * h.x + s.basis1 * h.y + b2 * h.z;
    l = -(v - 2.f * dot(h, v) * h);  // -reflect(v, h)
  } else {
    float3 hs = sample_hemisphere(ux, uy);
    l = s.basis0 * hs.x + s.basis1 * hs.y + b2 * hs.z;
    h = nrmz(v + l);
  }
  pdf = pdf_brdf(s, v, l, h);
  float3 brdf = brdf_eval(v, l, h, s);
  if (s.illum == 7) {
    float vh = dot(v, h);
    float fr = 1.f + (0.f - 1.f) * pow5(clampf(1.0f - vh, 0.0f, 1.0f));  // specularReflection(vec3(1), vec3(0), VdotH).x
    if (rng_next(re) < fr || !entering) {
      float t = !entering ? s.ior : 1.f / s.ior;
      float cos_i = dot(b2, l);
      float sin_t2 = t * t * (1.0f - cos_i * cos_i);
      if (sin_t2 <= 1.f) {
        l = l - 2.f * cos_i * b2;
        float cos_t = sqrtf(1.0f - sin_t2);
        l = t * l + (t * cos_i - cos_t) * b2;
      }
      brdf = s.transmissive;
      pdf = 1.f;
    } else {
      pdf = 1.f;
      brdf = f3(1.f);
    }
  }
  return brdf;
}

// lighting.glsl:6-10
PBRT_D float power_heuristic(float a, float b) {
  float f = a * a, g = b * b;
  return __fdividef(f, f + g);
}

// lighting.glsl:233-240
PBRT_D float3 sky_color(float3 dir) {
  float3 upper = srgb_to_linear(f3(0.3f, 0.5f, 0.92f));
  upper = mix3(f3(1.f), upper, fmaxf(dir.z, 0.f));
  float3 lower = f3(0.2f);
  float t = clampf((dir.z - (-0.02f)) / (0.02f - (-0.02f)), 0.f, 1.f);
  float w = t * t * (3.f - 2.f * t);
  return mix3(lower, upper, w);
}

// ---------------------------------------------------------------------------
// Scene access (geometry.glsl, layoutPTGeometry*.glsl).
// The texel pool holds each texture in 4 x 2-texel tiles, one 32-byte
// sector each, tiles in row-major order (texture_tile_index): a bilinear
// footprint touches 1.875 sectors on average instead of 2.25 row-major.
PBRT_HD uint32_t texture_tile_index(uint32_t w, uint32_t x, uint32_t y) {
  return (((y >> 1) * ((w + 3) >> 2) + (x >> 2)) << 3) + ((y & 1u) << 2) + (x & 3u);
}
PBRT_D float4 tex_fetch(const SceneView& sc, const DevTexture& t, int x, int y) {
  uchar4 c = sc.texels[t.offset + texture_tile_index(t.w, (uint32_t)x, (uint32_t)y)];
  return make_float4(u82f(c.x), u82f(c.y), u82f(c.z), u82f(c.w));
}
PBRT_D float4 tex_sample(const SceneView& sc, int tex, float u, float v) {
  const DevTexture t = sc.textures[tex];
  // a constant (1x1) texture: the texel itself (the bilinear weights sum to one)
  if (t.w == 1 && t.h == 1) return tex_fetch(sc, t, 0, 0);
  return bilinear((int)t.w, (int)t.h, u, v, [&](int i, int j) { return tex_fetch(sc, t, i, j); });
}
PBRT_D bool tex_is_1x1(const SceneView& sc, int tex) { return sc.textures[tex].w == 1 && sc.textures[tex].h == 1; }

// unpackIndex (geometry.glsl:4-26)
PBRT_D uint3 unpack_index(const SceneView& sc, uint32_t ibase, uint32_t prim, uint32_t stride) {
  const uint32_t* ind = sc.idx + ibase;
  if (stride == 4) return make_uint3(ind[3 * prim], ind[3 * prim + 1], ind[3 * prim + 2]);
  int full = 3 * (int)prim;
  uint32_t p = (uint32_t)((float)full * .5f);
  uint3 r;
  if (full & 1) {
    r.x = ind[p] >> 16;
    uint32_t t = ind[p + 1];
    r.z = t >> 16;
    r.y = t & 0xffffu;
  } else {
    uint32_t t = ind[p];
    r.y = t >> 16;
    r.x = t & 0xffffu;
    r.z = ind[p + 1] & 0xffffu;
  }
  return r;
}
PBRT_D float3 vload3(const float* pool, uint32_t v) { return f3(pool[3 * v], pool[3 * v + 1], pool[3 * v + 2]); }
PBRT_D float2 vload2(const float* pool, uint32_t v) { return make_float2(pool[2 * v], pool[2 * v + 1]); }

// ptAlphaHit.rahit: keep the candidate unless the diffuse alpha < .01.
PBRT_D bool alpha_accept(const SceneView& sc, uint32_t inst_id, uint32_t prim, float bu, float bv) {
  const DevInstance& inst = sc.instances[inst_id];
  if (inst.opaque) return true;
  const uint32_t vb = inst.vbase;
  uint3 ix = unpack_index(sc, inst.ibase, prim, inst.index_stride);
  float2 t0 = vload2(sc.uv, vb + ix.x), t1 = vload2(sc.uv, vb + ix.y), t2 = vload2(sc.uv, vb + ix.z);
  float b0 = 1.0f - bu - bv;
  float u = t0.x * b0 + t1.x * bu + t2.x * bv;
  float v = t0.y * b0 + t1.y * bu + t2.y * bv;
  float4 d = tex_sample(sc, inst.tex[0], u, v);
  return !(d.w < .01f);
}

// geometry.glsl:59-82
PBRT_D float3 get_tangent(float3 A, float3 B, float3 C, float2 Auv, float2 Buv, float2 Cuv) {
  float bv_cv = Buv.y - Cuv.y;
  if (bv_cv == 0.0f) return (B - C) * __fdividef(1.0f, Buv.x - Cuv.x);
  float q = __fdividef(Auv.y - Cuv.y, bv_cv);
  float3 D = C + (B - C) * q;
  float2 Duv = make_float2(Cuv.x + (Buv.x - Cuv.x) * q, Cuv.y + (Buv.y - Cuv.y) * q);
  return (D - A) * __fdividef(1.0f, Duv.x - Auv.x);
}
PBRT_D float3 project(float3 a, float3 b) { return __fdividef(dot(a, b), dot(b, b)) * b; }

// ptClosesthit.rchit:18-92 (plus the payload written by ptMiss.rmiss for
// misses). Returns the hit position; fills si and the material category.
PBRT_D float3 closest_hit(const SceneView& sc, float3 ray_dir, uint32_t inst_id, uint32_t prim, float bu, float bv,
                          SurfaceInfo& si, uint32_t& category) {
  const float eps = 1e-6f;
  const DevInstance& inst = sc.instances[inst_id];
  const int obj = inst.mesh;
  const uint32_t vb = inst.vbase;
  const int32_t* mtex = inst.tex;
  uint3 ix = unpack_index(sc, inst.ibase, prim, inst.index_stride);
  float3 p0 = vload3(sc.pos, vb + ix.x), p1 = vload3(sc.pos, vb + ix.y), p2 = vload3(sc.pos, vb + ix.z);
  float3 n0 = vload3(sc.nor, vb + ix.x), n1 = vload3(sc.nor, vb + ix.y), n2 = vload3(sc.nor, vb + ix.z);
  float2 t0 = vload2(sc.uv, vb + ix.x), t1 = vload2(sc.uv, vb + ix.y), t2 = vload2(sc.uv, vb + ix.z);
  const float b0 = 1.0f - bu - bv, b1 = bu, b2 = bv;
  float2 tc = make_float2(t0.x * b0 + t1.x * b1 + t2.x * b2, t0.y * b0 + t1.y * b1 + t2.y * b2);
  float4 dm = tex_sample(sc, mtex[0], tc.x, tc.y);
  float3 diffuse = srgb_to_linear(f3(dm.x, dm.y, dm.z));
  float diffuse_a = dm.w;
  diffuse = diffuse * diffuse_a;
  // unfused: the next rays start from this point and the G-buffer stores its distance
  const float3 position = mul_point_rn(inst.obj, add_rn(add_rn(mul_rn(p0, b0), mul_rn(p1, b1)), mul_rn(p2, b2)));
  // unfused, in the shader's order: the G-buffer stores this normal
  float3 normal = normalize_rn(add_rn(add_rn(mul_rn(n0, b0), mul_rn(n1, b1)), mul_rn(n2, b2)));
  if (isinf(normal.x) || isnan(normal.x)) normal = f3(0.f, 1.f, 0.f);
  const float3 c0 = f3(inst.nrm[0].x, inst.nrm[0].y, inst.nrm[0].z);
  const float3 c1 = f3(inst.nrm[1].x, inst.nrm[1].y, inst.nrm[1].z);
  const float3 c2 = f3(inst.nrm[2].x, inst.nrm[2].y, inst.nrm[2].z);
  normal = normalize_rn(add_rn(add_rn(mul_rn(c0, normal.x), mul_rn(c1, normal.y)), mul_rn(c2, normal.z)));
  if (t0.x == t1.x && t0.y == t1.y) t1.x += eps;
  if (t0.x == t2.x && t0.y == t2.y) t2.y += eps;
  if (t1.x == t2.x && t1.y == t2.y) {
    t2.x += eps;
    t2.y += eps;
  }
  float3 tg = get_tangent(p0, p1, p2, t0, t1, t2);
  float3 T = c0 * tg.x + c1 * tg.y + c2 * tg.z;
  float3 bt = get_tangent(p0, p2, p1, make_float2(t0.y, t0.x), make_float2(t2.y, t2.x), make_float2(t1.y, t1.x));
  float3 B = c0 * bt.x + c1 * bt.y + c2 * bt.z;
  // gramSchmidt (geometry.glsl:78-82)
  float3 tt = T - project(T, normal);
  float3 bb = B - project(B, tt) - project(B, normal);
  si.basis0 = nrmz(tt);
  si.basis1 = nrmz(bb);
  si.basis2 = normal;
  // getNormal (geometry.glsl:84-92)
  if (!tex_is_1x1(sc, mtex[2])) {
    float4 nm = tex_sample(sc, mtex[2], tc.x, tc.y);
    float3 tn = f3(nm.x * 2.0f - 1.0f, nm.y * 2.0f - 1.0f, nm.z * 2.0f - 1.0f);
    normal = normalize(si.basis0 * tn.x + si.basis1 * tn.y + si.basis2 * tn.z);
  }
  const DevMaterial mat = sc.materials[obj];
  diffuse = diffuse * f3(mat.diffuse_ior.x, mat.diffuse_ior.y, mat.diffuse_ior.z);
  float3 spec;
  float pr;
  if (tex_is_1x1(sc, mtex[4])) {
    spec = f3(mat.specular_dissolve.x, mat.specular_dissolve.y, mat.specular_dissolve.z);
    pr = mat.ambient_roughness.w;
  } else {
    float4 sm = tex_sample(sc, mtex[4], tc.x, tc.y);
    spec = srgb_to_linear(f3(sm.x, sm.y, sm.z));
    pr = sm.w;
  }
  float max_spec = fmaxf(fmaxf(spec.x, spec.y), spec.z);
  float metallic = convert_metallic(diffuse, spec, max_spec);
  float3 bc_diff = diffuse * __fdividef(__fdividef(1.0f - max_spec, 1 - kMinRoughness), fmaxf(1 - metallic, eps));
  float3 bc_spec = spec - (f3(kMinRoughness) * (1 - metallic) * __fdividef(1.0f, fmaxf(metallic, eps)));
  float3 base = mix3(bc_diff, bc_spec, metallic * metallic);
  float3 dcol = base * (f3(1.0f) - f3(0.04f));
  dcol = dcol * (1.0f - metallic);
  float3 scol = mix3(f3(0.04f), base, metallic);
  float refl = fmaxf(fmaxf(scol.x, scol.y), scol.z);
  float r90 = clampf(refl * 25.f, 0.f, 1.f);
  float3 v = nrmz(-ray_dir);
  float4 em = tex_sample(sc, mtex[3], tc.x, tc.y);
  float3 emissive = f3(mat.emission_texture_id.x, mat.emission_texture_id.y, mat.emission_texture_id.z) *
                    srgb_to_linear(f3(em.x, em.y, em.z));
  if (dot(v, normal) < 0.f) emissive = f3(0.f);
  si.perceptual_roughness = pr;
  si.metalness = metallic;
  si.alpha_roughness = pr * pr;
  si.illum = (int)mat.transmittance_illum.w;
  si.r0 = scol;
  si.r90 = f3(1.f) * r90;
  si.diffuse = dcol;
  si.specular = scol;
  si.emissive = emissive;
  si.transmissive = f3(mat.transmittance_illum.x, mat.transmittance_illum.y, mat.transmittance_illum.z);
  si.normal = normal;
  si.ior = mat.diffuse_ior.w;
  category = mat.category_id;
  return position;
}

// ptMiss.rmiss:7-25
PBRT_D void miss_payload(SurfaceInfo& si, float3& position, uint32_t& category) {
  position = f3(1.0e10f);
  category = 0xffffffffu;
  si.normal = f3(1.f);
  si.emissive = si.diffuse = si.specular = si.r0 = si.r90 = si.transmissive = f3(0.f);
  si.perceptual_roughness = si.metalness = si.alpha_roughness = 0.f;
  si.illum = 0;
  si.basis0 = si.basis1 = si.basis2 = f3(0.f);
  si.ior = 1.f;
}

}  // namespace pbrt
