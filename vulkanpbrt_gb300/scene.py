"""Seeded procedural scenes in the reference's scene data model.

What RayTracingSceneDescriptorCreationVisitor hands the shaders
(source/scene/RayTracingVisitor.{hpp,cpp}), produced directly:

* meshes: non-interleaved positions / normals / uvs and u16 or u32 indices
  (RayTracingVisitor.cpp:29-168; u16 indices are read as packed uint pairs,
  shaders/geometry.glsl:4-26);
* ObjectInstance {mat4 object_mat; int mesh_id; uint index_stride; pad}
  per instance (RayTracingVisitor.hpp:37-43), plus the per-instance
  opacity flag (diffuse alpha < 0.01 anywhere, RayTracingVisitor.cpp:319-343);
* WaveFrontMaterialPacked per mesh (RayTracingVisitor.hpp:44-53);
* PackedLight list (external/vsg/include/vsg/nodes/Light.h:23-37): every
  triangle of an emissive mesh is an area light with strengths (0,0,1) and
  ambient = diffuse = specular = emission (RayTracingVisitor.cpp:170-221);
  point lights are added directly (the visitor never collects them);
  inclusive strengths are prefix sums (RayTracingVisitor.cpp:428-441);
* five texture slots per mesh (diffuse, mr, normal, emissive, specular),
  slot 0 of the texture table being the 1x1 white default
  (RayTracingVisitor.cpp:3-15, 376-405).

Materials follow the metallic-roughness mapping: dielectric -> diffuse =
albedo, specular = 0; metal -> diffuse = 0, specular = albedo; roughness in
ambient_roughness.w (or the specular map's alpha).
"""
from __future__ import annotations

import concurrent.futures
import math
import os
from dataclasses import dataclass, field

import numpy as np

# texture slots per mesh (layoutPTGeometryImages.glsl bindings 6, 7, 8, 10, 11)
SLOT_DIFFUSE, SLOT_MR, SLOT_NORMAL, SLOT_EMISSIVE, SLOT_SPECULAR = range(5)
LIGHT_DIRECTIONAL, LIGHT_POINT, LIGHT_AREA = 1, 2, 5


@dataclass
class Mesh:
    positions: np.ndarray  # [nv, 3] f32
    normals: np.ndarray  # [nv, 3] f32
    uvs: np.ndarray  # [nv, 2] f32
    indices: np.ndarray  # [ni] u16 or u32

    @property
    def index_stride(self) -> int:
        return self.indices.dtype.itemsize

    @property
    def tri_count(self) -> int:
        return len(self.indices) // 3


@dataclass
class Scene:
    meshes: list = field(default_factory=list)
    instance_mats: list = field(default_factory=list)  # [4,4] float64, m[row, col]
    instance_mesh: list = field(default_factory=list)
    materials: list = field(default_factory=list)  # per mesh: np.float32[24] (96 B)
    textures: list = field(default_factory=list)  # uint8 [h, w, 4]
    mesh_textures: list = field(default_factory=list)  # per mesh: 5 texture ids
    lights: list = field(default_factory=list)  # np.float32[32] (128 B)
    camera_eye: tuple = (0.0, -3.0, 1.0)
    camera_center: tuple = (0.0, 0.0, 1.0)

    def __post_init__(self):
        if not self.textures:
            self.textures.append(np.full((1, 1, 4), 255, np.uint8))  # the 1x1 white default

    @property
    def tri_count(self) -> int:
        return sum(self.meshes[m].tri_count for m in self.instance_mesh)

    def add_mesh(self, mesh: Mesh, material: np.ndarray, textures=None) -> int:
        self.meshes.append(mesh)
        self.materials.append(np.asarray(material, np.float32))
        t = [0, 0, 0, 0, 0] if textures is None else list(textures)
        self.mesh_textures.append(t)
        return len(self.meshes) - 1

    def add_texture(self, rgba: np.ndarray) -> int:
        self.textures.append(np.ascontiguousarray(rgba, np.uint8))
        return len(self.textures) - 1

    def add_instance(self, mesh_id: int, mat: np.ndarray) -> int:
        self.instance_mesh.append(mesh_id)
        self.instance_mats.append(np.asarray(mat, np.float64))
        return len(self.instance_mesh) - 1

    def instance_opaque(self) -> np.ndarray:
        """RayTracingVisitor.cpp:319-343: non-opaque if any diffuse texel alpha < .01 * 255."""
        tex_opaque = [bool((t[..., 3] >= 0.01 * 255).all()) for t in self.textures]
        return np.array([tex_opaque[self.mesh_textures[m][SLOT_DIFFUSE]] for m in self.instance_mesh], bool)

    def add_emissive_lights(self, mesh_id: int, inst_mat: np.ndarray, emission) -> None:
        """One area light per triangle of an emissive mesh (RayTracingVisitor.cpp:170-221)."""
        m = self.meshes[mesh_id]
        idx = m.indices.astype(np.int64).reshape(-1, 3)
        for tri in idx:
            vs = []
            for k in tri:
                p = inst_mat @ np.append(m.positions[k].astype(np.float64), 1.0)
                vs.append(p[:3].astype(np.float32))
            self.lights.append(packed_light(LIGHT_AREA, vs[0], vs[1], vs[2], emission, (0.0, 0.0, 1.0)))

    def finalize_lights(self) -> None:
        """Inclusive strength prefix sums (RayTracingVisitor.cpp:428-441),
        after adding the default directional light to a scene without
        lights (RayTracingVisitor.cpp:409-423)."""
        if not self.lights:
            from .scene_import import default_light

            self.lights.append(default_light())
        acc = np.float32(0)
        for l in self.lights:
            s = np.float32(0)
            for c in (l[16:19], l[20:23], l[24:27]):
                for v in c:
                    s = np.float32(s + v)
            acc = np.float32(acc + s)
            l[31] = acc


def material(diffuse=(1, 1, 1), specular=(0, 0, 0), roughness=1.0, emission=(0, 0, 0), ior=1.0, dissolve=1.0,
             transmittance=(1, 1, 1), illum=0, alpha_cutoff=0.5, category=0) -> np.ndarray:
    """WaveFrontMaterialPacked (ptStructures.glsl:18-27): 24 floats."""
    m = np.zeros(24, np.float32)
    m[0:3] = diffuse  # ambient (unused by the shaders); keep = diffuse like PbrMaterial.baseColorFactor
    m[3] = roughness
    m[4:7] = diffuse
    m[7] = ior
    m[8:11] = specular
    m[11] = dissolve
    m[12:15] = transmittance
    m[15] = illum
    m[16:19] = emission
    m[19] = alpha_cutoff
    m[20:21] = np.array([category], np.uint32).view(np.float32)
    return m


def packed_light(kind, v0, v1=(0, 0, 0), v2=(0, 0, 0), color=(1, 1, 1), strengths=(0, 0, 1), direction=(0, 0, -1),
                 radius=0.0) -> np.ndarray:
    """vsg::Light::PackedLight (Light.h:23-37) with colour in ambient, diffuse and specular."""
    l = np.zeros(32, np.float32)
    l[0:3] = v0
    l[3] = kind
    l[4:7] = v1
    l[7] = radius
    l[8:11] = v2
    l[12:15] = direction
    l[16:19] = color
    l[20:23] = color
    l[24:27] = color
    l[28:31] = strengths
    return l


# ----------------------------------------------------------------------------
# geometry


def icosphere(subdivisions: int):
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
             (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
             (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
             (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        cache = {}

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    return np.array(verts), np.array(faces, np.int64)


def sphere_uv(p: np.ndarray) -> np.ndarray:
    u = np.arctan2(p[:, 1], p[:, 0]) / (2 * math.pi) + 0.5
    v = np.arccos(np.clip(p[:, 2], -1, 1)) / math.pi
    return np.stack([u, v], -1)


def _vertex_normals(pos: np.ndarray, faces: np.ndarray) -> np.ndarray:
    fn = np.cross(pos[faces[:, 1]] - pos[faces[:, 0]], pos[faces[:, 2]] - pos[faces[:, 0]])
    n = np.zeros_like(pos)
    for k in range(3):
        np.add.at(n, faces[:, k], fn)
    return n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-12)


def _indices(faces: np.ndarray, nv: int) -> np.ndarray:
    flat = faces.reshape(-1)
    return flat.astype(np.uint16 if nv < 65536 else np.uint32)


def make_icosphere(subdiv: int, displace=None) -> Mesh:
    v, f = icosphere(subdiv)
    pos = v * (1.0 + displace(v))[:, None] if displace is not None else v
    nor = _vertex_normals(pos, f) if displace is not None else v
    return Mesh(pos.astype(np.float32), nor.astype(np.float32), sphere_uv(v).astype(np.float32), _indices(f, len(v)))


def make_quad_grid(origin, du, dv, n: int, normal) -> tuple:
    o, du, dv = (np.asarray(x, np.float64) for x in (origin, du, dv))
    g = np.linspace(0, 1, n + 1)
    uu, vv = np.meshgrid(g, g, indexing="xy")
    pos = o + uu.reshape(-1, 1) * du + vv.reshape(-1, 1) * dv
    uv = np.stack([uu.reshape(-1), vv.reshape(-1)], -1)
    faces = []
    for j in range(n):
        for i in range(n):
            a = j * (n + 1) + i
            b, c, d = a + 1, a + n + 2, a + n + 1
            faces += [(a, b, c), (a, c, d)]
    nor = np.tile(np.asarray(normal, np.float64), (len(pos), 1))
    return pos, nor, uv, np.array(faces, np.int64)


def merge(parts) -> Mesh:
    P, N, U, F = [], [], [], []
    off = 0
    for pos, nor, uv, faces in parts:
        P.append(pos), N.append(nor), U.append(uv), F.append(faces + off)
        off += len(pos)
    pos = np.concatenate(P)
    return Mesh(pos.astype(np.float32), np.concatenate(N).astype(np.float32), np.concatenate(U).astype(np.float32),
                _indices(np.concatenate(F), len(pos)))


def make_box(n: int) -> Mesh:
    """Unit cube [-1,1]^3, n x n quads per face, outward normals."""
    parts = []
    for axis in range(3):
        for sgn in (-1.0, 1.0):
            nrm = np.zeros(3)
            nrm[axis] = sgn
            a1, a2 = (axis + 1) % 3, (axis + 2) % 3
            du, dv = np.zeros(3), np.zeros(3)
            du[a1], dv[a2] = 2.0, 2.0
            if sgn < 0:
                du, dv = dv, du
            origin = nrm - du / 2 - dv / 2
            parts.append(make_quad_grid(origin, du, dv, n, nrm))
    return merge(parts)


def translate_scale(t, s) -> np.ndarray:
    m = np.eye(4)
    m[:3, :3] *= s
    m[:3, 3] = t
    return m


def rot_z(a: float) -> np.ndarray:
    m = np.eye(4)
    c, s = math.cos(a), math.sin(a)
    m[0, 0], m[0, 1], m[1, 0], m[1, 1] = c, -s, s, c
    return m


# ----------------------------------------------------------------------------
# scenes


def cornell_spheres(seed: int = 0, spheres: int = 8, subdiv: int = 3, light_radiance: float = 20.0) -> Scene:
    """Small workload: Cornell-style box of 12 quads (24 tris), `spheres`
    icospheres of 1280 tris each with radius U[.1,.3], one 0.2 x 0.2 area light
    of radiance 20; albedo U[0,1]^3, roughness U[.05,1], metallic Bernoulli(.3)."""
    rng = np.random.default_rng(seed)
    sc = Scene()
    x0, x1, y0, y1, z0, z1 = -1.6, 1.6, -3.6, 1.6, 0.0, 2.6

    def wall(origin, du, dv, normal):
        return make_quad_grid(origin, du, dv, 1, normal)

    # each face split into two quads: 12 quads
    def split(origin, du, dv, normal):
        o, du, dv = (np.asarray(x, np.float64) for x in (origin, du, dv))
        return [wall(o, du / 2, dv, normal), wall(o + du / 2, du / 2, dv, normal)]

    white = split((x0, y0, z0), (x1 - x0, 0, 0), (0, y1 - y0, 0), (0, 0, 1))  # floor
    white += split((x0, y1, z1), (x1 - x0, 0, 0), (0, y0 - y1, 0), (0, 0, -1))  # ceiling
    white += split((x0, y1, z0), (x1 - x0, 0, 0), (0, 0, z1 - z0), (0, -1, 0))  # back
    white += split((x1, y0, z0), (x0 - x1, 0, 0), (0, 0, z1 - z0), (0, 1, 0))  # front (behind the camera)
    red = split((x0, y0, z0), (0, y1 - y0, 0), (0, 0, z1 - z0), (1, 0, 0))
    green = split((x1, y1, z0), (0, y0 - y1, 0), (0, 0, z1 - z0), (-1, 0, 0))
    eye = np.eye(4)
    for parts, col in ((white, (0.73, 0.73, 0.73)), (red, (0.63, 0.065, 0.05)), (green, (0.14, 0.45, 0.091))):
        mid = sc.add_mesh(merge(parts), material(diffuse=col, roughness=1.0))
        sc.add_instance(mid, eye)
    # spheres
    for _ in range(spheres):
        r = rng.uniform(0.1, 0.3)
        c = (rng.uniform(x0 + 0.4, x1 - 0.4), rng.uniform(-0.8, y1 - 0.4), rng.uniform(r, 1.8))
        albedo = rng.uniform(0, 1, 3)
        rough = rng.uniform(0.05, 1.0)
        metal = rng.random() < 0.3
        mat = material(diffuse=(0, 0, 0) if metal else albedo, specular=albedo if metal else (0, 0, 0), roughness=rough)
        mid = sc.add_mesh(make_icosphere(subdiv), mat)
        sc.add_instance(mid, translate_scale(c, r))
    # area light: 0.2 x 0.2 quad just below the ceiling, facing down
    half = 0.1
    lp, lnrm, luv, lf = make_quad_grid((-half, 0.1 + half, z1 - 0.01), (2 * half, 0, 0), (0, -2 * half, 0), 1, (0, 0, -1))
    lmesh = Mesh(lp.astype(np.float32), lnrm.astype(np.float32), luv.astype(np.float32), _indices(lf, len(lp)))
    e = (light_radiance,) * 3
    lid = sc.add_mesh(lmesh, material(diffuse=(0, 0, 0), roughness=1.0, emission=e))
    sc.add_instance(lid, eye)
    sc.add_emissive_lights(lid, eye, e)
    sc.finalize_lights()
    return sc


def instanced_field(seed: int = 0, instances: int = 2000, unique_meshes: int = 64, sphere_fraction: float = 20 / 64,
                    sphere_subdiv: int = 3, box_n: int = 4, texture_size: int = 1024, alpha_fraction: float = 0.05,
                    point_lights: int = 8, radius: float = 40.0, synth=None) -> Scene:
    """Full-size workload: `instances` instances (scale log-U[.05,2]) of seeded
    displaced icospheres and boxes on a ground plane (~1M triangles at the
    defaults), per-mesh texture_size^2 RGBA8 value-noise albedo / specular-
    roughness / normal maps, `alpha_fraction` of meshes alpha-masked,
    `point_lights` point lights and one area light."""
    rng = np.random.default_rng(seed)
    sc = Scene(camera_eye=(0.0, -radius * 0.6, radius * 0.2), camera_center=(0.0, 0.0, 1.0))
    if synth is None:
        from .texsynth import synth_texture as synth
    # textures are generated on a thread pool (numpy releases the GIL in its
    # array passes); ids are assigned in submission order
    pool = concurrent.futures.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1))
    jobs = []
    base = len(sc.textures)  # the 1x1 white default comes first

    def texture(*args) -> int:
        jobs.append(pool.submit(synth, *args))
        return base + len(jobs) - 1

    def textures(mesh_seed: int, albedo, metal: bool, alpha: bool, rough_lo: float, rough_hi: float):
        d = texture(mesh_seed, texture_size, "albedo", tuple(0 if metal else a for a in albedo), alpha)
        s = texture(mesh_seed + 1, texture_size, "specular", tuple(albedo if metal else (0, 0, 0)), False,
                    rough_lo, rough_hi)
        n = texture(mesh_seed + 2, texture_size, "normal", (0, 0, 0), False)
        return [d, 0, n, 0, s]

    # ground plane (u32 indices: exercises the full-index path)
    gp, gn, gu, gf = make_quad_grid((-radius * 3, -radius * 3, 0.0), (radius * 6, 0, 0), (0, radius * 6, 0), 4, (0, 0, 1))
    ground = Mesh(gp.astype(np.float32), gn.astype(np.float32), (gu * 24).astype(np.float32), gf.reshape(-1).astype(np.uint32))
    gid = sc.add_mesh(ground, material(diffuse=(1, 1, 1), roughness=1.0),
                      textures(seed * 1000 + 1, (0.5, 0.5, 0.45), False, False, 0.4, 0.9))
    sc.add_instance(gid, np.eye(4))
    # unique meshes
    n_sph = int(round(unique_meshes * sphere_fraction))
    mesh_ids, mesh_is_sphere = [], []
    for k in range(unique_meshes):
        sphere = k < n_sph
        if sphere:
            waves = [(rng.normal(0, 1, 3), rng.uniform(2, 6), rng.uniform(0, 6.28)) for _ in range(4)]
            amp = rng.uniform(0.05, 0.2)

            def disp(v, waves=waves, amp=amp):
                return amp * sum(np.sin(f * (v @ (d / np.linalg.norm(d))) + ph) for d, f, ph in waves) / len(waves)

            mesh = make_icosphere(sphere_subdiv, disp)
        else:
            mesh = make_box(box_n)
        albedo = rng.uniform(0.05, 0.95, 3)
        metal = rng.random() < 0.3
        alpha = rng.random() < alpha_fraction
        rlo = rng.uniform(0.05, 0.5)
        mat = material(diffuse=(1, 1, 1), specular=(0, 0, 0), roughness=rlo)
        mid = sc.add_mesh(mesh, mat, textures(seed * 1000 + 10 * k + 11, albedo, metal, alpha, rlo, min(1.0, rlo + 0.5)))
        mesh_ids.append(mid)
        mesh_is_sphere.append(sphere)
    # instances
    for _ in range(instances):
        k = int(rng.integers(0, unique_meshes))
        s = math.exp(rng.uniform(math.log(0.05), math.log(2.0)))
        rr = radius * math.sqrt(rng.random())
        a = rng.uniform(0, 2 * math.pi)
        pos = (rr * math.cos(a), rr * math.sin(a), s * rng.uniform(1.0, 1.6))
        m = translate_scale(pos, s) @ rot_z(rng.uniform(0, 2 * math.pi))
        sc.add_instance(mesh_ids[k], m)
    # lights: point lights above the field, one area light quad
    for _ in range(point_lights):
        p = (rng.uniform(-radius, radius) * 0.6, rng.uniform(-radius, radius) * 0.6, rng.uniform(6.0, 14.0))
        col = rng.uniform(30.0, 80.0) * np.array([1.0, rng.uniform(0.8, 1.0), rng.uniform(0.6, 1.0)])
        sc.lights.append(packed_light(LIGHT_POINT, p, color=col, strengths=(1.0, 0.0, 1.0)))
    ah = 2.0
    lp, lnrm, luv, lf = make_quad_grid((-ah, ah, 18.0), (2 * ah, 0, 0), (0, -2 * ah, 0), 1, (0, 0, -1))
    lmesh = Mesh(lp.astype(np.float32), lnrm.astype(np.float32), luv.astype(np.float32), _indices(lf, len(lp)))
    e = (60.0, 58.0, 55.0)
    lid = sc.add_mesh(lmesh, material(diffuse=(0, 0, 0), roughness=1.0, emission=e))
    sc.add_instance(lid, np.eye(4))
    sc.add_emissive_lights(lid, np.eye(4), e)
    sc.finalize_lights()
    assert len(sc.textures) == base, "texture ids are assigned in submission order"
    for j in jobs:
        sc.add_texture(j.result())
    pool.shutdown()
    return sc
