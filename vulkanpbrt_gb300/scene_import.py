"""Scene ingestion: what RayTracingSceneDescriptorCreationVisitor
(source/scene/RayTracingVisitor.cpp) does to the meshes, materials and
lights of a loaded scene graph, and a Wavefront OBJ/MTL loader that
produces the scene data model the way the reference's assimp path presents
an OBJ file to that visitor.

Visitor rules (`prepare_mesh`, `phong_material`, `pbr_material`,
`default_light`):
* a mesh whose first normal is zero gets area-weighted vertex normals
  (RayTracingVisitor.cpp:52-127; native, `pbrt_mesh_generate_normals`);
* a mesh without texture coordinates gets (0,0), (0,1), (1,0) per triangle
  corner (RayTracingVisitor.cpp:133-166; `pbrt_mesh_fill_uvs`);
* Phong materials: roughness = sqrt(2 / (shininess + 2)), illum 7 when the
  transmissive colour is not (1,1,1) (RayTracingVisitor.cpp:280-304); PBR
  materials as RayTracingVisitor.cpp:250-279;
* an emissive material (r + g + b != 0) makes every triangle of its meshes
  an area light (RayTracingVisitor.cpp:170-221; `Scene.add_emissive_lights`);
* a scene without lights gets one directional light
  (RayTracingVisitor.cpp:409-423; `Scene.finalize_lights`).

OBJ/MTL (`load_obj`), as vsgXchange's assimp reader hands it on
(external/vsgXchange/src/assimp/assimp.cpp:316, 400-470, 640-700): one mesh
per (object, material) run of faces; polygons fan-triangulated; one vertex
per face corner (no sharing, so generated normals are per face); missing
normals zero (then generated as above), missing texture coordinates zero;
v flipped (aiProcess_FlipUVs); uint16 indices below 65535 indices, else
uint32; Phong materials from Ka / Kd / Ks / Ke / Ns / Ni / Tf with
shininess < 0.01 clearing the specular colour; map_Kd -> diffuse, norm ->
normal, map_Ke -> emissive, map_Ks -> specular textures (PNG or PPM;
decoded here, forced to RGBA8). Triangle order is the file's (the
reference's cache-locality reordering changes only the order of equal
work).
"""
from __future__ import annotations

import ctypes as C
import os
import struct
import zlib
from typing import Dict, Optional

import numpy as np

from ._abi import check, lib
from .scene import LIGHT_DIRECTIONAL, SLOT_DIFFUSE, SLOT_EMISSIVE, SLOT_NORMAL, SLOT_SPECULAR, Mesh, Scene


def _p(a: np.ndarray) -> C.c_void_p:
    return a.ctypes.data_as(C.c_void_p)


def generate_normals(positions: np.ndarray, indices: np.ndarray, initial: Optional[np.ndarray] = None) -> np.ndarray:
    """Accumulates onto `initial` (the mesh's own normal array, as the
    visitor does; zeros when None): every referenced vertex is overwritten
    at its first triangle, unreferenced ones keep their value."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices)
    nor = np.zeros_like(pos) if initial is None else np.array(initial, np.float32).reshape(-1, 3)
    if nor.shape != pos.shape:
        raise ValueError("normals and positions differ in count")
    check(lib().pbrt_mesh_generate_normals(_p(pos), len(pos), _p(idx), len(idx), idx.dtype.itemsize, _p(nor)))
    return nor


def fill_uvs(vertex_count: int, indices: np.ndarray) -> np.ndarray:
    idx = np.ascontiguousarray(indices)
    uv = np.zeros((vertex_count, 2), np.float32)
    check(lib().pbrt_mesh_fill_uvs(vertex_count, _p(idx), len(idx), idx.dtype.itemsize, _p(uv)))
    return uv


def prepare_mesh(positions, normals, uvs, indices) -> Mesh:
    """A Mesh as the visitor hands it on: normals generated when the first
    one is zero (or none are given), uvs filled when none are given."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    idx = np.ascontiguousarray(indices)
    if idx.dtype not in (np.uint16, np.uint32):
        idx = idx.astype(np.uint16 if len(idx) < 65535 else np.uint32)
    nor = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    if nor is None or len(nor) == 0:
        nor = generate_normals(pos, idx)
    elif float(nor[0] @ nor[0]) == 0.0:  # length2(first normal) == 0
        nor = generate_normals(pos, idx, nor)
    uv = None if uvs is None else np.ascontiguousarray(uvs, np.float32).reshape(-1, 2)
    if uv is None or len(uv) == 0:
        uv = fill_uvs(len(pos), idx)
    return Mesh(pos, nor, uv, idx)


def _packed(ambient_roughness, diffuse_ior, specular_dissolve, transmittance_illum, emission_w, category) -> np.ndarray:
    m = np.zeros(24, np.float32)
    m[0:4] = ambient_roughness
    m[4:8] = diffuse_ior
    m[8:12] = specular_dissolve
    m[12:16] = transmittance_illum
    m[16:20] = emission_w
    m[20:21] = np.array([category], np.uint32).view(np.float32)
    return m


def phong_material(ambient=(0, 0, 0, 1), diffuse=(1, 1, 1, 1), specular=(0, 0, 0, 1), emissive=(0, 0, 0, 1),
                   transmissive=(1, 1, 1), shininess=0.0, alpha_mask=1.0, alpha_mask_cutoff=0.5,
                   index_of_refraction=1.0, category_id=0) -> np.ndarray:
    """WaveFrontMaterialPacked of a vsg::PhongMaterial (RayTracingVisitor.cpp:280-304)."""
    f = np.float32
    rough = np.sqrt(f(2) / (f(shininess) + f(2)))
    illum = 7.0 if tuple(np.float32(transmissive)) != (1.0, 1.0, 1.0) else 0.0
    return _packed((*ambient[:3], rough), (*diffuse[:3], index_of_refraction), (*specular[:3], alpha_mask),
                   (*transmissive[:3], illum), (*emissive[:3], alpha_mask_cutoff), category_id)


def pbr_material(base_color=(1, 1, 1, 1), emissive=(0, 0, 0, 1), diffuse=(1, 1, 1, 1), specular=(0, 0, 0, 1),
                 transmission=(1, 1, 1), metallic=1.0, roughness=1.0, alpha_mask=1.0, alpha_mask_cutoff=0.5,
                 index_of_refraction=1.0, category_id=0) -> np.ndarray:
    """WaveFrontMaterialPacked of a vsg::PbrMaterial (RayTracingVisitor.cpp:250-279;
    the metallic factor is not carried)."""
    illum = 7.0 if tuple(np.float32(transmission)) != (1.0, 1.0, 1.0) else 0.0
    return _packed((*base_color[:3], roughness), (*diffuse[:3], index_of_refraction), (*specular[:3], alpha_mask),
                   (*transmission[:3], illum), (*emissive[:3], alpha_mask_cutoff), category_id)


def is_emissive(material: np.ndarray) -> bool:
    m = np.asarray(material, np.float32)
    return bool(np.float32(np.float32(m[16] + m[17]) + m[18]) != 0)


def default_light() -> np.ndarray:
    """The directional light added to a scene without lights
    (RayTracingVisitor.cpp:412-422): ambient = diffuse = (2,2,2), specular 0,
    strengths (.5, 0, 0), direction normalize(0.1, 1, -5.1)."""
    d = np.array([0.1, 1.0, -5.1], np.float32)
    n = np.float32(np.sqrt(np.float32(np.float32(d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])))
    d = d * (np.float32(1) / n)
    l = np.zeros(32, np.float32)
    l[3] = LIGHT_DIRECTIONAL
    l[12:15] = d
    l[16:19] = 2.0
    l[20:23] = 2.0
    l[28:31] = (0.5, 0.0, 0.0)
    return l


# ---- images ------------------------------------------------------------------
def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def load_png(path) -> np.ndarray:
    """8- and 16-bit, non-interlaced PNG (grey, grey+alpha, RGB, RGBA,
    palette) -> RGBA8 [h, w, 4] (16-bit samples keep their high byte)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, plte, trns = 8, [], None, None
    w = h = depth = ctype = None
    while pos < len(data):
        n, typ = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if typ == b"IHDR":
            w, h, depth, ctype, _c, _f, interlace = struct.unpack(">IIBBBBB", body)
            if interlace:
                raise ValueError(f"{path}: interlaced PNG is not supported")
            if depth not in (8, 16) or ctype not in (0, 2, 3, 4, 6) or (ctype == 3 and depth != 8):
                raise ValueError(f"{path}: PNG bit depth {depth} / colour type {ctype} is not supported")
        elif typ == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif typ == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif typ == b"IDAT":
            idat.append(body)
        elif typ == b"IEND":
            break
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bpp = ch * depth // 8
    raw = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8)
    stride = w * bpp
    out = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        ft = raw[y * (stride + 1)]
        line = raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)].astype(np.int32)
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 0xFF
        elif ft == 1:
            cur = line.reshape(w, bpp).cumsum(0).reshape(-1) & 0xFF
        else:
            cur = line.copy()
            for i in range(stride):
                a = int(cur[i - bpp]) if i >= bpp else 0
                if ft == 3:
                    cur[i] = (cur[i] + ((a + int(prev[i])) >> 1)) & 0xFF
                elif ft == 4:
                    c = int(prev[i - bpp]) if i >= bpp else 0
                    cur[i] = (cur[i] + _paeth(a, int(prev[i]), c)) & 0xFF
                else:
                    raise ValueError(f"{path}: PNG filter {ft}")
        out[y] = cur
        prev = cur
    px = out.astype(np.uint8).reshape(h, w, ch * depth // 8)
    if depth == 16:
        px = px[..., 0::2]
    if ctype == 3:
        rgb = plte[px[..., 0]]
        alpha = np.full((h, w, 1), 255, np.uint8)
        if trns is not None:
            t = np.full(len(plte), 255, np.uint8)
            t[:len(trns)] = trns[:len(plte)]
            alpha = t[px[..., 0]][..., None]
        return np.concatenate([rgb, alpha], -1)
    if ch == 1:
        return np.concatenate([np.repeat(px, 3, -1), np.full((h, w, 1), 255, np.uint8)], -1)
    if ch == 2:
        return np.concatenate([np.repeat(px[..., :1], 3, -1), px[..., 1:2]], -1)
    if ch == 3:
        return np.concatenate([px, np.full((h, w, 1), 255, np.uint8)], -1)
    return np.ascontiguousarray(px)


def load_ppm(path) -> np.ndarray:
    """Binary PPM (P6, maxval 255) -> RGBA8."""
    with open(path, "rb") as f:
        data = f.read()
    toks, pos = [], 0
    while len(toks) < 4:
        while data[pos:pos + 1].isspace():
            pos += 1
        if data[pos:pos + 1] == b"#":
            pos = data.index(b"\n", pos) + 1
            continue
        end = pos
        while not data[end:end + 1].isspace():
            end += 1
        toks.append(data[pos:end])
        pos = end
    if toks[0] != b"P6" or int(toks[3]) != 255:
        raise ValueError(f"{path}: only binary 8-bit PPM (P6) is supported")
    w, h = int(toks[1]), int(toks[2])
    px = np.frombuffer(data, np.uint8, w * h * 3, pos + 1).reshape(h, w, 3)
    return np.concatenate([px, np.full((h, w, 1), 255, np.uint8)], -1)


def load_image(path) -> np.ndarray:
    ext = os.path.splitext(str(path))[1].lower()
    if ext == ".png":
        return load_png(path)
    if ext in (".ppm", ".pnm"):
        return load_ppm(path)
    raise ValueError(f"{path}: image format {ext} is not supported (PNG, PPM)")


# ---- OBJ / MTL -----------------------------------------------------------------
def _floats(parts, n, default):
    vals = [float(x) for x in parts[:n]]
    return tuple(vals + list(default[len(vals):]))


def load_mtl(path) -> Dict[str, dict]:
    mats: Dict[str, dict] = {}
    cur: Optional[dict] = None
    base = os.path.dirname(str(path))
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts or parts[0].startswith("#"):
                continue
            key, args = parts[0], parts[1:]
            if key == "newmtl":
                cur = mats.setdefault(" ".join(args), {})
            elif cur is None:
                continue
            elif key in ("Ka", "Kd", "Ks", "Ke", "Tf"):
                cur[key] = _floats(args, 3, (0.0, 0.0, 0.0))
            elif key in ("Ns", "Ni", "d"):
                cur[key] = float(args[0])
            elif key in ("map_Kd", "map_Ks", "map_Ke", "norm", "map_Bump", "bump"):
                cur[key] = os.path.join(base, args[-1])
    return mats


def _material_from_mtl(m: dict) -> np.ndarray:
    spec = (*m.get("Ks", (0.0, 0.0, 0.0)), 1.0)
    shin = m.get("Ns", None)
    if shin is None or shin < 0.01:  # assimp.cpp:674-689
        shin, spec = 0.0, (0.0, 0.0, 0.0, 0.0)
    return phong_material(ambient=(*m.get("Ka", (0.0, 0.0, 0.0)), 1.0), diffuse=(*m.get("Kd", (1.0, 1.0, 1.0)), 1.0),
                          specular=spec, emissive=(*m.get("Ke", (0.0, 0.0, 0.0)), 1.0),
                          transmissive=m.get("Tf", (1.0, 1.0, 1.0)), shininess=shin,
                          index_of_refraction=m.get("Ni", 1.0))


def load_obj(path, missing_textures: str = "error") -> Scene:
    """Wavefront OBJ (+ MTL) -> Scene (one instance per mesh, identity
    transforms). missing_textures: "error" or "white" (use the 1x1 default)."""
    base = os.path.dirname(str(path))
    V, VT, VN = [], [], []
    mtls: Dict[str, dict] = {}
    groups = []  # (material name, faces: list of [(v, vt, vn), ...])
    cur_mat, cur_faces = None, None

    def start(mat):
        nonlocal cur_mat, cur_faces
        cur_mat, cur_faces = mat, []
        groups.append((mat, cur_faces))

    start(None)

    def ref(tok, n, count):
        if not tok:
            return None
        i = int(tok)
        return i - 1 if i > 0 else count + i

    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts or parts[0].startswith("#"):
                continue
            key, args = parts[0], parts[1:]
            if key == "v":
                V.append([float(x) for x in args[:3]])
            elif key == "vt":
                VT.append([float(x) for x in (args + ["0"])[:2]])
            elif key == "vn":
                VN.append([float(x) for x in args[:3]])
            elif key == "f":
                corners = []
                for a in args:
                    t = (a.split("/") + ["", ""])[:3]
                    corners.append((ref(t[0], 0, len(V)), ref(t[1], 1, len(VT)), ref(t[2], 2, len(VN))))
                cur_faces.append(corners)
            elif key == "usemtl":
                start(" ".join(args))
            elif key in ("o", "g"):
                start(cur_mat)
            elif key == "mtllib":
                for name in args:
                    p = os.path.join(base, name)
                    if os.path.exists(p):
                        mtls.update(load_mtl(p))
    V = np.asarray(V, np.float32).reshape(-1, 3)
    VT = np.asarray(VT, np.float32).reshape(-1, 2)
    VN = np.asarray(VN, np.float32).reshape(-1, 3)
    sc = Scene()
    tex_cache: Dict[str, int] = {}

    def texture(p):
        if p is None:
            return 0
        if p not in tex_cache:
            try:
                tex_cache[p] = sc.add_texture(load_image(p))
            except (OSError, ValueError):
                if missing_textures != "white":
                    raise
                tex_cache[p] = 0
        return tex_cache[p]

    mat_ids: Dict[Optional[str], tuple] = {}
    for mname, faces in groups:
        tris = [(face[0], face[k], face[k + 1]) for face in faces for k in range(1, len(face) - 1)]
        if not tris:
            continue
        corners = [c for t in tris for c in t]
        pos = V[[c[0] for c in corners]]
        has_n = all(c[2] is not None for c in corners)
        has_t = all(c[1] is not None for c in corners)
        nor = VN[[c[2] for c in corners]] if has_n else np.zeros_like(pos)
        uv = VT[[c[1] for c in corners]] if has_t else np.zeros((len(pos), 2), np.float32)
        uv = np.stack([uv[:, 0], np.float32(1) - uv[:, 1]], -1)  # aiProcess_FlipUVs
        n = len(corners)
        idx = np.arange(n, dtype=np.uint16 if n < 65535 else np.uint32)
        mesh = prepare_mesh(pos, nor, uv, idx)
        if mname not in mat_ids:
            m = mtls.get(mname, {})
            tx = [texture(m.get("map_Kd")), 0, texture(m.get("norm")), texture(m.get("map_Ke")),
                  texture(m.get("map_Ks"))]
            mat_ids[mname] = (_material_from_mtl(m), tx)
        mat, tx = mat_ids[mname]
        t5 = [0] * 5
        t5[SLOT_DIFFUSE], t5[SLOT_NORMAL], t5[SLOT_EMISSIVE], t5[SLOT_SPECULAR] = tx[0], tx[2], tx[3], tx[4]
        mid = sc.add_mesh(mesh, mat, t5)
        sc.add_instance(mid, np.eye(4))
        if is_emissive(mat):
            sc.add_emissive_lights(mid, np.eye(4), tuple(mat[16:19]))
    sc.finalize_lights()
    return sc

