"""Oracle for the glTF scene ingestion (test infrastructure only: the tests import it as the checker;
the library never does).

An independent restatement, in numpy over Python's own json module, of what the reference's scene
parser produces from a glTF 2.0 file:
  * SceneParser::parse_scene_file (src/Scene/SceneParser.cpp:21-226) reads the file through ASSIMP
    with aiProcess_PreTransformVertices (every mesh instance moved to world space by its node's
    accumulated transform) and aiProcess_Triangulate, then concatenates the meshes' vertices and
    triangles with a running vertex offset (:104-190) and gives every triangle its mesh's
    material index (:174);
  * read_material_properties (src/Scene/SceneParser.cpp:391-438) maps the ASSIMP material keys
    into CPUMaterial (defaults src/HostDeviceCommon/Material/MaterialCPU.h:209-300), then
    CPUMaterial::make_safe (MaterialCPU.h:156-207) clamps it; emission_strength is baked into the
    emission afterwards (MaterialCPU.h:209-210).
ASSIMP is not available here, so the key each ASSIMP Get() reads is restated from the glTF field
ASSIMP's glTF 2 importer fills it from (baseColorFactor -> COLOR_DIFFUSE, emissiveFactor ->
COLOR_EMISSIVE, the KHR_materials_* extensions -> their keys, present only when the extension
is). Triangles are kept in node traversal order (depth first, children in file order); ASSIMP's
pre-transform step regroups meshes by material, which changes triangle order but no triangle.

Parity pinned against: the reference's own sample scenes (data/GLTFs/*.gltf of the reference tree
named by GBPT_REFERENCE_ROOT, when it is set) and synthetic files exercising every branch.
"""
from __future__ import annotations

import base64
import json
import os
import struct
import urllib.parse

import numpy as np

# CPUMaterial defaults (MaterialCPU.h:209-300), in the order of gbpt_principled_material's fields
DEFAULTS = {
    "base_color": (1.0, 1.0, 1.0), "roughness": 0.3, "emission": (0.0, 0.0, 0.0), "metallic": 0.0,
    "metallic_F82": (1.0, 1.0, 1.0), "metallic_F90_falloff_exponent": 5.0, "metallic_F90": (1.0, 1.0, 1.0),
    "anisotropy": 0.0, "anisotropy_rotation": 0.0, "second_roughness_weight": 0.0, "second_roughness": 0.5,
    "specular": 1.0, "specular_color": (1.0, 1.0, 1.0), "specular_tint": 1.0, "specular_darkening": 0.0,
    "coat": 0.0, "coat_roughness": 0.0, "coat_roughening": 1.0, "coat_medium_absorption": (1.0, 1.0, 1.0),
    "coat_medium_thickness": 5.0, "coat_darkening": 1.0, "coat_anisotropy": 0.0, "coat_anisotropy_rotation": 0.0,
    "coat_ior": 1.5, "sheen": 0.0, "ior": 1.4, "specular_transmission": 0.0, "diffuse_transmission": 0.0,
    "absorption_color": (1.0, 1.0, 1.0), "absorption_at_distance": 1.0, "thin_walled": 0,
}
FLT_MAX = float(np.finfo(np.float32).max)

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_WIDTH = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}


def _f32(x):
    return float(np.float32(x))


def _clamp(lo, hi, v):
    return _f32(min(hi, max(lo, _f32(v))))


def map_material(mat: dict) -> dict:
    """One glTF material object -> CPUMaterial fields after make_safe, emission scaled by strength."""
    m = dict(DEFAULTS)
    pbr = mat.get("pbrMetallicRoughness", {})
    bc = pbr.get("baseColorFactor", [1, 1, 1, 1])
    m["base_color"] = tuple(_f32(c) for c in bc[:3])
    m["metallic"] = _f32(pbr.get("metallicFactor", 1.0))
    m["roughness"] = _f32(pbr.get("roughnessFactor", 1.0))
    m["emission"] = tuple(_f32(c) for c in mat.get("emissiveFactor", [0, 0, 0]))
    ext = mat.get("extensions", {})
    strength = _f32(ext.get("KHR_materials_emissive_strength", {}).get("emissiveStrength", 1.0))
    if "KHR_materials_anisotropy" in ext:
        m["anisotropy"] = _f32(ext["KHR_materials_anisotropy"].get("anisotropyStrength", 0.0))
    if "KHR_materials_sheen" in ext:
        m["sheen"] = 1.0
    if "KHR_materials_specular" in ext:
        m["specular"] = _f32(ext["KHR_materials_specular"].get("specularFactor", 1.0))
        m["specular_tint"] = 1.0
        m["specular_color"] = (1.0, 1.0, 1.0)
    if "KHR_materials_clearcoat" in ext:
        e = ext["KHR_materials_clearcoat"]
        m["coat"] = _f32(e.get("clearcoatFactor", 0.0))
        m["coat_roughness"] = _f32(e.get("clearcoatRoughnessFactor", 0.0))
    if "KHR_materials_ior" in ext:
        m["ior"] = _f32(ext["KHR_materials_ior"].get("ior", 1.5))
    if "KHR_materials_transmission" in ext:
        m["specular_transmission"] = _f32(ext["KHR_materials_transmission"].get("transmissionFactor", 0.0))
    if "KHR_materials_volume" in ext:
        e = ext["KHR_materials_volume"]
        m["absorption_color"] = tuple(_f32(c) for c in e.get("attenuationColor", [1, 1, 1]))
        m["absorption_at_distance"] = _f32(e["attenuationDistance"]) if "attenuationDistance" in e else FLT_MAX
    # make_safe
    for k in ("base_color", "metallic_F82", "metallic_F90", "specular_color", "coat_medium_absorption"):
        m[k] = tuple(_clamp(0.0, 1.0, c) for c in m[k])
    m["absorption_color"] = tuple(_clamp(0.0, 1.0, max(_f32(c), _f32(1.0 / 512.0))) for c in m["absorption_color"])
    m["emission"] = tuple(max(0.0, c) for c in m["emission"])
    for k in ("metallic", "anisotropy", "anisotropy_rotation", "second_roughness_weight", "second_roughness",
              "specular", "specular_tint", "specular_darkening", "coat", "coat_roughening", "coat_darkening",
              "coat_anisotropy", "coat_anisotropy_rotation", "sheen", "specular_transmission"):
        m[k] = _clamp(0.0, 1.0, m[k])
    m["coat_roughness"] = _clamp(_f32(1e-4), 1.0, m["coat_roughness"])
    m["absorption_at_distance"] = max(_f32(m["absorption_at_distance"]), _f32(1e-4))
    m["emission"] = tuple(_f32(np.float32(c) * np.float32(strength)) for c in m["emission"])
    return m


def _node_matrix(node: dict) -> np.ndarray:
    if "matrix" in node:
        return np.asarray(node["matrix"], np.float64).reshape(4, 4).T  # column-major in the file
    t = np.asarray(node.get("translation", [0, 0, 0]), np.float64)
    x, y, z, w = node.get("rotation", [0, 0, 0, 1])
    s = np.asarray(node.get("scale", [1, 1, 1]), np.float64)
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]], np.float64)
    m = np.eye(4)
    m[:3, :3] = r * s[None, :]
    m[:3, 3] = t
    return m


class _Doc:
    def __init__(self, path: str):
        raw = open(path, "rb").read()
        bin_chunk = None
        if raw[:4] == b"glTF":
            _, _, total = struct.unpack_from("<4sII", raw, 0)
            at, chunks = 12, []
            while at + 8 <= total:
                ln, typ = struct.unpack_from("<II", raw, at)
                chunks.append((typ, raw[at + 8:at + 8 + ln]))
                at += 8 + ln
            text = chunks[0][1]
            bin_chunk = next((c for t, c in chunks[1:2] if t == 0x004E4942), None)
        else:
            text = raw
        self.j = json.loads(text.decode("utf-8"))
        base = os.path.dirname(path)
        self.buffers = []
        for i, b in enumerate(self.j.get("buffers", [])):
            uri = b.get("uri")
            if uri is None:
                data = bin_chunk
            elif uri.startswith("data:"):
                data = base64.b64decode(uri.split(",", 1)[1])
            else:
                data = open(os.path.join(base, urllib.parse.unquote(uri)), "rb").read()
            self.buffers.append(data[:b["byteLength"]])

    def accessor(self, i: int) -> np.ndarray:
        a = self.j["accessors"][i]
        dt = np.dtype(_COMPONENT[a["componentType"]]).newbyteorder("<")
        width, count = _WIDTH[a["type"]], a["count"]
        if "bufferView" not in a:
            return np.zeros((count, width), dt)
        v = self.j["bufferViews"][a["bufferView"]]
        elem = dt.itemsize * width
        stride = v.get("byteStride", elem)
        start = v.get("byteOffset", 0) + a.get("byteOffset", 0)
        buf = self.buffers[v["buffer"]]
        rows = [np.frombuffer(buf, dt, width, start + k * stride) for k in range(count)]
        return np.array(rows, dt).reshape(count, width)


def load(path: str) -> dict:
    """{'positions' (V,3) f32, 'indices' (T,3) i32, 'material_of' (T,) i32, 'materials' [dict],
    'camera' dict | None, 'normals' (V,3) f32 | None} of a .gltf/.glb file."""
    doc = _Doc(path)
    j = doc.j
    nodes = j.get("nodes", [])
    materials = [map_material(m) for m in j.get("materials", [])]
    default_material = [None]
    if j.get("scenes"):
        roots = j["scenes"][j.get("scene", 0)].get("nodes", [])
    else:
        children = {c for n in nodes for c in n.get("children", [])}
        roots = [i for i in range(len(nodes)) if i not in children]
    pos_out, tri_out, mat_out, nrm_out = [], [], [], []
    any_normals = False
    n_vertices = 0
    camera, camera_index = None, None

    def visit(i, parent):
        nonlocal n_vertices, camera, camera_index, any_normals
        node = nodes[i]
        world = parent @ _node_matrix(node)
        if "mesh" in node:
            mirrored = np.linalg.det(world[:3, :3]) < 0
            for prim in j["meshes"][node["mesh"]]["primitives"]:
                mode = prim.get("mode", 4)
                if mode < 4:
                    continue
                p = doc.accessor(prim["attributes"]["POSITION"]).astype(np.float64)
                nv = len(p)
                idx = (doc.accessor(prim["indices"]).reshape(-1).astype(np.int64) if "indices" in prim
                       else np.arange(nv, dtype=np.int64))
                if "material" in prim:
                    mi = prim["material"]
                else:
                    if default_material[0] is None:
                        default_material[0] = len(materials)
                        materials.append(map_material({}))
                    mi = default_material[0]
                wp = (p @ world[:3, :3].T + world[:3, 3]).astype(np.float32)
                if "NORMAL" in prim["attributes"]:
                    # inverse transpose of the node's 3x3 part, then normalised (ASSIMP's
                    # pre-transform step applies the same to normals)
                    nn = doc.accessor(prim["attributes"]["NORMAL"]).astype(np.float64) @ np.linalg.inv(world[:3, :3])
                    ln = np.linalg.norm(nn, axis=1, keepdims=True)
                    nn = np.where(ln > 0, nn / np.where(ln > 0, ln, 1.0), nn)
                    nrm_out.append(nn.astype(np.float32))
                    any_normals = True
                else:
                    nrm_out.append(np.zeros((nv, 3), np.float32))
                tris = []
                n = len(idx)
                if mode == 4:
                    tris = [(idx[t], idx[t + 1], idx[t + 2]) for t in range(0, n - 2, 3)]
                elif mode == 5:
                    tris = [(idx[t], idx[t + 1], idx[t + 2]) if t % 2 == 0 else (idx[t + 1], idx[t], idx[t + 2])
                            for t in range(n - 2)]
                else:
                    tris = [(idx[t], idx[t + 1], idx[0]) for t in range(1, n - 1)]
                if mirrored:
                    tris = [(a, c, b) for a, b, c in tris]
                pos_out.append(wp)
                tri_out.append(np.asarray(tris, np.int64).reshape(-1, 3) + n_vertices)
                mat_out.append(np.full(len(tris), mi, np.int32))
                n_vertices += nv
        if "camera" in node:
            c = j["cameras"][node["camera"]]
            if c.get("type") == "perspective" and "perspective" in c and (camera_index is None or node["camera"] < camera_index):
                camera_index = node["camera"]
                f = world[:3, :3] @ np.array([0.0, 0.0, -1.0])
                u = world[:3, :3] @ np.array([0.0, 1.0, 0.0])
                pp = c["perspective"]
                camera = {"position": tuple(world[:3, 3].astype(np.float32).tolist()),
                          "forward": tuple((f / np.linalg.norm(f)).astype(np.float32).tolist()),
                          "up": tuple((u / np.linalg.norm(u)).astype(np.float32).tolist()),
                          "yfov": _f32(pp.get("yfov", 0.0)), "aspect_ratio": _f32(pp.get("aspectRatio", 0.0)),
                          "znear": _f32(pp.get("znear", 0.0)), "zfar": _f32(pp.get("zfar", 0.0))}
        for c in node.get("children", []):
            visit(c, world)

    for r in roots:
        visit(r, np.eye(4))
    return {
        "positions": np.concatenate(pos_out) if pos_out else np.zeros((0, 3), np.float32),
        "indices": (np.concatenate(tri_out) if tri_out else np.zeros((0, 3), np.int64)).astype(np.int32),
        "material_of": np.concatenate(mat_out) if mat_out else np.zeros(0, np.int32),
        "materials": materials,
        "camera": camera,
        "normals": np.concatenate(nrm_out) if any_normals else None,
    }
