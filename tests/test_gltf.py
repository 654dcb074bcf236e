"""CPU: glTF 2.0 scene ingestion (gbpt_gltf_load) against the oracle's independent reader of the same
files: world-space positions, triangles, per-triangle materials, the principled records of the
reference's material mapping, and the camera; on synthetic files covering node hierarchies, TRS
and matrix transforms, mirrored instances, strided and 8/16/32-bit index accessors, strips, fans,
non-indexed primitives, missing materials, every read extension and make_safe's clamps, in all
three containers; on the reference's own sample scenes when they are present; and corrupt files
rejected with an error instead of a crash."""
import json
import math
import os
import sys

import numpy as np
import pytest

import gbpt
from gbpt import materials as M

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import gltf_oracle  # noqa: E402
from gltf_writer import GltfBuilder  # noqa: E402

import pyoracle  # noqa: E402

REFERENCE_SCENES = os.path.join(pyoracle.reference_root() or "", "data", "GLTFs")


def _quat(axis, deg):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    h = math.radians(deg) / 2
    return [*(a * math.sin(h)).tolist(), math.cos(h)]


MATERIALS = [
    # plain metallic-roughness with a base colour above 1 (clamped) and an emissive strength
    {"pbrMetallicRoughness": {"baseColorFactor": [1.5, 0.25, -0.5, 1], "metallicFactor": 0.25,
                              "roughnessFactor": 0.75},
     "emissiveFactor": [2.0, -1.0, 0.5],
     "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 7.5}}},
    # every extension the reference's mapping reads
    {"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 1]},
     "extensions": {"KHR_materials_ior": {"ior": 1.7},
                    "KHR_materials_transmission": {"transmissionFactor": 1.25},
                    "KHR_materials_clearcoat": {"clearcoatFactor": 0.5, "clearcoatRoughnessFactor": 0.0},
                    "KHR_materials_specular": {"specularFactor": 0.3},
                    "KHR_materials_volume": {"attenuationColor": [0.5, 0.001, 2.0], "attenuationDistance": 0.0},
                    "KHR_materials_anisotropy": {"anisotropyStrength": 0.6}}},
    # extensions present with their defaults; no pbrMetallicRoughness at all
    {"extensions": {"KHR_materials_ior": {}, "KHR_materials_clearcoat": {}, "KHR_materials_specular": {},
                    "KHR_materials_volume": {}}},
    # sheen: the reference turns it fully on
    {"extensions": {"KHR_materials_sheen": {"sheenColorFactor": [1, 1, 1]}}},
]


def synthetic(builder=None):
    """A scene with a node tree (matrix and TRS, a mirrored instance, an instanced mesh), index
    accessors of three widths (one strided), a strip, a fan, a non-indexed primitive, a line
    primitive (skipped), a primitive without a material and a camera under a rotated parent."""
    rng = np.random.default_rng(5)
    b = builder or GltfBuilder()
    b.j["materials"] = MATERIALS
    grid = rng.uniform(-1, 1, (12, 3)).astype(np.float32)
    p_grid = b.accessor(grid)
    p_grid_strided = b.accessor(grid, stride=20)
    tri8 = rng.integers(0, 12, 18).astype(np.uint8)
    tri16 = rng.integers(0, 12, 12).astype(np.uint16)
    tri32 = rng.integers(0, 12, 9).astype(np.uint32)
    strip = np.array([0, 1, 2, 3, 4, 5, 6], np.uint16)
    fan = np.array([7, 8, 9, 10, 11], np.uint32)
    normals = rng.normal(size=(12, 3)).astype(np.float32)
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    mesh_a = b.mesh([
        {"attributes": {"POSITION": p_grid, "NORMAL": b.accessor(normals)}, "indices": b.accessor(tri8), "material": 0},
        {"attributes": {"POSITION": p_grid_strided}, "indices": b.accessor(tri16, stride=4), "material": 1},
        {"attributes": {"POSITION": p_grid}, "indices": b.accessor(tri32)},  # no material
        {"attributes": {"POSITION": p_grid}, "indices": b.accessor(strip), "mode": 5, "material": 2},
        {"attributes": {"POSITION": p_grid}, "indices": b.accessor(fan), "mode": 6, "material": 3},
        {"attributes": {"POSITION": p_grid}, "indices": b.accessor(tri8[:4]), "mode": 1, "material": 0},  # lines
    ])
    soup = rng.uniform(-2, 2, (9, 3)).astype(np.float32)
    mesh_b = b.mesh([{"attributes": {"POSITION": b.accessor(soup)}, "material": 1}])  # not indexed

    m = np.eye(4)
    m[:3, :3] = [[0.0, -2.0, 0.0], [1.5, 0.0, 0.0], [0.0, 0.0, 0.5]]
    m[:3, 3] = [3.0, -1.0, 0.25]
    root = b.node(matrix=m.T.reshape(-1).tolist(), children=[])
    child = b.node(root=False, mesh=mesh_a, translation=[0.5, 1.0, -2.0], rotation=_quat([1, 2, 3], 37.0),
                   scale=[1.0, 2.0, 0.5])
    mirror = b.node(root=False, mesh=mesh_a, scale=[-1.0, 1.0, 1.0], children=[])
    grand = b.node(root=False, mesh=mesh_b, rotation=_quat([0, 1, 0], 90.0))
    b.j["nodes"][root]["children"] = [child, mirror]
    b.j["nodes"][mirror]["children"] = [grand]
    b.node(mesh=mesh_b, translation=[0, 0, 5])
    # two cameras: the one with the lower index wins whatever the traversal order
    b.j["cameras"] = [{"type": "perspective", "perspective": {"yfov": 0.5, "aspectRatio": 1.5, "znear": 0.1, "zfar": 50}},
                      {"type": "perspective", "perspective": {"yfov": 0.9, "znear": 0.2}}]
    b.node(camera=1, translation=[9, 9, 9])
    cam_parent = b.node(rotation=_quat([0, 1, 0], 30.0), translation=[1, 2, 3], children=[])
    cam = b.node(root=False, camera=0, rotation=_quat([1, 0, 0], -10.0), translation=[0, 0, 4])
    b.j["nodes"][cam_parent]["children"] = [cam]
    return b


def _compare(path):
    got = gbpt.load_gltf(path)
    want = gltf_oracle.load(path)
    assert got.indices.shape == want["indices"].shape
    np.testing.assert_array_equal(got.indices, want["indices"])
    np.testing.assert_array_equal(got.material_of_triangle, want["material_of"])
    assert got.positions.shape == want["positions"].shape
    scale = 1.0 + np.abs(want["positions"])
    assert np.all(np.abs(got.positions - want["positions"]) <= 2e-6 * scale)
    if want["normals"] is None:
        assert got.vertex_normals is None
    else:
        assert got.vertex_normals.shape == want["normals"].shape
        assert np.all(np.abs(got.vertex_normals - want["normals"]) <= 2e-6)
    expected = M.pack_many(want["materials"])
    assert got.principled.shape == expected.shape
    # material records are bit-identical (same float conversions and clamps)
    np.testing.assert_array_equal(got.principled.view(np.uint32), expected.view(np.uint32))
    if want["camera"] is None:
        assert got.camera is None
    else:
        for k, v in want["camera"].items():
            np.testing.assert_allclose(got.camera[k], v, rtol=1e-6, atol=1e-6, err_msg=k)
    return got, want


@pytest.mark.parametrize("container", ["file", "base64", "glb"])
def test_synthetic_scene_matches_oracle(tmp_path, container):
    path = synthetic().save(str(tmp_path / "scene"), container)
    got, want = _compare(path)
    # the counts the construction implies: mesh A twice (6 + 4 + 3 + 5 strip + 3 fan triangles,
    # the line primitive skipped), mesh B twice (3 triangles each)
    assert got.indices.shape[0] == 2 * (6 + 4 + 3 + 5 + 3) + 2 * 3
    # the default material is appended after the file's materials
    assert got.principled.shape[0] == len(MATERIALS) + 1
    assert set(np.unique(got.material_of_triangle)) == set(range(len(MATERIALS) + 1))
    assert got.camera["yfov"] == pytest.approx(0.5) and got.camera["aspect_ratio"] == pytest.approx(1.5)
    # normals: unit length where the primitive has them (the first primitive of each mesh A
    # instance), zero elsewhere
    ln = np.linalg.norm(got.vertex_normals, axis=1)
    assert np.all((np.abs(ln - 1) < 1e-6) | (ln == 0)) and 0 < np.count_nonzero(ln) < len(ln)


def test_containers_agree(tmp_path):
    outs = [gbpt.load_gltf(synthetic().save(str(tmp_path / c), c)) for c in ("file", "base64", "glb")]
    for o in outs[1:]:
        np.testing.assert_array_equal(o.positions, outs[0].positions)
        np.testing.assert_array_equal(o.indices, outs[0].indices)
        np.testing.assert_array_equal(o.principled, outs[0].principled)


def test_material_mapping_follows_reference_keys(tmp_path):
    """Spot values of the reference's mapping, independent of the oracle."""
    got = gbpt.load_gltf(synthetic().save(str(tmp_path / "scene"), "file"))
    p = got.principled
    f = np.float32
    # material 0: base colour clamped to [0, 1]; emission clamped at 0 then scaled by the strength
    assert list(M.get(p[0], "base_color")) == [1.0, 0.25, 0.0]
    assert list(M.get(p[0], "emission")) == [f(2.0) * f(7.5), 0.0, f(0.5) * f(7.5)]
    assert M.get(p[0], "metallic") == f(0.25) and M.get(p[0], "roughness") == f(0.75)
    assert M.get(p[0], "ior") == f(1.4)  # CPUMaterial's default without KHR_materials_ior
    # material 1: every extension
    assert M.get(p[1], "ior") == f(1.7) and M.get(p[1], "specular_transmission") == 1.0
    assert M.get(p[1], "coat") == 0.5 and M.get(p[1], "coat_roughness") == f(1e-4)
    assert M.get(p[1], "specular") == f(0.3) and M.get(p[1], "specular_tint") == 1.0
    assert list(M.get(p[1], "absorption_color")) == [0.5, f(1.0 / 512.0), 1.0]
    assert M.get(p[1], "absorption_at_distance") == f(1e-4)
    assert M.get(p[1], "anisotropy") == f(0.6)
    assert M.get(p[1], "metallic") == 1.0 and M.get(p[1], "roughness") == 1.0  # glTF defaults
    # material 2: extension defaults
    assert M.get(p[2], "ior") == f(1.5) and M.get(p[2], "specular") == 1.0 and M.get(p[2], "coat") == 0.0
    assert M.get(p[2], "absorption_at_distance") == np.finfo(np.float32).max
    # material 3: sheen on
    assert M.get(p[3], "sheen") == 1.0


def test_transforms_and_winding(tmp_path):
    """One triangle under a mirroring node keeps its facing: the loaded winding is flipped so the
    world-space geometric normal is the mirror image of the unmirrored one."""
    b = GltfBuilder()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    mesh = b.mesh([{"attributes": {"POSITION": b.accessor(tri)}}])
    b.node(mesh=mesh)
    b.node(mesh=mesh, scale=[-1, 1, 1], translation=[5, 0, 0])
    got = gbpt.load_gltf(b.save(str(tmp_path / "w"), "file"))
    p = got.positions
    n = [np.cross(p[t[1]] - p[t[0]], p[t[2]] - p[t[0]]) for t in got.indices]
    assert n[0][2] > 0 and n[1][2] > 0
    np.testing.assert_array_equal(p[3:], tri * [-1, 1, 1] + [5, 0, 0])


def test_normals_follow_the_inverse_transpose(tmp_path):
    """A non-uniform scale tilts normals the other way than positions: the loaded normal of a
    slanted face stays perpendicular to the scaled face."""
    b = GltfBuilder()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 1]], np.float32)
    n = np.cross(tri[1] - tri[0], tri[2] - tri[0])
    n = np.tile((n / np.linalg.norm(n)).astype(np.float32), (3, 1))
    b.node(mesh=b.mesh([{"attributes": {"POSITION": b.accessor(tri), "NORMAL": b.accessor(n)}}]), scale=[1, 3, 0.5])
    got = gbpt.load_gltf(b.save(str(tmp_path / "n"), "file"))
    p = got.positions
    face = np.cross(p[1] - p[0], p[2] - p[0])
    face /= np.linalg.norm(face)
    np.testing.assert_allclose(got.vertex_normals, np.tile(face, (3, 1)), atol=1e-6)


@pytest.mark.parametrize("name", ["cornell_pbr.gltf", "nested-dielectrics.gltf", "nested-dielectrics-complex.gltf",
                                  "multi-dispersion.gltf"])
def test_reference_sample_scenes(name):
    path = os.path.join(REFERENCE_SCENES, name)
    if not os.path.exists(path):
        pytest.skip("the reference's sample scenes are not present")
    got, want = _compare(path)
    assert got.indices.shape[0] > 0 and got.camera is not None
    # every index of the file's primitives is a triangle of the loaded scene
    j = json.load(open(path))
    expected = sum(j["accessors"][p["indices"]]["count"] // 3 for m in j["meshes"] for p in m["primitives"]
                   for n in j["nodes"] if n.get("mesh") == j["meshes"].index(m))
    assert got.indices.shape[0] == expected


def _bad(tmp_path, text=None, raw=None, name="bad.gltf"):
    path = tmp_path / name
    if raw is not None:
        path.write_bytes(raw)
    else:
        path.write_text(text if isinstance(text, str) else json.dumps(text))
    with pytest.raises(gbpt.GbptError) as e:
        gbpt.load_gltf(str(path))
    return str(e.value)


def test_corrupt_files_are_errors(tmp_path):
    with pytest.raises(gbpt.GbptError, match="cannot open"):
        gbpt.load_gltf(str(tmp_path / "missing.gltf"))
    assert "JSON" in _bad(tmp_path, "{\"asset\": {\"version\": \"2.0\"")
    assert "JSON" in _bad(tmp_path, "[1, 2,]")
    assert "JSON" in _bad(tmp_path, "{\"a\": 01}")
    assert "JSON" in _bad(tmp_path, "{\"a\": \"\\ud800\"}")
    assert "JSON" in _bad(tmp_path, "[" * 1000 + "]" * 1000)
    assert "version" in _bad(tmp_path, {"asset": {"version": "1.0"}})
    assert "extension" in _bad(tmp_path, {"asset": {"version": "2.0"}, "extensionsRequired": ["KHR_draco_mesh_compression"]})
    assert "GLB" in _bad(tmp_path, raw=b"glTF" + (2).to_bytes(4, "little") + (999).to_bytes(4, "little"), name="b.glb")

    b = synthetic()
    good = json.loads(json.dumps(b.j))
    blob_len = len(b.blob)

    def with_buffer(j):
        j = json.loads(json.dumps(j))
        import base64
        j["buffers"] = [{"byteLength": blob_len, "uri": "data:application/octet-stream;base64,"
                         + base64.b64encode(bytes(b.blob)).decode()}]
        for k in ("materials", "cameras"):
            if not j[k]:
                del j[k]
        return j

    j = with_buffer(good)
    j["accessors"][0]["count"] = 10 ** 6
    assert "past the end" in _bad(tmp_path, j)
    j = with_buffer(good)
    j["bufferViews"][0]["byteLength"] = blob_len * 2
    assert "past the end" in _bad(tmp_path, j)
    j = with_buffer(good)
    j["accessors"][0]["sparse"] = {"count": 1}
    assert "sparse" in _bad(tmp_path, j)
    j = with_buffer(good)
    j["nodes"][1]["children"] = [0]  # 0 -> 1 -> 0
    assert "cycle" in _bad(tmp_path, j)
    j = with_buffer(good)
    j["meshes"][0]["primitives"][0]["material"] = 99
    assert "material" in _bad(tmp_path, j)
    j = with_buffer(good)
    j["meshes"][0]["primitives"][0]["indices"] = j["meshes"][0]["primitives"][0]["attributes"]["POSITION"]
    assert "indices" in _bad(tmp_path, j)
    j = with_buffer(good)
    j["buffers"][0]["byteLength"] = blob_len + 1
    assert "shorter" in _bad(tmp_path, j)
    j = with_buffer(good)
    j["accessors"][0]["byteOffset"] = -4
    assert "non-negative" in _bad(tmp_path, j)

    # an index past the primitive's vertex count
    bb = GltfBuilder()
    tri = np.zeros((3, 3), np.float32)
    bb.node(mesh=bb.mesh([{"attributes": {"POSITION": bb.accessor(tri)}, "indices": bb.accessor(np.array([0, 1, 3], np.uint16))}]))
    with pytest.raises(gbpt.GbptError, match="out of range"):
        gbpt.load_gltf(bb.save(str(tmp_path / "oob"), "base64"))


def test_null_arguments():
    lib = gbpt.render._load()
    import ctypes
    h = ctypes.c_void_p()
    assert lib.gbpt_gltf_load(None, ctypes.byref(h)) == 1
    assert lib.gbpt_gltf_load(b"x.gltf", None) == 1
    assert lib.gbpt_gltf_scene_desc(None, None) == 1
    assert lib.gbpt_gltf_get_camera(None, None) == 1
    assert lib.gbpt_gltf_destroy(None) == 0
