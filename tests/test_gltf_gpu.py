"""GPU: a scene read from a glTF file (gbpt_gltf_load -> gbpt_scene_create) renders bit-identically
to the same scene built directly from the oracle reader's arrays and material records, with the
file's camera; so the loader feeds the path tracer exactly what the reference's parser would."""
import os
import sys

import numpy as np
import pytest
import torch

import gbpt
from gbpt import materials as M
from gbpt.render import BSDF_PRINCIPLED, LIGHT_POWER, RenderSettings

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
sys.path.insert(0, HERE)
import gltf_oracle  # noqa: E402
from gltf_writer import scene_file  # noqa: E402

GOLDEN = os.path.join(HERE, "golden", "pt_principled_cornell.npz")


def _gltf_materials(records):
    """glTF materials carrying the golden Cornell box's principled parameters that glTF can express."""
    out = []
    for r in records:
        e = np.asarray(M.get(r, "emission"), np.float64)
        strength = float(e.max()) if e.max() > 0 else 1.0
        out.append({
            "pbrMetallicRoughness": {"baseColorFactor": [*map(float, M.get(r, "base_color")), 1.0],
                                     "metallicFactor": float(M.get(r, "metallic")),
                                     "roughnessFactor": float(M.get(r, "roughness"))},
            "emissiveFactor": (e / strength).tolist(),
            "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": strength},
                           "KHR_materials_ior": {"ior": float(M.get(r, "ior"))},
                           "KHR_materials_transmission": {"transmissionFactor": float(M.get(r, "specular_transmission"))},
                           "KHR_materials_clearcoat": {"clearcoatFactor": float(M.get(r, "coat")),
                                                       "clearcoatRoughnessFactor": float(M.get(r, "coat_roughness"))}}})
    return out


def _image(scene, st, launches=2):
    r = gbpt.Renderer(scene, st)
    r.render(launches)
    torch.cuda.synchronize()
    return r.image_sums()[1]


@pytest.mark.parametrize("container", ["file", "glb"])
def test_loaded_scene_renders_like_direct_scene(cuda, tmp_path, container):
    g = np.load(GOLDEN)
    # the golden's camera as a camera node: its camera-to-world matrix and vertical field of view
    inv_view = np.asarray(g["inverse_view"], np.float64).reshape(4, 4)
    yfov = 2.0 * np.arctan(float(np.asarray(g["inverse_projection"]).reshape(4, 4)[1, 1]))
    camera = {"perspective": {"yfov": yfov, "aspectRatio": 1.0, "znear": 0.1, "zfar": 100.0},
              "transform": {"matrix": inv_view.T.reshape(-1).tolist()}}
    path = scene_file(str(tmp_path / "cornell"), g["positions"], g["indices"], g["material_of"],
                      _gltf_materials(g["materials"]), camera, container)
    loaded = gbpt.load_gltf(path)
    want = gltf_oracle.load(path)
    inv_view, inv_proj = loaded.camera_matrices()
    st = RenderSettings(width=48, height=48, samples_per_launch=4, nb_bounces=4, light_sampling=LIGHT_POWER,
                        bsdf=BSDF_PRINCIPLED, seed=11, inverse_view=inv_view, inverse_projection=inv_proj)
    via_file = loaded.create_scene()
    direct = gbpt.Scene(want["positions"], want["indices"], want["material_of"],
                        principled=M.pack_many(want["materials"]))
    a = _image(via_file, st)
    b = _image(direct, st)
    assert np.isfinite(a).all() and a.sum() > 0
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    la, lb = via_file.light_table(), direct.light_table()
    for k in ("emissive", "probas", "alias"):
        np.testing.assert_array_equal(la[k], lb[k])
    assert la["power_sum64"] == lb["power_sum64"] and la["emissive"].size > 0


def test_sheen_scene_loads_but_is_rejected(cuda, tmp_path):
    g = np.load(GOLDEN)
    mats = _gltf_materials(g["materials"])
    mats[0]["extensions"]["KHR_materials_sheen"] = {"sheenColorFactor": [1, 1, 1]}
    loaded = gbpt.load_gltf(scene_file(str(tmp_path / "s"), g["positions"], g["indices"], g["material_of"], mats))
    with pytest.raises(gbpt.GbptError, match="sheen"):
        loaded.create_scene()
