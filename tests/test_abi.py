"""CPU: libgbpt builds, loads and exports every entry point declared in include/*.h; argument
checks answer without touching the GPU; the material record layout matches the C struct."""
import ctypes
import os
import re

import pytest

import gbpt
from gbpt import _lib

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for h in sorted(os.listdir(INCLUDE)):
        if h.endswith(".h"):
            text = open(os.path.join(INCLUDE, h)).read()
            names |= set(re.findall(r"GBPT_API\s+[^;]*?\b(gbpt_\w+)\s*\(", text, re.S))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = gbpt.load()
    names = declared_symbols()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    from gbpt import bsdf, guide, render
    bound = ({n for n, _, _ in _lib.SIGNATURES} | {n for n, _, _ in render.RENDER_SIGNATURES}
             | {n for n, _, _ in bsdf.BSDF_SIGNATURES} | {n for n, _, _ in guide.GUIDE_SIGNATURES})
    assert bound == set(names)


def test_status_strings_and_version():
    lib = gbpt.load()
    assert lib.gbpt_version() >= 1
    assert lib.gbpt_status_string(0) == b"ok"
    assert lib.gbpt_status_string(2) == b"out of memory"


def test_invalid_arguments_are_reported_not_fatal():
    lib = gbpt.load()
    assert lib.gbpt_bvh_build(None, None, 0, 0, None, None) == 1
    assert b"out is NULL" in lib.gbpt_last_error()
    assert lib.gbpt_trace_closest(None, None, None, None, 10, None, None) == 1
    assert b"bvh is NULL" in lib.gbpt_last_error()
    h = ctypes.c_void_p()
    assert lib.gbpt_bvh_build(None, None, 0, 5, None, ctypes.byref(h)) == 1
    with pytest.raises(gbpt.GbptError):
        _lib.check(1)


def test_material_record_layout_matches_header():
    """gbpt.materials word offsets agree with gbpt_principled_material in include/gbpt_bsdf.h."""
    from gbpt import materials as M
    text = open(os.path.join(INCLUDE, "gbpt_bsdf.h")).read()
    body = text[text.index("typedef struct gbpt_principled_material {"):text.index("} gbpt_principled_material;")]
    off = 0
    seen = {}
    for m in re.finditer(r"(float|int32_t)\s+(\w+)(?:\[(\d+)\])?;", body):
        name, cnt = m.group(2), int(m.group(3) or 1)
        seen[name] = (off, cnt)
        off += cnt
    assert off == M.WORDS
    for name, (o, c) in M.OFFSETS.items():
        assert seen[name] == (o, c), name


def test_bsdf_entry_points_reject_bad_arguments():
    from gbpt import bsdf
    lib = bsdf._load()
    assert lib.gbpt_bsdf_eval(None, 0, None, None, -1, None, None, None) == 1
    assert lib.gbpt_bsdf_eval(None, 0, None, None, 0, None, None, None) == 0
    assert lib.gbpt_bsdf_sample(None, 0, None, None, None, 5, None, None, None, None, None) == 1
    assert b"device pointers" in lib.gbpt_last_error()


def test_guide_parameters_and_argument_checks():
    """gbpt_guide_params matches its C layout; bad parameters are rejected before any device work."""
    from gbpt import guide
    assert ctypes.sizeof(guide.GuideParams) == 72
    text = open(os.path.join(INCLUDE, "gbpt_guide.h")).read()
    for name in ("LEVELS", "TABLE", "FEATURES", "IN", "HIDDEN", "OUT", "LOBES", "ROW"):
        m = re.search(rf"#define GBPT_GUIDE_{name} (\d+)", text)
        assert m and int(m.group(1)) == getattr(guide, name), name
    p = guide.default_params()
    assert abs(p.learning_rate - 1e-2) < 1e-9 and p.max_batch == 1 << 18 and list(p.scene_max) == [1, 1, 1]
    lib = guide._load()
    h = ctypes.c_void_p()
    bad = guide.default_params(max_batch=0)
    assert lib.gbpt_guide_create(ctypes.byref(bad), ctypes.byref(h)) == 1 and not h.value
    bad = guide.default_params(scene_min=(0, 2, 0))
    assert lib.gbpt_guide_create(ctypes.byref(bad), ctypes.byref(h)) == 1
    assert b"empty scene box" in lib.gbpt_last_error()
    assert lib.gbpt_guide_train(None, None, None, None, None, None, None, 4, None, None) == 1
    assert lib.gbpt_guide_infer(None, None, None, None, 4, None, None) == 1
    assert lib.gbpt_guide_destroy(None) == 0


def test_world_descriptor_layout_defaults_and_checks():
    """gbpt_world_desc matches its C layout; defaults are the reference's; bad worlds are rejected
    before any device work."""
    from gbpt import render
    text = open(os.path.join(INCLUDE, "gbpt_render.h")).read()
    body = text[text.index("typedef struct gbpt_world_desc {"):text.index("} gbpt_world_desc;")]
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    names = [n.strip().split("[")[0] for decl in re.findall(r"(?:int32_t|float|const float\*)\s+([^;]+);", body)
             for n in decl.split(",")]
    assert names == [f for f, _ in render.WorldDescC._fields_]
    assert ctypes.sizeof(render.WorldDescC) == 128
    lib = render._load()
    w = render.WorldDescC()
    assert lib.gbpt_world_default(ctypes.byref(w)) == 0
    assert w.ambient == render.AMBIENT_NONE and w.envmap_intensity == 1.0
    assert w.envmap_sampling == render.ENVMAP_ALIAS_TABLE and w.envmap_bsdf_mis == 1 and w.envmap_bilinear == 0
    assert list(w.envmap_to_world) == [1, 0, 0, 0, 1, 0, 0, 0, 1] == list(w.world_to_envmap)
    assert lib.gbpt_scene_set_world(None, ctypes.byref(w), None) == 1
    assert lib.gbpt_scene_get_envmap_tables(None, None, None, None, None, None, None) == 1
