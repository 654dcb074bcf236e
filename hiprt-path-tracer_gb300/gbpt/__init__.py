"""gbpt — GB300-native render path (Python host side over the libgbpt C ABI).

The compute runs in hand-written CUDA kernels for sm_103a inside libgbpt.so; this package only
builds/loads the library, generates seeded synthetic scenes, and wraps the C entry points.
"""
from . import scenes  # noqa: F401
from ._lib import GbptError, load, lib_path  # noqa: F401
from .trace import BVH, hit_prim  # noqa: F401
from .render import (Batch, GltfScene, Renderer, RenderSettings, Scene, World, cornell_settings,  # noqa: F401
                     load_gltf, look_at_camera)
