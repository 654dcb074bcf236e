"""Seeded procedural scenes and ray batches.

One generator feeds both the GPU path and the CPU oracle, so both see bit-identical inputs.
Geometry is computed in float64 with numpy and rounded once to float32.

Scenes:
  * ``heightfield``: an n x n cell grid over [-1,1]^2 (2 triangles per cell) with heights from
    a seeded multi-octave value-noise fBm.
  * ``random_triangles``: small triangles with centres uniform in a box and vertex offsets
    drawn from N(0, sigma^2).
  * ``traversal_scene``: the union of the two, i.e. the BVH-traversal benchmark scene
    (1024 x 1024 cells + 200k random triangles = 2,297,152 triangles at full size).

Ray batches: pinhole primary rays; cosine-hemisphere bounce rays from primary hits (the hit
primitive becomes the self-hit filter's ``last_prim``, as in the reference's
src/Device/includes/PathTracing.h bounce loop); shadow rays to uniform points on an area-light
quad, with ``tmax = distance - 1e-4`` like the reference's shadow test
(src/Device/includes/Intersect.h:276-324).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

F32 = np.float32


@dataclass
class Mesh:
    positions: np.ndarray  # (V, 3) float32
    indices: np.ndarray  # (T, 3) int32

    @property
    def n_triangles(self) -> int:
        return int(self.indices.shape[0])

    def triangle_soup(self) -> np.ndarray:
        """(T, 9) float32: a, b, c per triangle (the oracle's input layout)."""
        return np.ascontiguousarray(self.positions[self.indices].reshape(-1, 9))


@dataclass
class RayBatch:
    origin_tmin: np.ndarray  # (N, 4) float32
    dir_tmax: np.ndarray  # (N, 4) float32
    last_prim: np.ndarray  # (N,) int32

    def __len__(self) -> int:
        return int(self.origin_tmin.shape[0])

    def slice(self, s: slice) -> "RayBatch":
        return RayBatch(self.origin_tmin[s], self.dir_tmax[s], self.last_prim[s])

    @staticmethod
    def concat(batches) -> "RayBatch":
        return RayBatch(np.concatenate([b.origin_tmin for b in batches]),
                        np.concatenate([b.dir_tmax for b in batches]),
                        np.concatenate([b.last_prim for b in batches]))


def _hash_u32(x: np.ndarray) -> np.ndarray:
    """Integer hash (a 32-bit avalanche mix) used for the value-noise lattice."""
    x = x.astype(np.uint64) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(16)
    x = (x * np.uint64(0x7FEB352D)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(15)
    x = (x * np.uint64(0x846CA68B)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(16)
    return x


def _lattice_value(ix: np.ndarray, iz: np.ndarray, seed: int, octave: int) -> np.ndarray:
    h = _hash_u32((ix.astype(np.int64) * 73856093) ^ (iz.astype(np.int64) * 19349663)
                  ^ np.int64(seed * 83492791 + octave * 2654435761))
    return h.astype(np.float64) / 4294967295.0 * 2.0 - 1.0


def value_noise_fbm(x: np.ndarray, z: np.ndarray, seed: int = 1, octaves: int = 6,
                    base_freq: float = 4.0) -> np.ndarray:
    """Seeded fBm of smoothstep-interpolated lattice value noise, roughly in [-1, 1]."""
    total = np.zeros_like(x, dtype=np.float64)
    amp, freq, norm = 1.0, base_freq, 0.0
    for o in range(octaves):
        fx, fz = x * freq, z * freq
        ix, iz = np.floor(fx), np.floor(fz)
        tx, tz = fx - ix, fz - iz
        sx, sz = tx * tx * (3 - 2 * tx), tz * tz * (3 - 2 * tz)
        ix, iz = ix.astype(np.int64), iz.astype(np.int64)
        v00 = _lattice_value(ix, iz, seed, o)
        v10 = _lattice_value(ix + 1, iz, seed, o)
        v01 = _lattice_value(ix, iz + 1, seed, o)
        v11 = _lattice_value(ix + 1, iz + 1, seed, o)
        a = v00 + (v10 - v00) * sx
        b = v01 + (v11 - v01) * sx
        total += amp * (a + (b - a) * sz)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def heightfield(cells: int = 1024, amplitude: float = 0.2, seed: int = 1, octaves: int = 6,
                extent: float = 1.0) -> Mesh:
    """cells x cells grid over [-extent, extent]^2 in x/z, y = amplitude * fBm(x, z)."""
    n = cells + 1
    lin = np.linspace(-extent, extent, n, dtype=np.float64)
    X, Z = np.meshgrid(lin, lin, indexing="xy")  # X varies along columns
    Y = amplitude * value_noise_fbm(X / extent, Z / extent, seed=seed, octaves=octaves)
    pos = np.stack([X, Y, Z], axis=-1).reshape(-1, 3).astype(F32)
    r, c = np.meshgrid(np.arange(cells), np.arange(cells), indexing="ij")
    v00 = (r * n + c).reshape(-1)
    v01 = v00 + 1
    v10 = v00 + n
    v11 = v10 + 1
    t0 = np.stack([v00, v10, v01], axis=1)
    t1 = np.stack([v01, v10, v11], axis=1)
    idx = np.stack([t0, t1], axis=1).reshape(-1, 3).astype(np.int32)
    return Mesh(pos, idx)


def random_triangles(count: int = 200_000, seed: int = 1, lo=(-1.0, 0.0, -1.0), hi=(1.0, 0.5, 1.0),
                     sigma: float = 0.01) -> Mesh:
    """Triangles with centres U[lo, hi] and each vertex = centre + N(0, sigma^2)^3."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(lo, hi, size=(count, 3))
    offs = rng.normal(0.0, sigma, size=(count, 3, 3))
    pos = (centres[:, None, :] + offs).reshape(-1, 3).astype(F32)
    idx = np.arange(count * 3, dtype=np.int32).reshape(-1, 3)
    return Mesh(pos, idx)


def merge(*meshes: Mesh) -> Mesh:
    pos, idx, base = [], [], 0
    for m in meshes:
        pos.append(m.positions)
        idx.append(m.indices + base)
        base += m.positions.shape[0]
    return Mesh(np.concatenate(pos).astype(F32), np.concatenate(idx).astype(np.int32))


def traversal_scene(cells: int = 1024, n_random: int = 200_000, seed: int = 1) -> Mesh:
    """Heightfield (fBm amplitude 0.2, 6 octaves) plus random triangles in [-1,1]x[0,0.5]x[-1,1]."""
    return merge(heightfield(cells, 0.2, seed, 6), random_triangles(n_random, seed + 1))


def _normalize(v: np.ndarray) -> np.ndarray:
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def band_order(width: int, height: int) -> np.ndarray:
    """Pixel index (row-major) of each position in band order: bands of 8 rows, each walked column by
    column (8 pixels of a column, then the next), so 32 consecutive rays cover a 4 x 8 tile; the
    last band has height % 8 rows. The order of the renderer's camera kernel (band_pixel)."""
    l = np.arange(width * height, dtype=np.int64)
    band = 8 * width
    full = height // 8
    x = np.empty_like(l)
    y = np.empty_like(l)
    m = l < full * band
    b, r = l[m] // band, l[m] % band
    x[m], y[m] = r >> 3, b * 8 + (r & 7)
    if (~m).any():
        bh = height - full * 8
        r = l[~m] - full * band
        x[~m], y[~m] = r // bh, full * 8 + r % bh
    return y * width + x


def pinhole_rays(width: int, height: int, eye=(0.0, 1.5, -2.5), target=(0.0, 0.0, 0.0),
                 vfov_deg: float = 60.0, up=(0.0, 1.0, 0.0), order: str = "rows") -> RayBatch:
    """One ray through each pixel centre: order "rows" is row-major from the top-left pixel,
    "bands" is band_order (4 x 8 pixel tiles per 32 rays, the coherent order a renderer emits)."""
    eye = np.asarray(eye, np.float64)
    fwd = _normalize(np.asarray(target, np.float64) - eye)
    right = _normalize(np.cross(np.asarray(up, np.float64), fwd))
    upv = np.cross(fwd, right)
    th = np.tan(np.radians(vfov_deg) * 0.5)
    aspect = width / height
    xs = ((np.arange(width) + 0.5) / width * 2.0 - 1.0) * th * aspect
    ys = (1.0 - (np.arange(height) + 0.5) / height * 2.0) * th
    YY, XX = np.meshgrid(ys, xs, indexing="ij")
    d = fwd[None, None, :] + XX[..., None] * right + YY[..., None] * upv
    d = _normalize(d).reshape(-1, 3)
    n = d.shape[0]
    o = np.empty((n, 4), F32)
    o[:, :3] = eye.astype(F32)
    o[:, 3] = 0.0
    dt = np.empty((n, 4), F32)
    dt[:, :3] = d.astype(F32)
    dt[:, 3] = np.inf
    if order == "bands":
        perm = band_order(width, height)
        o, dt = o[perm], dt[perm]
    elif order != "rows":
        raise ValueError(order)
    return RayBatch(o, dt, np.full(n, -1, np.int32))


def hit_points_normals(mesh: Mesh, rays: RayBatch, hits: np.ndarray):
    """World hit points (float32, origin + t*dir rounded like the reference's
    'ray.origin + hit.t * ray.direction') and unit geometric normals facing the ray."""
    prim = hits[:, 3].view(np.int32)
    t = hits[:, 0]
    p = rays.origin_tmin[:, :3] + t[:, None] * rays.dir_tmax[:, :3]
    tri = mesh.positions[mesh.indices[np.maximum(prim, 0)]].astype(np.float64)
    n = _normalize(np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0]))
    flip = np.sum(n * rays.dir_tmax[:, :3], axis=1) > 0
    n[flip] *= -1
    return p.astype(F32), n, prim


def bounce_rays(points: np.ndarray, normals: np.ndarray, prims: np.ndarray, seed: int = 3) -> RayBatch:
    """Cosine-weighted hemisphere directions around each normal; last_prim = the hit primitive."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = points.shape[0]
    u1, u2 = rng.random(n), rng.random(n)
    r, phi = np.sqrt(u1), 2.0 * np.pi * u2
    local = np.stack([r * np.cos(phi), r * np.sin(phi), np.sqrt(np.maximum(0.0, 1.0 - u1))], axis=1)
    nn = normals.astype(np.float64)
    a = np.where(np.abs(nn[:, :1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = _normalize(np.cross(a, nn))
    b = np.cross(nn, t)
    d = _normalize(local[:, :1] * t + local[:, 1:2] * b + local[:, 2:3] * nn)
    o = np.empty((n, 4), F32)
    o[:, :3] = points
    o[:, 3] = 0.0
    dt = np.empty((n, 4), F32)
    dt[:, :3] = d.astype(F32)
    dt[:, 3] = np.inf
    return RayBatch(o, dt, prims.astype(np.int32))


def shadow_rays(points: np.ndarray, prims: np.ndarray, seed: int = 4, centre=(0.0, 2.0, 0.0),
                size: float = 0.5):
    """Rays from each point to a uniform point on a size x size quad (normal -y) at 'centre'.
    Returns (batch, light_distance): batch.dir_tmax[:, 3] = light_distance - 1e-4 (float32)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n = points.shape[0]
    lp = np.empty((n, 3))
    lp[:, 0] = centre[0] + (rng.random(n) - 0.5) * size
    lp[:, 1] = centre[1]
    lp[:, 2] = centre[2] + (rng.random(n) - 0.5) * size
    v = lp - points.astype(np.float64)
    dist = np.linalg.norm(v, axis=1)
    d = v / dist[:, None]
    o = np.empty((n, 4), F32)
    o[:, :3] = points
    o[:, 3] = 0.0
    dt = np.empty((n, 4), F32)
    dt[:, :3] = d.astype(F32)
    dist32 = dist.astype(F32)
    dt[:, 3] = dist32 - F32(1.0e-4)
    return RayBatch(o, dt, prims.astype(np.int32)), dist32


# ---------------------------------------------------------------------------------------------
# Cornell box (the reference-CPU-runnable path-tracing scene)
# ---------------------------------------------------------------------------------------------
CORNELL_WHITE = (0.73, 0.73, 0.73)
CORNELL_RED = (0.63, 0.065, 0.05)
CORNELL_GREEN = (0.14, 0.45, 0.09)
CORNELL_LIGHT_EMISSION = (17.0, 12.0, 4.0)


@dataclass
class CornellBox:
    mesh: Mesh
    material_of_triangle: np.ndarray  # (T,) int32 index into albedo/emission
    albedo: np.ndarray  # (M, 3) float32
    emission: np.ndarray  # (M, 3) float32
    emissive_triangles: np.ndarray  # (E,) int32


def _quad(p0, p1, p2, p3):
    """Two triangles (p0,p1,p2), (p0,p2,p3)."""
    return [p0, p1, p2, p0, p2, p3]


def _box(size, angle_deg, base_centre):
    sx, sy, sz = size
    c, s = np.cos(np.radians(angle_deg)), np.sin(np.radians(angle_deg))
    corners = []
    for y in (0.0, sy):
        for (x, z) in ((-sx / 2, -sz / 2), (sx / 2, -sz / 2), (sx / 2, sz / 2), (-sx / 2, sz / 2)):
            corners.append((base_centre[0] + c * x + s * z, base_centre[1] + y, base_centre[2] - s * x + c * z))
    b = corners[:4]
    t = corners[4:]
    tris = []
    tris += _quad(b[0], b[3], b[2], b[1])  # bottom
    tris += _quad(t[0], t[1], t[2], t[3])  # top
    for i in range(4):
        j = (i + 1) % 4
        tris += _quad(b[i], b[j], t[j], t[i])
    return tris


def cornell_box() -> CornellBox:
    """The 36-triangle Cornell box inside [0, 5.5]^3, open towards -z.

    Five wall quads (10 triangles): floor y=0, ceiling y=5.5, back z=5.5 (white 0.73); red wall at
    x=5.5 and green wall at x=0 (the red wall is on the left of the image seen from the camera at
    (2.75, 2.75, -8) looking +z). Two boxes (12 triangles each): 1.65^3 rotated -18 degrees about y
    at (1.85, 0, 1.69), 1.65 x 3.3 x 1.65 rotated 15 degrees at (3.68, 0, 3.51). Area light: a
    1.3 x 1.05 quad centred at (2.75, 5.49, 2.75) facing down, emission (17, 12, 4).
    """
    L = 5.5
    tris, mats = [], []

    def add(ts, m):
        tris.extend(ts)
        mats.extend([m] * (len(ts) // 3))

    add(_quad((0, 0, 0), (0, 0, L), (L, 0, L), (L, 0, 0)), 0)  # floor
    add(_quad((0, L, 0), (L, L, 0), (L, L, L), (0, L, L)), 0)  # ceiling
    add(_quad((0, 0, L), (0, L, L), (L, L, L), (L, 0, L)), 0)  # back
    add(_quad((L, 0, 0), (L, 0, L), (L, L, L), (L, L, 0)), 1)  # red (x = 5.5)
    add(_quad((0, 0, 0), (0, L, 0), (0, L, L), (0, 0, L)), 2)  # green (x = 0)
    add(_box((1.65, 1.65, 1.65), -18.0, (1.85, 0.0, 1.69)), 0)
    add(_box((1.65, 3.3, 1.65), 15.0, (3.68, 0.0, 3.51)), 0)
    hx, hz, ly = 1.3 / 2, 1.05 / 2, 5.49
    add(_quad((2.75 - hx, ly, 2.75 - hz), (2.75 + hx, ly, 2.75 - hz), (2.75 + hx, ly, 2.75 + hz),
              (2.75 - hx, ly, 2.75 + hz)), 3)
    pos = np.asarray(tris, np.float64).astype(F32)
    idx = np.arange(pos.shape[0], dtype=np.int32).reshape(-1, 3)
    albedo = np.asarray([CORNELL_WHITE, CORNELL_RED, CORNELL_GREEN, (0.0, 0.0, 0.0)], F32)
    emission = np.asarray([(0, 0, 0), (0, 0, 0), (0, 0, 0), CORNELL_LIGHT_EMISSION], F32)
    mat = np.asarray(mats, np.int32)
    return CornellBox(Mesh(pos, idx), mat, albedo, emission, np.nonzero(mat == 3)[0].astype(np.int32))


def uv_sphere(centre, radius: float, n_lat: int = 8, n_lon: int = 16):
    """A latitude/longitude sphere: (Mesh, (V, 3) outward unit vertex normals). Coarse on purpose:
    shaded with its vertex normals it looks round, with its geometric normals faceted."""
    c = np.asarray(centre, np.float64)
    th = np.linspace(0.0, np.pi, n_lat + 1)
    ph = np.linspace(0.0, 2.0 * np.pi, n_lon + 1)
    dirs = np.stack([np.sin(th)[:, None] * np.cos(ph)[None, :], np.repeat(np.cos(th)[:, None], n_lon + 1, 1),
                     np.sin(th)[:, None] * np.sin(ph)[None, :]], -1).reshape(-1, 3)
    pos = (c + radius * dirs).astype(F32)
    tris = []
    for i in range(n_lat):
        for j in range(n_lon):
            a, b = i * (n_lon + 1) + j, i * (n_lon + 1) + j + 1
            cc, d = a + n_lon + 1, b + n_lon + 1
            if i > 0:
                tris.append((a, b, cc))  # outward winding
            if i < n_lat - 1:
                tris.append((b, d, cc))
    idx = np.asarray(tris, np.int32)
    return Mesh(pos, idx), (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(F32)


@dataclass
class SmoothScene:
    mesh: Mesh
    material_of_triangle: np.ndarray  # (T,) int32
    albedo: np.ndarray                # (M, 3)
    emission: np.ndarray              # (M, 3)
    vertex_normals: np.ndarray        # (V, 3): zero on the box, the sphere normals on the spheres

    def corner_normals(self) -> np.ndarray:
        """(T, 3, 3) normals at each triangle's corners (the oracle's layout)."""
        return np.ascontiguousarray(self.vertex_normals[self.mesh.indices])


def smooth_cornell() -> SmoothScene:
    """The Cornell box's walls and light (flat shading: zero vertex normals) with two coarse
    spheres shaded by their vertex normals in place of the boxes: a white one (material 0) of
    radius 1.1 at (1.85, 1.1, 1.69) and one of material 4 (a fifth material, white) of radius 1.3
    at (3.68, 1.3, 3.51)."""
    cb = cornell_box()
    keep = np.r_[0:10, 34:36]  # walls and light
    walls = Mesh(cb.mesh.positions[cb.mesh.indices[keep]].reshape(-1, 3),
                 np.arange(3 * len(keep), dtype=np.int32).reshape(-1, 3))
    s1, n1 = uv_sphere((1.85, 1.1, 1.69), 1.1)
    s2, n2 = uv_sphere((3.68, 1.3, 3.51), 1.3, n_lat=10, n_lon=20)
    mesh = merge(walls, s1, s2)
    mat = np.concatenate([cb.material_of_triangle[keep], np.zeros(s1.n_triangles, np.int32),
                          np.full(s2.n_triangles, 4, np.int32)])
    albedo = np.concatenate([cb.albedo, [[0.8, 0.8, 0.8]]]).astype(F32)
    emission = np.concatenate([cb.emission, [[0.0, 0.0, 0.0]]]).astype(F32)
    normals = np.concatenate([np.zeros((walls.positions.shape[0], 3), F32), n1, n2])
    return SmoothScene(mesh, mat, albedo, emission, normals)


def envmap_directions(width: int, height: int) -> np.ndarray:
    """World direction (identity rotation) of each texel centre of an equirectangular envmap, as the
    reference maps (u, v): phi = 2 pi u, theta = pi v, d = (-sin theta cos phi, -cos theta,
    -sin theta sin phi); row 0 is the -y pole. Returns (height, width, 3) float64."""
    u = (np.arange(width) + 0.5) / width
    v = (np.arange(height) + 0.5) / height
    phi = 2.0 * np.pi * u[None, :]
    theta = np.pi * v[:, None]
    return np.stack([-np.sin(theta) * np.cos(phi), -np.cos(theta) * np.ones_like(phi), -np.sin(theta) * np.sin(phi)],
                    axis=-1)


def sky_envmap(width: int = 64, height: int = 32, sun_dir=(0.35, 0.6, -0.72), sun_radius_deg: float = 8.0,
               sun_radiance=(30.0, 26.0, 20.0), seed: int = 1) -> np.ndarray:
    """Seeded synthetic outdoor envmap (height, width, 3) float32: a blue sky brightening towards
    the horizon, a dim brown ground below it, a warm sun disc of sun_radius_deg around sun_dir
    covering a few texels, and +-10% seeded texel noise."""
    d = envmap_directions(width, height)
    y = d[..., 1]
    sky = np.stack([0.25 + 0.35 * (1 - y), 0.45 + 0.3 * (1 - y), 0.9 + 0.1 * (1 - y)], -1) * (y >= 0)[..., None]
    ground = np.array([0.12, 0.09, 0.06]) * (y < 0)[..., None]
    sd = np.asarray(sun_dir, np.float64)
    sd = sd / np.linalg.norm(sd)
    sun = (d @ sd > np.cos(np.radians(sun_radius_deg)))[..., None] * np.asarray(sun_radiance)
    rng = np.random.Generator(np.random.PCG64(seed))
    img = (sky + ground + sun) * rng.uniform(0.9, 1.1, (height, width, 1))
    return img.astype(F32)


@dataclass
class ManyLightScene:
    mesh: Mesh
    material_of_triangle: np.ndarray  # (T,) int32
    materials: np.ndarray             # (M, 64) principled records (gbpt.materials layout)
    n_emitters: int
    box: tuple                        # scene bounds (lo xyz, hi xyz)
    eye: tuple                        # camera at frame 0 (orbits about the y axis through target)
    target: tuple
    vfov_deg: float


def many_light_scene(tile_cells: int = 128, grid=(32, 16), n_emitters: int = 10_000, seed: int = 1,
                     spacing: float = 2.0) -> ManyLightScene:
    """The many-light principled scene: grid[0] x grid[1] instances of a tile_cells^2-cell fBm
    heightfield tile (amplitude 0.2, 6 octaves, over [-1, 1]^2: the traversal scene's heightfield at
    a lower resolution), each rotated about y by U[0, 2 pi) and centred on a spacing-wide grid cell,
    flattened; one random principled material per instance (gbpt.materials.random_principled);
    n_emitters emissive triangles of side 0.05 (equilateral, facing down within 60 degrees of -y),
    centres uniform over the grid in x/z at U[0.1, 1.0] above the surface, radiance log-uniform in
    [1, 1000] times a colour U[0.2, 1]^3, one material each. Defaults: 512 x 32,768 = 16,777,216
    triangles + 10,000 emitters."""
    from . import materials as M
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    tile = heightfield(tile_cells, 0.2, seed, 6)
    nx, nz = grid
    n_inst = nx * nz
    ang = rng.uniform(0.0, 2.0 * np.pi, n_inst)
    cx = (np.arange(nx) - (nx - 1) / 2.0) * spacing
    cz = (np.arange(nz) - (nz - 1) / 2.0) * spacing
    centres = np.stack(np.meshgrid(cx, cz, indexing="xy"), -1).reshape(-1, 2)  # instance k = j * nx + i
    tp = tile.positions.astype(np.float64)
    c, s = np.cos(ang)[:, None], np.sin(ang)[:, None]
    X = c * tp[None, :, 0] + s * tp[None, :, 2] + centres[:, :1]
    Z = -s * tp[None, :, 0] + c * tp[None, :, 2] + centres[:, 1:]
    Y = np.broadcast_to(tp[None, :, 1], X.shape)
    pos = np.stack([X, Y, Z], -1).reshape(-1, 3)
    nv = tp.shape[0]
    idx = (tile.indices[None, :, :] + (np.arange(n_inst) * nv)[:, None, None]).reshape(-1, 3)
    mat_of = np.repeat(np.arange(n_inst, dtype=np.int32), tile.indices.shape[0])

    # emitters: surface height from the owning instance's fBm (local coordinates clamped to the tile)
    ex = rng.uniform(cx[0] - spacing / 2, cx[-1] + spacing / 2, n_emitters)
    ez = rng.uniform(cz[0] - spacing / 2, cz[-1] + spacing / 2, n_emitters)
    ii = np.clip(np.round((ex - cx[0]) / spacing).astype(int), 0, nx - 1)
    jj = np.clip(np.round((ez - cz[0]) / spacing).astype(int), 0, nz - 1)
    k = jj * nx + ii
    dx, dz = ex - centres[k, 0], ez - centres[k, 1]
    lx = np.clip(np.cos(ang[k]) * dx - np.sin(ang[k]) * dz, -1, 1)
    lz = np.clip(np.sin(ang[k]) * dx + np.cos(ang[k]) * dz, -1, 1)
    ground = 0.2 * value_noise_fbm(lx, lz, seed=seed, octaves=6)
    ey = ground + rng.uniform(0.1, 1.0, n_emitters)
    # equilateral triangle of side 0.05 in a plane whose normal is within 60 degrees of -y
    theta = np.arccos(rng.uniform(np.cos(np.radians(60.0)), 1.0, n_emitters))
    phi = rng.uniform(0, 2 * np.pi, n_emitters)
    nrm = np.stack([np.sin(theta) * np.cos(phi), -np.cos(theta), np.sin(theta) * np.sin(phi)], -1)
    a = np.where(np.abs(nrm[:, :1]) < 0.9, np.array([[1.0, 0, 0]]), np.array([[0.0, 0, 1]]))
    u = _normalize(np.cross(nrm, a))
    v = np.cross(nrm, u)
    r = 0.05 / np.sqrt(3.0)  # circumradius
    beta = rng.uniform(0, 2 * np.pi, n_emitters)[:, None]
    corners = []
    for q in range(3):
        t = beta + q * 2.0 * np.pi / 3.0
        corners.append(np.stack([ex, ey, ez], -1) + r * (np.cos(t) * u + np.sin(t) * v))
    # winding so that the geometric normal (b - a) x (c - a) is nrm
    tri = np.stack([corners[0], corners[2], corners[1]], 1)
    g = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    flip = (g * nrm).sum(-1) < 0
    tri[flip] = tri[flip][:, [0, 2, 1]]
    e_pos = tri.reshape(-1, 3)
    e_idx = np.arange(3 * n_emitters).reshape(-1, 3) + pos.shape[0]
    rad = np.exp(rng.uniform(0.0, np.log(1000.0), n_emitters))[:, None] * rng.uniform(0.2, 1.0, (n_emitters, 3))

    mats = M.pack_many(M.random_principled(rng, n_inst))
    emat = np.stack([M.pack(base_color=(0.0, 0.0, 0.0), emission=tuple(float(x) for x in e)) for e in rad])
    mesh = Mesh(np.concatenate([pos, e_pos]).astype(F32), np.concatenate([idx, e_idx]).astype(np.int32))
    mat_of = np.concatenate([mat_of, n_inst + np.arange(n_emitters, dtype=np.int32)])
    lo = tuple(float(x) for x in mesh.positions.min(0))
    hi = tuple(float(x) for x in mesh.positions.max(0))
    return ManyLightScene(mesh, mat_of, np.concatenate([mats, emat]).astype(F32), n_emitters, (lo, hi),
                          eye=(0.0, 7.0, -26.0), target=(0.0, 0.0, 0.0), vfov_deg=45.0)
