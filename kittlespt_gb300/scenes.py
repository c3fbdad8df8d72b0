"""Seeded synthetic scenes for the path-tracing workloads.

The reference ships no scene files (its SampleApp loads glTF files that are not
in its repository), so every workload here is procedural.  All generators are
numpy-only and deterministic for a given seed (PCG64).

Conventions follow the reference renderer:

* matrices are column-major ``Mat4`` (``KittlesPT/src/maths/matrix_maths.cuh:172``);
  numpy arrays here are ``M[row, col]`` and are flattened with ``M.T`` when
  they cross the C boundary;
* the camera is given by its inverse projection and inverse view matrices
  (``Camera::setView(inv_proj, inv_view)``, ``shaders/camera.cuh:28-36``); the
  inverse view has columns ``[right, up, forward, position]`` like the
  SampleApp camera (``SampleApp/src/sample_app/camera_controller.cpp:85-97``),
  and the projection is a left-handed perspective
  (``renderer.cu:81-83``);
* a mesh is a list of triangles with per-vertex position, normal and uv and a
  per-triangle material id (``pod_types.hpp:125-147``); an instance places a
  mesh with a model matrix and may override its material.
"""

from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

F32 = np.float32

# Reference defaults: pod_types.hpp:37-57 and atmosphere.cuh:292-310.
DEFAULT_SUN_ANGULAR_DIAMETER = 0.0087
DEFAULT_SUN_PHI = 4.18879
DEFAULT_SUN_THETA = math.radians(17.0)
RAYLEIGH_SIGMA_S = (3.8e-6, 13.5e-6, 33.1e-6)
MIE_SIGMA_S = 21e-6
MIE_SIGMA_A = 21e-6 * 0.1
RAYLEIGH_SCALE_HEIGHT = 7994.0
MIE_SCALE_HEIGHT = 1200.0

MATERIAL_DTYPE = np.dtype([
    ("albedo", F32, 3), ("metallic", F32), ("roughness", F32),
    ("transmission", F32), ("ior", F32), ("emission", F32, 3),
    ("emission_scale", F32), ("normal_scale", F32),
    ("albedo_tex", np.int32), ("orm_tex", np.int32),
    ("transmission_tex", np.int32), ("emission_tex", np.int32),
    ("normal_tex", np.int32), ("pad", np.int32),
])
assert MATERIAL_DTYPE.itemsize == 72

ENV_DTYPE = np.dtype([
    ("sun_angular_diameter", F32), ("sun_phi", F32), ("sun_theta", F32),
    ("sun_emission_factor", F32), ("rayleigh", F32, 3), ("mie", F32),
    ("mie_absorption", F32), ("rayleigh_height", F32), ("mie_height", F32),
    ("pad", F32),
])
assert ENV_DTYPE.itemsize == 48

SETTINGS_DTYPE = np.dtype([
    ("max_depth", np.int32), ("bloom", np.int32), ("karis", np.int32),
    ("auto_exposure", np.int32), ("bloom_final_blend", F32),
    ("bloom_internal_blend", F32), ("frame_delta_ms", F32), ("pad", F32),
])
assert SETTINGS_DTYPE.itemsize == 32

EXPOSURE_DTYPE = np.dtype([
    ("aperture", F32), ("iso", F32), ("shutter", F32), ("ev_comp", F32),
    ("white_ev", F32), ("black_ev", F32), ("max_iso", F32), ("min_iso", F32),
    ("max_shutter", F32), ("min_shutter", F32), ("pad0", F32), ("pad1", F32),
])
assert EXPOSURE_DTYPE.itemsize == 48


def material(albedo=(0.8, 0.8, 0.8), metallic=0.0, roughness=0.5,
             transmission=0.0, ior=1.45, emission=(0.0, 0.0, 0.0),
             emission_scale=1.0):
    """One material record; defaults are the device ``Material`` defaults
    (``shaders/material.cuh:56-74``)."""
    m = np.zeros((), MATERIAL_DTYPE)
    m["albedo"] = albedo
    m["metallic"] = metallic
    m["roughness"] = roughness
    m["transmission"] = transmission
    m["ior"] = ior
    m["emission"] = emission
    m["emission_scale"] = emission_scale
    m["normal_scale"] = 1.0
    for k in ("albedo_tex", "orm_tex", "transmission_tex", "emission_tex", "normal_tex"):
        m[k] = -1
    return m


def environment(sun_theta=DEFAULT_SUN_THETA, sun_phi=DEFAULT_SUN_PHI,
                sun_angular_diameter=DEFAULT_SUN_ANGULAR_DIAMETER,
                sun_emission_factor=1.0, rayleigh=RAYLEIGH_SIGMA_S,
                mie=MIE_SIGMA_S, mie_absorption=MIE_SIGMA_A,
                rayleigh_height=RAYLEIGH_SCALE_HEIGHT, mie_height=MIE_SCALE_HEIGHT):
    e = np.zeros((), ENV_DTYPE)
    e["sun_angular_diameter"] = sun_angular_diameter
    e["sun_phi"] = sun_phi
    e["sun_theta"] = sun_theta
    e["sun_emission_factor"] = sun_emission_factor
    e["rayleigh"] = rayleigh
    e["mie"] = mie
    e["mie_absorption"] = mie_absorption
    e["rayleigh_height"] = rayleigh_height
    e["mie_height"] = mie_height
    return e


def settings(max_depth=3, bloom=False, karis=False, auto_exposure=False,
             bloom_final_blend=0.175, bloom_internal_blend=0.65,
             frame_delta_ms=16.0):
    """Renderer settings; defaults follow ``RendererSettings``
    (``pod_types.hpp:46-57``)."""
    s = np.zeros((), SETTINGS_DTYPE)
    s["max_depth"] = max_depth
    s["bloom"] = int(bloom)
    s["karis"] = int(karis)
    s["auto_exposure"] = int(auto_exposure)
    s["bloom_final_blend"] = bloom_final_blend
    s["bloom_internal_blend"] = bloom_internal_blend
    s["frame_delta_ms"] = frame_delta_ms
    return s


def exposure(aperture=11.0, iso=100.0, shutter=0.004, ev_comp=0.0,
             white_ev=6.5, black_ev=-10.0, max_iso=6400.0, min_iso=100.0,
             max_shutter=1.0 / 30.0, min_shutter=1.0 / 400.0):
    """Camera exposure state; defaults are the SampleApp daytime preset
    (``SampleApp/src/sample_app/camera_controller.hpp:55-60``)."""
    x = np.zeros((), EXPOSURE_DTYPE)
    for k, v in dict(aperture=aperture, iso=iso, shutter=shutter, ev_comp=ev_comp,
                     white_ev=white_ev, black_ev=black_ev, max_iso=max_iso,
                     min_iso=min_iso, max_shutter=max_shutter,
                     min_shutter=min_shutter).items():
        x[k] = v
    return x


# ----------------------------------------------------------------------------
# matrices (float64 maths, stored as float32)

def translate(x, y, z):
    m = np.eye(4)
    m[:3, 3] = (x, y, z)
    return m


def scale(s):
    m = np.eye(4)
    m[0, 0] = m[1, 1] = m[2, 2] = s
    return m


def rot_y(a):
    c, s = math.cos(a), math.sin(a)
    m = np.eye(4)
    m[0, 0], m[0, 2], m[2, 0], m[2, 2] = c, s, -s, c
    return m


def perspective_fov_lh(fov_y, width, height, near, far):
    """Left-handed perspective with clip-space depth in [-1, 1]: the standard
    published formula the reference gets from its math library."""
    h = math.cos(0.5 * fov_y) / math.sin(0.5 * fov_y)
    w = h * height / width
    m = np.zeros((4, 4))
    m[0, 0] = w
    m[1, 1] = h
    m[2, 2] = (far + near) / (far - near)
    m[3, 2] = 1.0
    m[2, 3] = -(2.0 * far * near) / (far - near)
    return m


def look_at_inv_view(eye, target, world_up=(0.0, 1.0, 0.0)):
    """Inverse view with columns [right, up, forward, eye], the SampleApp
    convention (right = forward x up, up = right x forward)."""
    eye = np.asarray(eye, float)
    f = np.asarray(target, float) - eye
    f /= np.linalg.norm(f)
    r = np.cross(f, world_up)
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    u /= np.linalg.norm(u)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = r, u, f, eye
    return m


@dataclasses.dataclass
class Camera:
    inv_proj: np.ndarray     # (4,4) float32, M[row, col]
    inv_view: np.ndarray     # (4,4) float32

    @staticmethod
    def look_at(eye, target, fov_y_deg, width, height):
        proj = perspective_fov_lh(math.radians(fov_y_deg), width, height, 0.1, 100.0)
        return Camera(np.linalg.inv(proj).astype(F32),
                      look_at_inv_view(eye, target).astype(F32))


# ----------------------------------------------------------------------------
# geometry

@dataclasses.dataclass
class Mesh:
    positions: np.ndarray    # (T,3,3) float32
    normals: np.ndarray      # (T,3,3) float32
    uvs: np.ndarray          # (T,3,2) float32
    material: np.ndarray     # (T,) int32

    @property
    def ntris(self):
        return int(self.positions.shape[0])


def _mesh(pos, nrm, uv, mat_id=0):
    t = pos.shape[0]
    return Mesh(np.ascontiguousarray(pos, F32), np.ascontiguousarray(nrm, F32),
                np.ascontiguousarray(uv, F32), np.full(t, mat_id, np.int32))


def uv_sphere(slices=64, stacks=32, radius=1.0, mat_id=0):
    """UV sphere: one triangle per slice in each cap, two per slice in each
    of the stacks-2 middle bands (64x32 -> 3968 triangles)."""
    th = np.linspace(0.0, math.pi, stacks + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, slices + 1)
    T, P = np.meshgrid(th, ph, indexing="ij")
    n = np.stack([np.sin(T) * np.cos(P), np.cos(T), np.sin(T) * np.sin(P)], -1)
    uv = np.stack([P / (2 * math.pi), 1.0 - T / math.pi], -1)
    tris = []
    for i in range(stacks):
        for j in range(slices):
            a, b, c, d = (i, j), (i, j + 1), (i + 1, j), (i + 1, j + 1)
            if i != 0:
                tris.append((a, b, d))
            if i != stacks - 1:
                tris.append((a, d, c))
    idx = np.array(tris)                      # (T, 3, 2)
    nn = n[idx[..., 0], idx[..., 1]]
    return _mesh(nn * radius, nn, uv[idx[..., 0], idx[..., 1]], mat_id)


def quad(size_x, size_z, y=0.0, facing_up=True, mat_id=0):
    """Axis-aligned quad in the xz plane centred on the origin (2 triangles)."""
    hx, hz = 0.5 * size_x, 0.5 * size_z
    p = np.array([[-hx, y, -hz], [hx, y, -hz], [hx, y, hz], [-hx, y, hz]])
    uv = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], float)
    tri = [(0, 2, 1), (0, 3, 2)] if facing_up else [(0, 1, 2), (0, 2, 3)]
    pos = np.stack([p[list(t)] for t in tri])
    e1, e2 = pos[:, 1] - pos[:, 0], pos[:, 2] - pos[:, 0]
    n = np.cross(e1, e2)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    nrm = np.repeat(n[:, None, :], 3, 1)
    uvs = np.stack([uv[list(t)] for t in tri])
    return _mesh(pos, nrm, uvs, mat_id)


def _icosahedron():
    t = (1.0 + math.sqrt(5.0)) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    return v, f


def _subdivide(v, f):
    edge = {}
    verts = list(v)

    def mid(a, b):
        k = (a, b) if a < b else (b, a)
        if k not in edge:
            p = verts[a] + verts[b]
            verts.append(p / np.linalg.norm(p))
            edge[k] = len(verts) - 1
        return edge[k]

    nf = []
    for a, b, c in f:
        ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
        nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
    return np.array(verts), np.array(nf)


def value_noise3(p, seed, freq=4.0):
    """Seeded 3-D value noise in [-1, 1]: random lattice values, trilinear
    interpolation with a smoothstep fade."""
    rng = np.random.Generator(np.random.PCG64(seed))
    table = rng.uniform(-1.0, 1.0, 4096)
    perm = rng.permutation(4096)
    q = p * freq
    i0 = np.floor(q).astype(np.int64)
    fr = q - i0
    fr = fr * fr * (3.0 - 2.0 * fr)

    def lat(ix, iy, iz):
        h = perm[(ix * 73856093 ^ iy * 19349663 ^ iz * 83492791) % 4096]
        return table[h]

    out = 0.0
    for dx in (0, 1):
        wx = fr[:, 0] if dx else 1.0 - fr[:, 0]
        for dy in (0, 1):
            wy = fr[:, 1] if dy else 1.0 - fr[:, 1]
            for dz in (0, 1):
                wz = fr[:, 2] if dz else 1.0 - fr[:, 2]
                out = out + wx * wy * wz * lat(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
    return out


def displaced_icosphere(subdiv=6, amplitude=0.1, seed=0, mat_id=0):
    """Icosphere (20 * 4**subdiv triangles) displaced along the normal by
    seeded value noise of the given amplitude."""
    v, f = _icosahedron()
    for _ in range(subdiv):
        v, f = _subdivide(v, f)
    d = amplitude * value_noise3(v, seed)
    p = v * (1.0 + d)[:, None]
    # smooth vertex normals of the displaced surface (area weighted)
    fn = np.cross(p[f[:, 1]] - p[f[:, 0]], p[f[:, 2]] - p[f[:, 0]])
    vn = np.zeros_like(p)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    vn /= np.linalg.norm(vn, axis=1, keepdims=True)
    uv = np.stack([0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * math.pi),
                   0.5 + np.arcsin(np.clip(v[:, 1], -1, 1)) / math.pi], -1)
    return _mesh(p[f], vn[f], uv[f], mat_id)


# ----------------------------------------------------------------------------
# scenes

@dataclasses.dataclass
class Instance:
    mesh: int
    model: np.ndarray                 # (4,4) float32
    material: int = -1                # -1: use the mesh's per-triangle ids


@dataclasses.dataclass
class Scene:
    meshes: List[Mesh]
    instances: List[Instance]
    materials: np.ndarray             # MATERIAL_DTYPE array
    camera: Camera
    env: np.ndarray
    settings: np.ndarray
    exposure: np.ndarray
    width: int
    height: int
    spp: int
    name: str = ""
    # 8-bit textures (TextureSceneEntity, pod_types.hpp): [h, w, channels] uint8 each
    textures: List[np.ndarray] = dataclasses.field(default_factory=list)
    # arithmetic of the sky and the sun's constants (kpt_settings.sky_arith):
    # 0 IEEE single precision, as the oracle and the reference's host build
    # compute them; 1 that of the reference's GPU build
    sky_arith: int = 0
    # arithmetic of the temporal reprojection (kpt_settings.temporal_arith):
    # 0 IEEE, as the oracle restates it; 1 that of the reference's GPU build
    temporal_arith: int = 0

    def texture_arrays(self):
        """(desc int32 [n, 4] = width, height, channels, byte offset; pixels
        uint8) as kpt_set_textures takes them."""
        desc = np.zeros((len(self.textures), 4), np.int32)
        off = 0
        for k, t in enumerate(self.textures):
            h, w, ch = t.shape
            desc[k] = (w, h, ch, off)
            off += t.size
        pix = (np.concatenate([np.ascontiguousarray(t, np.uint8).reshape(-1) for t in self.textures])
               if self.textures else np.zeros(1, np.uint8))
        return desc, pix

    @property
    def ntris_expanded(self):
        return sum(self.meshes[i.mesh].ntris for i in self.instances)

    def expanded(self):
        """The scene with every instance turned into its own mesh, the
        reference's layout (it has no instancing: one mesh = one BLAS with its
        own triangle copies, ``renderer.cu:386-417``)."""
        pos, nrm, uv, mat, tri_off, tri_cnt, models = [], [], [], [], [], [], []
        off = 0
        for inst in self.instances:
            m = self.meshes[inst.mesh]
            pos.append(m.positions)
            nrm.append(m.normals)
            uv.append(m.uvs)
            mat.append(np.full(m.ntris, inst.material, np.int32)
                       if inst.material >= 0 else m.material)
            tri_off.append(off)
            tri_cnt.append(m.ntris)
            models.append(inst.model)
            off += m.ntris
        return dict(positions=np.ascontiguousarray(np.concatenate(pos), F32),
                    normals=np.ascontiguousarray(np.concatenate(nrm), F32),
                    uvs=np.ascontiguousarray(np.concatenate(uv), F32),
                    material=np.ascontiguousarray(np.concatenate(mat), np.int32),
                    mesh_offset=np.array(tri_off, np.int32),
                    mesh_count=np.array(tri_cnt, np.int32),
                    models=np.ascontiguousarray(np.stack(models), F32))


def scene_small(width=256, height=256, spp=1, max_depth=4, seed=1):
    """Small plain-method scene: a 64x32 UV sphere (radius 1) as one mesh with
    two instances at x = -1.5 (diffuse albedo 0.8) and x = +1.5 (GGX
    conductor, roughness 0.3, F0 (0.95, 0.64, 0.54)) over a 20x20 ground quad
    at y = -1; pinhole camera at (0,1,5) looking at the origin with a 45 deg
    vertical field of view; Nishita sky with the sun 30 deg above the
    horizon.  The diffuse material is the reference's opaque dielectric
    (GGX glossy + Lambert) at its default roughness 0.5 and the ground is a
    grey (0.5) opaque dielectric."""
    mats = np.stack([
        material(albedo=(0.8, 0.8, 0.8), roughness=0.5),
        material(albedo=(0.95, 0.64, 0.54), metallic=1.0, roughness=0.3),
        material(albedo=(0.5, 0.5, 0.5), roughness=0.5),
    ])
    meshes = [uv_sphere(64, 32, 1.0, 0), quad(20.0, 20.0, 0.0, True, 2)]
    inst = [Instance(0, translate(-1.5, 0, 0).astype(F32), 0),
            Instance(0, translate(1.5, 0, 0).astype(F32), 1),
            Instance(1, translate(0, -1.0, 0).astype(F32), 2)]
    cam = Camera.look_at((0.0, 1.0, 5.0), (0.0, 0.0, 0.0), 45.0, width, height)
    return Scene(meshes, inst, mats, cam,
                 environment(sun_theta=math.radians(30.0)),
                 settings(max_depth=max_depth), exposure(), width, height, spp,
                 name="sphere_pair_256")


# Value-noise seeds of the five icosphere variants of the full-frame scene.
# Among seeds 1000-1999 these are the first five whose subdivision-6 mesh
# gets a BLAS (binned SAH, leaves of at most 8 triangles) with no interior
# node deeper than 14: the reference's traversal keeps 16-entry stacks
# (shaders/blas.cuh:37, shaders/tlas.cuh:10) and pushes both children of an
# interior node of depth d onto at most d pending entries, so these trees
# never overflow them.  Most seeds give depth 15.
FULL_FRAME_VARIANT_SEEDS = (1019, 1081, 1160, 1232, 1321)


def scene_full(width=1920, height=1080, spp=16, max_depth=8, seed=2,
               n_variants=5, subdiv=6, grid=8, n_lights=16, variant_seeds=None):
    """Full-frame plain-method scene: 5 displaced icospheres (subdivision 6,
    81,920 triangles each, value-noise amplitude 0.1), 64 instances on an 8x8
    grid with spacing 3, random yaw U(0, 2pi) and scale U(0.5, 1.5),
    per-instance material drawn from {opaque dielectric, transparent
    dielectric IOR 1.5, conductor} with roughness U(0.05, 1) and albedo
    U(0.1, 0.9)^3; 16 downward-facing emissive 0.5x0.5 quads of radiance 20
    on a 4x4 grid at height 3; Nishita sky and sun (default sun angles);
    post chain with 6-level bloom, auto exposure and AgX.  The camera sits at
    (0, 4, 22) looking at (0, 1, 0) with a 45 deg field of view, so that the
    upper part of the frame shows the sky above the horizon.  The variants'
    noise seeds are ``variant_seeds`` (default FULL_FRAME_VARIANT_SEEDS)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    vs = FULL_FRAME_VARIANT_SEEDS if variant_seeds is None else variant_seeds
    meshes = [displaced_icosphere(subdiv, 0.1, seed=vs[k]) for k in range(n_variants)]
    meshes.append(quad(0.5, 0.5, 0.0, facing_up=False, mat_id=0))
    light_mesh = len(meshes) - 1
    mats = []
    inst = []
    half = (grid - 1) / 2.0
    for gi in range(grid):
        for gj in range(grid):
            kind = int(rng.integers(0, 3))
            rough = float(rng.uniform(0.05, 1.0))
            alb = tuple(float(a) for a in rng.uniform(0.1, 0.9, 3))
            if kind == 0:
                mats.append(material(albedo=alb, roughness=rough))
            elif kind == 1:
                mats.append(material(albedo=alb, roughness=rough, transmission=1.0, ior=1.5))
            else:
                mats.append(material(albedo=alb, roughness=rough, metallic=1.0))
            yaw = float(rng.uniform(0.0, 2.0 * math.pi))
            s = float(rng.uniform(0.5, 1.5))
            v = int(rng.integers(0, n_variants))
            model = translate((gi - half) * 3.0, 0.0, (gj - half) * 3.0) @ rot_y(yaw) @ scale(s)
            inst.append(Instance(v, model.astype(F32), len(mats) - 1))
    mats.append(material(albedo=(0.8, 0.8, 0.8), emission=(1.0, 1.0, 1.0), emission_scale=20.0))
    lmat = len(mats) - 1
    lg = int(round(math.sqrt(n_lights)))
    for li in range(lg):
        for lj in range(lg):
            model = translate((li - (lg - 1) / 2.0) * 6.0, 3.0, (lj - (lg - 1) / 2.0) * 6.0)
            inst.append(Instance(light_mesh, model.astype(F32), lmat))
    cam = Camera.look_at((0.0, 4.0, 22.0), (0.0, 1.0, 0.0), 45.0, width, height)
    return Scene(meshes, inst, np.stack(mats), cam, environment(),
                 settings(max_depth=max_depth, bloom=True, auto_exposure=True),
                 exposure(), width, height, spp, name="icosphere_grid_1080p")


def random_triangles(n=2_000_000, seed=3, mu=-5.0, sigma=0.5):
    """n triangles with centroids uniform in the unit cube and vertices at the
    centroid plus edge vectors of log-normal length (mu, sigma) in uniform
    random directions."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(0.0, 1.0, (n, 1, 3))
    d = rng.normal(size=(n, 3, 3))
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    ln = rng.lognormal(mu, sigma, (n, 3, 1))
    pos = (c + d * ln).astype(F32)
    e1, e2 = pos[:, 1] - pos[:, 0], pos[:, 2] - pos[:, 0]
    g = np.cross(e1.astype(np.float64), e2.astype(np.float64))
    g /= np.maximum(np.linalg.norm(g, axis=1, keepdims=True), 1e-30)
    nrm = np.repeat(g[:, None, :], 3, 1).astype(F32)
    uv = np.zeros((n, 3, 2), F32)
    return Mesh(pos, nrm, uv, np.zeros(n, np.int32))


def random_rays(n=1_048_576, seed=4, center=(0.5, 0.5, 0.5), radius=None):
    """Origins uniform on the bounding sphere of the unit cube, directions
    uniform on the unit sphere (incoherent)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    if radius is None:
        radius = math.sqrt(3.0) / 2.0 + 1e-3
    o = rng.normal(size=(n, 3))
    o /= np.linalg.norm(o, axis=1, keepdims=True)
    o = np.asarray(center) + radius * o
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(F32), d.astype(F32)


def scene_traversal(ntris=2_000_000, seed=3):
    """Traversal stress scene: one BLAS of random triangles, identity
    instance."""
    mesh = random_triangles(ntris, seed)
    mats = np.stack([material()])
    cam = Camera.look_at((0.5, 0.5, 3.0), (0.5, 0.5, 0.5), 45.0, 64, 64)
    return Scene([mesh], [Instance(0, np.eye(4, dtype=F32), 0)], mats, cam,
                 environment(), settings(), exposure(), 64, 64, 1,
                 name="random_tris")


def scene_small_n(width, height, spp, max_depth, n_instances, seed=11):
    """Variant of the small scene with n sphere instances (for batched
    jobs)."""
    sc = scene_small(width, height, spp, max_depth)
    rng = np.random.Generator(np.random.PCG64(seed))
    inst = [sc.instances[-1]]
    for k in range(n_instances):
        x, z = rng.uniform(-6, 6), rng.uniform(-6, 2)
        inst.append(Instance(0, translate(x, 0, z).astype(F32), int(rng.integers(0, 2))))
    sc.instances = inst
    return sc
