"""Generates the golden fixtures in this directory from the reference's own
code compiled for the host (oracle/_ref/libkpt_ref_host.so, built by
oracle/build_ref.sh from the reference source tree).

The reference ships no tests or golden vectors, so these fixtures are the
pin for the CPU oracle: tests/test_oracle_golden.py checks that the oracle
reproduces every array here bit for bit.  The right-to-left RNG argument order
of this host build (g++), all three unspecified-order call sites right to
left, is recorded as rng_order=7.

Run from the repository root:  python tests/golden/make_golden.py
"""

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from kittlespt_gb300 import scenes as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def bvh_digest(sc):
    b = sc.bvh()
    return digest(b["left_first"], b["count"], b["bounds"], b["tri_index"], b["blas_root"],
                  b["blas_bounds"], b["blas_inv"], b["tlas_lr"], b["tlas_blas"], b["tlas_bounds"])


def small_scene():
    return S.scene_small(48, 48, 2, 4)


def full_scene():
    return S.scene_full(64, 36, 2, 8, n_variants=2, subdiv=3, grid=3, n_lights=4, variant_seeds=(1000, 1001))


def traversal_scene():
    return S.scene_traversal(20000)


def textured_scene():
    """The small scene with every texture slot of the material in use
    (Material::getBSDF and Texture::evaluate, material.cu:17-70,
    texture.cuh:34-66; Light::L, light.cu:21-33): an sRGB albedo texture and
    a normal map on the diffuse sphere, an occlusion-roughness-metallic
    texture on the conductor, the albedo texture again on the ground, a
    glass pane with a transmission texture and an emitter with an emission
    texture above the spheres.  Textures have 3 or 4 channels and odd sizes;
    the last texel of the last texture sits at the end of the pixel buffer.
    The roughness channel of the ORM texture stays at or above 64/255 (a
    roughness of at least 0.15 on the conductor): below ~0.03 (alpha < 1e-3)
    the reference treats the lobe as smooth -- no light sample, D clamped --
    yet samples its microfacet normal with the raw alpha, where the normal's
    cosine is within ~alpha^2 of 1 and a fast-maths build's ulps move the
    sampled angle by percent: no two builds agree there, and the scene
    measures texture parity instead."""
    sc = S.scene_small(40, 40, 2, 4)
    rng = np.random.default_rng(77)
    tex = [rng.integers(0, 256, (9, 13, 3), dtype=np.uint8),    # albedo (sRGB)
           rng.integers(0, 256, (8, 8, 4), dtype=np.uint8),     # normal map
           rng.integers(0, 256, (5, 7, 3), dtype=np.uint8),     # occlusion, roughness, metallic
           rng.integers(0, 256, (6, 6, 3), dtype=np.uint8),     # transmission
           rng.integers(0, 256, (4, 11, 3), dtype=np.uint8)]    # emission
    m = [S.material(albedo=(0.9, 0.8, 0.7), roughness=0.4),
         S.material(albedo=(0.95, 0.64, 0.54), metallic=1.0, roughness=0.6),
         S.material(albedo=(0.6, 0.6, 0.6), roughness=0.7),
         S.material(albedo=(0.9, 0.95, 1.0), roughness=0.2, transmission=1.0, ior=1.5),
         S.material(albedo=(0.8, 0.8, 0.8), emission=(1.0, 0.9, 0.8), emission_scale=15.0)]
    m[0]["albedo_tex"], m[0]["normal_tex"], m[0]["normal_scale"] = 0, 1, 0.8
    m[1]["orm_tex"] = 2
    m[2]["albedo_tex"] = 0
    m[3]["transmission_tex"] = 3
    m[4]["emission_tex"] = 4
    sc.materials = np.stack(m)
    sc.meshes = [S.uv_sphere(32, 16, 1.0, 0), S.quad(20.0, 20.0, 0.0, True, 2), S.quad(2.0, 2.0, 0.0, True, 3),
                 S.quad(1.0, 1.0, 0.0, False, 4)]
    sc.instances = [S.Instance(0, S.translate(-1.5, 0, 0).astype(np.float32), 0),
                    S.Instance(0, S.translate(1.5, 0, 0).astype(np.float32), 1),
                    S.Instance(1, S.translate(0, -1.0, 0).astype(np.float32), 2),
                    S.Instance(2, S.translate(0.5, 1.3, 0.5).astype(np.float32), 3),
                    S.Instance(3, S.translate(0, 2.5, 0).astype(np.float32), 4)]
    tex[2][..., 1] = 64 + (tex[2][..., 1].astype(np.int32) * 191) // 255
    sc.textures = tex
    return sc


def tricky_scene():
    """Random triangles plus exact duplicates of a third of them, triangles
    with two equal vertices, collinear vertices and slivers, in one mesh
    placed three times: instances 0 and 1 coincide, instance 2 is moved and
    turned.  Equal hit distances are frequent, so the hit that wins depends
    on the traversal order."""
    rng = np.random.default_rng(5)
    n = 3000
    c = rng.uniform(-2.0, 2.0, (n, 1, 3))
    p = (c + rng.normal(0.0, 0.3, (n, 3, 3))).astype(np.float32)
    dup = p[rng.choice(n, n // 3, replace=False)]
    deg = p[:200].copy()
    deg[:100, 2] = deg[:100, 1]                                                    # two equal vertices
    deg[100:, 2] = deg[100:, 0] + np.float32(2.0) * (deg[100:, 1] - deg[100:, 0])  # collinear
    sliver = p[200:400].copy()
    sliver[:, 2] = sliver[:, 0] + (sliver[:, 1] - sliver[:, 0]) * np.float32(0.5) + np.float32(1e-6)
    pos = np.concatenate([p, dup, deg, sliver]).astype(np.float32)
    pos = pos[rng.permutation(pos.shape[0])]
    nrm = np.repeat(np.cross(pos[:, 1] - pos[:, 0], pos[:, 2] - pos[:, 0])[:, None, :], 3, 1)
    nrm /= np.maximum(np.linalg.norm(nrm, axis=-1, keepdims=True), 1e-12)
    mesh = S.Mesh(pos, nrm.astype(np.float32), np.zeros((pos.shape[0], 3, 2), np.float32),
                  np.zeros(pos.shape[0], np.int32))
    base = S.scene_small(8, 8, 1, 2)
    ident = np.eye(4, dtype=np.float32)
    inst = [S.Instance(0, ident, 0), S.Instance(0, ident, 1),
            S.Instance(0, (S.translate(0.5, 0.25, -0.5) @ S.rot_y(0.7)).astype(np.float32), 2)]
    return S.Scene([mesh], inst, base.materials, base.camera, base.env, base.settings, base.exposure, 8, 8, 1)


def tricky_rays(sc, m=60000):
    """Rays aimed at points inside random triangles of the tricky scene's mesh
    (a tenth of them on an edge), from points around the cloud."""
    pos = sc.meshes[0].positions
    rng = np.random.default_rng(9)
    k = rng.integers(0, pos.shape[0], m)
    b = rng.dirichlet((1.0, 1.0, 1.0), m).astype(np.float32)
    b[: m // 10, 2] = 0.0
    b[: m // 10] /= b[: m // 10].sum(1, keepdims=True)
    target = np.einsum("nk,nkj->nj", b, pos[k]).astype(np.float32)
    o = (target + rng.normal(0.0, 1.0, (m, 3)) * np.float32(4.0)).astype(np.float32)
    d = target - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def main():
    if not O.available("ref"):
        O.build(ref=True)
    rng = np.random.default_rng(2024)
    out = {}

    # plain method, small scene
    r = O.Scene(small_scene(), "ref")
    rs = r.render_samples(0, 2)
    o, d = S.random_rays(4096, 5, center=(0, 0, 0), radius=6.0)
    h = r.trace(o, d)
    out.update(small_radiance=rs["radiance"], small_albedo=rs["albedo"], small_first_hit=rs["first_hit"],
               small_first_t=rs["first_t"], small_ray_o=o, small_ray_d=d, small_prim=h["prim"],
               small_inst=h["inst"], small_t=h["t"], small_bvh=np.array(bvh_digest(r)))

    # plain method, reduced full scene (lights, MIS, three material kinds)
    r = O.Scene(full_scene(), "ref")
    rs = r.render_samples(0, 2)
    out.update(full_radiance=rs["radiance"], full_albedo=rs["albedo"], full_first_hit=rs["first_hit"],
               full_bvh=np.array(bvh_digest(r)))

    # traversal scene: closest hits and the 4-bounce chain
    r = O.Scene(traversal_scene(), "ref")
    o, d = S.random_rays(4096, 4)
    h = r.trace(o, d)
    b = r.trace_bounces(o, d, 4)
    out.update(trav_ray_o=o, trav_ray_d=d, trav_prim=h["prim"], trav_t=h["t"],
               trav_bounce_prim=b["prim"], trav_bounce_t=b["t"], trav_bvh=np.array(bvh_digest(r)))

    # sky
    dirs = rng.normal(size=(512, 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    env = S.environment(sun_theta=np.radians(30.0))
    out.update(sky_dirs=dirs, sky_rgb=O.sky(env, dirs, "ref"))

    # BSDF lobes
    n = 4096
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    p = np.zeros((n, 12), np.float32)
    p[:, 0:3] = nrm
    p[:, 3:6] = rng.uniform(0.05, 0.95, (n, 3))
    kind = rng.integers(0, 3, n)
    p[:, 6] = kind == 2
    p[:, 7] = rng.uniform(0.0, 1.0, n)
    p[:, 8] = kind == 1
    p[:, 9] = rng.choice([1.45, 1.5], n)
    p[:, 10] = rng.integers(0, 2, n)
    p[:, 11] = rng.integers(0, 2, n)
    dd = rng.normal(size=(n, 6))
    dd[:, :3] /= np.linalg.norm(dd[:, :3], axis=1, keepdims=True)
    dd[:, 3:] /= np.linalg.norm(dd[:, 3:], axis=1, keepdims=True)
    dd = dd.astype(np.float32)
    u = rng.uniform(0, 1, (n, 4)).astype(np.float32)
    out.update(bsdf_params=p, bsdf_dirs=dd, bsdf_u=u, bsdf_out=O.bsdf_eval(p, dd, u, "ref"))

    # post chain on the reduced full-scene frame
    acc = out["full_radiance"][0] + out["full_radiance"][1]
    render = O.modulate(acc, 2, out["full_albedo"], "ref")
    bl = O.bloom(render, False, 0.65, "ref")
    blk = O.bloom(render, True, 0.65, "ref")
    ex = S.exposure()
    es = O.exposure_scalar(ex)
    img = O.post_image(render, bl, 0.175, es, prefix="ref")
    hist = O.histogram(render, prefix="ref")
    expo = O.exposure(hist, ex, 0.5, 16.0, "ref")
    Y = np.exp(rng.uniform(np.log(1e-4), np.log(2e3), 8192)).astype(np.float32)
    out.update(post_acc=acc, post_render=render, post_bloom=bl, post_bloom_karis=blk, post_expo_scalar=np.float32(es),
               post_image=img, post_hist_float=hist, post_exposure=expo, lum=Y,
               lum_bins=O.lum_bins(Y, prefix="ref"), meter_96x54=O.metering_weights(96, 54, "ref"),
               meter_100x37=O.metering_weights(100, 37, "ref"))

    # upscaling of the same render to the output size it is rendered for
    # (64x36 = 160x90 / 2.5): bilinear, and the FSR path (EASU + RCAS) also on
    # a high-dynamic-range image with zero patches and an odd ratio
    hdr = np.exp(rng.normal(0.0, 3.0, (27, 48, 4))).astype(np.float32)
    hdr[::3, ::5] = 0.0
    hdr[10:16, 20:30] = 0.25
    easu, sharp = O.fsr(render, 160, 90, "ref")
    easu_hdr, sharp_hdr = O.fsr(hdr, 121, 67, "ref")
    out.update(up_bilinear=O.upscale(render, 160, 90, "ref"), up_easu=easu, up_fsr=sharp, up_hdr=hdr,
               up_hdr_easu=easu_hdr, up_hdr_fsr=sharp_hdr)
    # every texture slot (albedo, normal map, ORM, transmission, emission)
    r = O.Scene(textured_scene(), "ref")
    rs = r.render_samples(0, 2)
    out.update(tex_radiance=rs["radiance"], tex_albedo=rs["albedo"], tex_first_hit=rs["first_hit"],
               tex_first_t=rs["first_t"])
    # closest hits where equal distances are common (duplicated and
    # coincident triangles): which one wins is the reference's traversal order
    r = O.Scene(tricky_scene(), "ref")
    o, d = tricky_rays(tricky_scene(), 8192)
    h = r.trace(o, d)
    out.update(tricky_prim=h["prim"], tricky_t=h["t"], tricky_bvh=np.array(bvh_digest(r)))
    np.savez_compressed(os.path.join(OUT, "reference_host.npz"), **out)
    print("wrote", os.path.join(OUT, "reference_host.npz"))


if __name__ == "__main__":
    main()
