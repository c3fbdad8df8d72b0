"""The CPU oracle reproduces the reference's own code bit for bit.

The fixtures in tests/golden/reference_host.npz were produced by
tests/golden/make_golden.py from the reference source compiled for the host
(oracle/build_ref.sh).  RNG argument order there is right-to-left at all
three call sites whose order C++ leaves unspecified (rng_order=7).
"""

import numpy as np
import pytest

from kittlespt_gb300 import scenes as S
from oracle import oracle as O

from tests.golden.make_golden import (bvh_digest, full_scene, small_scene, textured_scene, traversal_scene,
                                     tricky_rays, tricky_scene)


def bits(a):
    a = np.ascontiguousarray(a, np.float32)
    return a.view(np.uint32)


def test_small_scene_bvh_matches_reference(golden):
    assert bvh_digest(O.Scene(small_scene())) == str(golden["small_bvh"])


def test_full_scene_bvh_matches_reference(golden):
    assert bvh_digest(O.Scene(full_scene())) == str(golden["full_bvh"])


def test_traversal_scene_bvh_matches_reference(golden):
    assert bvh_digest(O.Scene(traversal_scene())) == str(golden["trav_bvh"])


def test_small_scene_closest_hits(golden):
    sc = O.Scene(small_scene())
    h = sc.trace(golden["small_ray_o"], golden["small_ray_d"])
    np.testing.assert_array_equal(h["prim"], golden["small_prim"])
    np.testing.assert_array_equal(h["inst"], golden["small_inst"])
    np.testing.assert_array_equal(bits(h["t"]), bits(golden["small_t"]))


def test_brute_force_agrees_with_bvh(golden):
    sc = O.Scene(small_scene())
    h = sc.trace(golden["small_ray_o"], golden["small_ray_d"], brute=True)
    np.testing.assert_array_equal(h["prim"], golden["small_prim"])


def test_small_scene_per_sample_radiance(golden):
    r = O.Scene(small_scene()).render_samples(0, 2, rng_order=7)
    np.testing.assert_array_equal(bits(r["radiance"]), bits(golden["small_radiance"]))
    np.testing.assert_array_equal(bits(r["albedo"]), bits(golden["small_albedo"]))
    np.testing.assert_array_equal(r["first_hit"], golden["small_first_hit"])
    np.testing.assert_array_equal(bits(r["first_t"]), bits(golden["small_first_t"]))


def test_full_scene_per_sample_radiance(golden):
    r = O.Scene(full_scene()).render_samples(0, 2, rng_order=7)
    np.testing.assert_array_equal(bits(r["radiance"]), bits(golden["full_radiance"]))
    np.testing.assert_array_equal(bits(r["albedo"]), bits(golden["full_albedo"]))
    np.testing.assert_array_equal(r["first_hit"], golden["full_first_hit"])


def test_traversal_hits_and_bounces(golden):
    sc = O.Scene(traversal_scene())
    h = sc.trace(golden["trav_ray_o"], golden["trav_ray_d"])
    np.testing.assert_array_equal(h["prim"], golden["trav_prim"])
    np.testing.assert_array_equal(bits(h["t"]), bits(golden["trav_t"]))
    b = sc.trace_bounces(golden["trav_ray_o"], golden["trav_ray_d"], 4)
    np.testing.assert_array_equal(b["prim"], golden["trav_bounce_prim"])
    np.testing.assert_array_equal(bits(b["t"]), bits(golden["trav_bounce_t"]))


def test_sky(golden):
    env = S.environment(sun_theta=np.radians(30.0))
    np.testing.assert_array_equal(bits(O.sky(env, golden["sky_dirs"])), bits(golden["sky_rgb"]))


def test_bsdf_lobes(golden):
    out = O.bsdf_eval(golden["bsdf_params"], golden["bsdf_dirs"], golden["bsdf_u"])
    ref = golden["bsdf_out"]
    same = (bits(out) == bits(ref)) | (np.isnan(out) & np.isnan(ref))
    assert same.all()


def test_post_chain(golden):
    render = O.modulate(golden["post_acc"], 2, golden["full_albedo"])
    np.testing.assert_array_equal(bits(render), bits(golden["post_render"]))
    np.testing.assert_array_equal(bits(O.bloom(render, False, 0.65)), bits(golden["post_bloom"]))
    np.testing.assert_array_equal(bits(O.bloom(render, True, 0.65)), bits(golden["post_bloom_karis"]))
    img = O.post_image(render, golden["post_bloom"], 0.175, float(golden["post_expo_scalar"]))
    np.testing.assert_array_equal(bits(img), bits(golden["post_image"]))


def test_ties_are_broken_in_the_reference_order(golden):
    """Duplicated, coincident, degenerate and sliver triangles: trees, hit
    distances and the winning triangle among equal distances are the
    reference's; brute force (lowest index) disagrees on many of them."""
    r = O.Scene(tricky_scene())
    assert bvh_digest(r) == str(golden["tricky_bvh"])
    o, d = tricky_rays(tricky_scene(), 8192)
    h = r.trace(o, d)
    np.testing.assert_array_equal(h["prim"], golden["tricky_prim"])
    np.testing.assert_array_equal(bits(h["t"]), bits(golden["tricky_t"]))
    brute = r.trace(o, d, brute=True)
    np.testing.assert_array_equal(bits(brute["t"]), bits(golden["tricky_t"]))
    assert (brute["prim"] != h["prim"]).mean() > 0.05


def test_upscale_bilinear_and_fsr(golden):
    """upscale (upscale.cuh:260-291) and the FSR path (EASU + RCAS, compiled in
    with USE_FSR), bit for bit, on the post-chain render and on a
    high-dynamic-range image with zero patches at an odd ratio."""
    render = golden["post_render"]
    np.testing.assert_array_equal(bits(O.upscale(render, 160, 90)), bits(golden["up_bilinear"]))
    easu, sharp = O.fsr(render, 160, 90)
    np.testing.assert_array_equal(bits(easu), bits(golden["up_easu"]))
    np.testing.assert_array_equal(bits(sharp), bits(golden["up_fsr"]))
    easu, sharp = O.fsr(golden["up_hdr"], 121, 67)
    np.testing.assert_array_equal(bits(easu), bits(golden["up_hdr_easu"]))
    np.testing.assert_array_equal(bits(sharp), bits(golden["up_hdr_fsr"]))
    # a constant image stays that constant through EASU and RCAS
    flat = np.full((20, 24, 4), 0.3, np.float32)
    assert (O.fsr(flat, 60, 50)[1][..., :3] == np.float32(0.3)).all()


def test_histogram_bins_and_weights(golden):
    np.testing.assert_array_equal(O.lum_bins(golden["lum"]), golden["lum_bins"])
    np.testing.assert_array_equal(bits(O.metering_weights(96, 54)), bits(golden["meter_96x54"]))
    np.testing.assert_array_equal(bits(O.metering_weights(100, 37)), bits(golden["meter_100x37"]))


def test_histogram_and_exposure_close_to_float_reference(golden):
    # the reference sums float weights with atomics (order dependent); the
    # oracle sums 2^-24 fixed point, so agreement is to float rounding
    h = O.histogram(golden["post_render"])
    np.testing.assert_allclose(h.astype(np.float64) / 2 ** 24, golden["post_hist_float"], rtol=1e-5, atol=1e-4)
    e = O.exposure(h, S.exposure(), 0.5, 16.0)
    np.testing.assert_allclose(e, golden["post_exposure"], rtol=1e-4)


def test_sensitivity_probe_is_inert_at_zero_and_deterministic():
    """The rounding-sensitivity probe (tests/parity_rule.py): with eps = 0 it
    re-renders every sample exactly; its unperturbed radiance is
    render_samples'; the same call gives the same responses; and a probe
    of the size of fast-maths errors leaves most samples unmoved."""
    sc = small_scene()
    o = O.Scene(sc)
    ref = o.render_samples(0, 2, rng_order=0)
    z = o.render_sensitivity(0, 2, 0, eps=0.0, eps_pos=0.0, ncopies=2)
    assert np.array_equal(z["radiance"], ref["radiance"])
    assert not z["response"].any()
    a = o.render_sensitivity(0, 2, 0, eps=1e-4, eps_pos=1e-5, ncopies=4)
    b = o.render_sensitivity(0, 2, 0, eps=1e-4, eps_pos=1e-5, ncopies=4)
    assert np.array_equal(a["response"], b["response"])
    assert np.median(a["response"]) < 1e-4


def test_textured_scene_per_sample_radiance(golden):
    """Every texture slot -- sRGB albedo, normal map, occlusion-roughness-
    metallic, transmission, emission (through light sampling) -- against the
    reference's own Material::getBSDF / Texture::evaluate / Light::L
    (material.cu:17-70, texture.cuh:34-66, light.cu:21-33), bit for bit."""
    r = O.Scene(textured_scene()).render_samples(0, 2, rng_order=7)
    np.testing.assert_array_equal(bits(r["radiance"]), bits(golden["tex_radiance"]))
    np.testing.assert_array_equal(bits(r["albedo"]), bits(golden["tex_albedo"]))
    np.testing.assert_array_equal(r["first_hit"], golden["tex_first_hit"])
    np.testing.assert_array_equal(bits(r["first_t"]), bits(golden["tex_first_t"]))
