"""Edge cases of the path against the oracle, with the tolerances of
tests/test_gpu_parity.py (ids and distances bit-exact, per-sample radiance
1e-4 relative, render and histogram bit-exact, display image 2e-5):

  * a frame in which every camera ray leaves the scene (sky only), and an
    empty scene, which kpt_commit_scene refuses without harming the context;
  * ragged image sizes, down to 1 x 1 (bloom mip chain with no levels);
  * the depth limits 0 and 1;
  * degenerate, sliver and coincident triangles, in one mesh and in two
    instances at the same place: equal hit distances are decided by the
    order of the traversal, which must be the reference's.
"""

import numpy as np
import pytest

from kittlespt_gb300 import scenes as S
from oracle import oracle as O

from tests.golden.make_golden import tricky_rays, tricky_scene
from tests.test_gpu_parity import bits, global_prim, gpu_trace, make_renderer, render_samples

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _radiance_close(rad, ref, what):
    err = np.abs(rad - ref).max(-1) / np.maximum(np.abs(ref).max(-1), 1e-3)
    frac = (err <= 1e-4).mean()
    assert frac >= 0.99, f"{what}: {frac:.4f} of samples within 1e-4"


def _frame_matches_oracle(sc, n):
    """Renders n samples per pixel with bloom and auto exposure, then checks
    render, histogram, exposure and display image against the oracle's post
    chain run on the GPU's accumulation."""
    sc.settings["bloom"] = 1
    sc.settings["auto_exposure"] = 1
    r = make_renderer(sc)
    try:
        r.execute_rendering(16.0, n)
        r.synchronize()
        acc = r.read_accumulation()[..., :3]
        alb = r.read_albedo()[..., :3]
        render = r.read_render()
        hist = r.read_histogram()
        st = r.stats()
        img = r.get_render_target()
    finally:
        r.shutdown()
    ref_render = O.modulate(acc, n, alb)
    np.testing.assert_array_equal(bits(render), bits(ref_render))
    ref_hist = O.histogram(ref_render)
    np.testing.assert_array_equal(hist, ref_hist)
    e = O.exposure(ref_hist, sc.exposure, 0.0, float(sc.settings["frame_delta_ms"]))
    np.testing.assert_array_equal(bits(np.array([st.avg_bin, st.avg_luminance, st.adapted_luminance,
                                                 st.exposure_scalar, st.iso, st.shutter], np.float32)), bits(e))
    bl = O.bloom(ref_render, False, float(sc.settings["bloom_internal_blend"]))
    ref_img = O.post_image(ref_render, bl, float(sc.settings["bloom_final_blend"]), float(e[3]))
    assert np.abs(img - ref_img).max() <= 2e-5


def _all_miss_scene(w, h, spp):
    sc = S.scene_small(w, h, spp, 3)
    # every instance moved 40 units behind the camera (at z = 5, looking at -z)
    sc.instances = [S.Instance(i.mesh, (S.translate(0.0, 0.0, 40.0) @ i.model).astype(np.float32), i.material)
                    for i in sc.instances]
    return sc


def test_every_camera_ray_misses():
    sc = _all_miss_scene(24, 16, 2)
    r = make_renderer(sc)
    try:
        rad, hit, alb = render_samples(r, sc, 2)
    finally:
        r.shutdown()
    ref = O.Scene(sc).render_samples(0, 2)
    assert (ref["first_hit"][..., 0] < 0).all()
    np.testing.assert_array_equal(global_prim(sc, hit[..., 0], hit[..., 1]), ref["first_hit"][..., 0])
    _radiance_close(rad, ref["radiance"], "sky only")
    _frame_matches_oracle(_all_miss_scene(24, 16, 2), 2)


def test_empty_scene_is_refused_and_the_context_stays_usable():
    from kittlespt_gb300 import _lib as K
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_small(16, 16, 1, 2)
    empty = S.scene_small(16, 16, 1, 2)
    empty.instances = []
    r = Renderer(0)
    r.initialize()
    try:
        with pytest.raises(K.KptError):
            r.load_scene(empty)
        r.load_scene(sc)
        rad, _, _ = render_samples(r, sc, 1)
    finally:
        r.shutdown()
    _radiance_close(rad, O.Scene(sc).render_samples(0, 1)["radiance"], "after a refused commit")


@pytest.mark.parametrize("w,h", [(1, 1), (7, 3), (33, 17), (3, 29)])
def test_ragged_sizes(w, h):
    sc = S.scene_small(w, h, 2, 3)
    r = make_renderer(sc)
    try:
        rad, hit, alb = render_samples(r, sc, 2)
    finally:
        r.shutdown()
    ref = O.Scene(sc).render_samples(0, 2)
    np.testing.assert_array_equal(global_prim(sc, hit[..., 0], hit[..., 1]), ref["first_hit"][..., 0])
    np.testing.assert_array_equal(bits(hit[..., 2].view(np.float32)), bits(ref["first_t"]))
    if w * h * 2 >= 100:
        _radiance_close(rad, ref["radiance"], f"{w}x{h}")
    else:   # too few samples for a fraction: each within 1e-4, or the path flipped a decision
        err = np.abs(rad - ref["radiance"]).max(-1) / np.maximum(np.abs(ref["radiance"]).max(-1), 1e-3)
        assert (err <= 1e-4).sum() >= err.size - 1, err
    _frame_matches_oracle(S.scene_small(w, h, 2, 3), 2)


@pytest.mark.parametrize("depth", [0, 1])
def test_depth_limits(depth):
    sc = S.scene_full(48, 27, 2, depth, n_variants=2, subdiv=3, grid=3, n_lights=4)
    r = make_renderer(sc)
    try:
        rad, hit, alb = render_samples(r, sc, 2)
    finally:
        r.shutdown()
    ref = O.Scene(sc).render_samples(0, 2)
    np.testing.assert_array_equal(global_prim(sc, hit[..., 0], hit[..., 1]), ref["first_hit"][..., 0])
    _radiance_close(rad, ref["radiance"], f"depth {depth}")


def test_degenerate_and_coincident_triangles():
    sc = tricky_scene()
    o, d = tricky_rays(sc)
    r = make_renderer(sc)
    try:
        gi, gt, t = gpu_trace(r, o, d)
    finally:
        r.shutdown()
    ref = O.Scene(sc).trace(o, d)
    np.testing.assert_array_equal(global_prim(sc, gi, gt), ref["prim"])
    np.testing.assert_array_equal(bits(t), bits(ref["t"]))
    # hits land on the coincident pair and on the moved instance
    assert (ref["prim"] >= 0).mean() > 0.5
    assert (gi == 0).any() and (gi == 2).any()
