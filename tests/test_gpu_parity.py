"""GPU parity: the CUDA path behind include/kpt.h against the CPU oracle.

Tolerances (from the parity targets of the path):
  * closest-hit triangle ids and hit distances: bit-exact (the traversal
    runs in IEEE arithmetic; the oracle is pinned to the reference's own code);
  * Nishita sky: 1e-4 relative (fast-maths exp/sqrt as in the reference's
    GPU build);
  * per-sample radiance: within 1e-4 relative, or explained by the oracle's
    rounding-sensitivity probe (tests/parity_rule.py);
  * modulate, histogram, exposure: bit-exact on the same inputs;
  * display image: 2e-5 absolute (CUDA powf/log2f vs the C library).
"""

import numpy as np
import pytest

from kittlespt_gb300 import scenes as S
from oracle import oracle as O
from tests.parity_rule import PROBE_COPIES, PROBE_EPS, PROBE_EPS_POS, check_samples

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from kittlespt_gb300 import build
    build.build()
    O.build(ref=False)


def make_renderer(scene):
    from kittlespt_gb300.renderer import Renderer
    r = Renderer(0)
    r.initialize()
    r.load_scene(scene)
    return r


def global_prim(scene, inst, tri):
    ex = scene.expanded()
    base = np.concatenate([[0], np.cumsum(ex["mesh_count"])[:-1]]).astype(np.int64)
    return np.where(inst >= 0, base[np.maximum(inst, 0)] + tri, -1)


def gpu_trace(r, o, d):
    n = o.shape[0]
    dev = "cuda:0"
    to = torch.from_numpy(np.ascontiguousarray(o, np.float32)).to(dev)
    td = torch.from_numpy(np.ascontiguousarray(d, np.float32)).to(dev)
    inst = torch.empty(n, dtype=torch.int32, device=dev)
    tri = torch.empty(n, dtype=torch.int32, device=dev)
    t = torch.empty(n, dtype=torch.float32, device=dev)
    r.trace_device(n, to.data_ptr(), td.data_ptr(), inst.data_ptr(), tri.data_ptr(), t.data_ptr())
    r.synchronize()
    return inst.cpu().numpy(), tri.cpu().numpy(), t.cpu().numpy()


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("which", ["small", "full"])
def test_closest_hits_bit_exact(which):
    if which == "small":
        sc = S.scene_small(64, 64, 1, 4)
        o, d = S.random_rays(50000, 7, center=(0, 0, 0), radius=6.0)
    else:
        sc = S.scene_full(64, 36, 1, 8, n_variants=2, subdiv=4, grid=4, n_lights=4)
        o, d = S.random_rays(50000, 8, center=(0, 1, 0), radius=9.0)
    r = make_renderer(sc)
    try:
        inst, tri, t = gpu_trace(r, o, d)
    finally:
        r.shutdown()
    ref = O.Scene(sc).trace(o, d)
    np.testing.assert_array_equal(global_prim(sc, inst, tri), ref["prim"])
    np.testing.assert_array_equal(inst, ref["inst"])
    np.testing.assert_array_equal(bits(t), bits(ref["t"]))
    assert (ref["prim"] >= 0).mean() > 0.05


def test_random_triangles_hits_and_bounces_bit_exact():
    sc = S.scene_traversal(200000)
    o, d = S.random_rays(65536, 9)
    r = make_renderer(sc)
    try:
        inst, tri, t = r.trace_bounces(o, d, 4)
    finally:
        r.shutdown()
    ref = O.Scene(sc).trace_bounces(o, d, 4)
    np.testing.assert_array_equal(np.where(inst >= 0, tri, -1), ref["prim"])
    np.testing.assert_array_equal(bits(t), bits(ref["t"]))
    assert (ref["prim"][4] >= 0).sum() > 0


def test_sky_matches_oracle():
    rng = np.random.default_rng(3)
    dirs = rng.normal(size=(8192, 3)).astype(np.float32)
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    sc = S.scene_small(8, 8, 1, 1)
    r = make_renderer(sc)
    try:
        td = torch.from_numpy(dirs).cuda()
        out = torch.empty_like(td)
        r.sky_device(dirs.shape[0], td.data_ptr(), out.data_ptr())
        r.synchronize()
        g = out.cpu().numpy()
    finally:
        r.shutdown()
    ref = O.sky(sc.env, dirs)
    scale = np.maximum(np.abs(ref), 1e-3 * np.abs(ref).max())
    assert (np.abs(g - ref) / scale).max() <= 1e-4


def render_samples(r, sc, n):
    rad = torch.zeros((n, sc.height, sc.width, 4), dtype=torch.float32, device="cuda:0")
    hit = torch.zeros((sc.height, sc.width, 4), dtype=torch.int32, device="cuda:0")
    alb = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda:0")
    r.render_samples_device(0, n, rad.data_ptr(), hit.data_ptr(), alb.data_ptr())
    r.synchronize()
    return rad[..., :3].cpu().numpy(), hit.cpu().numpy(), alb[..., :3].cpu().numpy()


@pytest.mark.parametrize("which,n,order", [("small", 4, 0), ("small", 2, 7), ("small", 2, 5), ("full", 2, 0),
                                           ("textured", 4, 0)])
def test_per_sample_radiance(which, n, order):
    if which == "small":
        sc = S.scene_small(64, 64, n, 4)
    elif which == "textured":   # every texture slot; its oracle is pinned to the reference's own code
        from tests.golden.make_golden import textured_scene
        sc = textured_scene()
        sc.spp = n
    else:
        sc = S.scene_full(96, 54, n, 8, n_variants=2, subdiv=3, grid=3, n_lights=4)
    r = make_renderer(sc)
    try:
        r.set_renderer_settings(rng_order=order)
        rad, hit, alb = render_samples(r, sc, n)
    finally:
        r.shutdown()
    o = O.Scene(sc)
    ref = o.render_samples(0, n, rng_order=order)
    # first hits: exact
    np.testing.assert_array_equal(global_prim(sc, hit[..., 0], hit[..., 1]), ref["first_hit"][..., 0])
    np.testing.assert_array_equal(bits(hit[..., 2].view(np.float32)), bits(ref["first_t"]))
    hitmask = ref["first_hit"][..., 0] >= 0
    if which == "textured":
        # the sRGB decoding of the albedo texture is powf, fast on the GPU as
        # in the reference's GPU build: a few ulps
        np.testing.assert_allclose(alb[hitmask], ref["albedo"][hitmask], rtol=1e-6, atol=0)
    else:
        np.testing.assert_array_equal(bits(alb[hitmask]), bits(ref["albedo"][hitmask]))
    probe = o.render_sensitivity(0, n, order, eps=PROBE_EPS, eps_pos=PROBE_EPS_POS, ncopies=PROBE_COPIES)
    check_samples(rad, ref["radiance"], probe["response"], f"{which} x{n}, rng order {order}")
    # the mean over samples converges to the same image
    assert np.abs(rad.mean(0) - ref["radiance"].mean(0)).mean() <= 1e-2 * max(ref["radiance"].mean(), 1e-3)


def test_frame_post_chain_bit_exact():
    sc = S.scene_small(96, 64, 2, 4)
    sc.settings["bloom"] = 1
    sc.settings["auto_exposure"] = 1
    r = make_renderer(sc)
    try:
        r.execute_rendering(16.0, 3)
        r.synchronize()
        acc = r.read_accumulation()[..., :3]
        alb = r.read_albedo()[..., :3]
        render = r.read_render()
        hist = r.read_histogram()
        st = r.stats()
        img = r.get_render_target()
        assert st.frame_index == 3
    finally:
        r.shutdown()
    ref_render = O.modulate(acc, 3, alb)
    np.testing.assert_array_equal(bits(render), bits(ref_render))
    ref_hist = O.histogram(ref_render)
    np.testing.assert_array_equal(hist, ref_hist)
    e = O.exposure(ref_hist, sc.exposure, 0.0, float(sc.settings["frame_delta_ms"]))
    np.testing.assert_array_equal(bits(np.array([st.avg_bin, st.avg_luminance, st.adapted_luminance,
                                                 st.exposure_scalar, st.iso, st.shutter], np.float32)), bits(e))
    bl = O.bloom(ref_render, False, float(sc.settings["bloom_internal_blend"]))
    ref_img = O.post_image(ref_render, bl, float(sc.settings["bloom_final_blend"]), float(e[3]))
    assert np.abs(img - ref_img).max() <= 2e-5


def test_accumulation_is_sample_order_sum():
    sc = S.scene_small(32, 32, 4, 3)
    r = make_renderer(sc)
    try:
        rad, _, _ = render_samples(r, sc, 4)
        r.execute_rendering(16.0, 2)
        r.execute_rendering(16.0, 2)
        r.synchronize()
        acc = r.read_accumulation()[..., :3]
    finally:
        r.shutdown()
    s = np.zeros_like(rad[0])
    for k in range(4):
        s = (s + rad[k]).astype(np.float32)
    np.testing.assert_array_equal(bits(acc), bits(s))


def test_level_counts_agree_with_the_ray_counts():
    """kpt_get_level_counts: level 0 shades every camera-ray hit of every
    sample, each level's paths and shadow rays add up to the frame's ray
    counters, and fewer paths continue than enter."""
    from kittlespt_gb300 import _lib as K
    sc = S.scene_full(64, 36, 3, 6, n_variants=2, subdiv=3, grid=3, n_lights=4)
    r = make_renderer(sc)
    try:
        with pytest.raises(K.KptError):
            r.level_counts()        # no frame yet
        st0 = r.stats()
        r.execute_rendering(16.0, 3)
        r.synchronize()
        st1 = r.stats()
        lc = r.level_counts()
        hits = int((render_samples(r, sc, 1)[1][..., 0] >= 0).sum())
    finally:
        r.shutdown()
    assert lc.shape == (7, 3)
    assert lc[0, 0] == hits * 3
    assert (np.diff(lc[:, 0]) <= 0).all() and lc[1, 0] > 0
    assert (lc[:, 1] + lc[:, 2] <= lc[:, 0]).all()
    assert lc[1:, 0].sum() == st1.path_rays - st0.path_rays
    assert lc[:, 1:].sum() == st1.shadow_rays - st0.shadow_rays


def test_api_errors_and_state():
    sc = S.scene_small(16, 16, 1, 2)
    r = make_renderer(sc)
    try:
        assert r.set_material(999, sc.materials[0]) is False
        assert r.set_mesh_transform(999, np.eye(4)) is False
        with pytest.raises(IndexError):
            r.get_material(999)
        m = r.get_mesh_transform(1)
        np.testing.assert_allclose(m, sc.instances[1].model)
        assert r.get_materials_count() == 3 and r.get_mesh_count() == 3
        assert r.set_mesh_transform(1, S.translate(1.0, 0.5, 0.0)) is True
        r.execute_rendering(16.0, 1)
        r.synchronize()
        assert r.stats().frame_index == 1
        assert r.launch_count() > 0
    finally:
        r.shutdown()
