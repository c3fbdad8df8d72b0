"""GPU parity on the workloads' stated sizes, through the C ABI, against the
CPU oracle on the same seeded inputs.

  * plain method, small: 256x256, depth 4, every pixel; first hits and
    visible-surface albedo bit-exact, per-sample radiance by the rule of
    tests/parity_rule.py;
  * plain method, full frame: 1920x1080, 16 spp, depth 8 on the five-variant
    8x8 icosphere grid with 16 lights; camera-ray hits of every pixel
    bit-exact, per-sample radiance of every sample of four bands of rows
    spread over the frame by the same rule; no ray of the oracle's paths
    needs more than the reference's 16-entry traversal stack;
  * traversal stress: 2,000,000 random triangles, 1,048,576 incoherent rays
    plus 4 diffuse bounces; every id and distance bit-exact; the rays for
    which the reference's 16-entry stack would overflow are counted and
    reported (its traversal would drop nodes there; ours and the oracle's do
    not).
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


def global_prim(scene, inst, tri):
    ex = scene.expanded()
    base = np.concatenate([[0], np.cumsum(ex["mesh_count"])[:-1]]).astype(np.int64)
    return np.where(inst >= 0, base[np.maximum(inst, 0)] + tri, -1)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def gpu_samples(sc, n, rows=None):
    """Per-sample radiance [n][H][W][3] (only `rows` if given), camera-ray
    hits [H][W][4] and albedo [H][W][3] of the CUDA path."""
    from kittlespt_gb300.renderer import Renderer
    with Renderer(0) as r:
        r.load_scene(sc)
        rad = torch.zeros((n, sc.height, sc.width, 4), dtype=torch.float32, device="cuda:0")
        hit = torch.zeros((sc.height, sc.width, 4), dtype=torch.int32, device="cuda:0")
        alb = torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda:0")
        r.render_samples_device(0, n, rad.data_ptr(), hit.data_ptr(), alb.data_ptr())
        r.synchronize()
        if rows is not None:
            rad = rad[:, rows]
        out = rad[..., :3].cpu().numpy(), hit.cpu().numpy(), alb[..., :3].cpu().numpy()
        del rad
        return out


def test_small_config_every_pixel():
    sc = S.scene_small(256, 256, 4, 4)
    n = 4
    rad, hit, alb = gpu_samples(sc, n)
    o = O.Scene(sc)
    ref = o.render_samples(0, n, rng_order=0)
    np.testing.assert_array_equal(global_prim(sc, hit[..., 0], hit[..., 1]), ref["first_hit"][..., 0])
    np.testing.assert_array_equal(bits(hit[..., 2].view(np.float32)), bits(ref["first_t"]))
    m = ref["first_hit"][..., 0] >= 0
    np.testing.assert_array_equal(bits(alb[m]), bits(ref["albedo"][m]))
    probe = o.render_sensitivity(0, n, 0, eps=PROBE_EPS, eps_pos=PROBE_EPS_POS, ncopies=PROBE_COPIES)
    assert np.array_equal(bits(probe["radiance"]), bits(ref["radiance"]))
    check_samples(rad, ref["radiance"], probe["response"], "256x256 x4, depth 4")


@pytest.fixture(scope="module")
def full_frame():
    sc = S.scene_full()   # 1920x1080, 16 spp, depth 8, 64 icospheres + 16 lights
    return sc, O.Scene(sc)


BANDS = [(90, 4), (400, 4), (710, 4), (1020, 4)]


def test_full_frame_camera_hits_every_pixel(full_frame):
    sc, o = full_frame
    _, hit, alb = gpu_samples(sc, 1, rows=[0])
    ref = o.render_samples(0, 1, rng_order=0, max_depth=0, want_radiance=False)
    np.testing.assert_array_equal(global_prim(sc, hit[..., 0], hit[..., 1]), ref["first_hit"][..., 0])
    np.testing.assert_array_equal(bits(hit[..., 2].view(np.float32)), bits(ref["first_t"]))
    m = ref["first_hit"][..., 0] >= 0
    np.testing.assert_array_equal(bits(alb[m]), bits(ref["albedo"][m]))
    assert 0.2 < m.mean() < 0.9


def test_full_frame_per_sample_radiance_bands(full_frame):
    sc, o = full_frame
    n = sc.spp
    rows = np.concatenate([np.arange(r0, r0 + k) for r0, k in BANDS])
    rad, _, _ = gpu_samples(sc, n, rows=rows)
    refs, resp = [], []
    overflow = 0
    for r0, k in BANDS:
        ref = o.render_samples(0, n, rng_order=0, row0=r0, nrows=k)
        overflow += int(ref["counters"][7])
        probe = o.render_sensitivity(0, n, 0, row0=r0, nrows=k, eps=PROBE_EPS, eps_pos=PROBE_EPS_POS,
                                     ncopies=PROBE_COPIES)
        assert np.array_equal(bits(probe["radiance"]), bits(ref["radiance"]))
        refs.append(ref["radiance"])
        resp.append(probe["response"])
    ref = np.concatenate(refs, axis=1)
    response = np.concatenate(resp, axis=1)
    print(f"1080p bands: rays over the reference's 16-entry stack: {overflow}")
    assert overflow == 0
    check_samples(rad, ref, response, f"1920x1080 x{n}, depth 8, {len(rows)} rows")
    # the bands converge to the same image
    assert np.abs(rad.mean(0) - ref.mean(0)).mean() <= 1e-2 * max(float(ref.mean()), 1e-3)


def test_traversal_stress_full_size():
    sc = S.scene_traversal(2_000_000)
    o, d = S.random_rays(1_048_576, 9)
    from kittlespt_gb300.renderer import Renderer
    with Renderer(0) as r:
        r.load_scene(sc)
        inst, tri, t = r.trace_bounces(o, d, 4)
    ref = O.Scene(sc).trace_bounces(o, d, 4)
    np.testing.assert_array_equal(np.where(inst >= 0, tri, -1), ref["prim"])
    np.testing.assert_array_equal(bits(t), bits(ref["t"]))
    print(f"2M triangles: {(ref['prim'][0] >= 0).mean():.3f} of 1,048,576 rays hit; rays over the reference's "
          f"16-entry stack: {int(ref['counters'][7])}; deepest stack {int(ref['counters'][6])}")
    assert (ref["prim"][4] >= 0).sum() > 0
