"""Parity against the reference's own GPU build.

The reference's CUDA megakernel (computePathTraceSamplesMegaKernel,
shaders/kernels.cu:385-451) is built unmodified for sm_103a with its GPU
build's -use_fast_math from the staged reference sources
(oracle/build_ref.sh gpu) and driven by oracle/ref_harness/ref_gpu_harness.cu.
These tests put the CUDA path behind include/kpt.h beside it on the plain
method's small configuration at its stated size (256x256, depth 4, the
reference's frame index = the sample index), through the C ABI, with the sky
in the GPU build's arithmetic (kpt_settings.sky_arith = 1, the default) and
the RNG argument order of that build (rng_order = 0, the default):

  * camera-ray closest hits: our camera rays and traversal are IEEE, the
    reference's fast maths (its camera direction is normalised with the
    approximate reciprocal square root, its Moller-Trumbore divides
    approximately), so ids agree on every pixel and t within 5e-5 relative
    (measured: 1.24e-5);
  * per-sample radiance (the megakernel's accumulation after one frame from
    zero is exactly that frame's clamped sample): at least 99.8% of the
    samples within 1e-4 relative (measured: 99.88%); the rest lie where the
    two builds' traversal rounding or the ill-conditioned sky altitude
    differ.  Under IEEE sky arithmetic only ~78% agree, and under any other
    RNG argument order 35-85%.

They are skipped where the reference's sources were not staged (no
oracle/_ref/libkpt_ref_gpu.so).
"""

import numpy as np
import pytest

from kittlespt_gb300 import scenes as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    if not O.available("refgpu"):
        pytest.skip("reference GPU build absent (reference sources not staged)")
    from kittlespt_gb300 import build
    build.build()
    O.build(ref=False)


def global_prim(scene, inst, tri):
    ex = scene.expanded()
    base = np.concatenate([[0], np.cumsum(ex["mesh_count"])[:-1]]).astype(np.int64)
    return np.where(inst >= 0, base[np.maximum(inst, 0)] + tri, -1)


def ours(sc, n):
    from kittlespt_gb300.renderer import Renderer
    with Renderer(0) as r:
        assert r.get_renderer_settings().rng_order == 0 and r.get_renderer_settings().sky_arith == 1
        r.load_scene(sc)
        r.set_renderer_settings(sky_arith=1)
        rad = torch.zeros((n, sc.height, sc.width, 4), dtype=torch.float32, device="cuda:0")
        hit = torch.zeros((sc.height, sc.width, 4), dtype=torch.int32, device="cuda:0")
        r.render_samples_device(0, n, rad.data_ptr(), hit.data_ptr())
        r.synchronize()
        return rad[..., :3].cpu().numpy(), hit.cpu().numpy()


@pytest.fixture(scope="module")
def small():
    sc = S.scene_small(256, 256, 4, 4)
    n = 4
    g = O.RefGpuScene(sc)
    try:
        depth = g.tree_depth()
        hits = g.first_hits()
        rad_ref = g.render_samples(0, n)
    finally:
        g.close()
    rad, hit = ours(sc, n)
    return sc, depth, hits, rad_ref, rad, hit


def test_tree_fits_the_reference_stacks(small):
    _, depth, *_ = small
    assert depth["blas"] <= 14 and depth["tlas"] <= 14


def test_camera_hits_match_the_reference_gpu_build(small):
    sc, _, ref, _, _, hit = small
    prim = global_prim(sc, hit[..., 0], hit[..., 1])
    same = prim == ref["prim"]
    frac = same.mean()
    print(f"camera-ray ids equal on {frac:.6f} of {same.size} pixels ({(~same).sum()} differ)")
    assert frac >= 0.999
    t = hit[..., 2].view(np.float32)
    both = same & (prim >= 0)
    rel = np.abs(t[both] - ref["t"][both]) / np.abs(ref["t"][both])
    print(f"t: max relative difference {rel.max():.3e} where ids agree")
    assert rel.max() <= 5e-5
    # every pixel whose id differs hits near an edge of the IEEE oracle's triangle
    if (~same).any():
        ys, xs = np.nonzero(~same)
        o, d = camera_rays(sc, xs, ys)
        tr = O.Scene(sc).trace(o, d)
        margin = tr["bary"].min(-1)
        print(f"barycentric margin of the differing pixels: max {margin.max():.3e}")
        assert (margin < 1e-4).all()


def camera_rays(sc, xs, ys):
    """Camera::generateRay (camera.cuh:16-25) in IEEE single precision for
    pixels (xs, ys), as the oracle computes them."""
    W, H = sc.width, sc.height
    f = np.float32
    uv = np.stack([(xs.astype(f) + f(0.5)) / f(W), (ys.astype(f) + f(0.5)) / f(H)], -1)
    ndc = f(2.0) * uv - f(1.0)
    p = np.concatenate([ndc, np.ones((len(xs), 2), f)], -1)
    cs = (sc.camera.inv_proj.astype(f) @ p.T).T
    v = cs[:, :3] / cs[:, 3:4]
    v = v / np.linalg.norm(v, axis=1, keepdims=True)
    ws = (sc.camera.inv_view.astype(f) @ np.concatenate([v, np.zeros((len(xs), 1), f)], -1).T).T[:, :3]
    d = (ws / np.linalg.norm(ws, axis=1, keepdims=True)).astype(f)
    o = np.repeat(sc.camera.inv_view[:3, 3][None, :].astype(f), len(xs), 0)
    return o, d


def test_per_sample_radiance_matches_the_reference_gpu_build(small):
    sc, _, ref, rad_ref, rad, hit = small
    prim = global_prim(sc, hit[..., 0], hit[..., 1])
    same_first = prim == ref["prim"]
    err = np.abs(rad - rad_ref).max(-1) / np.maximum(np.abs(rad_ref).max(-1), 1e-3)
    ok = err <= 1e-4
    print(f"per-sample radiance within 1e-4: {ok.mean():.6f} of {ok.size}; "
          f"where the first hit agrees {ok[:, same_first].mean():.6f}; max err {err.max():.3e}")
    assert ok.mean() >= 0.998
    # the converged image agrees
    m, mr = rad.mean(0), rad_ref.mean(0)
    assert np.abs(m - mr).mean() <= 1e-2 * max(float(mr.mean()), 1e-3)


@pytest.fixture(scope="module")
def full_frame():
    """The full-frame workload (1920x1080, 16 spp, depth 8, the 8x8
    icosphere grid with 16 lights): the megakernel's 16 frames and our 16
    samples of the same frame indices."""
    sc = S.scene_full()
    sc.sky_arith = 1
    g = O.RefGpuScene(sc)
    try:
        depth = g.tree_depth()
        hits = g.first_hits()
        rad_ref = g.render_samples(0, sc.spp)
    finally:
        g.close()
    rad, hit = ours(sc, sc.spp)
    return sc, depth, hits, rad_ref, rad, hit


def test_full_frame_matches_the_reference_gpu_build(full_frame):
    sc, depth, ref, rad_ref, rad, hit = full_frame
    assert depth["blas"] <= 14 and depth["tlas"] <= 14
    prim = global_prim(sc, hit[..., 0], hit[..., 1])
    same = prim == ref["prim"]
    print(f"1080p camera-ray ids equal on {same.mean():.6f} of {same.size} pixels ({(~same).sum()} differ)")
    assert same.mean() >= 0.999
    t = hit[..., 2].view(np.float32)
    both = same & (prim >= 0)
    rel = np.abs(t[both] - ref["t"][both]) / np.abs(ref["t"][both])
    print(f"1080p t: max relative difference {rel.max():.3e}, 99.99th percentile {np.quantile(rel, 0.9999):.3e}")
    err = np.abs(rad - rad_ref).max(-1) / np.maximum(np.abs(rad_ref).max(-1), 1e-3)
    ok = err <= 1e-4
    print(f"1080p x{sc.spp} per-sample radiance within 1e-4: {ok.mean():.6f} of {ok.size}; "
          f"where the first hit agrees {ok[:, same].mean():.6f}; quantiles 0.5/0.99/0.999 "
          f"{np.quantile(err, [0.5, 0.99, 0.999]).tolist()}")
    assert ok.mean() >= 0.995
    m, mr = rad.mean(0), rad_ref.mean(0)
    assert np.abs(m - mr).mean() <= 1e-2 * max(float(mr.mean()), 1e-3)
