"""Temporal accumulation (kpt_settings.temporal_accumulation, the reference's
integrator_use_temporal_accumulation, kernels.cu:164-327 and :422-428): each
sample of a call is one reference frame, blended into the previous frame's
image reprojected along the visible surface's motion.  The GPU image after
every call of a sequence with camera and instance motion is compared with
the oracle's restatement (oracle/kpt_oracle.cpp orc_temporal_frame) driven
by the oracle's own samples: reprojection decisions depend on exact
geometry (camera rays, first hits and distances are bit-exact), the blended
colors on the per-sample radiance (1e-4 relative), so >= 99% of the pixels
must agree within 1e-4 relative."""

import copy

import numpy as np
import pytest

from kittlespt_gb300 import scenes as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _oracle_call(sc, frame_index, n, state):
    """Advances the oracle's temporal state by one render call of n samples."""
    ref = O.Scene(sc).render_samples(frame_index, n)
    inst = ref["first_hit"][..., 1]
    t = np.where(inst >= 0, ref["first_t"], np.float32(np.inf)).astype(np.float32)
    H, W = inst.shape
    for k in range(n):
        prev_cam = state["cam_prev"] if k == 0 else state["cam"]
        prev_depth = state["depth"] if k == 0 else t
        sample = np.zeros((H, W, 4), np.float32)
        sample[..., :3] = ref["radiance"][k]
        state["hist"] = O.temporal_frame(prev_cam, state["cam"], state["models"], state["models_prev"], inst, t,
                                         sample, prev_depth, state["hist"])
    state["depth"] = t
    state["cam_prev"] = state["cam"]
    return O.modulate(state["hist"][..., :3], 1, ref["albedo"])[..., :3]


def _close(gpu, ref, what):
    err = np.abs(gpu - ref).max(-1) / np.maximum(np.abs(ref).max(-1), 1e-3)
    frac = (err <= 1e-4).mean()
    assert frac >= 0.99, f"{what}: {frac:.4f} of pixels within 1e-4"


def test_temporal_sequence_matches_oracle():
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_small_n(64, 48, 1, 3, 4)
    r = Renderer(0)
    r.initialize()
    try:
        r.load_scene(sc)
        r.set_renderer_settings(temporal_accumulation=1)
        cam = (sc.camera.inv_proj.astype(np.float32), sc.camera.inv_view.astype(np.float32))
        models = [np.asarray(i.model, np.float32) for i in sc.instances]
        state = dict(hist=np.zeros((48, 64, 4), np.float32), depth=np.zeros((48, 64), np.float32),
                     cam=cam, cam_prev=cam, models=list(models), models_prev=list(models))
        frame = 0
        steps = [("render", 2), ("camera", (0.06, 0.03, 0.0)), ("render", 1), ("instance", (1, 0.15)),
                 ("render", 3), ("render", 1), ("camera", (-0.1, 0.0, 0.05)), ("instance", (2, -0.2)),
                 ("render", 2)]
        seen_history = False
        for kind, arg in steps:
            if kind == "camera":
                iv = state["cam"][1].copy()
                iv[:3, 3] += np.asarray(arg, np.float32)
                state["cam_prev"], state["cam"] = state["cam"], (state["cam"][0], iv)
                sc = copy.deepcopy(sc)
                sc.camera.inv_view = iv
                r.set_camera_inverse(state["cam"][0], iv)
            elif kind == "instance":
                k, dx = arg
                m = state["models"][k].copy()
                m[0, 3] += dx
                # TriangleMesh::setTransform (triangle.cuh:142-146): only this
                # instance's previous transform changes; another instance
                # moved earlier keeps its old previous transform (and velocity)
                state["models_prev"][k] = state["models"][k]
                state["models"][k] = m
                sc = copy.deepcopy(sc)
                sc.instances[k] = S.Instance(sc.instances[k].mesh, m, sc.instances[k].material)
                r.set_mesh_transform(k, m)
            else:
                r.execute_rendering(16.0, arg)
                r.synchronize()
                gpu = r.read_render()[..., :3]
                ref = _oracle_call(sc, frame, arg, state)
                frame += arg
                _close(gpu, ref, f"after {frame} frames")
                seen_history |= bool((state["hist"][..., 3] >= 2).any())
        # the history did carry over between frames (reprojection succeeded)
        assert seen_history
    finally:
        r.shutdown()


def test_temporal_long_history_matches_oracle():
    """A static camera over 20 frames in one call: the history reaches the cap
    of 16 frames."""
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_small(48, 32, 1, 2)
    r = Renderer(0)
    r.initialize()
    try:
        r.load_scene(sc)
        r.set_renderer_settings(temporal_accumulation=1)
        r.execute_rendering(16.0, 20)
        r.synchronize()
        gpu = r.read_render()[..., :3]
    finally:
        r.shutdown()
    cam = (sc.camera.inv_proj.astype(np.float32), sc.camera.inv_view.astype(np.float32))
    models = [np.asarray(i.model, np.float32) for i in sc.instances]
    state = dict(hist=np.zeros((32, 48, 4), np.float32), depth=np.zeros((32, 48), np.float32),
                 cam=cam, cam_prev=cam, models=list(models), models_prev=list(models))
    ref = _oracle_call(sc, 0, 20, state)
    assert state["hist"][..., 3].max() >= 16
    _close(gpu, ref, "20 frames")


@pytest.mark.parametrize("arith", [1, 0])
def test_temporal_sequence_matches_reference_gpu(arith):
    """The same sequence of camera and instance motion through the
    reference's own megakernel with temporal accumulation on (its GPU build,
    driven frame by frame as Renderer::executeRendering does:
    oracle/ref_harness/ref_gpu_harness.cu refgpu_temporal_frame), with the
    CUDA path in the same build's sky arithmetic, and its temporal
    reprojection in that build's arithmetic (temporal_arith = 1) or in IEEE
    (0).  The reference computes the velocity from four approximate matrix
    inverses per pixel, so even a still camera gives velocities of a few
    ulps, and its reprojection truncates the previous pixel coordinate: a
    pixel whose coordinate lands an ulp below an integer takes its history
    length (point-sampled) and bilinear weights from the texel one over.
    Those ulps also follow the visible-surface position and depth, which
    temporal_arith 1 recomputes as that build does (its fast-maths camera
    ray, the hit triangle's distance by its fast-maths triangle test, o + t
    d).  Measured (history lengths equal to the reference's / modulated
    images within 1e-4 relative, after 2, 3, 6, 7 and 9 frames):
    temporal_arith 1: 100/99.97, 100/100, 100/99.97, 100/99.97, 100/99.93%;
    temporal_arith 0 (IEEE, the oracle's arithmetic): 94.2/99.97, 94.3/94.2,
    89.2/88.9, 88.9/88.4, 87.1/89.2% -- a pixel whose decision differed once
    keeps a different history until it saturates at 16 frames.  The test
    asserts 99.9% / 99.5% after every call for temporal_arith 1, 85% for
    IEEE."""
    from kittlespt_gb300.renderer import Renderer
    if not O.available("refgpu"):
        pytest.skip("reference GPU build absent (reference sources not staged)")
    sc = S.scene_small_n(64, 48, 1, 3, 4)
    sc.sky_arith = 1
    sc.temporal_arith = arith
    g = O.RefGpuScene(sc)
    r = Renderer(0)
    r.initialize()
    try:
        r.load_scene(sc)
        r.set_renderer_settings(temporal_accumulation=1)
        cam = (sc.camera.inv_proj.astype(np.float32), sc.camera.inv_view.astype(np.float32))
        models = [np.asarray(i.model, np.float32) for i in sc.instances]
        state = dict(hist=np.zeros((48, 64, 4), np.float32), depth=np.zeros((48, 64), np.float32),
                     cam=cam, cam_prev=cam, models=list(models), models_prev=list(models))
        frame, first, seen = 0, True, []
        steps = [("render", 2), ("camera", (0.06, 0.03, 0.0)), ("render", 1), ("instance", (1, 0.15)),
                 ("render", 3), ("render", 1), ("camera", (-0.1, 0.0, 0.05)), ("instance", (2, -0.2)),
                 ("render", 2)]
        for kind, arg in steps:
            if kind == "camera":
                iv = state["cam"][1].copy()
                iv[:3, 3] += np.asarray(arg, np.float32)
                state["cam_prev"], state["cam"] = state["cam"], (state["cam"][0], iv)
                sc = copy.deepcopy(sc)
                sc.camera.inv_view = iv
                r.set_camera_inverse(state["cam"][0], iv)
            elif kind == "instance":
                k, dx = arg
                m = state["models"][k].copy()
                m[0, 3] += dx
                state["models_prev"][k] = state["models"][k]
                state["models"][k] = m
                sc = copy.deepcopy(sc)
                sc.instances[k] = S.Instance(sc.instances[k].mesh, m, sc.instances[k].material)
                r.set_mesh_transform(k, m)
            else:
                r.execute_rendering(16.0, arg)
                r.synchronize()
                gpu = r.read_render()[..., :3]
                for f in range(frame, frame + arg):
                    rimg, racc = g.temporal_frame(f, reset=first, camera=state["cam"], models=state["models"])
                    first = False
                _oracle_call(sc, frame, arg, state)
                frame += arg
                same_oracle = (racc[..., 3] == state["hist"][..., 3]).mean()
                same_hist = (racc[..., 3] == r.read_history()[..., 3]).mean()
                err = np.abs(gpu - rimg[..., :3]).max(-1) / np.maximum(np.abs(rimg[..., :3]).max(-1), 1e-3)
                close = (err <= 1e-4).mean()
                print(f"temporal_arith {arith}, after {frame} frames: history lengths equal on {same_hist:.4f} "
                      f"(oracle's: {same_oracle:.4f}), images within 1e-4 on {close:.4f} of the pixels")
                seen.append((frame, same_hist, close))
        floor_h, floor_c = (0.999, 0.995) if arith == 1 else (0.85, 0.85)
        assert all(h >= floor_h and c >= floor_c for _, h, c in seen), seen
        assert (racc[..., 3] >= 2).any()
    finally:
        r.shutdown()
        g.close()


def test_temporal_settings_and_history_errors():
    """temporal_arith takes 0 or 1; the history readback needs a frame
    rendered with temporal accumulation; the history's alpha counts the
    blended frames (at most one per sample)."""
    from kittlespt_gb300 import _lib as K
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_small(32, 24, 1, 2)
    r = Renderer(0)
    r.initialize()
    try:
        r.load_scene(sc)
        assert r.get_renderer_settings().temporal_arith == 0   # the scene's (oracle) arithmetic
        with pytest.raises(K.KptError):
            r.set_renderer_settings(temporal_arith=2)
        with pytest.raises(K.KptError):
            r.read_history()                       # no temporal frame yet
        r.set_renderer_settings(temporal_accumulation=1, temporal_arith=1)
        r.execute_rendering(16.0, 3)
        r.synchronize()
        hist = r.read_history()
        assert hist.shape == (24, 32, 4)
        # history lengths are frame counts: at most one per sample, and
        # camera hits carry history after 3 samples; sky pixels none
        counts = hist[..., 3]
        assert set(np.unique(counts).tolist()) <= {0.0, 1.0, 2.0, 3.0}, np.unique(counts)
        assert counts.max() >= 2.0
    finally:
        r.shutdown()
