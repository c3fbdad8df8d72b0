"""BLAS refit on the GPU (kpt_refit_mesh): new positions, the same tree.
Every node's child boxes must be the bounds of the triangles under them
(recomputed here from the tree and the new positions), closest hits the
oracle's brute force over the deformed scene, and frames those of the
deformed scene loaded afresh (whose tree differs, which changes no hit)."""

import copy

import numpy as np
import pytest

from kittlespt_gb300 import scenes as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _deformed(sc, mesh, seed):
    rng = np.random.default_rng(seed)
    m = sc.meshes[mesh]
    pos = m.positions.astype(np.float32).copy()
    pos *= np.float32(1.15)
    pos += rng.normal(0.0, 0.01, pos.shape).astype(np.float32)
    sc2 = copy.deepcopy(sc)
    sc2.meshes[mesh] = S.Mesh(pos, m.normals, m.uvs, m.material)
    return sc2, pos


def _expected_boxes(blas, pos):
    """Child boxes of every node from the tree and the positions."""
    boxes, refs, order = blas["boxes"], blas["refs"], blas["order"]
    tri = pos.reshape(-1, 9)[order]                      # leaf order
    lo_t = np.minimum(np.minimum(tri[:, 0:3], tri[:, 3:6]), tri[:, 6:9])
    hi_t = np.maximum(np.maximum(tri[:, 0:3], tri[:, 3:6]), tri[:, 6:9])
    out = np.zeros_like(boxes)
    done = np.zeros(len(boxes), bool)

    def child(ref, cnt):
        if cnt > 0:
            return lo_t[ref:ref + cnt].min(0), hi_t[ref:ref + cnt].max(0)
        node(ref)
        b = out[ref]
        return np.minimum(b[0:3], b[6:9]), np.maximum(b[3:6], b[9:12])

    def node(k):
        if done[k]:
            return
        for s in range(2):
            lo, hi = child(refs[k, 2 * s], refs[k, 2 * s + 1])
            out[k, 6 * s:6 * s + 3], out[k, 6 * s + 3:6 * s + 6] = lo, hi
        done[k] = True

    for k in range(len(boxes) - 1, -1, -1):
        node(k)
    return out


def test_refit_boxes_hits_and_frames():
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_full(96, 54, 2, 4, n_variants=2, subdiv=4, grid=3, n_lights=4)
    mesh = 0
    sc2, pos = _deformed(sc, mesh, 3)
    o, d = S.random_rays(40000, 9, center=(0, 1, 0), radius=9.0)
    r = Renderer(0)
    r.initialize()
    try:
        r.load_scene(sc)
        before = r.get_blas(mesh)
        r.refit_mesh(mesh, pos)
        after = r.get_blas(mesh)
        # the tree is kept; every box is the bounds of the triangles below it
        np.testing.assert_array_equal(before["refs"], after["refs"])
        np.testing.assert_array_equal(before["order"], after["order"])
        assert np.array_equal(after["boxes"], _expected_boxes(after, pos))
        assert not np.array_equal(before["boxes"], after["boxes"])
        # closest hits: the oracle's brute force over the deformed scene
        from tests.test_gpu_parity import bits, global_prim, gpu_trace
        inst, tri, t = gpu_trace(r, o, d)
        ref = O.Scene(sc2).trace(o, d, brute=True)
        np.testing.assert_array_equal(global_prim(sc2, inst, tri), ref["prim"])
        np.testing.assert_array_equal(bits(t), bits(ref["t"]))
        assert (ref["prim"] >= 0).mean() > 0.02
        r.execute_rendering(16.0, 2)
        r.synchronize()
        img_refit = r.get_render_target()
    finally:
        r.shutdown()
    r2 = Renderer(0)
    r2.initialize()
    try:
        r2.load_scene(sc2)
        r2.execute_rendering(16.0, 2)
        r2.synchronize()
        img_fresh = r2.get_render_target()
    finally:
        r2.shutdown()
    same = (img_refit.view(np.uint32) == img_fresh.view(np.uint32)).all(-1)
    assert same.mean() >= 0.999, same.mean()


def test_refit_errors():
    from kittlespt_gb300 import _lib as K
    L = K.load()
    assert L.kpt_refit_mesh(None, 0, None, None) == -1
