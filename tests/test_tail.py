"""The wave's tail (kpt_tuning.tail_paths): once few paths enter a level, one
thread finishes each of them -- shading, shadow ray, continuation -- instead
of the remaining per-level launches.  It must change no result: the
per-sample radiance, the camera-ray hits and the level counters are the same
bit for bit with the tail off, at its default threshold, and taking over
from the first level (every bounce then runs in the tail)."""

import numpy as np
import pytest

from kittlespt_gb300 import scenes as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def render(sc, n, tail_paths):
    from kittlespt_gb300.renderer import Renderer
    with Renderer(0) as r:
        r.load_scene(sc)
        r.set_tuning(tail_paths=tail_paths)
        rad = torch.zeros((n, sc.height, sc.width, 4), dtype=torch.float32, device="cuda:0")
        hit = torch.zeros((sc.height, sc.width, 4), dtype=torch.int32, device="cuda:0")
        r.render_samples_device(0, n, rad.data_ptr(), hit.data_ptr())
        r.synchronize()
        levels = r.level_counts()
        r.execute_rendering(16.0, n)
        r.synchronize()
        img = r.get_render_target()
        return rad.cpu().numpy(), hit.cpu().numpy(), levels, img


@pytest.mark.parametrize("which", ["small", "full", "textured"])
def test_tail_changes_no_result(which):
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    if which == "small":
        sc = S.scene_small(96, 64, 4, 6)
    elif which == "full":
        sc = S.scene_full(160, 90, 4, 8, n_variants=2, subdiv=4, grid=4, n_lights=4)
        sc.sky_arith = 1
    else:
        from tests.golden.make_golden import textured_scene
        sc = textured_scene()
        sc.spp = 4
    n = sc.spp
    off = render(sc, n, -1)
    for tp in (0, 1 << 30):
        on = render(sc, n, tp)
        np.testing.assert_array_equal(on[0].view(np.uint32), off[0].view(np.uint32))
        np.testing.assert_array_equal(on[1], off[1])
        np.testing.assert_array_equal(on[2], off[2])
        np.testing.assert_array_equal(on[3].view(np.uint32), off[3].view(np.uint32))
    assert off[2][2:, 0].sum() > 0   # paths did go past level 1
