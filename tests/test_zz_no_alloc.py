"""kpt_trace_bounces_noalloc: the ray-bounce call for callers that must not
allocate device memory (a stall-free frame loop, a fixed device-memory
budget, or work issued while another library captures a CUDA graph).  It
stages rays and hits in a fixed array inside the library instead of
cudaMalloc'd buffers, and must return exactly what kpt_trace_bounces returns.

This file is collected last on purpose (pytest orders files by name), so a
run that stops at the first failure has run every other test first.  It
passes alone in a fresh process and after the other tests.
"""

import ctypes as C

import numpy as np
import pytest

from kittlespt_gb300 import scenes as S

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def renderer():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from kittlespt_gb300 import build
    build.build()
    from kittlespt_gb300.renderer import Renderer
    r = Renderer(0)
    r.initialize()
    r.load_scene(S.scene_traversal(100000))
    yield r
    r.shutdown()


def noalloc(r, o, d, nb):
    from kittlespt_gb300 import _lib as K
    n = int(o.shape[0])
    inst = np.full((nb + 1) * n, -7, np.int32)
    tri = np.full_like(inst, -7)
    t = np.full((nb + 1) * n, -7.0, np.float32)
    K.check(r._L.kpt_trace_bounces_noalloc(r.ctx, n, K.fptr(np.ascontiguousarray(o, np.float32).reshape(-1)),
                                           K.fptr(np.ascontiguousarray(d, np.float32).reshape(-1)), nb,
                                           K.iptr(inst), K.iptr(tri), K.fptr(t)))
    return inst.reshape(nb + 1, n), tri.reshape(nb + 1, n), t.reshape(nb + 1, n)


def test_matches_the_allocating_call_on_two_calls_in_a_row(renderer):
    # hit ids are integers and t is computed identically, so the tolerance is exact
    for seed, n in ((21, 60000), (22, 23457)):
        o, d = S.random_rays(n, seed)
        a = renderer.trace_bounces(o, d, 4)
        b = noalloc(renderer, o, d, 4)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(np.ascontiguousarray(x).view(np.uint32),
                                          np.ascontiguousarray(y).view(np.uint32))
        assert (a[0][0] >= 0).sum() > 0


def test_rejects_requests_larger_than_the_staging_array(renderer):
    from kittlespt_gb300 import _lib as K
    nb = 4
    n = (8 << 20) // (24 + 12 * (nb + 1)) + 1
    o, d = S.random_rays(n, 23)
    inst = np.zeros((nb + 1) * n, np.int32)
    t = np.zeros((nb + 1) * n, np.float32)
    st = renderer._L.kpt_trace_bounces_noalloc(renderer.ctx, n, K.fptr(o.reshape(-1)), K.fptr(d.reshape(-1)), nb,
                                               K.iptr(inst), K.iptr(inst.copy()), K.fptr(t))
    assert st == -1
    assert b"8 MiB" in renderer._L.kpt_last_error()
