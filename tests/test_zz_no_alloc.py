"""kpt_trace_bounces_noalloc: the ray-bounce call for callers that must not
allocate device memory (a frame loop that must not stall on cudaMalloc or
cudaFree, or an application with a fixed device-memory budget).  It stages
rays and hits in a fixed array inside the library instead of cudaMalloc'd
buffers, and must return exactly what kpt_trace_bounces returns.

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


def test_no_device_memory_is_taken(renderer):
    o, d = S.random_rays(30000, 24)
    noalloc(renderer, o, d, 3)            # warm-up: module loading, staging look-up
    torch.cuda.synchronize()
    before = torch.cuda.mem_get_info(0)[0]
    for _ in range(3):
        noalloc(renderer, o, d, 3)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == before


def test_zero_rays_and_zero_bounces(renderer):
    from kittlespt_gb300 import _lib as K
    z = np.zeros(3, np.float32)
    zi = np.zeros(1, np.int32)
    assert renderer._L.kpt_trace_bounces_noalloc(renderer.ctx, 0, K.fptr(z), K.fptr(z), 4, K.iptr(zi),
                                                 K.iptr(zi.copy()), K.fptr(z.copy())) == 0
    o, d = S.random_rays(5000, 25)
    a = renderer.trace_bounces(o, d, 0)
    b = noalloc(renderer, o, d, 0)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(np.ascontiguousarray(x).view(np.uint32).reshape(-1),
                                      np.ascontiguousarray(y).view(np.uint32).reshape(-1))


def test_rejects_bounce_counts_whose_size_would_overflow(renderer):
    from kittlespt_gb300 import _lib as K
    o, d = S.random_rays(4, 26)
    buf = np.zeros(64, np.int32)
    t = np.zeros(64, np.float32)
    for n, nb in ((4, 2**31 - 1), (700_000_000, 2**31 - 2), (1, (8 << 20) // 12)):
        st = renderer._L.kpt_trace_bounces_noalloc(renderer.ctx, n, K.fptr(o.reshape(-1)), K.fptr(d.reshape(-1)),
                                                   nb, K.iptr(buf), K.iptr(buf.copy()), K.fptr(t))
        assert st == -1, (n, nb)


def test_refuses_a_pending_transform_change():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from kittlespt_gb300 import _lib as K
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_small(16, 16, 1, 2)
    with Renderer(0) as r:
        r.load_scene(sc)
        o, d = S.random_rays(1000, 27, center=(0, 0, 0), radius=6.0)
        noalloc(r, o, d, 2)
        assert r.set_mesh_transform(0, S.translate(-1.4, 0.1, 0.0))
        inst = np.zeros(3 * 1000, np.int32)
        t = np.zeros(3 * 1000, np.float32)
        st = r._L.kpt_trace_bounces_noalloc(r.ctx, 1000, K.fptr(o.reshape(-1)), K.fptr(d.reshape(-1)), 2,
                                            K.iptr(inst), K.iptr(inst.copy()), K.fptr(t))
        assert st == -3
        # after the allocating call has rebuilt the top level, the no-alloc call
        # agrees with it on the moved scene
        a = r.trace_bounces(o, d, 2)
        b = noalloc(r, o, d, 2)
        for x, y in zip(a, b):
            np.testing.assert_array_equal(np.ascontiguousarray(x).view(np.uint32),
                                          np.ascontiguousarray(y).view(np.uint32))
