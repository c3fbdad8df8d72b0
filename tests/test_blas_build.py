"""Device BLAS build (kpt_set_blas_build): the tree of the host build (the
reference's binned SAH, as_builder.cuh:110-261) -- every node's child boxes,
child references, the leaf ranges and the triangle order inside each leaf --
and therefore the same images.  Boxes are compared by value (a zero may
differ in sign: the device reduces min/max in another order); everything
else bit for bit."""

import ctypes as C

import numpy as np
import pytest

from kittlespt_gb300 import _lib as K
from kittlespt_gb300 import scenes as S


def _sequential_partition(goes_left):
    """The reference's in-place partition (as_builder.cuh:196-203) on positions."""
    a = list(range(len(goes_left)))
    i, j = 0, len(a) - 1
    while i <= j:
        if goes_left[a[i]]:
            i += 1
        else:
            a[i], a[j] = a[j], a[i]
            j -= 1
    return a


def _closed_form(goes_left):
    """The closed form each thread of kpt_build.cu's partition evaluates."""
    n = len(goes_left)
    L = np.asarray(goes_left, bool)
    R = ~L
    nl, nr = int(L.sum()), int(R.sum())
    xr = np.nonzero(R)[0]                                   # XR(m) = xr[m - 1]
    yl = np.concatenate([[0], n - np.nonzero(L)[0][::-1]])  # YL(m) = yl[m]
    ev = None
    for m in range(1, min(nr, nl) + 2):
        if m > nr or xr[m - 1] >= n - yl[m - 1]:
            ev = (m, True)
            break
        if m > nl or n - yl[m] <= xr[m - 1]:
            ev = (m, False)
            break
    m, xfail = ev
    a = n - yl[m - 1] if xfail else xr[m - 1] + 1
    r_before = np.concatenate([[0], np.cumsum(R)])[:-1]
    l_after = nl - np.cumsum(L)
    out = [None] * n
    for p in range(n):
        if p < a:
            dst = p if L[p] else n - 1 - yl[r_before[p]]
        else:
            dst = xr[l_after[p]] if L[p] else p - 1
        assert out[dst] is None
        out[dst] = p
    return out


def test_partition_closed_form_matches_sequential():
    rng = np.random.default_rng(5)
    for _ in range(3000):
        n = int(rng.integers(1, 64))
        flags = list(rng.random(n) < rng.random())
        assert _closed_form(flags) == _sequential_partition(flags), flags
    for n in (1, 2, 9, 33):
        for flags in ([True] * n, [False] * n, [i % 2 == 0 for i in range(n)], [i >= n // 2 for i in range(n)]):
            assert _closed_form(flags) == _sequential_partition(flags)


def _meshes():
    rng = np.random.default_rng(17)
    out = []
    for n, seed in ((1, 1), (8, 2), (9, 3), (100, 4), (5000, 5), (200_000, 6)):
        out.append((f"random{n}", S.random_triangles(n, seed=seed).positions))
    out.append(("icosphere5", S.displaced_icosphere(subdiv=5, amplitude=0.1, seed=3).positions))
    out.append(("uv_sphere", S.uv_sphere(48, 24).positions))
    out.append(("quad", S.quad(4.0, 4.0).positions))
    # a flat grid: every centroid has the same y
    g = []
    for i in range(40):
        for j in range(40):
            a, b, c, d = (i, 0, j), (i + 1, 0, j), (i + 1, 0, j + 1), (i, 0, j + 1)
            g += [a + b + c, a + c + d]
    out.append(("grid", np.asarray(g, np.float32).reshape(-1, 9) * 0.1))
    # identical triangles: no axis has distinct centroids
    t = rng.random(9).astype(np.float32)
    out.append(("identical", np.tile(t, (50, 1))))
    # duplicated random triangles, and a few far outliers
    p = S.random_triangles(3000, seed=9).positions.reshape(-1, 9)
    p = np.concatenate([p, p[:1500], p[:10] + 50.0]).astype(np.float32)
    out.append(("duplicates", p))
    return out


def _upload(L, ctx, pos):
    pos = np.ascontiguousarray(pos, np.float32).reshape(-1)
    n = pos.size // 9
    mat = np.zeros(n, np.int32)
    mesh = C.c_int()
    K.check(L.kpt_upload_mesh(ctx, n, K.fptr(pos), None, None, K.iptr(mat), C.byref(mesh)))
    return mesh.value


def _blas(L, ctx, mesh):
    info = np.zeros(5, np.int32)
    K.check(L.kpt_get_blas(ctx, mesh, K.iptr(info), None, None, None))
    raw = np.zeros((max(int(info[0]), 1), 16), np.float32)
    order = np.zeros(int(info[4]), np.int32)
    bounds = np.zeros(6, np.float32)
    K.check(L.kpt_get_blas(ctx, mesh, K.iptr(info), K.fptr(raw.reshape(-1)), K.iptr(order), K.fptr(bounds)))
    k = int(info[0])
    return info, raw[:k, :12].copy(), raw[:k, 12:].view(np.int32).copy(), order, bounds


@pytest.mark.gpu
def test_device_blas_equals_host_blas():
    L = K.load()
    ctx = C.c_void_p()
    K.check(L.kpt_create(0, C.byref(ctx)))
    try:
        for name, pos in _meshes():
            K.check(L.kpt_set_blas_build(ctx, 0))
            mh = _upload(L, ctx, pos)
            K.check(L.kpt_set_blas_build(ctx, 1))
            md = _upload(L, ctx, pos)
            ih, bh, rh, oh, nh = _blas(L, ctx, mh)
            idv, bd, rd, od, nd = _blas(L, ctx, md)
            np.testing.assert_array_equal(ih, idv, err_msg=name)
            np.testing.assert_array_equal(rh, rd, err_msg=name)
            np.testing.assert_array_equal(oh, od, err_msg=name)
            assert np.array_equal(bh, bd), name
            assert np.array_equal(nh, nd), name
        assert L.kpt_set_blas_build(ctx, 2) == -1
    finally:
        L.kpt_destroy(ctx)


@pytest.mark.gpu
def test_device_blas_frame_is_bit_identical():
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_full(128, 72, 2, 5, n_variants=2, subdiv=4, grid=3, n_lights=4)
    imgs = []
    for device in (False, True):
        r = Renderer(0)
        r.initialize()
        try:
            r.set_blas_build(device)
            r.load_scene(sc)
            r.execute_rendering(16.0, 2)
            r.synchronize()
            imgs.append((r.get_render_target(), r.read_accumulation()))
        finally:
            r.shutdown()
    for a, b in zip(imgs[0], imgs[1]):
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
