"""Batched requests (kpt_submit_batch / kpt_wait_batch / kpt_autotune_batch).

A batch renders one frame of each job in one CUDA graph: with shared queues
(the default) each level's extension and shadow rays of all jobs are traced
by one launch in the jobs' merged scene, otherwise each job's frame is a
branch of the graph.  Every job's samples are computed exactly as by
kpt_render_frame, so images and accumulations must be bit-identical to
rendering the jobs one by one, in either mode, under any lane count and any
launch tuning (grid share, wave capacity -- a small one forces many waves and
the branch mode --, shading block size, octant sort of the extension rays,
lobe grouping)."""

import ctypes as C

import numpy as np
import pytest

from kittlespt_gb300 import _lib as K


def test_tuning_defaults_and_errors():
    L = K.load()
    t = K.Tuning()
    L.kpt_tuning_default(C.byref(t))
    assert (t.grid_scale, t.wave_cap, t.shade_block, t.sort_rays, t.fetch_batch, t.group_lobes) == (1.0, 0, 256, 0, 7, 2048)
    assert L.kpt_set_tuning(None, C.byref(t)) == -1
    assert L.kpt_get_tuning(None, C.byref(t)) == -1
    assert L.kpt_submit_batch(None, 1, None, None, 0) == -1
    assert L.kpt_wait_batch(None, None, None) == -1
    assert L.kpt_autotune_batch(None, 1, None, None, 1, None, None, None) == -1
    assert L.kpt_batch_destroy(None) == 0


def _jobs():
    from kittlespt_gb300 import scenes as S
    return [
        (S.scene_small_n(96, 64, 2, 4, 3), 2),
        (S.scene_small(128, 72, 3, 3), 3),
        (S.scene_full(160, 90, 1, 5), 1),
        (S.scene_small_n(64, 64, 4, 6, 8, seed=5), 4),
    ]


def _renderers(jobs):
    from kittlespt_gb300.renderer import Renderer
    rs = []
    for sc, _ in jobs:
        r = Renderer(0)
        r.initialize()
        r.load_scene(sc)
        rs.append(r)
    return rs


def _outputs(rs):
    for r in rs:
        r.synchronize()
    return [(r.get_render_target(), r.read_accumulation()) for r in rs]


def _same(a, b, images=True):
    for (ia, aa), (ib, ab) in zip(a, b):
        if images:
            np.testing.assert_array_equal(ia.view(np.uint32), ib.view(np.uint32))
        np.testing.assert_array_equal(aa.view(np.uint32), ab.view(np.uint32))


@pytest.fixture(scope="module")
def reference_frames():
    """Two frames of every job, rendered one by one."""
    jobs = _jobs()
    rs = _renderers(jobs)
    for _ in range(2):
        for r, (_, spp) in zip(rs, jobs):
            r.execute_rendering(16.0, spp)
    out = _outputs(rs)
    for r in rs:
        r.shutdown()
    return jobs, out


@pytest.mark.gpu
@pytest.mark.parametrize("lanes,tuning", [
    (0, None),
    (2, None),
    (1, dict(grid_scale=0.25, wave_cap=1024, shade_block=64)),
    (3, dict(grid_scale=0.5, wave_cap=4096, shade_block=256, sort_rays=1)),
    (0, dict(sort_rays=1)),
    (2, dict(fetch_batch=1)),
    (0, dict(fetch_batch=32)),
    (0, dict(group_lobes=-1)),
    (2, dict(group_lobes=64, shade_block=128)),
    (0, dict(group_lobes=256, shade_block=64)),
])
@pytest.mark.parametrize("shared", [True, False])
def test_batch_matches_one_by_one(reference_frames, lanes, tuning, shared):
    from kittlespt_gb300.renderer import Batch
    jobs, ref = reference_frames
    rs = _renderers(jobs)
    spp = [s for _, s in jobs]
    try:
        if tuning:
            for r in rs:
                r.set_tuning(**tuning)
        with Batch(0) as b:
            assert b.shared
            b.shared = shared
            for _ in range(2):
                b.submit(rs, spp, lanes=lanes)
                job_ms, total = b.wait()
                assert job_ms.shape == (len(rs),) and np.all(job_ms > 0)
                assert total == pytest.approx(float(job_ms.max()))
        _same(_outputs(rs), ref)
        assert all(r.stats().frame_index == 2 * s for r, s in zip(rs, spp))
    finally:
        for r in rs:
            r.shutdown()


@pytest.mark.gpu
def test_batch_errors():
    from kittlespt_gb300.renderer import Batch
    from kittlespt_gb300 import scenes as S
    rs = _renderers([(S.scene_small(32, 32, 1, 2), 1)])
    try:
        with Batch(0) as b:
            with pytest.raises(K.KptError):
                b.submit(rs + rs, [1, 1])       # one context twice
            with pytest.raises(K.KptError):
                b.submit(rs, [0])               # no samples
            with pytest.raises(K.KptError):
                b.wait()                        # nothing submitted
            b.submit(rs, [1])
            with pytest.raises(K.KptError):
                b.submit(rs, [1])               # previous batch not waited for
            b.wait()
        with Batch(0) as b:
            with pytest.raises(K.KptError):
                b.shared = 2                    # not a mode
            b.submit(rs, [1])
            with pytest.raises(K.KptError):
                b.shared = False                # a batch is pending
            b.wait()
        with pytest.raises(K.KptError):
            rs[0].set_tuning(grid_scale=0.0)
        with pytest.raises(K.KptError):
            rs[0].set_tuning(wave_cap=100)
        with pytest.raises(K.KptError):
            rs[0].set_tuning(shade_block=96)
        with pytest.raises(K.KptError):
            rs[0].set_tuning(sort_rays=2)
        with pytest.raises(K.KptError):
            rs[0].set_tuning(fetch_batch=33)
        for g in (1, 96, 4096):
            with pytest.raises(K.KptError):
                rs[0].set_tuning(group_lobes=g)
    finally:
        for r in rs:
            r.shutdown()


@pytest.mark.gpu
def test_autotune_applies_and_caches(reference_frames):
    from kittlespt_gb300.renderer import Batch
    jobs, ref = reference_frames
    rs = _renderers(jobs)
    spp = [s for _, s in jobs]
    try:
        with Batch(0) as b:
            t1, lanes1, ms1 = b.autotune(rs, spp, reps=1)
            assert 0.0 < t1["grid_scale"] <= 1.0 and t1["shade_block"] in (64, 128, 256)
            assert 1 <= lanes1 <= len(rs) and ms1 > 0.0
            assert all(r.tuning() == t1 for r in rs)
            assert all(r.stats().frame_index == 0 for r in rs)   # tuning frames discarded
            t2, lanes2, ms2 = b.autotune(rs, spp, reps=1)          # cached: same choice, no rendering
            assert (t2, lanes2, ms2) == (t1, lanes1, ms1)
            for _ in range(2):
                b.submit(rs, spp, lanes=lanes1)
                b.wait()
        # the eye adaptation of the discarded frames persists (resetAccumulation
        # keeps it, renderer.cu:336-340): only the accumulation is compared
        _same(_outputs(rs), ref, images=False)
    finally:
        for r in rs:
            r.shutdown()


@pytest.mark.gpu
def test_batch_matches_oracle():
    """One batch of the four jobs against the CPU oracle directly: each job's
    accumulation (the clamped samples of its frame, summed in sample order)
    against the oracle's samples of the same frame indices summed in the same
    order.  A pixel's sum differs beyond 1e-4 relative only where one of its
    samples does (the per-sample rule of tests/parity_rule.py, checked on
    these scenes in tests/test_gpu_parity.py): >= 99% of the pixels of every
    job within 1e-4, and the mean images within 1e-3."""
    from kittlespt_gb300.renderer import Batch
    from oracle import oracle as O
    jobs = _jobs()
    rs = _renderers(jobs)
    try:
        spp = [s for _, s in jobs]
        with Batch(0) as b:
            b.submit(rs, spp, lanes=0)
            b.wait()
        accs = [r.read_accumulation()[..., :3] for r in rs]
    finally:
        for r in rs:
            r.shutdown()
    for (sc, n), acc in zip(jobs, accs):
        ref = O.Scene(sc).render_samples(0, n, rng_order=0)["radiance"]
        s = np.zeros_like(ref[0])
        for k in range(n):
            s = (s + ref[k]).astype(np.float32)
        err = np.abs(acc - s).max(-1) / np.maximum(np.abs(s).max(-1), 1e-3 * n)
        print(f"{sc.width}x{sc.height}x{n}: {(err <= 1e-4).mean():.5f} of pixels within 1e-4")
        assert (err <= 1e-4).mean() >= 0.99
        assert np.abs(acc - s).mean() <= 1e-3 * max(float(np.abs(s).mean()), 1e-3)


@pytest.mark.gpu
def test_batch_follows_scene_changes():
    """The shared queues trace in a merged copy of the jobs' scenes, rebuilt
    when a job's scene changes: after an instance moves in one job and a
    mesh is refit in another, the next batch still matches the same jobs
    rendered one by one, bit for bit."""
    from kittlespt_gb300.renderer import Batch
    jobs = _jobs()
    spp = [s for _, s in jobs]
    batched, single = _renderers(jobs), _renderers(jobs)

    def change(rs):
        sc0 = jobs[0][0]
        m = np.array(sc0.instances[-1].model, np.float32)
        m[0, 3] += 0.2
        assert rs[0].set_mesh_transform(len(sc0.instances) - 1, m)
        pos = jobs[2][0].meshes[0].positions * np.float32(1.05)
        rs[2].refit_mesh(0, pos)

    try:
        with Batch(0) as b:
            assert b.shared
            b.submit(batched, spp)
            b.wait()
            for r, s in zip(single, spp):
                r.execute_rendering(16.0, s)
            _same(_outputs(batched), _outputs(single))
            change(batched)
            change(single)
            for _ in range(2):
                b.submit(batched, spp)
                b.wait()
                for r, s in zip(single, spp):
                    r.execute_rendering(16.0, s)
            _same(_outputs(batched), _outputs(single))
    finally:
        for r in batched + single:
            r.shutdown()


@pytest.mark.gpu
@pytest.mark.parametrize("shared", [True, False])
def test_batch_with_post_features(shared):
    """Jobs whose post chains differ -- temporal accumulation, lens effects,
    FSR upscaling, auto exposure off -- batched, against the same jobs
    rendered one by one: every job's display image and accumulation
    bit-identical, over three submissions (the temporal history carries
    over between them)."""
    from kittlespt_gb300.renderer import Batch
    from kittlespt_gb300 import scenes as S
    jobs = [(S.scene_small(96, 64, 2, 4), 2), (S.scene_small_n(80, 48, 1, 5, 3), 3), (S.scene_full(128, 72, 1, 3), 1)]
    settings = [dict(temporal_accumulation=1), dict(postprocess_effects=1, upscale=2), dict(auto_exposure=0, bloom=0)]
    spp = [s for _, s in jobs]

    def make():
        rs = _renderers(jobs)
        for r, kw in zip(rs, settings):
            r.set_renderer_settings(**kw)
        return rs

    batched, single = make(), make()
    try:
        with Batch(0) as b:
            b.shared = shared
            for _ in range(3):
                b.submit(batched, spp)
                b.wait()
                for r, s in zip(single, spp):
                    r.execute_rendering(16.0, s)
        for ra, rb in zip(batched, single):
            ra.synchronize()
            rb.synchronize()
            np.testing.assert_array_equal(ra.get_render_target().view(np.uint32),
                                          rb.get_render_target().view(np.uint32))
            np.testing.assert_array_equal(ra.read_render().view(np.uint32), rb.read_render().view(np.uint32))
    finally:
        for r in batched + single:
            r.shutdown()
