"""Lens effects (kpt_settings.postprocess_effects, the reference's
postprocess_enable_effects: computeEffects with getFishEyeUV,
kernels.cu:340-374, 506-527).  The frame with effects is the frame without
them resampled by the oracle's restatement: every output texel is a copy of
one input texel, so pixels compare exactly; a pixel may pick a neighbouring
texel where CUDA's tanf / powf and the host's round a coordinate across a
texel edge."""

import numpy as np
import pytest

from kittlespt_gb300 import scenes as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("w,h", [(96, 64), (80, 80), (67, 45)])
def test_effects_match_oracle(w, h):
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_small(w, h, 1, 3)
    sc.settings["bloom"] = 1
    imgs = []
    for fx in (0, 1):
        r = Renderer(0)
        r.initialize()
        try:
            r.load_scene(sc)
            r.set_renderer_settings(postprocess_effects=fx)
            r.execute_rendering(16.0, 2)
            r.synchronize()
            imgs.append(r.get_render_target())
        finally:
            r.shutdown()
    ref = O.effects(imgs[0])
    same = (imgs[1] == ref).all(-1)
    assert same.mean() >= 0.995, f"{same.mean():.4f} of pixels equal"
    assert not np.array_equal(imgs[0], imgs[1])   # the effects changed the image
    if O.available("refgpu"):
        # the reference's own computeEffects kernel (its GPU build, fast
        # maths) on the same image: it pins the oracle's restatement and the
        # CUDA path alike, up to texels whose coordinate its fast tanf / powf
        # round across an edge
        rg = O.ref_gpu_effects(imgs[0])
        so = (rg == ref).all(-1).mean()
        sg = (rg == imgs[1]).all(-1).mean()
        print(f"{w}x{h}: reference GPU effects equal the oracle's on {so:.4f}, ours on {sg:.4f} of pixels")
        assert so >= 0.99 and sg >= 0.99


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("bloom", [0, 1])
def test_upscale_matches_oracle(bloom, mode):
    """kpt_settings.upscale (the reference's upscale_enable): the render at the
    output resolution / 2.5, upscaled bilinearly (1) or by the FSR path, EASU
    then RCAS (2), then bloom and tonemapping at the output resolution."""
    from kittlespt_gb300.renderer import Renderer
    sc = S.scene_small(80, 60, 1, 3)
    sc.settings["bloom"] = bloom
    r = Renderer(0)
    r.initialize()
    try:
        r.load_scene(sc)
        r.set_renderer_settings(upscale=mode)
        assert r.render_size() == (32, 24)
        with pytest.raises(Exception):
            r.set_renderer_settings(upscale=3)
        assert r.get_renderer_settings().upscale == mode
        r.execute_rendering(16.0, 2)
        r.synchronize()
        render = r.read_render()
        img = r.get_render_target()
    finally:
        r.shutdown()
    assert render.shape == (24, 32, 4) and img.shape == (60, 80, 4)
    out = O.upscale(render, 80, 60) if mode == 1 else O.fsr(render, 80, 60)[1]
    if mode == 2:   # the sharpened image is not the bilinear one
        assert np.abs(out - O.upscale(render, 80, 60)).max() > 1e-3
    bl = O.bloom(out, False, float(sc.settings["bloom_internal_blend"])) if bloom else None
    ref = O.post_image(out, bl, float(sc.settings["bloom_final_blend"]), O.exposure_scalar(sc.exposure))
    err = np.abs(img - ref).max(-1)
    assert err.max() <= 2e-5, f"{(err > 2e-5).mean():.4f} of pixels off, worst {err.max()} at {np.argwhere(err > 2e-5)[:8]}"
