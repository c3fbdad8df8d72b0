"""Path-replay adjoint (kpt_adjoint*): gradients of an image loss with respect
to per-material albedo and roughness and the Nishita sky coefficients.

Checks (GPU):
  * against an FP64 host oracle: the adjoint's frozen path records are
    re-evaluated in double precision (oracle/adjoint_oracle.cpp) and the
    gradient is compared with central differences (h = 1e-3 relative) of
    that estimator, for every parameter: <= 1e-3 relative;
  * against central differences (h = 1e-3) of the GPU forward renderer for
    the sky parameters, which no sampling decision depends on: <= 5e-3, the
    resolution of the single-precision sky's derivative at the sun;
  * through a torch.autograd.Function wrapper (test harness only) on an L2
    image loss between a target rendered with other samples (seed 7) and an
    initial guess perturbed by up to +-20%.
Sizes are reduced versions of the differentiation workload (the small
sphere-pair scene, depth 6)."""

import ctypes as C

import numpy as np
import pytest

from kittlespt_gb300 import _lib as K

W, H, SPP, DEPTH = 48, 40, 4, 6
REL = 1e-3
# central differences of the single-precision forward renderer: at the sun
# direction (every sun light sample) the float sky's derivative is only
# determined to ~3e-3 (measured: float differences with h = 1e-2 and 1e-3
# spread 0.3% around the double-precision derivative the adjoint uses)
RENDERER_REL = 5e-3


def test_adjoint_api_errors_without_context():
    L = K.load()
    n = C.c_int()
    assert L.kpt_adjoint_param_count(None, C.byref(n)) == -1
    assert L.kpt_adjoint(None, 0, 1, None, None, None) == -1
    assert L.kpt_adjoint_forward_device(None, 0, 1, None) == -1
    assert L.kpt_adjoint_backward_device(None, None, None) == -1
    assert L.kpt_adjoint_record_size() == 192


def _scene(seed=3, width=W, height=H, spp=SPP):
    """The sphere-pair scene with random materials and a 400 x 400 ground, so
    that no path leaves the scene below the horizon: there the reference's
    single-precision sky march (the earth's interior on the view ray) is off
    from its exact value by up to ~1%, and the FP64 comparison would measure
    that instead of the adjoint."""
    from kittlespt_gb300 import scenes as S
    sc = S.scene_small(width, height, spp, DEPTH)
    sc.meshes[1] = S.quad(400.0, 400.0, 0.0, True, 2)
    rng = np.random.Generator(np.random.PCG64(seed))
    mats = sc.materials.copy()
    for m in mats:
        m["albedo"] = rng.uniform(0.1, 0.9, 3)
        m["roughness"] = rng.uniform(0.05, 1.0)
    sc.materials = mats
    env = sc.env.copy()
    env["rayleigh_height"] = 8000.0
    env["mie_height"] = 1200.0
    sc.env = env
    return sc


def _theta(sc):
    t = []
    for m in sc.materials:
        t += [float(x) for x in m["albedo"]] + [float(m["roughness"])]
    e = sc.env
    t += [float(x) for x in e["rayleigh"]] + [float(e["mie"]), float(e["rayleigh_height"]), float(e["mie_height"])]
    return np.array(t, np.float64)


def _apply(r, sc, theta):
    for k, m in enumerate(sc.materials):
        mm = m.copy()
        mm["albedo"] = theta[4 * k:4 * k + 3]
        mm["roughness"] = theta[4 * k + 3]
        assert r.set_material(k, mm)
    e = sc.env.copy()
    e["rayleigh"] = theta[-6:-3]
    e["mie"], e["rayleigh_height"], e["mie_height"] = theta[-3], theta[-2], theta[-1]
    r.set_procedural_environment_data(e)


def _fixed(sc):
    e = sc.env
    cp, sp = np.cos(np.float32(e["sun_phi"])), np.sin(np.float32(e["sun_phi"]))
    ct, st = np.cos(np.float32(e["sun_theta"])), np.sin(np.float32(e["sun_theta"]))
    d = np.array([cp * ct, st, sp * ct], np.float64)
    d /= np.linalg.norm(d)
    return [d[0], d[1], d[2], float(e["sun_emission_factor"]), float(e["mie_absorption"]), 6378137.0, 6438137.0]


def _records(r, adjoint, sample0=0, nsamples=SPP, max_rec=1 << 18):
    import torch
    n = C.c_int()
    K.check(r._L.kpt_adjoint_param_count(r.ctx, C.byref(n)))
    adj = torch.from_numpy(np.ascontiguousarray(adjoint, np.float32)).cuda()
    grad = torch.zeros(n.value, dtype=torch.float64, device="cuda")
    rec = torch.zeros(max_rec * 192, dtype=torch.uint8, device="cuda")
    cnt = C.c_int()
    K.check(r._L.kpt_adjoint_records_device(r.ctx, sample0, nsamples, adj.data_ptr(), grad.data_ptr(),
                                            rec.data_ptr(), max_rec, C.byref(cnt)))
    assert 0 < cnt.value <= max_rec
    return grad.cpu().numpy(), rec[:cnt.value * 192].cpu().numpy().tobytes(), cnt.value


def _oracle_fd(records, n, theta, nmat, fixed):
    from oracle import oracle as O

    def E(t):
        return O.adjoint_estimate(records, n, t[:4 * nmat].reshape(nmat, 4)[:, :3], t[:4 * nmat].reshape(nmat, 4)[:, 3],
                                  t[4 * nmat:], fixed)[0]
    g = np.zeros_like(theta)
    for i in range(theta.size):
        h = 1e-3 * abs(theta[i])
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        g[i] = (E(tp) - E(tm)) / (2.0 * h)
    return g, E(theta)


def _compare(gpu, ref, theta, names, rel=REL):
    # relative sensitivities theta_i dE/dtheta_i, compared per parameter with a
    # floor of rel * 1e-2 of the largest one
    sg, sr = gpu * theta, ref * theta
    floor = 1e-2 * np.abs(sr).max()
    bad = [(names[i], sg[i], sr[i]) for i in range(theta.size)
           if abs(sg[i] - sr[i]) > rel * max(abs(sr[i]), floor)]
    assert not bad, "\n".join(f"{n}: adjoint {a:.6e} reference {b:.6e}" for n, a, b in bad)


def _renderer(sc):
    from kittlespt_gb300.renderer import Renderer
    r = Renderer(0)
    r.initialize()
    r.load_scene(sc)
    return r


def _mean_image(r, sample0, nsamples):
    """Per-pixel mean of the forward renderer's clamped samples."""
    import torch
    buf = torch.zeros((nsamples, H, W, 4), dtype=torch.float32, device="cuda")
    r.render_samples_device(sample0, nsamples, buf.data_ptr())
    r.synchronize()
    return buf.mean(dim=0).cpu().numpy().astype(np.float64)


@pytest.mark.gpu
def test_adjoint_matches_fp64_oracle_fd():
    from kittlespt_gb300.renderer import adjoint_param_names
    sc = _scene()
    r = _renderer(sc)
    try:
        theta = _theta(sc)
        nmat = len(sc.materials)
        rng = np.random.Generator(np.random.PCG64(11))
        adj = np.zeros((H, W, 4), np.float32)
        adj[..., :3] = rng.uniform(-1.0, 1.0, (H, W, 3))
        # the records cover the replayed paths of hit pixels; camera-miss
        # pixels (sky only) get no weight here and are checked by the
        # renderer differences below
        hit = _hit_mask(r)
        assert 0 < hit.sum() < hit.size
        adj_hits = adj * hit[..., None]
        grad, records, n = _records(r, adj_hits)
        assert np.isfinite(grad).all(), grad
        assert np.abs(grad).max() > 0
        fd, _ = _oracle_fd(records, n, theta, nmat, _fixed(sc))
        _compare(grad, fd, theta, adjoint_param_names(nmat))
        # the replay's image is the forward renderer's (mean of the clamped
        # samples): per pixel within 1e-4 except where a last-bit difference
        # flips a path decision
        _, img = r.adjoint(0, SPP, adj_hits, want_image=True)
        fwd = _mean_image(r, 0, SPP)
        close = np.abs(img[..., :3] - fwd[..., :3]) <= 1e-4 * np.maximum(np.abs(fwd[..., :3]), 1e-3)
        assert close.all(axis=-1).mean() >= 0.99
    finally:
        r.shutdown()


@pytest.mark.gpu
def test_adjoint_matches_fp64_oracle_fd_at_workload_spp():
    """The same check with the differentiation workload's 32 samples per
    pixel and depth 6 (on 128x96 pixels instead of 512x512): 393,216 paths
    replayed, their frozen records re-evaluated in double by the oracle, all
    18 parameters within 1e-3 of its central differences."""
    from kittlespt_gb300.renderer import adjoint_param_names
    w, h, spp = 128, 96, 32
    sc = _scene(5, w, h, spp)
    r = _renderer(sc)
    try:
        theta = _theta(sc)
        nmat = len(sc.materials)
        rng = np.random.Generator(np.random.PCG64(13))
        adj = np.zeros((h, w, 4), np.float32)
        adj[..., :3] = rng.uniform(-1.0, 1.0, (h, w, 3))
        adj *= _hit_mask(r, w, h)[..., None]
        grad, records, n = _records(r, adj, 0, spp, max_rec=1 << 22)
        assert np.isfinite(grad).all() and np.abs(grad).max() > 0
        print(f"{w}x{h}x{spp}: {n} vertex records")
        fd, _ = _oracle_fd(records, n, theta, nmat, _fixed(sc))
        _compare(grad, fd, theta, adjoint_param_names(nmat))
    finally:
        r.shutdown()


def _above_horizon(sc, min_elevation=0.05):
    """1 for pixels whose camera ray rises more than min_elevation (y
    component) above the horizon: near the horizon the reference's
    single-precision sky is noisy, and so are central differences of the
    forward renderer there."""
    cam = sc.camera
    x, y = np.meshgrid(np.arange(W), np.arange(H))
    ndc = np.stack([2.0 * (x + 0.5) / W - 1.0, 2.0 * (y + 0.5) / H - 1.0, np.ones_like(x, float),
                    np.ones_like(x, float)], -1)
    v = ndc @ np.asarray(cam.inv_proj, np.float64).T
    v = v[..., :3] / v[..., 3:]
    v /= np.linalg.norm(v, axis=-1, keepdims=True)
    w = v @ np.asarray(cam.inv_view, np.float64)[:3, :3].T
    w /= np.linalg.norm(w, axis=-1, keepdims=True)
    return (w[..., 1] > min_elevation).astype(np.float32)


def _hit_mask(r, width=W, height=H):
    """1 where the pixel's camera ray hits the scene."""
    import torch
    buf = torch.zeros((1, height, width, 4), dtype=torch.float32, device="cuda")
    fh = torch.zeros((height, width, 4), dtype=torch.int32, device="cuda")
    r.render_samples_device(0, 1, buf.data_ptr(), fh.data_ptr())
    r.synchronize()
    return (fh[..., 0] >= 0).cpu().numpy().astype(np.float32)


@pytest.mark.gpu
def test_adjoint_sky_matches_renderer_fd():
    from kittlespt_gb300.renderer import SKY_PARAM_NAMES
    sc = _scene(5)
    r = _renderer(sc)
    try:
        theta = _theta(sc)
        nmat = len(sc.materials)
        rng = np.random.Generator(np.random.PCG64(12))
        adj = np.zeros((H, W, 4), np.float32)
        adj[..., :3] = rng.uniform(0.0, 1.0, (H, W, 3))
        hit = _hit_mask(r)
        adj *= np.maximum(hit, _above_horizon(sc))[..., None]   # no sky pixels at the horizon
        assert adj.any()
        grad, _ = r.adjoint(0, SPP, adj)

        def E(t):
            _apply(r, sc, t)
            return float((adj[..., :3] * _mean_image(r, 0, SPP)[..., :3]).sum())
        fd = np.zeros(6)
        for k in range(6):
            i = 4 * nmat + k
            h = 1e-3 * abs(theta[i])
            tp, tm = theta.copy(), theta.copy()
            tp[i] += h
            tm[i] -= h
            fd[k] = (E(tp) - E(tm)) / (2.0 * h)
        _apply(r, sc, theta)
        _compare(grad[4 * nmat:], fd, theta[4 * nmat:], list(SKY_PARAM_NAMES), rel=RENDERER_REL)
    finally:
        r.shutdown()


@pytest.mark.gpu
def test_adjoint_depth_limit():
    sc = _scene()
    r = _renderer(sc)
    try:
        r.set_renderer_settings(max_depth=17)
        with pytest.raises(K.KptError):
            r.adjoint(0, 1, np.zeros((H, W, 4), np.float32))
    finally:
        r.shutdown()


@pytest.mark.gpu
def test_autograd_function_l2_loss():
    """torch.autograd.Function over the C ABI: forward = the renderer's mean
    clamped radiance, backward = kpt_adjoint.  L2 loss against a target
    rendered from other samples (seed 7) at the true parameters, from an
    initial guess perturbed by up to +-20%."""
    import torch
    from kittlespt_gb300.renderer import adjoint_param_names
    sc = _scene(7)
    r = _renderer(sc)
    nmat = len(sc.materials)
    try:
        theta_true = _theta(sc)
        rng = np.random.Generator(np.random.PCG64(7))
        theta0 = theta_true * (1.0 + rng.uniform(-0.2, 0.2, theta_true.size))
        theta0[:4 * nmat] = np.clip(theta0[:4 * nmat], 0.02, 0.98)

        # pixel weights of the loss: every hit pixel, sky pixels away from the horizon
        wpix = torch.from_numpy(np.maximum(_hit_mask(r), _above_horizon(sc))[..., None].astype(np.float64))

        class KptImage(torch.autograd.Function):
            @staticmethod
            def forward(ctx, theta):
                _apply(r, sc, theta.detach().cpu().numpy())
                return torch.from_numpy(_mean_image(r, 0, SPP)[..., :3])

            @staticmethod
            def backward(ctx, grad_img):
                adj = np.zeros((H, W, 4), np.float32)
                adj[..., :3] = grad_img.detach().cpu().numpy()
                g, _ = r.adjoint(0, SPP, adj)
                return torch.from_numpy(g)

        _apply(r, sc, theta_true)
        target = torch.from_numpy(_mean_image(r, 7 * SPP, SPP)[..., :3])   # seed 7: other samples
        theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
        loss = (wpix * (KptImage.apply(theta) - target) ** 2).sum()
        loss.backward()
        g = theta.grad.numpy()
        assert np.isfinite(g).all() and np.abs(g).max() > 0
        # materials: against the FP64 oracle on the same adjoint (hit pixels
        # only carry material dependence)
        _apply(r, sc, theta0)
        img0 = _mean_image(r, 0, SPP)[..., :3]
        adj = np.zeros((H, W, 4), np.float32)
        hit = _hit_mask(r)
        assert 0 < hit.sum() < hit.size
        adj[..., :3] = 2.0 * (img0 - target.numpy()) * hit[..., None]
        grad, records, n = _records(r, adj)
        fd, _ = _oracle_fd(records, n, theta0, nmat, _fixed(sc))
        assert np.abs(fd[:4 * nmat]).max() > 0
        names = adjoint_param_names(nmat)
        _compare(g[:4 * nmat], fd[:4 * nmat], theta0[:4 * nmat], names[:4 * nmat])
        # sky: against central differences of the loss through the forward renderer
        def lossf(t):
            _apply(r, sc, t)
            return float((wpix.numpy() * (_mean_image(r, 0, SPP)[..., :3] - target.numpy()) ** 2).sum())
        fd_sky = np.zeros(6)
        for k in range(6):
            i = 4 * nmat + k
            h = 1e-3 * abs(theta0[i])
            tp, tm = theta0.copy(), theta0.copy()
            tp[i] += h
            tm[i] -= h
            fd_sky[k] = (lossf(tp) - lossf(tm)) / (2.0 * h)
        _compare(g[4 * nmat:], fd_sky, theta0[4 * nmat:], names[4 * nmat:], rel=RENDERER_REL)
    finally:
        r.shutdown()


def _sky_theta_fixed(sc):
    e = sc.env
    sky = [float(x) for x in e["rayleigh"]] + [float(e["mie"]), float(e["rayleigh_height"]), float(e["mie_height"])]
    return np.array(sky, np.float64), _fixed(sc)


def _sky_grad_gpu(r, dirs):
    import torch
    d = torch.from_numpy(np.ascontiguousarray(dirs, np.float32)).cuda()
    out = torch.zeros((dirs.shape[0], 7, 3), dtype=torch.float32, device="cuda")
    K.check(r._L.kpt_sky_grad_device(r.ctx, dirs.shape[0], d.data_ptr(), out.data_ptr()))
    r.synchronize()
    return out.cpu().numpy().astype(np.float64)


@pytest.mark.gpu
def test_sky_gradient_matches_fp64_fd():
    """The sky's Jacobian (forward-mode through the 16 x 8 march) against
    central differences of the double-precision sky, direction by direction,
    above the horizon and around the sun."""
    from oracle import oracle as O
    sc = _scene()
    r = _renderer(sc)
    try:
        sky, fixed = _sky_theta_fixed(sc)
        rng = np.random.Generator(np.random.PCG64(21))
        d = rng.normal(size=(512, 3))
        d[:64] = np.array(fixed[:3]) + 0.05 * rng.normal(size=(64, 3))
        d[:, 1] = np.abs(d[:, 1]) + 0.02   # above the horizon (see _scene)
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        d = d.astype(np.float32)
        out = _sky_grad_gpu(r, d)
        L0 = O.sky_double(d, sky, fixed)
        # the single-precision march itself is within 1e-3 of the exact sky here
        np.testing.assert_allclose(out[:, 0], L0, rtol=1e-3, atol=1e-6 * np.abs(L0).max())
        for k in range(6):
            h = 1e-3 * abs(sky[k])
            sp, sm = sky.copy(), sky.copy()
            sp[k] += h
            sm[k] -= h
            fd = (O.sky_double(d, sp, fixed) - O.sky_double(d, sm, fixed)) / (2.0 * h)
            J = out[:, 1 + k]
            scale = np.abs(fd * sky[k]).max()
            err = np.abs((J - fd) * sky[k])
            assert err.max() <= 1e-3 * scale, (k, err.max() / scale)
    finally:
        r.shutdown()


@pytest.mark.gpu
def test_split_adjoint_matches_one_call():
    """kpt_adjoint_forward_device + kpt_adjoint_backward_device (one replay,
    its records kept for the sweep) against kpt_adjoint_device (replay and
    sweep in one call): the same image and gradient up to the order of
    their atomic sums; the backward half refuses to run without kept records
    for the current state."""
    import torch
    sc = _scene()
    r = _renderer(sc)
    try:
        n = C.c_int()
        K.check(r._L.kpt_adjoint_param_count(r.ctx, C.byref(n)))
        rng = np.random.Generator(np.random.PCG64(5))
        adj = torch.from_numpy(rng.uniform(-1.0, 1.0, (H, W, 4)).astype(np.float32)).cuda()
        g1 = torch.zeros(n.value, dtype=torch.float64, device="cuda")
        g2 = torch.zeros_like(g1)
        img1 = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
        img2 = torch.zeros_like(img1)
        K.check(r._L.kpt_adjoint_device(r.ctx, 0, SPP, adj.data_ptr(), g1.data_ptr(), img1.data_ptr()))
        r.adjoint_forward_device(0, SPP, img2.data_ptr())
        r.adjoint_backward_device(adj.data_ptr(), g2.data_ptr())
        r.synchronize()
        a, b = g1.cpu().numpy(), g2.cpu().numpy()
        np.testing.assert_allclose(b, a, rtol=1e-9, atol=1e-12 * np.abs(a).max())
        np.testing.assert_allclose(img2.cpu().numpy(), img1.cpu().numpy(), rtol=1e-6, atol=1e-7)
        with pytest.raises(K.KptError):
            r.adjoint_backward_device(adj.data_ptr(), g2.data_ptr())     # one backward per forward
        r.adjoint_forward_device(0, SPP, img2.data_ptr())
        r.execute_rendering(16.0, 1)
        with pytest.raises(K.KptError):
            r.adjoint_backward_device(adj.data_ptr(), g2.data_ptr())     # a frame in between
        r.adjoint_forward_device(0, SPP, img2.data_ptr())
        m = sc.materials[0].copy()
        m["roughness"] = 0.5 * m["roughness"]
        assert r.set_material(0, m)
        with pytest.raises(K.KptError):
            r.adjoint_backward_device(adj.data_ptr(), g2.data_ptr())     # a parameter changed
        r.adjoint_forward_device(0, SPP, img2.data_ptr())
        model = np.array(sc.instances[0].model, np.float32)
        model[1, 3] += 0.25
        assert r.set_mesh_transform(0, model)
        with pytest.raises(K.KptError):
            r.adjoint_backward_device(adj.data_ptr(), g2.data_ptr())     # an instance moved
    finally:
        r.shutdown()
