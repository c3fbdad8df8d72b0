"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/libkpt_oracle.so`` (our FP32 restatement of the reference hot
path, built by ``oracle/build_oracle.sh``) or, with ``prefix="ref"``,
``oracle/_ref/libkpt_ref_host.so`` (the reference's own code compiled for the
host by ``oracle/build_ref.sh`` from its staged sources).  Both export the
same C ABI, so every helper below drives either one.  ``RefGpuScene`` drives
``oracle/_ref/libkpt_ref_gpu.so``: the reference's own CUDA megakernel, built
for the GPU by ``oracle/build_ref.sh gpu``.

Only tests, the smoke check and the benchmark's CPU-baseline leg use this
module; the product path (``kittlespt_gb300``) never imports it.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libkpt_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libkpt_ref_host.so")
REF_GPU_SO = os.path.join(HERE, "_ref", "libkpt_ref_gpu.so")
REF_SRC = os.path.join(HERE, "_ref", "src", "KittlesPT", "src", "shaders")

_f = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_u64 = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_v = C.c_void_p

_libs = {}


def build(ref: bool = False, what: str = "all") -> None:
    """Builds the oracle, or with ref=True the reference's own code
    (build_ref.sh `what`: stage, host, gpu or all)."""
    cmd = ["sh", os.path.join(HERE, "build_ref.sh"), what] if ref else ["sh", os.path.join(HERE, "build_oracle.sh")]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL)


def ref_staged() -> bool:
    """True where the reference's sources have been staged for building."""
    return os.path.isdir(REF_SRC)


def available(prefix: str = "orc") -> bool:
    path = {"ref": REF_SO, "refgpu": REF_GPU_SO}.get(prefix, ORACLE_SO)
    return os.path.exists(path)


def lib(prefix: str = "orc"):
    if prefix in _libs:
        return _libs[prefix]
    path = REF_SO if prefix == "ref" else ORACLE_SO
    if not os.path.exists(path):
        if prefix == "ref":
            raise FileNotFoundError(path)
        build(False)
    L = C.CDLL(path)
    g = lambda n: getattr(L, f"{prefix}_{n}")
    g("scene_create").restype = _v
    g("scene_create").argtypes = [C.c_int, _f, _f, _f, _i, C.c_int, _i, _i, _f, C.c_int, _v,
                                  C.c_int, _v, C.c_longlong, _v]
    g("scene_destroy").argtypes = [_v]
    g("scene_counts").argtypes = [_v, _i64]
    g("scene_bvh").argtypes = [_v, _i, _u, _f, _i, _i64, _f, _f]
    g("scene_tlas").argtypes = [_v, _u, _i, _f]
    g("trace").argtypes = [_v, C.c_int, _f, _f, C.c_float, C.c_float, _i, _i, _f, _v, C.c_int, _v, C.c_int]
    g("trace_bounces").argtypes = [_v, C.c_int, _f, _f, C.c_int, _i, _f, _v, C.c_int]
    g("render_samples").argtypes = [_v, _f, _f, _v, _v, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_int, _v, _v, _v, _v, _v, C.c_int]
    g("sky").argtypes = [_v, C.c_int, _f, _f]
    g("bsdf_eval").argtypes = [C.c_int, _f, _f, _f, _f]
    g("lum_bins").argtypes = [C.c_int, _f, C.c_float, C.c_float, _i]
    g("modulate").argtypes = [C.c_int, C.c_int, _f, C.c_int, _f, _f]
    g("bloom").argtypes = [C.c_int, C.c_int, _f, C.c_int, C.c_float, _f]
    g("post_image").argtypes = [C.c_int, C.c_int, _f, _v, C.c_int, C.c_float, C.c_float, C.c_float,
                                C.c_float, _f]
    g("metering_weights").argtypes = [C.c_int, C.c_int, _f]
    g("upscale").argtypes = [C.c_int, C.c_int, _f, C.c_int, C.c_int, _f]
    g("fsr").argtypes = [C.c_int, C.c_int, _f, C.c_int, C.c_int, _f, _f]
    if prefix == "orc":
        g("sky_double").argtypes = [C.c_int, _v, _v, _v, _v]
        g("adjoint_estimate").restype = C.c_int
        g("adjoint_estimate").argtypes = [_v, C.c_int, _v, _v, _v, _v, _v]
        g("render_sensitivity").argtypes = [_v, _f, _f, _v, _v, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                            C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, _v, _f, C.c_int]
        g("histogram").argtypes = [C.c_int, C.c_int, _f, C.c_float, C.c_float, _u64]
        g("exposure").argtypes = [_u64, _v, C.c_float, C.c_float, _f]
        g("hist_thresholds").argtypes = [C.c_float, C.c_float, _f]
        g("temporal_frame").argtypes = [C.c_int, C.c_int, _f, _f, _f, _f, C.c_int, _f, _f, _i, _f, _f, _f, _f, _f]
        g("effects").argtypes = [C.c_int, C.c_int, _f, _f]
    else:
        g("histogram").argtypes = [C.c_int, C.c_int, _f, C.c_float, C.c_float, _f]
        g("exposure").argtypes = [_f] + [C.c_float] * 12 + [_f]
    _libs[prefix] = L
    return L


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Scene:
    """A scene in the reference's layout (one mesh per instance)."""

    def __init__(self, scene, prefix: str = "orc"):
        self.prefix = prefix
        self.L = lib(prefix)
        ex = scene.expanded()
        self.ex = ex
        self._keep = ex
        self.materials = np.ascontiguousarray(scene.materials)
        fn = getattr(self.L, f"{prefix}_scene_create")
        n = int(ex["positions"].shape[0])
        self.h = fn(n, ex["positions"].reshape(-1), ex["normals"].reshape(-1), ex["uvs"].reshape(-1),
                    ex["material"], len(ex["mesh_offset"]), ex["mesh_offset"], ex["mesh_count"],
                    np.ascontiguousarray(np.transpose(ex["models"], (0, 2, 1))).reshape(-1),
                    len(self.materials), _ptr(self.materials), *self._textures(scene))
        self.scene = scene

    def _textures(self, scene):
        tex = getattr(scene, "textures", None)
        if not tex:
            return 0, None, 0, None
        desc, pix = scene.texture_arrays()
        self._tex = (desc, pix)
        return len(tex), _ptr(desc), int(pix.size), _ptr(pix)

    def close(self):
        if self.h:
            getattr(self.L, f"{self.prefix}_scene_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _fn(self, n):
        return getattr(self.L, f"{self.prefix}_{n}")

    def counts(self):
        out = np.zeros(5, np.int64)
        self._fn("scene_counts")(self.h, out)
        return dict(nodes=int(out[0]), tri_index=int(out[1]), tlas_nodes=int(out[2]),
                    lights=int(out[3]), meshes=int(out[4]))

    def bvh(self):
        c = self.counts()
        nn, nt, nb = c["nodes"], c["tri_index"], c["meshes"]
        lf = np.zeros(nn, np.int32); cnt = np.zeros(nn, np.uint32); bd = np.zeros(nn * 6, np.float32)
        ti = np.zeros(nt, np.int32); br = np.zeros(nb, np.int64); bb = np.zeros(nb * 6, np.float32)
        bi = np.zeros(nb * 16, np.float32)
        self._fn("scene_bvh")(self.h, lf, cnt, bd, ti, br, bb, bi)
        nt_ = c["tlas_nodes"]
        lr = np.zeros(nt_, np.uint32); tb = np.zeros(nt_, np.int32); tbd = np.zeros(nt_ * 6, np.float32)
        self._fn("scene_tlas")(self.h, lr, tb, tbd)
        return dict(left_first=lf, count=cnt, bounds=bd.reshape(-1, 6), tri_index=ti, blas_root=br,
                    blas_bounds=bb.reshape(-1, 6), blas_inv=bi.reshape(-1, 16),
                    tlas_lr=lr, tlas_blas=tb, tlas_bounds=tbd.reshape(-1, 6))

    def trace(self, o, d, tmin=0.0, tmax=np.inf, brute=False, nthreads=None):
        n = int(o.shape[0])
        o = np.ascontiguousarray(o, np.float32).reshape(-1)
        d = np.ascontiguousarray(d, np.float32).reshape(-1)
        prim = np.zeros(n, np.int32); inst = np.zeros(n, np.int32); t = np.zeros(n, np.float32)
        bary = np.zeros(n * 3, np.float32); cnt = np.zeros(8, np.int64)
        self._fn("trace")(self.h, n, o, d, tmin, tmax, prim, inst, t, _ptr(bary), int(brute), _ptr(cnt),
                          nthreads or os.cpu_count())
        return dict(prim=prim, inst=inst, t=t, bary=bary.reshape(-1, 3), counters=cnt)

    def trace_bounces(self, o, d, nbounces, nthreads=None):
        n = int(o.shape[0])
        prim = np.zeros((nbounces + 1) * n, np.int32); t = np.zeros((nbounces + 1) * n, np.float32)
        cnt = np.zeros(8, np.int64)
        self._fn("trace_bounces")(self.h, n, np.ascontiguousarray(o, np.float32).reshape(-1),
                                  np.ascontiguousarray(d, np.float32).reshape(-1), nbounces, prim, t,
                                  _ptr(cnt), nthreads or os.cpu_count())
        return dict(prim=prim.reshape(nbounces + 1, n), t=t.reshape(nbounces + 1, n), counters=cnt)

    def render_samples(self, sample0=0, nsamples=1, rng_order=0, width=None, height=None,
                       row0=0, nrows=0, max_depth=None, nthreads=None, want_radiance=True):
        sc = self.scene
        W = width or sc.width
        H = height or sc.height
        rows = nrows if nrows > 0 else H - row0
        st = sc.settings.copy()
        if max_depth is not None:
            st["max_depth"] = max_depth
        rad = np.zeros((nsamples, rows, W, 3), np.float32) if want_radiance else None
        alb = np.zeros((rows, W, 3), np.float32)
        fh = np.zeros((rows, W, 2), np.int32)
        ft = np.zeros((rows, W), np.float32)
        cnt = np.zeros(8, np.int64)
        ip = np.ascontiguousarray(sc.camera.inv_proj.T, np.float32).reshape(-1)
        iv = np.ascontiguousarray(sc.camera.inv_view.T, np.float32).reshape(-1)
        env = np.ascontiguousarray(sc.env)
        self._fn("render_samples")(self.h, ip, iv, _ptr(env), _ptr(st), W, H, sample0, nsamples, rng_order,
                                   row0, nrows, _ptr(rad) if rad is not None else None, _ptr(alb), _ptr(fh),
                                   _ptr(ft), _ptr(cnt), nthreads or os.cpu_count())
        return dict(radiance=rad, albedo=alb, first_hit=fh, first_t=ft, counters=cnt)


    def render_sensitivity(self, sample0=0, nsamples=1, rng_order=0, row0=0, nrows=0, eps=2e-6, eps_pos=2e-7,
                           ncopies=4, nthreads=None):
        """The rounding-sensitivity probe of the oracle (orc_render_sensitivity):
        per sample, the largest relative change of its radiance over `ncopies`
        re-renders with scattered directions, normals and throughput moved by a
        relative eps and surface and light-sample points by a relative eps_pos.  Returns dict(radiance
        [nsamples][rows][W][3], response [nsamples][rows][W])."""
        sc = self.scene
        W, H = sc.width, sc.height
        rows = nrows if nrows > 0 else H - row0
        rad = np.zeros((nsamples, rows, W, 3), np.float32)
        resp = np.zeros((nsamples, rows, W), np.float32)
        ip = np.ascontiguousarray(sc.camera.inv_proj.T, np.float32).reshape(-1)
        iv = np.ascontiguousarray(sc.camera.inv_view.T, np.float32).reshape(-1)
        env = np.ascontiguousarray(sc.env)
        st = sc.settings.copy()
        self._fn("render_sensitivity")(self.h, ip, iv, _ptr(env), _ptr(st), W, H, sample0, nsamples, rng_order,
                                       row0, nrows, float(eps), float(eps_pos), int(ncopies), _ptr(rad), resp,
                                       nthreads or os.cpu_count())
        return dict(radiance=rad, response=resp)


def sky(env, dirs, prefix="orc"):
    dirs = np.ascontiguousarray(dirs, np.float32)
    out = np.zeros_like(dirs)
    e = np.ascontiguousarray(env)
    getattr(lib(prefix), f"{prefix}_sky")(_ptr(e), int(dirs.shape[0]), dirs.reshape(-1), out.reshape(-1))
    return out


def bsdf_eval(params, dirs, u, prefix="orc"):
    n = int(params.shape[0])
    out = np.zeros((n, 12), np.float32)
    getattr(lib(prefix), f"{prefix}_bsdf_eval")(n, np.ascontiguousarray(params, np.float32).reshape(-1),
                                                np.ascontiguousarray(dirs, np.float32).reshape(-1),
                                                np.ascontiguousarray(u, np.float32).reshape(-1), out.reshape(-1))
    return out


def lum_bins(Y, black_ev=-10.0, white_ev=6.5, prefix="orc"):
    Y = np.ascontiguousarray(Y, np.float32)
    out = np.zeros(Y.shape[0], np.int32)
    getattr(lib(prefix), f"{prefix}_lum_bins")(int(Y.shape[0]), Y, black_ev, white_ev, out)
    return out


def hist_thresholds(black_ev=-10.0, white_ev=6.5):
    thr = np.zeros(255, np.float32)
    lib("orc").orc_hist_thresholds(black_ev, white_ev, thr)
    return thr


def _cm(m):
    """4x4 numpy M[row, col] -> 16 floats column-major."""
    return np.ascontiguousarray(np.asarray(m, np.float32).T, np.float32).reshape(-1)


def temporal_frame(prev_cam, curr_cam, curr_models, prev_models, vis_inst, vis_t, sample, prev_depth, hist_in):
    """One reference frame of temporal accumulation (kernels.cu:164-327,
    :422-428) for every pixel.  Cameras are (inv_proj, inv_view) pairs of 4x4
    M[row, col]; models [n, 4, 4]; vis_inst / vis_t [H, W] (first-hit
    instance, -1 for a miss, and distance); sample, hist_in [H, W, 4];
    prev_depth [H, W].  Returns the new history image [H, W, 4]."""
    H, W = vis_inst.shape
    n = len(curr_models)
    cm = np.concatenate([_cm(m) for m in curr_models]) if n else np.zeros(16, np.float32)
    pm = np.concatenate([_cm(m) for m in prev_models]) if n else np.zeros(16, np.float32)
    out = np.zeros((H, W, 4), np.float32)
    lib().orc_temporal_frame(W, H, _cm(prev_cam[0]), _cm(prev_cam[1]), _cm(curr_cam[0]), _cm(curr_cam[1]), n, cm, pm,
                             np.ascontiguousarray(vis_inst, np.int32).reshape(-1),
                             np.ascontiguousarray(vis_t, np.float32).reshape(-1),
                             np.ascontiguousarray(sample, np.float32).reshape(-1),
                             np.ascontiguousarray(prev_depth, np.float32).reshape(-1),
                             np.ascontiguousarray(hist_in, np.float32).reshape(-1), out.reshape(-1))
    return out


def effects(image):
    """computeEffects (kernels.cu:506-527): fisheye and chromatic aberration of
    a tonemapped image [H, W, 4]."""
    H, W = image.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    lib().orc_effects(W, H, np.ascontiguousarray(image, np.float32).reshape(-1), out.reshape(-1))
    return out


def upscale(render, width, height, prefix="orc"):
    """upscale without FSR (upscale.cuh:260-291) of a render [h, w, 4] to
    [height, width, 4]."""
    sh, sw = render.shape[:2]
    out = np.zeros((height, width, 4), np.float32)
    getattr(lib(prefix), prefix + "_upscale")(sw, sh, np.ascontiguousarray(render, np.float32).reshape(-1),
                                              width, height, out.reshape(-1))
    return out


def fsr(render, width, height, prefix="orc"):
    """The reference's FSR 1.0 upscale (EASU, upscale.cuh:13-258) and sharpen
    (RCAS, upscale.cuh:300-433) of a render [h, w, 4] to [height, width, 4]:
    returns (EASU image, sharpened image)."""
    sh, sw = render.shape[:2]
    easu = np.zeros((height, width, 4), np.float32)
    out = np.zeros((height, width, 4), np.float32)
    getattr(lib(prefix), prefix + "_fsr")(sw, sh, np.ascontiguousarray(render, np.float32).reshape(-1),
                                          width, height, easu.reshape(-1), out.reshape(-1))
    return easu, out


def modulate(acc_sum, nsamples, albedo, prefix="orc"):
    H, W = acc_sum.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    getattr(lib(prefix), f"{prefix}_modulate")(W, H, np.ascontiguousarray(acc_sum, np.float32).reshape(-1),
                                               nsamples, np.ascontiguousarray(albedo, np.float32).reshape(-1),
                                               out.reshape(-1))
    return out


def bloom(render, karis=False, internal_blend=0.65, prefix="orc"):
    H, W = render.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    getattr(lib(prefix), f"{prefix}_bloom")(W, H, np.ascontiguousarray(render, np.float32).reshape(-1),
                                            int(karis), internal_blend, out.reshape(-1))
    return out


def post_image(render, bloom_img, final_blend, expo, white_ev=6.5, black_ev=-10.0, prefix="orc"):
    H, W = render.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    b = np.ascontiguousarray(bloom_img, np.float32) if bloom_img is not None else None
    getattr(lib(prefix), f"{prefix}_post_image")(W, H, np.ascontiguousarray(render, np.float32).reshape(-1),
                                                 _ptr(b) if b is not None else None, int(b is not None),
                                                 final_blend, expo, white_ev, black_ev, out.reshape(-1))
    return out


def metering_weights(W, H, prefix="orc"):
    out = np.zeros((H, W), np.float32)
    getattr(lib(prefix), f"{prefix}_metering_weights")(W, H, out.reshape(-1))
    return out


def histogram(render, black_ev=-10.0, white_ev=6.5, prefix="orc"):
    """orc: fixed-point (2^24) uint64 bins; ref: float bins."""
    H, W = render.shape[:2]
    r = np.ascontiguousarray(render, np.float32).reshape(-1)
    if prefix == "orc":
        out = np.zeros(256, np.uint64)
        lib("orc").orc_histogram(W, H, r, black_ev, white_ev, out)
    else:
        out = np.zeros(256, np.float32)
        lib("ref").ref_histogram(W, H, r, black_ev, white_ev, out)
    return out


def exposure(hist, expo, last_lum, delta_ms, prefix="orc"):
    """[avg bin, avg lum, adapted lum, exposure scalar, iso, shutter]."""
    out = np.zeros(6, np.float32)
    if prefix == "orc":
        e = np.ascontiguousarray(expo)
        lib("orc").orc_exposure(np.ascontiguousarray(hist, np.uint64), _ptr(e), last_lum, delta_ms, out)
    else:
        e = expo
        lib("ref").ref_exposure(np.ascontiguousarray(hist, np.float32), float(e["aperture"]), float(e["iso"]),
                                float(e["shutter"]), float(e["ev_comp"]), float(e["white_ev"]),
                                float(e["black_ev"]), float(e["min_iso"]), float(e["max_iso"]),
                                float(e["min_shutter"]), float(e["max_shutter"]), last_lum, delta_ms, out)
    return out


def exposure_scalar(expo) -> float:
    """Film exposure scalar for fixed camera values
    (AutoExposureProgram::getStandardOutputBasedExposure), in double."""
    N = float(expo["aperture"])
    lavg = (10.0 / 0.65) * ((N * N) / (float(expo["iso"]) * float(expo["shutter"])))
    return float(np.float32(0.18 / lavg))


def sky_double(dirs, sky, fixed):
    """Nishita radiance in double precision for [n][3] directions (sky and
    fixed as for adjoint_estimate)."""
    L = lib("orc")
    d = np.ascontiguousarray(dirs, np.float32)
    s = np.ascontiguousarray(sky, np.float64)
    f = np.ascontiguousarray(fixed, np.float64)
    out = np.zeros((d.shape[0], 3), np.float64)
    L.orc_sky_double(d.shape[0], _ptr(d), _ptr(s), _ptr(f), _ptr(out))
    return out


def adjoint_estimate(records: bytes, n: int, albedo, roughness, sky, fixed):
    """E(theta) = sum over samples of g . L(theta) on the adjoint's frozen
    path records, in double precision (adjoint_oracle.cpp).  albedo [M][3],
    roughness [M], sky (Rayleigh r, g, b, Mie, Rayleigh height, Mie height),
    fixed (sun direction xyz, sun emission factor, Mie absorption, earth
    radius, atmosphere radius).  Returns (E, number of samples)."""
    L = lib("orc")
    buf = np.frombuffer(records, np.uint8)
    a = np.ascontiguousarray(albedo, np.float64).reshape(-1)
    r = np.ascontiguousarray(roughness, np.float64)
    s = np.ascontiguousarray(sky, np.float64)
    f = np.ascontiguousarray(fixed, np.float64)
    out = np.zeros(1, np.float64)
    items = L.orc_adjoint_estimate(_ptr(buf), n, _ptr(a), _ptr(r), _ptr(s), _ptr(f), _ptr(out))
    return float(out[0]), int(items)


class RefGpuScene:
    """The reference's own CUDA megakernel on the GPU, over a scene in its
    layout (oracle/_ref/libkpt_ref_gpu.so, built by ``build_ref.sh gpu``).
    Construction raises RuntimeError if a tree is deeper than the reference's
    16-entry traversal stacks allow; no kernel has run then."""

    _L = None

    @classmethod
    def lib(cls):
        if cls._L is None:
            if not os.path.exists(REF_GPU_SO):
                raise FileNotFoundError(REF_GPU_SO)
            L = C.CDLL(REF_GPU_SO)
            L.refgpu_last_error.restype = C.c_char_p
            L.refgpu_scene_create.restype = _v
            L.refgpu_scene_create.argtypes = [C.c_int, C.c_int, _f, _f, _f, _i, C.c_int, _i, _i, _f, C.c_int, _v,
                                              C.c_int, _v, C.c_longlong, _v]
            L.refgpu_scene_destroy.argtypes = [_v]
            L.refgpu_tree_depth.argtypes = [_v, _i]
            L.refgpu_render.restype = C.c_int
            L.refgpu_render.argtypes = [_v, _f, _f, _v, _v, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _v, _v]
            L.refgpu_temporal_frame.restype = C.c_int
            L.refgpu_temporal_frame.argtypes = [_v, _v, _v, _v, _v, C.c_int, C.c_int, C.c_int, _v, C.c_int, _v, _v]
            L.refgpu_effects.restype = C.c_int
            L.refgpu_effects.argtypes = [C.c_int, C.c_int, _f, _f]
            L.refgpu_first_hits.restype = C.c_int
            L.refgpu_first_hits.argtypes = [_v, _f, _f, _v, _v, C.c_int, C.c_int, _i, _i, _f]
            cls._L = L
        return cls._L

    def __init__(self, scene, device: int = 0):
        L = self.lib()
        ex = scene.expanded()
        self._keep = ex
        self.materials = np.ascontiguousarray(scene.materials)
        tex = getattr(scene, "textures", None)
        targs = (0, None, 0, None)
        if tex:
            desc, pix = scene.texture_arrays()
            self._tex = (desc, pix)
            targs = (len(tex), _ptr(desc), int(pix.size), _ptr(pix))
        n = int(ex["positions"].shape[0])
        self.h = L.refgpu_scene_create(device, n, ex["positions"].reshape(-1), ex["normals"].reshape(-1),
                                       ex["uvs"].reshape(-1), ex["material"], len(ex["mesh_offset"]),
                                       ex["mesh_offset"], ex["mesh_count"],
                                       np.ascontiguousarray(np.transpose(ex["models"], (0, 2, 1))).reshape(-1),
                                       len(self.materials), _ptr(self.materials), *targs)
        if not self.h:
            raise RuntimeError(L.refgpu_last_error().decode())
        self.scene = scene

    def close(self):
        if getattr(self, "h", None):
            self.lib().refgpu_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tree_depth(self):
        out = np.zeros(2, np.int32)
        self.lib().refgpu_tree_depth(self.h, out)
        return dict(blas=int(out[0]), tlas=int(out[1]))

    def _view(self, max_depth):
        sc = self.scene
        st = sc.settings.copy()
        if max_depth is not None:
            st["max_depth"] = max_depth
        ip = np.ascontiguousarray(sc.camera.inv_proj.T, np.float32).reshape(-1)
        iv = np.ascontiguousarray(sc.camera.inv_view.T, np.float32).reshape(-1)
        env = np.ascontiguousarray(sc.env)
        self._st = (st, env)
        return ip, iv, _ptr(env), _ptr(st)

    def render(self, frame0=0, nframes=1, clear=True, max_depth=None, want_accum=True):
        """Frames frame0 .. frame0+nframes-1 (one sample per pixel each, the
        reference's frame index = the sample index).  Returns (accumulation
        [H][W][4] or None, kernel milliseconds per frame)."""
        sc = self.scene
        ip, iv, env, st = self._view(max_depth)
        acc = np.zeros((sc.height, sc.width, 4), np.float32) if want_accum else None
        ms = np.zeros(max(nframes, 1), np.float32)
        rc = self.lib().refgpu_render(self.h, ip, iv, env, st, sc.width, sc.height, frame0, nframes, int(clear),
                                      _ptr(acc) if acc is not None else None, _ptr(ms))
        if rc != 0:
            raise RuntimeError(self.lib().refgpu_last_error().decode())
        return acc, ms[:nframes]

    def render_samples(self, sample0=0, nsamples=1, max_depth=None):
        """Per-sample clamped radiance [nsamples][H][W][3]: each sample is one
        frame rendered into a cleared accumulation."""
        sc = self.scene
        out = np.zeros((nsamples, sc.height, sc.width, 3), np.float32)
        for k in range(nsamples):
            acc, _ = self.render(sample0 + k, 1, clear=True, max_depth=max_depth)
            out[k] = acc[..., :3]
        return out

    def temporal_frame(self, frame_index, reset=False, camera=None, models=None):
        """One frame of the reference's temporal accumulation
        (refgpu_temporal_frame): camera = (inv_proj, inv_view) 4x4 row-major or
        None to keep it; models = per-mesh 4x4 model matrices in the
        reference's mesh order or None.  Returns (modulated render,
        accumulation) [H][W][4] each."""
        sc = self.scene
        ip, iv, env, st = self._view(None)
        if camera is not None:
            ip = np.ascontiguousarray(np.asarray(camera[0], np.float32).T).reshape(-1)
            iv = np.ascontiguousarray(np.asarray(camera[1], np.float32).T).reshape(-1)
        elif not reset:
            ip = iv = None
        mp = None
        if models is not None:
            mp = np.ascontiguousarray(np.transpose(np.asarray(models, np.float32), (0, 2, 1))).reshape(-1)
        render = np.zeros((sc.height, sc.width, 4), np.float32)
        acc = np.zeros_like(render)
        rc = self.lib().refgpu_temporal_frame(self.h, _ptr(ip) if ip is not None else None,
                                              _ptr(iv) if iv is not None else None, env, st, sc.width, sc.height,
                                              frame_index, _ptr(mp) if mp is not None else None, int(reset),
                                              _ptr(render), _ptr(acc))
        if rc != 0:
            raise RuntimeError(self.lib().refgpu_last_error().decode())
        return render, acc

    def first_hits(self):
        sc = self.scene
        ip, iv, env, st = self._view(None)
        prim = np.zeros((sc.height, sc.width), np.int32)
        inst = np.zeros_like(prim)
        t = np.zeros((sc.height, sc.width), np.float32)
        rc = self.lib().refgpu_first_hits(self.h, ip, iv, env, st, sc.width, sc.height, prim, inst, t)
        if rc != 0:
            raise RuntimeError(self.lib().refgpu_last_error().decode())
        return dict(prim=prim, inst=inst, t=t)


def ref_gpu_effects(image):
    """The reference's own lens-effects kernel (computeEffects) on the GPU for
    an [H][W][4] float image (the backbuffer); returns the output texture."""
    L = RefGpuScene.lib()
    img = np.ascontiguousarray(image, np.float32)
    H, W = img.shape[:2]
    out = np.zeros((H, W, 4), np.float32)
    if L.refgpu_effects(W, H, img.reshape(-1), out.reshape(-1)) != 0:
        raise RuntimeError(L.refgpu_last_error().decode())
    return out
