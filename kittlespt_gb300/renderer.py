"""Python mirror of KittlesPT::Renderer (KittlesPT/src/renderer.hpp:13-58)
over the C ABI of libkpt.so.

Method names follow the reference (snake_case), with the same argument
meaning and error behaviour: setters on an index out of range return False
(the reference's bool), getters raise IndexError (the reference asserts).
``get_render_target`` replaces getRenderTargetTexture(GLuint): there is no
graphics stack, so the display image is copied into a numpy array.
"""

from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as K
from . import scenes as S


def _m16(m) -> np.ndarray:
    """numpy M[row, col] (4x4) -> 16 floats column-major."""
    a = np.asarray(m, np.float32)
    if a.shape == (4, 4):
        a = a.T
    return np.ascontiguousarray(a.reshape(16), np.float32)


def _mat(rec) -> K.Material:
    m = K.Material()
    for name, ctype in K.Material._fields_:
        v = rec[name]
        if name in ("albedo", "emission"):
            getattr(m, name)[:] = [float(x) for x in v]
        elif ctype is C.c_float:
            setattr(m, name, float(v))
        else:
            setattr(m, name, int(v))
    return m


class Renderer:
    """One GPU path tracer: scene, camera, settings, accumulation, post chain."""

    def __init__(self, device: int = 0):
        self._L = K.load()
        self._ctx = C.c_void_p()
        self._device = device
        self._open = False

    # -- lifetime (renderer.cu:22-53) ----------------------------------------
    def initialize(self):
        K.check(self._L.kpt_create(self._device, C.byref(self._ctx)))
        self._open = True

    def shutdown(self):
        if self._open:
            K.check(self._L.kpt_destroy(self._ctx))
            self._open = False

    def __enter__(self):
        self.initialize()
        return self

    def __exit__(self, *exc):
        self.shutdown()

    @property
    def ctx(self):
        return self._ctx

    # -- resolution (renderer.cu:55-101) -------------------------------------
    def resize_resolution(self, width: int, height: int):
        K.check(self._L.kpt_resize(self._ctx, width, height))
        self.width, self.height = width, height

    # -- scene (renderer.cu:356-436) -----------------------------------------
    def load_scene(self, scene: S.Scene, commit: bool = True):
        """Materials, meshes (BLAS built on upload), instances, camera,
        environment, settings and exposure of a synthetic scene."""
        L = self._L
        K.check(L.kpt_clear_scene(self._ctx))
        mats = (K.Material * len(scene.materials))(*[_mat(m) for m in scene.materials])
        K.check(L.kpt_set_materials(self._ctx, len(scene.materials), mats))
        if getattr(scene, "textures", None):
            desc, pix = scene.texture_arrays()
            K.check(L.kpt_set_textures(self._ctx, len(scene.textures), K.iptr(desc.reshape(-1)), pix.size,
                                       pix.ctypes.data_as(C.POINTER(C.c_uint8))))
        for m in scene.meshes:
            out = C.c_int()
            K.check(L.kpt_upload_mesh(self._ctx, m.ntris, K.fptr(m.positions.reshape(-1)),
                                      K.fptr(m.normals.reshape(-1)), K.fptr(m.uvs.reshape(-1)),
                                      K.iptr(np.ascontiguousarray(m.material, np.int32)), C.byref(out)))
        for inst in scene.instances:
            out = C.c_int()
            K.check(L.kpt_add_instance(self._ctx, inst.mesh, K.fptr(_m16(inst.model)), inst.material, C.byref(out)))
        if commit:
            K.check(L.kpt_commit_scene(self._ctx))
        self.resize_resolution(scene.width, scene.height)
        self.set_camera_inverse(scene.camera.inv_proj, scene.camera.inv_view)
        self.set_procedural_environment_data(scene.env)
        st = scene.settings
        self.set_renderer_settings(max_depth=int(st["max_depth"]), bloom=bool(st["bloom"]),
                                   karis=bool(st["karis"]), auto_exposure=bool(st["auto_exposure"]),
                                   bloom_final_blend=float(st["bloom_final_blend"]),
                                   bloom_internal_blend=float(st["bloom_internal_blend"]),
                                   frame_delta_ms=float(st["frame_delta_ms"]),
                                   sky_arith=int(getattr(scene, "sky_arith", 0)),
                                   temporal_arith=int(getattr(scene, "temporal_arith", 0)))
        self.set_exposure(scene.exposure)
        self.scene = scene

    # -- BLAS build (no reference counterpart) --------------------------------
    def set_blas_build(self, device: bool):
        """Build the BLAS of meshes uploaded from now on on the GPU (True) or
        the host (False, the default); the trees are the same."""
        K.check(self._L.kpt_set_blas_build(self._ctx, 1 if device else 0))

    def refit_mesh(self, mesh: int, positions, normals=None):
        """New positions (and optionally normals) for an uploaded mesh of the
        committed scene; the BLAS keeps its tree and is refit on the GPU."""
        p = np.ascontiguousarray(positions, np.float32).reshape(-1)
        n = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1)
        K.check(self._L.kpt_refit_mesh(self._ctx, mesh, K.fptr(p), K.fptr(n) if n is not None else None))

    def get_blas(self, mesh: int) -> dict:
        """The device-format BLAS of an uploaded mesh: nodes (float32 [k, 12]
        child boxes, int32 [k, 4] child references and counts), leaf order,
        root (-1: a leaf of leaf_count triangles from leaf_first), bounds."""
        info = np.zeros(5, np.int32)
        K.check(self._L.kpt_get_blas(self._ctx, mesh, K.iptr(info), None, None, None))
        k, ntris = int(info[0]), int(info[4])
        raw = np.zeros((max(k, 1), 16), np.float32)
        order = np.zeros(ntris, np.int32)
        bounds = np.zeros(6, np.float32)
        K.check(self._L.kpt_get_blas(self._ctx, mesh, K.iptr(info), K.fptr(raw.reshape(-1)), K.iptr(order),
                                     K.fptr(bounds)))
        return {"boxes": raw[:k, :12].copy(), "refs": raw[:k, 12:].view(np.int32).copy(),
                "order": order, "root": int(info[1]), "leaf_first": int(info[2]),
                "leaf_count": int(info[3]), "bounds": bounds}

    def get_materials_count(self) -> int:
        n = C.c_int()
        K.check(self._L.kpt_counts(self._ctx, C.byref(n), None, None, None))
        return n.value

    def get_mesh_count(self) -> int:
        """Instances: the reference's meshes (it copies one mesh per instance)."""
        n = C.c_int()
        K.check(self._L.kpt_counts(self._ctx, None, None, C.byref(n), None))
        return n.value

    def get_light_count(self) -> int:
        n = C.c_int()
        K.check(self._L.kpt_counts(self._ctx, None, None, None, C.byref(n)))
        return n.value

    # -- materials (renderer.cu:207-248) -------------------------------------
    def set_material(self, index: int, material) -> bool:
        rec = material if isinstance(material, K.Material) else _mat(material)
        st = self._L.kpt_set_material(self._ctx, index, C.byref(rec))
        if st == K.KPT_OK:
            return True
        if st == -1:
            return False
        K.check(st)

    def get_material(self, index: int) -> np.ndarray:
        m = K.Material()
        st = self._L.kpt_get_material(self._ctx, index, C.byref(m))
        if st == -1:
            raise IndexError(f"material {index} out of range")
        K.check(st)
        out = np.zeros((), S.MATERIAL_DTYPE)
        for name, _ in K.Material._fields_:
            v = getattr(m, name)
            out[name] = list(v) if name in ("albedo", "emission") else v
        return out

    # -- mesh transforms (renderer.cu:250-278) -------------------------------
    def set_mesh_transform(self, index: int, model) -> bool:
        st = self._L.kpt_set_instance_transform(self._ctx, index, K.fptr(_m16(model)))
        if st == K.KPT_OK:
            return True
        if st == -1:
            return False
        K.check(st)

    def get_mesh_transform(self, index: int) -> np.ndarray:
        out = np.zeros(16, np.float32)
        st = self._L.kpt_get_instance_transform(self._ctx, index, K.fptr(out))
        if st == -1:
            raise IndexError(f"mesh {index} out of range")
        K.check(st)
        return out.reshape(4, 4).T.copy()

    # -- camera (renderer.cu:342-354) ----------------------------------------
    def set_view(self, projection, view):
        K.check(self._L.kpt_set_view(self._ctx, K.fptr(_m16(projection)), K.fptr(_m16(view))))

    def set_camera_inverse(self, inv_projection, inv_view):
        K.check(self._L.kpt_set_camera_inverse(self._ctx, K.fptr(_m16(inv_projection)), K.fptr(_m16(inv_view))))

    # -- environment, settings, exposure (renderer.cu:290-334) ---------------
    def set_procedural_environment_data(self, env):
        e = K.Environment()
        for name, _ in K.Environment._fields_:
            if name == "rayleigh":
                e.rayleigh[:] = [float(x) for x in env["rayleigh"]]
            else:
                setattr(e, name, float(env[name]))
        K.check(self._L.kpt_set_environment(self._ctx, C.byref(e)))

    def get_procedural_environment_data(self) -> K.Environment:
        e = K.Environment()
        K.check(self._L.kpt_get_environment(self._ctx, C.byref(e)))
        return e

    def set_renderer_settings(self, **kw):
        s = K.Settings()
        K.check(self._L.kpt_get_settings(self._ctx, C.byref(s)))
        for k, v in kw.items():
            setattr(s, k, type(getattr(s, k))(v))
        K.check(self._L.kpt_set_settings(self._ctx, C.byref(s)))

    def get_renderer_settings(self) -> K.Settings:
        s = K.Settings()
        K.check(self._L.kpt_get_settings(self._ctx, C.byref(s)))
        return s

    def set_exposure(self, exposure):
        x = K.Exposure()
        for name, _ in K.Exposure._fields_:
            setattr(x, name, float(exposure[name]))
        K.check(self._L.kpt_set_exposure(self._ctx, C.byref(x)))

    def get_exposure(self) -> K.Exposure:
        x = K.Exposure()
        K.check(self._L.kpt_get_exposure(self._ctx, C.byref(x)))
        return x

    def reset_accumulation(self):
        K.check(self._L.kpt_reset_accumulation(self._ctx))

    # -- rendering (renderer.cu:103-195) -------------------------------------
    def execute_rendering(self, delta_time_ms: float = 16.0, spp: int = 1):
        K.check(self._L.kpt_render_frame(self._ctx, spp, delta_time_ms))

    def synchronize(self):
        K.check(self._L.kpt_synchronize(self._ctx))

    def _read(self, fn, shape=None):
        out = np.zeros((self.height, self.width, 4) if shape is None else shape, np.float32)
        K.check(fn(self._ctx, K.fptr(out.reshape(-1))))
        return out

    def get_render_target(self) -> np.ndarray:
        """Display image (AgX, non-linear sRGB), [H][W][4] float."""
        return self._read(self._L.kpt_read_image)

    def get_debug_render_target(self) -> np.ndarray:
        """getDebugRenderTargetTexture (renderer.cu:202-205): the reference's
        debug texture, whose only write is commented out (kernels.cu:436-448),
        so it holds zeros; [H][W][4] float at the output size."""
        return np.zeros((self.height, self.width, 4), np.float32)

    def render_size(self):
        """(width, height) of the render resolution (the output's unless upscaling)."""
        w, h = C.c_int(), C.c_int()
        K.check(self._L.kpt_get_render_size(self._ctx, C.byref(w), C.byref(h)))
        return w.value, h.value

    def _read_render_res(self, fn):
        w, h = self.render_size()
        return self._read(fn, (h, w, 4))

    def read_render(self) -> np.ndarray:
        return self._read_render_res(self._L.kpt_read_render)

    def read_accumulation(self) -> np.ndarray:
        return self._read_render_res(self._L.kpt_read_accumulation)

    def read_albedo(self) -> np.ndarray:
        return self._read_render_res(self._L.kpt_read_albedo)

    def read_history(self) -> np.ndarray:
        """Temporal accumulation's blended history: rgb, history length in alpha."""
        return self._read_render_res(self._L.kpt_read_history)

    def read_histogram(self) -> np.ndarray:
        out = np.zeros(256, np.uint64)
        K.check(self._L.kpt_read_histogram(self._ctx, out.ctypes.data_as(C.POINTER(C.c_uint64))))
        return out

    def stats(self) -> K.Stats:
        s = K.Stats()
        K.check(self._L.kpt_get_stats(self._ctx, C.byref(s)))
        return s

    def level_counts(self, max_levels: int = 65) -> np.ndarray:
        """[levels, 3]: paths shaded, sun shadow rays and area-light shadow
        rays per level of the last wave of the last frame (kpt_get_level_counts)."""
        buf = (C.c_int32 * (3 * max_levels))()
        n = C.c_int32()
        K.check(self._L.kpt_get_level_counts(self._ctx, max_levels, buf, C.byref(n)))
        return np.array(buf[:3 * n.value], np.int64).reshape(n.value, 3)

    def launch_count(self) -> int:
        n = C.c_uint64()
        K.check(self._L.kpt_launch_count(self._ctx, C.byref(n)))
        return n.value

    def stream(self) -> int:
        p = C.c_void_p()
        K.check(self._L.kpt_get_stream(self._ctx, C.byref(p)))
        return p.value or 0

    # -- device-pointer entry points (torch tensors or raw pointers) ---------
    def render_samples_device(self, sample0: int, nsamples: int, radiance_ptr: int, first_hit_ptr: int = 0,
                              albedo_ptr: int = 0):
        K.check(self._L.kpt_render_samples_device(self._ctx, sample0, nsamples, radiance_ptr or None,
                                                  first_hit_ptr or None, albedo_ptr or None))

    def trace_device(self, n, o_ptr, d_ptr, inst_ptr, tri_ptr, t_ptr, uv_ptr=0, tmin=0.0, tmax=float("inf")):
        K.check(self._L.kpt_trace_device(self._ctx, n, o_ptr, d_ptr, tmin, tmax, inst_ptr, tri_ptr, t_ptr,
                                         uv_ptr or None))

    def occluded_device(self, n, o_ptr, d_ptr, tmax_ptr, out_ptr, tmin=0.0):
        K.check(self._L.kpt_occluded_device(self._ctx, n, o_ptr, d_ptr, tmin, tmax_ptr, out_ptr))

    def trace_bounces_device(self, n, o_ptr, d_ptr, nbounces, inst_ptr, tri_ptr, t_ptr):
        K.check(self._L.kpt_trace_bounces_device(self._ctx, n, o_ptr, d_ptr, nbounces, inst_ptr, tri_ptr, t_ptr))

    def trace_bounces(self, o: np.ndarray, d: np.ndarray, nbounces: int):
        n = int(o.shape[0])
        inst = np.zeros((nbounces + 1) * n, np.int32)
        tri = np.zeros_like(inst)
        t = np.zeros((nbounces + 1) * n, np.float32)
        K.check(self._L.kpt_trace_bounces(self._ctx, n, K.fptr(np.ascontiguousarray(o, np.float32).reshape(-1)),
                                          K.fptr(np.ascontiguousarray(d, np.float32).reshape(-1)), nbounces,
                                          K.iptr(inst), K.iptr(tri), K.fptr(t)))
        return (inst.reshape(nbounces + 1, n), tri.reshape(nbounces + 1, n), t.reshape(nbounces + 1, n))

    def sky_device(self, n, dirs_ptr, out_ptr):
        K.check(self._L.kpt_sky_device(self._ctx, n, dirs_ptr, out_ptr))

    # -- path-replay adjoint (no reference counterpart) -----------------------
    def adjoint(self, sample0: int, nsamples: int, adjoint: np.ndarray, want_image: bool = False):
        """dLoss/dtheta for dLoss/dimage = adjoint ([H][W][4] float32, host);
        returns (grad float64 in adjoint_param_names order, image or None)."""
        n = C.c_int()
        K.check(self._L.kpt_adjoint_param_count(self._ctx, C.byref(n)))
        a = np.ascontiguousarray(adjoint, np.float32).reshape(-1)
        if a.size != self.width * self.height * 4:
            raise ValueError("adjoint must be [H][W][4]")
        g = np.zeros(n.value, np.float64)
        img = np.zeros((self.height, self.width, 4), np.float32) if want_image else None
        K.check(self._L.kpt_adjoint(self._ctx, sample0, nsamples, K.fptr(a), g.ctypes.data_as(C.POINTER(C.c_double)),
                                    K.fptr(img.reshape(-1)) if want_image else None))
        return g, img

    def adjoint_forward_device(self, sample0: int, nsamples: int, image_ptr: int):
        """The split adjoint's forward half: replays the samples once, keeps
        the records, writes the image ([H][W][4] float32, device pointer)."""
        K.check(self._L.kpt_adjoint_forward_device(self._ctx, sample0, nsamples, image_ptr))

    def adjoint_backward_device(self, adjoint_ptr: int, grad_ptr: int):
        """The split adjoint's backward half: dLoss/dimage ([H][W][4] float32,
        device pointer) -> gradient (float64, device pointer)."""
        K.check(self._L.kpt_adjoint_backward_device(self._ctx, adjoint_ptr, grad_ptr))

    # -- launch parameters (no reference counterpart) -------------------------
    def set_tuning(self, grid_scale: float = 1.0, wave_cap: int = 0, shade_block: int = 0, sort_rays: int = 0,
                   fetch_batch: int = 0, group_lobes: int = 0):
        t = K.Tuning(grid_scale=grid_scale, wave_cap=wave_cap, shade_block=shade_block, sort_rays=sort_rays,
                     fetch_batch=fetch_batch, group_lobes=group_lobes)
        K.check(self._L.kpt_set_tuning(self._ctx, C.byref(t)))

    def tuning(self) -> dict:
        t = K.Tuning()
        K.check(self._L.kpt_get_tuning(self._ctx, C.byref(t)))
        return {"grid_scale": t.grid_scale, "wave_cap": t.wave_cap, "shade_block": t.shade_block,
                "sort_rays": t.sort_rays, "fetch_batch": t.fetch_batch, "group_lobes": t.group_lobes}


class Batch:
    """Batched requests (no reference counterpart): one frame of each of many
    renderers -- each its own scene, camera, resolution and settings -- in
    one CUDA graph (kpt_submit_batch): by default each level's extension and
    shadow rays of every job traced by one launch from one queue spanning the
    jobs (shared = True), else each job's frame a concurrent branch; and the
    autotuner that picks their launch parameters (kpt_autotune_batch)."""

    def __init__(self, device: int = 0):
        self._L = K.load()
        self._b = C.c_void_p()
        K.check(self._L.kpt_batch_create(device, C.byref(self._b)))
        self._n = 0

    def close(self):
        if self._b:
            K.check(self._L.kpt_batch_destroy(self._b))
            self._b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _args(self, renderers, spp):
        n = len(renderers)
        jobs = (C.c_void_p * n)(*[r._ctx.value for r in renderers])
        s = np.ascontiguousarray(np.broadcast_to(np.asarray(spp, np.int32), (n,)))
        return n, jobs, s

    @property
    def shared(self) -> bool:
        v = np.zeros(1, np.int32)
        K.check(self._L.kpt_batch_get_shared(self._b, K.iptr(v)))
        return bool(v[0])

    @shared.setter
    def shared(self, on: bool):
        K.check(self._L.kpt_batch_set_shared(self._b, int(on)))

    def submit(self, renderers, spp, lanes: int = 0):
        n, jobs, s = self._args(renderers, spp)
        K.check(self._L.kpt_submit_batch(self._b, n, jobs, K.iptr(s), lanes))
        self._n = n

    def wait(self):
        """Per-job device latency from the batch start (ms) and the batch's device time."""
        job = np.zeros(max(self._n, 1), np.float32)
        total = np.zeros(1, np.float32)
        K.check(self._L.kpt_wait_batch(self._b, K.fptr(job), K.fptr(total)))
        return job[:self._n], float(total[0])

    def autotune(self, renderers, spp, reps: int = 2):
        n, jobs, s = self._args(renderers, spp)
        t = K.Tuning()
        lanes = np.zeros(1, np.int32)
        ms = np.zeros(1, np.float32)
        K.check(self._L.kpt_autotune_batch(self._b, n, jobs, K.iptr(s), reps, C.byref(t), K.iptr(lanes),
                                           K.fptr(ms)))
        return ({"grid_scale": t.grid_scale, "wave_cap": t.wave_cap, "shade_block": t.shade_block,
                 "sort_rays": t.sort_rays, "fetch_batch": t.fetch_batch, "group_lobes": t.group_lobes}, int(lanes[0]), float(ms[0]))


# -- path-replay adjoint (no reference counterpart) ----------------------------

SKY_PARAM_NAMES = ("rayleigh_r", "rayleigh_g", "rayleigh_b", "mie", "rayleigh_height", "mie_height")


def adjoint_param_names(nmat: int):
    """Order of kpt_adjoint's gradient: per material (albedo r, g, b,
    roughness), then the sky."""
    names = []
    for m in range(nmat):
        names += [f"m{m}.albedo_r", f"m{m}.albedo_g", f"m{m}.albedo_b", f"m{m}.roughness"]
    return names + list(SKY_PARAM_NAMES)
