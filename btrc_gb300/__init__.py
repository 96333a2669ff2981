"""btrc_gb300: GB300-native wavefront path tracer with Btrc's scene format.

Python mirror of the C ABI in include/btrc.h (ctypes). The compute path is the in-tree
CUDA library btrc_gb300/_build/libbtrc_gb300.so; there is no CPU fallback: when the
library is missing or no GPU is present, the calls raise.

Typical use (the reference's CLI flow, src/cli/main.cpp:17-81):

    ctx = btrc_gb300.Context(0)
    scene = ctx.load_scene("scene.json")   # parse JSON, load OBJ files
    scene.build()                          # SAH BVH + upload
    image = ctx.render(scene)              # float32 (H, W, 3) radiance / weight
"""
from __future__ import annotations

import ctypes as C
import os
import weakref
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libbtrc_gb300.so"

OK = 0
STATUS_NAMES = {
    0: "OK", 1: "INVALID_ARG", 2: "IO", 3: "PARSE", 4: "CUDA", 5: "OOM",
    6: "TIMEOUT", 7: "CANCELLED", 8: "UNSUPPORTED", 9: "INTERNAL",
}
HIT_BIT = 1 << 30

# exported symbols and their ctypes signatures (kept in sync with include/btrc.h)
_vp = C.c_void_p


class SceneInfo(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32),
        ("min_depth", C.c_int32), ("max_depth", C.c_int32), ("state_count", C.c_int32),
        ("sampler", C.c_int32), ("filter", C.c_int32),
        ("instances", C.c_int32), ("geometries", C.c_int32), ("materials", C.c_int32),
        ("area_lights", C.c_int32), ("media", C.c_int32), ("has_envir_light", C.c_int32),
        ("triangles", C.c_uint64), ("bvh_nodes", C.c_int32), ("bvh_depth", C.c_int32),
        ("bvh_bytes", C.c_uint64), ("world_min", C.c_float * 3), ("world_max", C.c_float * 3),
        ("build_ms", C.c_double), ("bvh_ms", C.c_double), ("bvh_builder", C.c_int32), ("two_level", C.c_int32),
    ]


class BuildOpts(C.Structure):
    _fields_ = [("threads", C.c_int32), ("builder", C.c_int32), ("two_level", C.c_int32)]


BUILDERS = {"host": 0, "device": 1}


class RenderOpts(C.Structure):
    _fields_ = [("spp", C.c_int32), ("state_count", C.c_int32), ("output_on_device", C.c_int32),
                ("use_graphs", C.c_int32), ("profile", C.c_int32), ("post_process", C.c_int32),
                ("albedo_out", _vp), ("normal_out", _vp)]


class NrcRenderOpts(C.Structure):
    _fields_ = [("frame", C.c_uint32), ("terminate_vertex", C.c_int32), ("train_stride", C.c_int32),
                ("train_steps", C.c_int32), ("train_batch", C.c_int32), ("output_on_device", C.c_int32),
                ("spread_threshold", C.c_float)]


class NrcFrameStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("queries", C.c_uint64), ("train_samples", C.c_uint64),
                ("train_steps", C.c_int32), ("loss", C.c_float), ("render_ms", C.c_double), ("wall_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchOpts(C.Structure):
    _fields_ = [("lanes", C.c_int32), ("autotune", C.c_int32), ("output_on_device", C.c_int32),
                ("merged", C.c_int32)]


class BatchSceneStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("ms", C.c_double), ("lane", C.c_int32), ("capacity", C.c_uint32),
                ("grid_pct", C.c_int32), ("block", C.c_int32), ("done_ms", C.c_double)]


STAGES = ("control", "generate", "trace", "medium", "shade", "shadow")


class Stats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("bounces", C.c_uint32), ("traversal_errors", C.c_uint32), ("device_ms", C.c_double),
                ("wall_ms", C.c_double), ("kernel_launches", C.c_uint64), ("stage_ms", C.c_double * 6),
                ("stage_launches", C.c_uint64 * 6), ("node_visits", C.c_uint64), ("tri_tests", C.c_uint64)]

    def as_dict(self) -> dict:
        d = {}
        for k, _ in self._fields_:
            v = getattr(self, k)
            d[k] = dict(zip(STAGES, list(v))) if k in ("stage_ms", "stage_launches") else v
        return d


SIGNATURES = {
    "btrc_version": (C.c_char_p, []),
    "btrc_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "btrc_ctx_destroy": (None, [_vp]),
    "btrc_last_error": (C.c_char_p, [_vp]),
    "btrc_cancel": (None, [_vp]),
    "btrc_scene_load_json": (C.c_int, [_vp, C.c_char_p, C.POINTER(_vp)]),
    "btrc_scene_build": (C.c_int, [_vp, C.POINTER(BuildOpts)]),
    "btrc_scenes_load_build": (C.c_int, [_vp, C.POINTER(C.c_char_p), C.c_uint32, C.POINTER(BuildOpts),
                                         C.POINTER(_vp)]),
    "btrc_scene_info_get": (C.c_int, [_vp, C.POINTER(SceneInfo)]),
    "btrc_scene_destroy": (None, [_vp]),
    "btrc_scene_export_triangles": (C.c_int, [_vp, _vp, _vp, C.c_uint64]),
    "btrc_scene_export_bvh": (C.c_int, [_vp, _vp, C.c_uint64, _vp, C.c_uint64]),
    "btrc_render": (C.c_int, [_vp, _vp, C.POINTER(RenderOpts), _vp, C.POINTER(Stats)]),
    "btrc_render_noalloc": (C.c_int, [_vp, _vp, C.c_int32, _vp, C.POINTER(Stats)]),
    "btrc_trace_closest": (C.c_int, [_vp, _vp, _vp, C.c_uint64, _vp, _vp, _vp]),
    "btrc_trace_any": (C.c_int, [_vp, _vp, _vp, C.c_uint64, _vp, _vp]),
    "btrc_trace_stats": (C.c_int, [_vp, _vp, _vp, C.c_uint64, _vp, _vp, _vp]),
    "btrc_sampler_batch": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_int32, _vp, _vp, C.c_uint64, C.c_uint32,
                                     _vp, _vp]),
    "btrc_bsdf_batch": (C.c_int, [_vp, C.c_int32, _vp, _vp, _vp, C.c_uint64, _vp, _vp]),
    "btrc_medium_tr_batch": (C.c_int, [_vp, _vp, C.c_int32, _vp, _vp, C.c_uint64, _vp, _vp]),
    "btrc_tonemap_aces": (C.c_int, [_vp, _vp, C.c_int32, C.c_int32, C.c_int32, C.c_float, _vp]),
    "btrc_denoise_atrous": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32, _vp]),
    "btrc_image_save": (C.c_int, [_vp, C.c_char_p, _vp, C.c_int32, C.c_int32, C.c_int32, C.c_float]),
    "btrc_nrc_create": (C.c_int, [_vp, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_uint64, C.POINTER(_vp)]),
    "btrc_nrc_destroy": (None, [_vp]),
    "btrc_nrc_infer": (C.c_int, [_vp, _vp, _vp, C.c_uint64, _vp, _vp]),
    "btrc_nrc_train": (C.c_int, [_vp, _vp, _vp, C.c_uint64, C.c_int32, C.POINTER(C.c_float)]),
    "btrc_nrc_params": (C.c_int, [_vp, _vp, C.c_int32, _vp, C.c_uint64, C.c_int32]),
    "btrc_render_batch": (C.c_int, [_vp, C.POINTER(_vp), C.c_uint32, C.POINTER(BatchOpts), C.POINTER(_vp),
                                    C.POINTER(BatchSceneStats), C.POINTER(C.c_double)]),
    "btrc_render_nrc_frame": (C.c_int, [_vp, _vp, _vp, C.POINTER(NrcRenderOpts), _vp, C.POINTER(NrcFrameStats)]),
    "btrc_image_load": (C.c_int, [_vp, C.c_char_p, _vp, C.c_uint64, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_int32)]),
}

_lib = None


class BtrcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def load_library(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load the CUDA library (built by btrc_gb300._build.build()). Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"native library {p} is missing: run btrc_gb300._build.build() first")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def version() -> str:
    return load_library().btrc_version().decode()


def _ptr(x) -> int | None:
    """Raw address of a torch tensor / numpy array / int."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    raise TypeError(f"cannot take a pointer of {type(x)}")


class Context:
    """One CUDA device + stream (btrc_ctx)."""

    def __init__(self, device: int = 0):
        self._lib = load_library()
        h = _vp()
        st = self._lib.btrc_ctx_create(device, C.byref(h))
        if st != OK:
            raise BtrcError(st, f"btrc_ctx_create(device={device}) failed")
        self.handle = h
        self.device = device
        self._scenes = weakref.WeakSet()

    def _check(self, status: int):
        if status != OK:
            msg = self._lib.btrc_last_error(self.handle)
            raise BtrcError(status, msg.decode() if msg else "")

    def close(self):
        """Destroy the context; scenes still open on it are destroyed with it."""
        if getattr(self, "handle", None):
            for sc in list(getattr(self, "_scenes", ())):
                sc.handle = None  # owned by the context from here on
            self._lib.btrc_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def load_scene(self, path: str | os.PathLike) -> "Scene":
        h = _vp()
        self._check(self._lib.btrc_scene_load_json(self.handle, str(path).encode(), C.byref(h)))
        sc = Scene(self, h)
        self._scenes.add(sc)
        return sc

    def load_build_scenes(self, paths: list, threads: int = 0, builder: str = "host",
                          two_level: bool = False) -> list:
        """Load and build many scenes at once on one pool of host threads
        (btrc_scenes_load_build); builder "device" builds the BVHs on the GPU.
        Returns the built scenes in order."""
        n = len(paths)
        arr_p = (C.c_char_p * n)(*[str(p).encode() for p in paths])
        arr_s = (_vp * n)()
        opts = BuildOpts(threads, BUILDERS[builder], 1 if two_level else 0)
        self._check(self._lib.btrc_scenes_load_build(self.handle, arr_p, n, C.byref(opts), arr_s))
        out = []
        for h in arr_s:
            sc = Scene(self, _vp(h))
            self._scenes.add(sc)
            out.append(sc)
        return out

    def cancel(self):
        self._lib.btrc_cancel(self.handle)

    def render(self, scene: "Scene", spp: int = 0, state_count: int = 0, out=None, use_graphs: bool = True,
               stats: dict | None = None, profile: int = 0, post_process: bool = False, albedo=None,
               normal=None) -> np.ndarray:
        """Render the scene's frame. `out` may be a CUDA tensor (rendered in place) or None
        (a new host float32 array of shape (H, W, 3) is returned). `albedo` / `normal`
        receive the first-hit g-buffers (arrays in the same memory space as `out`);
        post_process runs the scene's post_processors (tonemap, denoise, save) on the result."""
        info = scene.info()
        on_dev = out is not None and hasattr(out, "is_cuda") and out.is_cuda
        if out is None:
            out = np.zeros((info.height, info.width, 3), np.float32)
        opts = RenderOpts(spp, state_count, 1 if on_dev else 0, 1 if use_graphs else 0, profile,
                          1 if post_process else 0, _ptr(albedo) if albedo is not None else None,
                          _ptr(normal) if normal is not None else None)
        st = Stats()
        self._check(self._lib.btrc_render(self.handle, scene.handle, C.byref(opts), _ptr(out), C.byref(st)))
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def render_batch(self, scenes: list, outs: list, lanes: int = 4, autotune: bool = True,
                     merged: bool = False) -> tuple[list, float]:
        """Render many built scenes (btrc_render_batch): through concurrent lanes, or with
        merged=True in one pass of one path queue through one set of stage kernels. outs are
        CUDA tensors or host arrays of each scene's (H, W, 3). Returns (per-scene stats,
        total wall ms)."""
        n = len(scenes)
        on_dev = n > 0 and hasattr(outs[0], "is_cuda") and outs[0].is_cuda
        arr_s = (_vp * n)(*[s.handle for s in scenes])
        arr_o = (_vp * n)(*[_ptr(o) for o in outs])
        st = (BatchSceneStats * n)()
        total = C.c_double()
        opts = BatchOpts(lanes, 1 if autotune else 0, 1 if on_dev else 0, 1 if merged else 0)
        self._check(self._lib.btrc_render_batch(self.handle, arr_s, n, C.byref(opts), arr_o, st, C.byref(total)))
        return [{k: getattr(x, k) for k, _ in BatchSceneStats._fields_} for x in st], total.value

    def render_noalloc(self, scene: "Scene", out, spp: int = 0, stats: dict | None = None):
        """Allocation-free render into a caller-owned CUDA tensor of shape (H, W, 3)
        (btrc_render_noalloc: fixed scratch, film up to 512x512 pixels).

        `out` must be a contiguous float32 CUDA tensor on this context's device with at
        least H*W*3 elements; anything else raises BtrcError(INVALID_ARG) before the
        library is called. Work already queued on torch's current stream (a fill of
        `out`, say) is finished first, since the render runs on the context's own stream."""
        info = scene.info()
        need = info.width * info.height * 3
        if not (hasattr(out, "is_cuda") and out.is_cuda):
            raise BtrcError(1, "render_noalloc: out must be a CUDA tensor (device memory)")
        import torch
        if out.dtype != torch.float32 or not out.is_contiguous():
            raise BtrcError(1, "render_noalloc: out must be a contiguous float32 tensor")
        if out.device.index != self.device:
            raise BtrcError(1, f"render_noalloc: out is on cuda:{out.device.index}, the context on cuda:{self.device}")
        if out.numel() < need:
            raise BtrcError(1, f"render_noalloc: out holds {out.numel()} floats, the film needs {need}")
        torch.cuda.current_stream(out.device).synchronize()
        st = Stats()
        self._check(self._lib.btrc_render_noalloc(self.handle, scene.handle, spp, _ptr(out), C.byref(st)))
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def trace_closest(self, scene: "Scene", rays, n: int, flags, hits, stream: int | None = None):
        self._check(self._lib.btrc_trace_closest(self.handle, scene.handle, _ptr(rays), n, _ptr(flags),
                                                 _ptr(hits), stream))

    def trace_any(self, scene: "Scene", rays, n: int, occluded, stream: int | None = None):
        self._check(self._lib.btrc_trace_any(self.handle, scene.handle, _ptr(rays), n, _ptr(occluded), stream))

    def trace_stats(self, scene: "Scene", rays, n: int, node_visits, tri_tests, stream: int | None = None):
        self._check(self._lib.btrc_trace_stats(self.handle, scene.handle, _ptr(rays), n, _ptr(node_visits),
                                               _ptr(tri_tests), stream))

    def sampler_batch(self, kind: int, width: int, height: int, pixel_xy, sample_index, n: int, dims: int, out,
                      stream: int | None = None):
        self._check(self._lib.btrc_sampler_batch(self.handle, kind, width, height, _ptr(pixel_xy),
                                                 _ptr(sample_index), n, dims, _ptr(out), stream))

    def bsdf_batch(self, op: int, material, wo, wi_or_u, n: int, out, stream: int | None = None):
        self._check(self._lib.btrc_bsdf_batch(self.handle, op, _ptr(material), _ptr(wo), _ptr(wi_or_u), n,
                                              _ptr(out), stream))

    def medium_tr_batch(self, scene: "Scene", medium_id: int, seg, seeds, n: int, out, stream: int | None = None):
        self._check(self._lib.btrc_medium_tr_batch(self.handle, scene.handle, medium_id, _ptr(seg), _ptr(seeds),
                                                   n, _ptr(out), stream))

    def tonemap_aces(self, pixels, width: int, height: int, channels: int = 3, exposure: float = 1.0,
                     stream: int | None = None):
        """In-place ACES tone map of a device buffer (tonemap post-processor)."""
        self._check(self._lib.btrc_tonemap_aces(self.handle, _ptr(pixels), width, height, channels, exposure,
                                                stream))

    def denoise_atrous(self, pixels, width: int, height: int, albedo=None, normal=None, stream: int | None = None):
        """In-place edge-avoiding a-trous denoise of a device RGB buffer, optionally guided by
        device albedo / normal images (denoise post-processor)."""
        self._check(self._lib.btrc_denoise_atrous(self.handle, _ptr(pixels), _ptr(albedo), _ptr(normal), width,
                                                  height, stream))

    def image_load(self, filename: str) -> tuple[np.ndarray, int]:
        """Decode a .png / .hdr texture file: ((H, W, 4) float32 texels, file channels)."""
        w, h, c = C.c_int32(), C.c_int32(), C.c_int32()
        fn = str(filename).encode()
        self._check(self._lib.btrc_image_load(self.handle, fn, None, 0, C.byref(w), C.byref(h), C.byref(c)))
        out = np.zeros((h.value, w.value, 4), np.float32)
        self._check(self._lib.btrc_image_load(self.handle, fn, _ptr(out), out.size, C.byref(w), C.byref(h),
                                              C.byref(c)))
        return out, c.value

    def image_save(self, filename: str, pixels: np.ndarray, gamma: float = 1.0):
        """Write an (H, W, 3|4) float image to .png / .exr / .hdr (save post-processor)."""
        px = np.ascontiguousarray(pixels, np.float32)
        h, w, c = px.shape
        self._check(self._lib.btrc_image_save(self.handle, str(filename).encode(), _ptr(px), w, h, c, gamma))


NRC_QUERY_FLOATS = 13
NRC_SAMPLE_FLOATS = 16
NRC_WEIGHTS = 22528
NRC_HASH_FLOATS = 16 * (1 << 19) * 2


class RadianceCache:
    """btrc_nrc: hash-grid + SH encoded 5x64 BF16 MLP radiance cache trained with Adam."""

    def __init__(self, ctx: "Context", bbox_min, bbox_max, seed: int = 1):
        self.ctx = ctx
        lo = (C.c_float * 3)(*map(float, bbox_min))
        hi = (C.c_float * 3)(*map(float, bbox_max))
        h = _vp()
        ctx._check(ctx._lib.btrc_nrc_create(ctx.handle, lo, hi, seed, C.byref(h)))
        self.handle = h

    def infer(self, queries, n: int, out, stream: int | None = None):
        self.ctx._check(self.ctx._lib.btrc_nrc_infer(self.ctx.handle, self.handle, _ptr(queries), n, _ptr(out),
                                                     stream))

    def train(self, samples, n: int, apply_adam: bool = True) -> float:
        loss = C.c_float()
        self.ctx._check(self.ctx._lib.btrc_nrc_train(self.ctx.handle, self.handle, _ptr(samples), n,
                                                     1 if apply_adam else 0, C.byref(loss)))
        return loss.value

    def params(self, which: int) -> np.ndarray:
        n = NRC_WEIGHTS if which in (0, 2) else NRC_HASH_FLOATS
        out = np.zeros(n, np.float32)
        self.ctx._check(self.ctx._lib.btrc_nrc_params(self.ctx.handle, self.handle, which, _ptr(out), n, 0))
        return out

    def render_frame(self, scene: "Scene", frame: int, out=None, terminate_vertex: int = 1, train_stride: int = 16,
                     train_steps: int = 4, train_batch: int = 16384, stats: dict | None = None,
                     spread_threshold: float = 0.0):
        """One frame (one path per pixel) with cache termination, training and inference
        (btrc_render_nrc_frame). spread_threshold > 0 ends paths by the path-spread rule
        instead of at terminate_vertex. Returns the frame image (H, W, 3)."""
        info = scene.info()
        on_dev = out is not None and hasattr(out, "is_cuda") and out.is_cuda
        if out is None:
            out = np.zeros((info.height, info.width, 3), np.float32)
        opts = NrcRenderOpts(frame, terminate_vertex, train_stride, train_steps, train_batch, 1 if on_dev else 0,
                             spread_threshold)
        st = NrcFrameStats()
        self.ctx._check(self.ctx._lib.btrc_render_nrc_frame(self.ctx.handle, scene.handle, self.handle, C.byref(opts),
                                                            _ptr(out), C.byref(st)))
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def set_params(self, which: int, values: np.ndarray):
        v = np.ascontiguousarray(values, np.float32)
        self.ctx._check(self.ctx._lib.btrc_nrc_params(self.ctx.handle, self.handle, which, _ptr(v), v.size, 1))

    def close(self):
        if self.handle:
            self.ctx._lib.btrc_nrc_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    """A loaded scene (btrc_scene). build() constructs the BVH and uploads to HBM."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    def build(self, threads: int = 0, builder: str = "host", two_level: bool = False) -> "Scene":
        """btrc_scene_build; builder "host" (binned SAH on the host threads) or "device"
        (PLOC on the GPU, then the same 8-wide collapse and node layout); two_level builds
        one tree per geometry under a top level over the instances."""
        opts = BuildOpts(threads, BUILDERS[builder], 1 if two_level else 0)
        self.ctx._check(self.ctx._lib.btrc_scene_build(self.handle, C.byref(opts)))
        return self

    def info(self) -> SceneInfo:
        info = SceneInfo()
        self.ctx._check(self.ctx._lib.btrc_scene_info_get(self.handle, C.byref(info)))
        return info

    def export_triangles(self) -> tuple[np.ndarray, np.ndarray]:
        n = self.info().triangles
        xyz = np.zeros((n, 9), np.float32)
        ids = np.zeros((n, 2), np.uint32)
        self.ctx._check(self.ctx._lib.btrc_scene_export_triangles(self.handle, xyz.ctypes.data, ids.ctypes.data, n))
        return xyz, ids

    def export_bvh(self) -> tuple[np.ndarray, np.ndarray]:
        """(nodes, tris) as raw uint8 arrays of shape (N, 80) and (M, 48)."""
        info = self.info()
        nodes = np.zeros((info.bvh_nodes, 80), np.uint8)
        tris = np.zeros((info.triangles, 48), np.uint8)
        self.ctx._check(self.ctx._lib.btrc_scene_export_bvh(self.handle, nodes.ctypes.data, len(nodes),
                                                            tris.ctypes.data, len(tris)))
        return nodes, tris

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            self.ctx._lib.btrc_scene_destroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
