"""ORACLE — test infrastructure only (CPU restatement of the reference path).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU baseline as the checker;
never by the product package. See oracle/oracle.cpp for what is restated and how each
part is pinned.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_vp = C.c_void_p
_lib = None
_ref = None


class OracleScene(C.Structure):
    _fields_ = [
        ("tris", _vp), ("ids", _vp), ("ntri", C.c_uint64),
        ("ninst", C.c_int32), ("inst_l2w", _vp), ("inst_w2l", _vp), ("inst_geo", _vp), ("inst_mat", _vp),
        ("inst_light", _vp), ("inst_inner", _vp), ("inst_outer", _vp),
        ("ngeo", C.c_int32), ("geo_offset", _vp), ("geo_count", _vp), ("geo_area_total", _vp), ("shade", _vp),
        ("total_geo_tris", C.c_uint64), ("tri_area", _vp), ("local_pos", _vp),
        ("nmat", C.c_int32), ("mat", _vp),
        ("nlight", C.c_int32), ("light_inst", _vp), ("light_geo", _vp), ("light_scale", _vp),
        ("light_intensity", _vp),
        ("env_type", C.c_int32), ("env_lower", C.c_float * 3), ("env_upper", C.c_float * 3),
        ("env_up", C.c_float * 3),
        ("vacuum_medium", C.c_int32), ("world_diagonal", C.c_float),
        ("nmed", C.c_int32), ("med", _vp), ("med_grid_offset", _vp), ("grids", _vp),
        ("eye", C.c_float * 3), ("lbc", C.c_float * 3), ("film_x", C.c_float * 3), ("film_y", C.c_float * 3),
        ("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("min_depth", C.c_int32),
        ("max_depth", C.c_int32), ("rr_threshold", C.c_float), ("rr_cont_prob", C.c_float),
        ("sampler", C.c_int32), ("filter", C.c_int32), ("filter_radius", C.c_float), ("filter_alpha", C.c_float),
        ("nvol", C.c_int32), ("vol", _vp), ("vol_off", _vp),
        ("ntex_img", C.c_int32), ("tex_img", _vp), ("tex_texels", _vp), ("tex_instr", _vp), ("mat_tex", _vp),
        ("mat_texrow", _vp), ("env_prog", C.c_int32), ("env_lut_w", C.c_int32), ("env_lut_h", C.c_int32),
    ]


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(str(path))
        L.oracle_bvh_build.restype = _vp
        L.oracle_bvh_build.argtypes = [_vp, _vp, C.c_uint64]
        L.oracle_bvh_free.argtypes = [_vp]
        L.oracle_trace_closest.argtypes = [_vp, _vp, C.c_uint64, _vp, _vp, C.c_int]
        L.oracle_trace_any.argtypes = [_vp, _vp, C.c_uint64, _vp, C.c_int]
        L.oracle_sampler_batch.argtypes = [C.c_int, C.c_int, C.c_int, _vp, _vp, C.c_uint64, C.c_uint32, _vp]
        L.oracle_pcg32_stream.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, _vp]
        L.oracle_murmur64a.restype = C.c_uint64
        L.oracle_murmur64a.argtypes = [_vp, C.c_uint64, C.c_uint64]
        L.oracle_bsdf_batch.argtypes = [C.c_int, _vp, _vp, _vp, C.c_uint64, _vp]
        L.oracle_bsdf_batch_f32.argtypes = [C.c_int, _vp, _vp, _vp, C.c_uint64, _vp]
        L.oracle_prepare.restype = _vp
        L.oracle_prepare.argtypes = [C.POINTER(OracleScene)]
        L.oracle_medium_tr_batch.argtypes = [C.POINTER(OracleScene), C.c_int, _vp, _vp, C.c_uint64, _vp]
        L.oracle_release.argtypes = [_vp]
        L.oracle_wide_bvh_counts.argtypes = [_vp, _vp, _vp, C.c_uint64, _vp, _vp, C.c_int]
        L.oracle_render.argtypes = [_vp, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, _vp, C.c_int]
        L.oracle_render_aov.argtypes = [_vp, C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32, _vp, _vp, C.c_int]
        _lib = L
    return _lib


def ref_lib() -> C.CDLL | None:
    """The reference tree's vendored lib/bvh (oracle/_ref), or None when not built."""
    global _ref
    if _ref is None:
        path = _build.build_ref()
        if path is None or not Path(path).exists():
            return None
        L = C.CDLL(str(path))
        L.ref_build.restype = _vp
        L.ref_build.argtypes = [_vp, C.c_uint64]
        L.ref_free.argtypes = [_vp]
        L.ref_closest.argtypes = [_vp, _vp, C.c_uint64, _vp, _vp]
        _ref = L
    return _ref


def _p(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


class OracleBvh:
    """Closest / any hit over world-space triangles (9 floats) with (inst, prim) ids."""

    def __init__(self, tris: np.ndarray, ids: np.ndarray):
        self.tris = np.ascontiguousarray(tris, np.float32)
        self.ids = np.ascontiguousarray(ids, np.uint32)
        self.h = lib().oracle_bvh_build(_p(self.tris), _p(self.ids), len(self.tris))

    def closest(self, rays: np.ndarray, threads: int = 0) -> tuple[np.ndarray, np.ndarray]:
        rays = np.ascontiguousarray(rays, np.float32)
        flags = np.zeros(len(rays), np.uint32)
        hits = np.zeros((len(rays), 4), np.float32)
        lib().oracle_trace_closest(self.h, _p(rays), len(rays), _p(flags), _p(hits), threads)
        return flags, hits

    def any(self, rays: np.ndarray, threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, np.float32)
        occ = np.zeros(len(rays), np.uint32)
        lib().oracle_trace_any(self.h, _p(rays), len(rays), _p(occ), threads)
        return occ

    def __del__(self):
        try:
            lib().oracle_bvh_free(self.h)
        except Exception:
            pass


def _xf_rows(m: np.ndarray, v: np.ndarray, translate: bool) -> np.ndarray:
    """Rows of (N, 3) float32 vectors through a 3x4 matrix, ((m0 x + m1 y) + m2 z) (+ m3)
    with every product and sum rounded to FP32: the host's Transform::point order."""
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    cols = []
    for r in range(3):
        a = (m[r, 0] * x).astype(np.float32)
        a = (a + (m[r, 1] * y).astype(np.float32)).astype(np.float32)
        a = (a + (m[r, 2] * z).astype(np.float32)).astype(np.float32)
        if translate:
            a = (a + m[r, 3]).astype(np.float32)
        cols.append(a)
    return np.stack(cols, axis=1).astype(np.float32)


def two_level_trace(S, rays: np.ndarray, threads: int = 0):
    """Closest and any hit through per-instance object-space rays (the two-level form of
    the acceleration structure): every instance's world-to-local matrix takes the rays
    into object space, the geometry's own triangles are intersected there with the
    oracle's watertight test, and hits combine in (t, instance, primitive) order, as
    OptiX's IAS over GASes does (core/btrc/core/scene.cpp:196-209). S is an
    oracle.scene.Scene. Returns (flags, hits, occluded) in btrc_trace_* layout."""
    rays = np.ascontiguousarray(rays, np.float32)
    n = len(rays)
    best_t = np.full(n, np.inf, np.float32)
    best_inst = np.full(n, 0xFFFFFFFF, np.uint64)
    best_prim = np.full(n, 0xFFFFFFFF, np.uint64)
    hits = np.zeros((n, 4), np.float32)
    occ = np.zeros(n, np.uint32)
    trees = {}
    for i, g in enumerate(S.inst_geo):
        g = int(g)
        cnt, off = int(S.geo_count[g]), int(S.geo_offset[g])
        if cnt == 0:
            continue
        if g not in trees:
            ids = np.stack([np.zeros(cnt, np.uint32), np.arange(cnt, dtype=np.uint32)], 1)
            trees[g] = OracleBvh(S.local_pos[off:off + cnt], ids)
        w = S.inst_w2l[i].reshape(3, 4).astype(np.float32)
        r = rays.copy()
        r[:, 0:3] = _xf_rows(w, rays[:, 0:3], True)
        r[:, 4:7] = _xf_rows(w, rays[:, 4:7], False)
        f, h = trees[g].closest(r, threads)
        t = h[:, 0]
        prim = h[:, 1].view(np.uint32).astype(np.uint64)
        better = (f != 0) & ((t < best_t) | ((t == best_t) & ((i < best_inst) | ((i == best_inst) & (prim < best_prim)))))
        best_t[better] = t[better]
        best_inst[better] = i
        best_prim[better] = prim[better]
        hits[better] = h[better]
        occ |= trees[g].any(r, threads)
    hit = best_inst != 0xFFFFFFFF
    flags = np.where(hit, best_inst.astype(np.uint32) | np.uint32(1 << 30), np.uint32(0)).astype(np.uint32)
    hits[~hit] = 0.0
    return flags, hits, occ


def sampler_batch(kind: int, width: int, height: int, pixel_xy: np.ndarray, sample_index: np.ndarray,
                  dims: int) -> np.ndarray:
    pixel_xy = np.ascontiguousarray(pixel_xy, np.uint32)
    sample_index = np.ascontiguousarray(sample_index, np.uint32)
    out = np.zeros((len(pixel_xy), dims), np.float32)
    lib().oracle_sampler_batch(kind, width, height, _p(pixel_xy), _p(sample_index), len(pixel_xy), dims, _p(out))
    return out


def pcg32_stream(initstate: int, initseq: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().oracle_pcg32_stream(initstate, initseq, n, _p(out))
    return out


def murmur64a(data: bytes, seed: int = 0) -> int:
    buf = np.frombuffer(data, np.uint8).copy() if data else np.zeros(1, np.uint8)
    return int(lib().oracle_murmur64a(_p(buf), len(data), seed))


def wide_bvh_counts(nodes: np.ndarray, tris: np.ndarray, rays: np.ndarray, threads: int = 0):
    """Node visits and triangle tests per ray of a sequential, exact-box closest-hit
    traversal of the library's exported 8-wide BVH (nodes: (n, 80) uint8, tris: (m, 48)
    uint8 as btrc_scene_export_bvh writes them; rays: (k, 8) float32)."""
    nodes = np.ascontiguousarray(nodes, np.uint8)
    tris = np.ascontiguousarray(tris).view(np.uint8)
    rays = np.ascontiguousarray(rays, np.float32)
    nv = np.zeros(len(rays), np.uint32)
    tt = np.zeros(len(rays), np.uint32)
    lib().oracle_wide_bvh_counts(_p(nodes), _p(tris), _p(rays), len(rays), _p(nv), _p(tt), threads)
    return nv, tt


def bsdf_batch(op: int, material: np.ndarray, wo: np.ndarray, wi_or_u: np.ndarray, fp32: bool = False) -> np.ndarray:
    """Local-space BSDF in FP64 (or the same code in FP32). material: (n, 16) float32,
    type in column 15. op 0: (f.rgb, pdf); op 1: (f.rgb, pdf, wi.xyz); op 2 (FP64 only):
    (drawn, 0, 0, 0, wi.xyz), the sampled direction before Disney's bad-sample rejection."""
    material = np.ascontiguousarray(material, np.float32)
    wo = np.ascontiguousarray(wo, np.float64)
    wu = np.ascontiguousarray(wi_or_u, np.float64)
    out = np.zeros((len(material), 4 if op == 0 else 7), np.float64)
    fn = lib().oracle_bsdf_batch_f32 if fp32 else lib().oracle_bsdf_batch
    fn(op, _p(material), _p(wo), _p(wu), len(material), _p(out))
    return out


def ref_closest(tris: np.ndarray, rays: np.ndarray) -> tuple[np.ndarray, np.ndarray] | None:
    """Closest hit with the reference tree's lib/bvh; None when it is not built."""
    L = ref_lib()
    if L is None:
        return None
    tris = np.ascontiguousarray(tris, np.float32)
    rays = np.ascontiguousarray(rays, np.float32)
    h = L.ref_build(_p(tris), len(tris))
    prim = np.zeros(len(rays), np.int64)
    t = np.zeros(len(rays), np.float32)
    try:
        L.ref_closest(h, _p(rays), len(rays), _p(prim), _p(t))
    finally:
        L.ref_free(h)
    return prim, t
