"""ctypes binding of liblrx.so (include/lrx.h).

The library is the product: this module loads it from luxcore_gb300/lib/
and raises if it is missing -- there is no CPU fallback.  Device buffers are
passed as raw device addresses (ints), streams as raw cudaStream_t handles;
PyTorch, when used by callers, only provides that memory and those streams.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "liblrx.so")

LRX_TRACE_CLOSEST = 0
LRX_TRACE_ANY = 1
LRX_OBJECT_INSTANCE = 0x1
LRX_OBJECT_HAS_INVERSE = 0x2
LRX_ERR_INVALID_ARGUMENT = 1
LRX_ERR_NOT_SUPPORTED = 6

# lrx_trace_config.variant bits (include/lrx.h)
LRX_VARIANT_MINMAX3 = 0x1
LRX_VARIANT_SCENE_L2_KEEP = 0x2
LRX_VARIANT_STREAM_RAYS = 0x4
LRX_VARIANT_OCCUPANCY = 0x8
LRX_VARIANT_SORT_RAYS = 0x10
LRX_VARIANT_SORT_OCTANT = 0x20
LRX_VARIANT_PERSISTENT = 0x40
LRX_VARIANT_SMEM_STACK = 0x80
LRX_VARIANT_COMPACT = 0x100
LRX_VARIANT_SMEM_STACK16 = 0x400
LRX_VARIANT_SMEM_STACK32 = 0x800
LRX_VARIANT_DRAIN_SPLIT = 0x2000

STATUS_NAMES = {0: "LRX_OK", 1: "LRX_ERR_INVALID_ARGUMENT", 2: "LRX_ERR_CUDA", 3: "LRX_ERR_OUT_OF_MEMORY",
                4: "LRX_ERR_BUILD", 5: "LRX_ERR_DEVICE", 6: "LRX_ERR_NOT_SUPPORTED", 7: "LRX_ERR_BUDGET",
                8: "LRX_ERR_BUSY", 9: "LRX_ERR_TIMEOUT"}

# Every function include/lrx.h declares (checked by the CPU tests).
EXPORTED = ["lrx_abi_version", "lrx_last_error", "lrx_scene_create", "lrx_scene_destroy",
            "lrx_scene_update_instances", "lrx_scene_get_info", "lrx_trace", "lrx_trace_host",
            "lrx_trace_counted", "lrx_scene_device_status", "lrx_trace_host_noalloc",
            "lrx_scene_set_trace_config", "lrx_scene_get_trace_config", "lrx_trace_batches",
            "lrx_scene_autotune", "lrx_trace_batches_ex", "lrx_server_create", "lrx_server_destroy",
            "lrx_server_add_scene",
            "lrx_server_submit", "lrx_server_wait", "lrx_server_get_stats", "lrx_server_reset_stats",
            "lrx_ply_load", "lrx_ply_free", "lrx_scene_key", "lrx_scene_save", "lrx_scene_load",
            "lrx_scene_create_motion", "lrx_trace_host_batches", "lrx_scene_create_autotuned"]
LRX_SERVE_BATCHED = 0
LRX_SERVE_PLAIN = 1
LRX_NOALLOC_MAX_RAYS = 131072


class LrxError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class MeshDesc(ctypes.Structure):
    _fields_ = [("vertices", ctypes.c_void_p), ("triangles", ctypes.c_void_p),
                ("vertex_count", ctypes.c_uint32), ("triangle_count", ctypes.c_uint32)]


class ObjectDesc(ctypes.Structure):
    _fields_ = [("mesh", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("transform", ctypes.c_float * 16), ("inverse", ctypes.c_float * 16)]


class BuildOpts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("leaf_max", ctypes.c_uint32),
                ("treelet_passes", ctypes.c_uint32), ("node_width", ctypes.c_uint32),
                ("node_layout", ctypes.c_uint32)]


LRX_NODES_WIDE8 = 0      # 80-byte records, up to 8 children
LRX_NODES_COMPACT4 = 1   # 64-byte records, up to 4 children (node_width 4, flat scenes)


class TraceConfig(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("block_size", ctypes.c_uint32),
                ("postpone", ctypes.c_uint32), ("variant", ctypes.c_uint32), ("modes", ctypes.c_uint32),
                ("refill", ctypes.c_uint32), ("max_visits", ctypes.c_uint32), ("deadline_us", ctypes.c_uint32)]


class MotionDesc(ctypes.Structure):
    _fields_ = [("object", ctypes.c_uint32), ("count", ctypes.c_uint32), ("times", ctypes.c_void_p),
                ("transforms", ctypes.c_void_p)]


class HostBatch(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("h_rays", ctypes.c_void_p), ("h_hits", ctypes.c_void_p),
                ("count", ctypes.c_uint32), ("mode", ctypes.c_uint32)]


class PlyMesh(ctypes.Structure):
    _fields_ = [("vertices", ctypes.POINTER(ctypes.c_float)), ("triangles", ctypes.POINTER(ctypes.c_uint32)),
                ("vertex_count", ctypes.c_uint32), ("triangle_count", ctypes.c_uint32)]


class SceneInfo(ctypes.Structure):
    _fields_ = [("triangle_count", ctypes.c_uint64), ("unique_triangle_count", ctypes.c_uint64),
                ("object_count", ctypes.c_uint32), ("instance_count", ctypes.c_uint32),
                ("blas_count", ctypes.c_uint32), ("two_level", ctypes.c_uint32),
                ("node_count", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64),
                ("max_depth", ctypes.c_uint32), ("node_bytes", ctypes.c_uint32),
                ("build_ms", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None
_lock = threading.Lock()


def load(path: str | None = None):
    """Loads liblrx.so; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RuntimeError(f"liblrx.so not found at {p}: run luxcore_gb300/build.py "
                               "(there is no CPU fallback)")
        L = ctypes.CDLL(p)
        vp, u32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64
        st = ctypes.c_int
        L.lrx_abi_version.restype = u32
        L.lrx_last_error.restype = ctypes.c_char_p
        L.lrx_scene_create.restype = st
        L.lrx_scene_create.argtypes = [vp, u32, vp, u32, vp, vp, ctypes.POINTER(vp)]
        L.lrx_scene_create_motion.restype = st
        L.lrx_scene_create_motion.argtypes = [vp, u32, vp, u32, vp, u32, vp, vp, ctypes.POINTER(vp)]
        L.lrx_scene_destroy.restype = st
        L.lrx_scene_destroy.argtypes = [vp]
        L.lrx_scene_update_instances.restype = st
        L.lrx_scene_update_instances.argtypes = [vp, vp, u32, vp]
        L.lrx_scene_get_info.restype = st
        L.lrx_scene_get_info.argtypes = [vp, ctypes.POINTER(SceneInfo)]
        L.lrx_trace.restype = st
        L.lrx_trace.argtypes = [vp, vp, vp, u32, u32, vp]
        L.lrx_trace_host.restype = st
        L.lrx_trace_host.argtypes = [vp, vp, vp, u32, u32, vp]
        L.lrx_scene_set_trace_config.restype = st
        L.lrx_scene_set_trace_config.argtypes = [vp, ctypes.POINTER(TraceConfig)]
        L.lrx_scene_get_trace_config.restype = st
        L.lrx_scene_get_trace_config.argtypes = [vp, ctypes.POINTER(TraceConfig)]
        L.lrx_server_create.restype = st
        L.lrx_server_create.argtypes = [ctypes.POINTER(ServerOpts), ctypes.POINTER(vp)]
        L.lrx_server_destroy.restype = st
        L.lrx_server_destroy.argtypes = [vp]
        L.lrx_server_add_scene.restype = st
        L.lrx_server_add_scene.argtypes = [vp, vp, u32, vp, u32, ctypes.POINTER(u32)]
        L.lrx_server_submit.restype = st
        L.lrx_server_submit.argtypes = [vp, u32, vp, vp, u32, u32, ctypes.POINTER(u64)]
        L.lrx_server_wait.restype = st
        L.lrx_server_wait.argtypes = [vp, u64, u32]
        L.lrx_server_get_stats.restype = st
        L.lrx_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
        L.lrx_server_reset_stats.restype = st
        L.lrx_server_reset_stats.argtypes = [vp]
        L.lrx_scene_autotune.restype = st
        L.lrx_scene_autotune.argtypes = [vp, vp, u32, u32, vp, ctypes.POINTER(TraceConfig)]
        L.lrx_trace_batches.restype = st
        L.lrx_trace_batches.argtypes = [vp, u32, vp]
        L.lrx_trace_host_noalloc.restype = st
        L.lrx_trace_host_noalloc.argtypes = [vp, vp, vp, u32, u32, vp]
        L.lrx_trace_counted.restype = st
        L.lrx_trace_counted.argtypes = [vp, vp, vp, u32, u32, vp, vp]
        L.lrx_scene_device_status.restype = st
        L.lrx_scene_device_status.argtypes = [vp, ctypes.POINTER(u32), vp]
        L.lrx_ply_load.restype = st
        L.lrx_ply_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(PlyMesh)]
        L.lrx_ply_free.restype = None
        L.lrx_ply_free.argtypes = [ctypes.POINTER(PlyMesh)]
        L.lrx_scene_key.restype = st
        L.lrx_scene_key.argtypes = [vp, u32, vp, u32, vp, ctypes.POINTER(u64)]
        L.lrx_scene_save.restype = st
        L.lrx_scene_save.argtypes = [vp, vp, ctypes.POINTER(ctypes.c_size_t), vp]
        L.lrx_scene_load.restype = st
        L.lrx_scene_load.argtypes = [vp, ctypes.c_size_t, vp, ctypes.POINTER(vp)]
        _lib = L
        return L


def rank_slice(count: int, rank: int, world_size: int) -> tuple:
    """Ray range [begin, end) that replica `rank` of `world_size` traces of a
    RayBuffer of `count` rays: contiguous, sizes differing by at most one,
    in rank order -- so the ranks' hit slices concatenated in rank order are
    the whole buffer's hits.  Each GPU holds a full scene replica and traces
    its slice with no exchange between GPUs, as the reference gives each
    intersection device its own tasks (src/slg/engines/pathocl/pathocl.cpp:217-247)."""
    if world_size < 1 or not 0 <= rank < world_size or count < 0:
        raise ValueError("bad rank / world size / count")
    base, extra = divmod(count, world_size)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def check(status: int):
    if status != 0:
        raise LrxError(status, load().lrx_last_error().decode(errors="replace"))


class Batch(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_void_p), ("d_rays", ctypes.c_void_p), ("d_hits", ctypes.c_void_p),
                ("count", ctypes.c_uint32), ("mode", ctypes.c_uint32)]


def batch_array(batches):
    """ctypes array of lrx_batch from (Scene, d_rays, d_hits, count, mode) tuples."""
    arr = (Batch * max(1, len(batches)))()
    for k, (s, r, h, n, m) in enumerate(batches):
        arr[k].scene = s.handle.value if isinstance(s.handle, ctypes.c_void_p) else s.handle
        arr[k].d_rays = r
        arr[k].d_hits = h
        arr[k].count = n
        arr[k].mode = m
    return arr


def host_batch_array(batches):
    """ctypes array of lrx_host_batch from (Scene, h_rays, h_hits, count, mode) tuples (host addresses)."""
    arr = (HostBatch * max(1, len(batches)))()
    for k, (s, r, h, n, m) in enumerate(batches):
        arr[k].scene = s.handle.value if isinstance(s.handle, ctypes.c_void_p) else s.handle
        arr[k].h_rays = r
        arr[k].h_hits = h
        arr[k].count = n
        arr[k].mode = m
    return arr


def trace_host_batches(batches, stream: int = 0, arr=None):
    """lrx_trace_host_batches: host batches whose copies and traces overlap;
    returns when every hit is in host memory."""
    if arr is None:
        arr = host_batch_array(batches)
    check(load().lrx_trace_host_batches(arr, len(batches), ctypes.c_void_p(stream)))


def trace_batches(batches, stream: int = 0, d_tile_counters: int = 0, d_done_flags: int = 0, arr=None):
    """lrx_trace_batches over (Scene, d_rays, d_hits, count, mode) tuples (or a
    prebuilt batch_array); with device addresses of per-batch counters and
    flags, lrx_trace_batches_ex."""
    if arr is None:
        arr = batch_array(batches)
    if d_tile_counters or d_done_flags:
        check(load().lrx_trace_batches_ex(arr, len(batches), ctypes.c_void_p(stream), ctypes.c_void_p(d_tile_counters),
                                          ctypes.c_void_p(d_done_flags)))
    else:
        check(load().lrx_trace_batches(arr, len(batches), ctypes.c_void_p(stream)))


class ServerOpts(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("policy", ctypes.c_uint32), ("budget_bytes", ctypes.c_uint64),
                ("streams", ctypes.c_uint32), ("max_requests_per_launch", ctypes.c_uint32),
                ("host_cache_bytes", ctypes.c_uint64), ("max_rays_per_launch", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("requests_done", ctypes.c_uint64), ("rays_done", ctypes.c_uint64),
                ("requests_failed", ctypes.c_uint64), ("scene_builds", ctypes.c_uint64),
                ("scene_evictions", ctypes.c_uint64), ("resident_bytes", ctypes.c_uint64),
                ("peak_resident_bytes", ctypes.c_uint64), ("launches", ctypes.c_uint64),
                ("latency_p50_us", ctypes.c_double), ("latency_p99_us", ctypes.c_double),
                ("latency_mean_us", ctypes.c_double), ("latency_max_us", ctypes.c_double),
                ("busy_seconds", ctypes.c_double), ("scene_reloads", ctypes.c_uint64),
                ("host_cache_bytes", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def _mesh_array(scene: W.SceneDesc):
    keep = []
    meshes = (MeshDesc * max(1, len(scene.meshes)))()
    for i, m in enumerate(scene.meshes):
        v = np.ascontiguousarray(m.vertices, np.float32)
        t = np.ascontiguousarray(m.triangles, np.uint32)
        keep += [v, t]
        meshes[i].vertices = v.ctypes.data
        meshes[i].triangles = t.ctypes.data
        meshes[i].vertex_count = v.shape[0]
        meshes[i].triangle_count = t.shape[0]
    return meshes, keep


class Server:
    """lrx_server: scenes kept resident under an HBM budget and ray-batch
    requests served by continuous batching (policy LRX_SERVE_BATCHED) or one
    launch per request (LRX_SERVE_PLAIN)."""

    def __init__(self, policy: int = LRX_SERVE_BATCHED, budget_bytes: int = 0, streams: int = 0,
                 max_requests_per_launch: int = 0, host_cache_bytes: int = 0, max_rays_per_launch: int = 0):
        """host_cache_bytes: blobs of evicted scenes (0 = library default,
        2**64 - 1 = no cache).  max_rays_per_launch: rays a batched launch
        takes before it stops admitting requests (0 = library default,
        2**64 - 1 = no cap)."""
        o = ServerOpts(ctypes.sizeof(ServerOpts), policy, budget_bytes, streams, max_requests_per_launch,
                       host_cache_bytes, max_rays_per_launch)
        h = ctypes.c_void_p()
        check(load().lrx_server_create(ctypes.byref(o), ctypes.byref(h)))
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            load().lrx_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_scene(self, scene: W.SceneDesc) -> int:
        if scene.has_motion:
            raise ValueError("the server's scene registry takes static scenes only (no motion systems)")
        meshes, keep = _mesh_array(scene)
        objs = _object_array(scene)
        has_inst = scene.has_instances
        sid = ctypes.c_uint32()
        check(load().lrx_server_add_scene(self.handle, meshes, len(scene.meshes), objs if has_inst else None,
                                          len(scene.objects) if has_inst else 0, ctypes.byref(sid)))
        del keep  # the server copied the geometry
        return sid.value

    def submit(self, scene_id: int, d_rays: int, d_hits: int, count: int, mode: int = LRX_TRACE_CLOSEST) -> int:
        t = ctypes.c_uint64()
        check(load().lrx_server_submit(self.handle, scene_id, ctypes.c_void_p(d_rays), ctypes.c_void_p(d_hits),
                                       count, mode, ctypes.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000) -> int:
        """LRX_OK (0) when done; raises LrxError on failure or timeout."""
        check(load().lrx_server_wait(self.handle, ticket, timeout_ms))
        return 0

    def stats(self) -> dict:
        s = ServerStats()
        check(load().lrx_server_get_stats(self.handle, ctypes.byref(s)))
        return s.as_dict()

    def reset_stats(self):
        check(load().lrx_server_reset_stats(self.handle))


def _object_array(scene: W.SceneDesc):
    objs = (ObjectDesc * max(1, len(scene.objects)))()
    for i, (mi, m) in enumerate(scene.objects):
        objs[i].mesh = mi
        if isinstance(m, W.Motion):
            objs[i].flags = LRX_OBJECT_INSTANCE  # the motion system replaces the transform
        elif m is not None:
            objs[i].flags = LRX_OBJECT_INSTANCE
            flat = np.asarray(m, np.float32).reshape(16)
            for k in range(16):
                objs[i].transform[k] = float(flat[k])
    return objs


def _motion_array(scene: W.SceneDesc, keep: list):
    """lrx_motion_desc array of the scene's Motion objects."""
    ms = [(i, m) for i, (_, m) in enumerate(scene.objects) if isinstance(m, W.Motion)]
    arr = (MotionDesc * max(1, len(ms)))()
    for k, (i, m) in enumerate(ms):
        t = np.ascontiguousarray(m.times, np.float32).reshape(-1)
        x = np.ascontiguousarray(m.transforms, np.float32).reshape(-1)
        if x.size != 16 * t.size:
            raise ValueError("motion: one 4x4 matrix per keyframe time")
        keep += [t, x]
        arr[k].object = i
        arr[k].count = t.size
        arr[k].times = t.ctypes.data
        arr[k].transforms = x.ctypes.data
    return arr, len(ms)


def ply_load(path: str) -> W.Mesh:
    """lrx_ply_load: the geometry of a PLY file as a Mesh."""
    L = load()
    pm = PlyMesh()
    check(L.lrx_ply_load(os.fsencode(path), ctypes.byref(pm)))
    try:
        v = np.ctypeslib.as_array(pm.vertices, shape=(pm.vertex_count, 3)).copy()
        t = np.ctypeslib.as_array(pm.triangles, shape=(pm.triangle_count, 3)).copy()
    finally:
        L.lrx_ply_free(ctypes.byref(pm))
    return W.Mesh(v, t)


def _mesh_descs(scene: W.SceneDesc, keep: list):
    meshes = (MeshDesc * max(1, len(scene.meshes)))()
    for i, m in enumerate(scene.meshes):
        v = np.ascontiguousarray(m.vertices, np.float32)
        t = np.ascontiguousarray(m.triangles, np.uint32)
        keep += [v, t]
        meshes[i].vertices = v.ctypes.data
        meshes[i].triangles = t.ctypes.data
        meshes[i].vertex_count = v.shape[0]
        meshes[i].triangle_count = t.shape[0]
    return meshes


def scene_key(scene: W.SceneDesc, leaf_max: int = 3, treelet_passes: int = 2, node_width: int = 8,
              node_layout: int = LRX_NODES_WIDE8) -> int:
    """lrx_scene_key: content key of a scene's inputs and build options."""
    keep = []
    meshes = _mesh_descs(scene, keep)
    objs = _object_array(scene)
    opts = BuildOpts(ctypes.sizeof(BuildOpts), leaf_max, treelet_passes, node_width, node_layout)
    k = ctypes.c_uint64()
    check(load().lrx_scene_key(meshes, len(scene.meshes), objs, len(scene.objects), ctypes.byref(opts),
                               ctypes.byref(k)))
    return k.value


class Scene:
    """A device-resident scene (lrx_scene): meshes + objects of a SceneDesc."""

    def __init__(self, scene: W.SceneDesc | None, stream: int = 0, leaf_max: int = 3, treelet_passes: int = 2,
                 node_width: int = 8, node_layout: int = LRX_NODES_WIDE8, _handle=None):
        L = load()
        if _handle is not None:  # from_blob
            self.handle = _handle
            self.desc = scene
            return
        self._keep = []
        meshes = _mesh_descs(scene, self._keep)
        objs = _object_array(scene)
        opts = BuildOpts(ctypes.sizeof(BuildOpts), leaf_max, treelet_passes, node_width, node_layout)
        h = ctypes.c_void_p()
        if scene.has_motion:
            motions, n_motion = _motion_array(scene, self._keep)
            check(L.lrx_scene_create_motion(meshes, len(scene.meshes), objs, len(scene.objects), motions, n_motion,
                                            ctypes.byref(opts), ctypes.c_void_p(stream), ctypes.byref(h)))
        else:
            check(L.lrx_scene_create(meshes, len(scene.meshes), objs, len(scene.objects), ctypes.byref(opts),
                                     ctypes.c_void_p(stream), ctypes.byref(h)))
        self._keep = None  # the library copied the geometry
        self.handle = h
        self.desc = scene

    def close(self):
        if getattr(self, "handle", None):
            load().lrx_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def save(self, stream: int = 0) -> bytes:
        """lrx_scene_save: the built scene as a blob."""
        L = load()
        n = ctypes.c_size_t(0)
        check(L.lrx_scene_save(self.handle, None, ctypes.byref(n), ctypes.c_void_p(stream)))
        buf = ctypes.create_string_buffer(n.value)
        check(L.lrx_scene_save(self.handle, buf, ctypes.byref(n), ctypes.c_void_p(stream)))
        return buf.raw[:n.value]

    @classmethod
    def autotuned(cls, scene: W.SceneDesc, d_rays: int, count: int, mode: int = LRX_TRACE_CLOSEST, stream: int = 0,
                  treelet_passes: int = 2):
        """lrx_scene_create_autotuned: the fastest of the candidate builds (node
        width and record x leaf size) on the sample rays, each at its
        autotuned launch configuration.  Returns (scene, build options, trace
        config) dicts."""
        if scene.has_motion:
            raise ValueError("autotuned builds take static scenes")
        L = load()
        keep = []
        meshes = _mesh_descs(scene, keep)
        objs = _object_array(scene)
        opts = BuildOpts(ctypes.sizeof(BuildOpts), 0, treelet_passes, 0, 0)
        chosen = BuildOpts(ctypes.sizeof(BuildOpts), 0, 0, 0, 0)
        cfg = TraceConfig()
        cfg.struct_size = ctypes.sizeof(TraceConfig)
        h = ctypes.c_void_p()
        check(L.lrx_scene_create_autotuned(meshes, len(scene.meshes), objs, len(scene.objects), ctypes.byref(opts),
                                           ctypes.c_void_p(d_rays), count, mode, ctypes.c_void_p(stream),
                                           ctypes.byref(h), ctypes.byref(chosen), ctypes.byref(cfg)))
        sc = cls(scene, _handle=h)
        return (sc, {"leaf_max": chosen.leaf_max, "treelet_passes": chosen.treelet_passes,
                     "node_width": chosen.node_width, "node_layout": chosen.node_layout},
                {"block_size": cfg.block_size, "postpone": cfg.postpone, "variant": cfg.variant, "refill": cfg.refill})

    @classmethod
    def from_blob(cls, blob: bytes, stream: int = 0, desc: W.SceneDesc | None = None) -> "Scene":
        """lrx_scene_load: a scene from a blob of lrx_scene_save, without a build."""
        h = ctypes.c_void_p()
        buf = ctypes.create_string_buffer(bytes(blob), len(blob))
        check(load().lrx_scene_load(buf, len(blob), ctypes.c_void_p(stream), ctypes.byref(h)))
        return cls(desc, _handle=h)

    def info(self) -> dict:
        inf = SceneInfo()
        check(load().lrx_scene_get_info(self.handle, ctypes.byref(inf)))
        return inf.as_dict()

    def set_trace_config(self, block_size: int = 64, postpone: int = 0, variant: int = 0, modes: int = 0,
                         refill: int = 0, max_visits: int = 0, deadline_us: int = 0):
        """modes: 1 = closest-hit launches, 2 = any-hit launches, 0 = both.
        refill: with LRX_VARIANT_PERSISTENT, idle lanes that trigger a warp's
        next ray claim (0 = the library default).  max_visits / deadline_us:
        the failure bounds (0 = the scene's own visit bound / the default
        launch deadline)."""
        c = TraceConfig(ctypes.sizeof(TraceConfig), block_size, postpone, variant, modes, refill, max_visits,
                        deadline_us)
        check(load().lrx_scene_set_trace_config(self.handle, ctypes.byref(c)))

    def trace_config(self, mode: int = LRX_TRACE_CLOSEST, bounds: bool = False) -> dict:
        """The launch configuration of `mode`; with bounds, also its failure
        bounds (max_visits, deadline_us)."""
        c = TraceConfig()
        c.struct_size = ctypes.sizeof(TraceConfig)
        c.modes = 2 if mode == LRX_TRACE_ANY else 1
        check(load().lrx_scene_get_trace_config(self.handle, ctypes.byref(c)))
        out = {"block_size": c.block_size, "postpone": c.postpone, "variant": c.variant, "refill": c.refill}
        if bounds:
            out.update(max_visits=c.max_visits, deadline_us=c.deadline_us)
        return out

    def autotune(self, d_rays: int, count: int, mode: int = LRX_TRACE_CLOSEST, stream: int = 0) -> dict:
        """Picks this scene's fastest launch configuration for `mode` on a
        device-resident sample of rays."""
        c = TraceConfig()
        c.struct_size = ctypes.sizeof(TraceConfig)
        check(load().lrx_scene_autotune(self.handle, ctypes.c_void_p(d_rays), count, mode,
                                        ctypes.c_void_p(stream), ctypes.byref(c)))
        return {"block_size": c.block_size, "postpone": c.postpone, "variant": c.variant, "refill": c.refill}

    def update_instances(self, scene: W.SceneDesc, stream: int = 0):
        objs = _object_array(scene)
        check(load().lrx_scene_update_instances(self.handle, objs, len(scene.objects), ctypes.c_void_p(stream)))
        self.desc = scene

    def trace(self, d_rays: int, d_hits: int, count: int, mode: int = LRX_TRACE_CLOSEST, stream: int = 0):
        """Device buffers (raw addresses); asynchronous on `stream`."""
        check(load().lrx_trace(self.handle, ctypes.c_void_p(d_rays), ctypes.c_void_p(d_hits), count, mode,
                               ctypes.c_void_p(stream)))

    def trace_counted(self, d_rays: int, d_hits: int, count: int, mode: int, d_counters: int, stream: int = 0):
        check(load().lrx_trace_counted(self.handle, ctypes.c_void_p(d_rays), ctypes.c_void_p(d_hits), count, mode,
                                       ctypes.c_void_p(d_counters), ctypes.c_void_p(stream)))

    def trace_host(self, rays: np.ndarray, hits: np.ndarray | None = None, mode: int = LRX_TRACE_CLOSEST,
                   stream: int = 0) -> np.ndarray:
        """Host rays in, host hits out (copies inside the call)."""
        rays = np.ascontiguousarray(rays, W.RAY_DTYPE)
        if hits is None:
            hits = np.zeros(rays.shape[0], W.HIT_DTYPE)
        check(load().lrx_trace_host(self.handle, rays.ctypes.data, hits.ctypes.data, rays.shape[0], mode,
                                    ctypes.c_void_p(stream)))
        return hits

    def trace_host_ptr(self, h_rays: int, h_hits: int, count: int, mode: int = LRX_TRACE_CLOSEST,
                       stream: int = 0):
        """lrx_trace_host on raw host addresses (e.g. pinned buffers)."""
        check(load().lrx_trace_host(self.handle, ctypes.c_void_p(h_rays), ctypes.c_void_p(h_hits), count, mode,
                                    ctypes.c_void_p(stream)))

    def device_status(self, stream: int = 0) -> int:
        v = ctypes.c_uint32()
        rc = load().lrx_scene_device_status(self.handle, ctypes.byref(v), ctypes.c_void_p(stream))
        if rc not in (0, 5):
            check(rc)
        return v.value
