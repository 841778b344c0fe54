"""A PATHOCL-style wavefront caller of the engine, on device buffers.

The reference's PathOCL render threads keep `taskCount` paths in flight
and, every iteration, trace one RayBuffer holding one ray per task --
path rays and shadow (direct light) rays mixed, tasks with nothing to
trace marked RAY_FLAGS_MASKED -- then run AdvancePaths, which reads the
hits, advances each task's state machine and writes the next rays into the
same buffer (src/slg/engines/pathoclbase/pathoclopenclthread.cpp:126-200,
the trace at :185 through HardwareIntersectionKernel::EnqueueTraceRayBuffer).

This module reproduces that calling pattern: the buffers are allocated once
and traced in place with lrx_trace (the EnqueueTraceRayBuffer replacement),
and a small AdvancePaths written with torch element-wise ops on the device
stands in for the reference's shading kernels (which are out of scope):
Lambertian surfaces of one albedo, one point light, a pinhole camera, a
fixed depth limit, and finished paths restarted as new camera samples so
the buffer stays full.  Plain and instanced objects are shaded (an
instance's normal is its mesh's, under the inverse transpose of the
instance transform); motion-blurred objects are not.

Task states:
  NEXT_VERTEX  the task's ray is a path ray (camera or bounce); after the
               trace a miss adds the background and restarts the task, a
               hit stores the vertex and moves to DIRECT_LIGHT;
  DIRECT_LIGHT the task's ray is a shadow ray to the light (closest hit
               with maxt just short of the light, as PATHOCL traces them);
               a miss adds the light's contribution; then the path either
               bounces (cosine-weighted, back to NEXT_VERTEX) or, past the
               depth limit, restarts.  A vertex facing away from the light
               has no shadow ray: its ray is masked for that iteration.
"""
from __future__ import annotations

import math

import numpy as np

from . import lrx
from . import workloads as W

NEXT_VERTEX, DIRECT_LIGHT = 0, 1
RAY_WORDS, HIT_WORDS = 12, 5


class WavefrontPaths:
    """taskCount = width * height tasks, one per pixel, traced in place."""

    def __init__(self, scene: lrx.Scene, desc: W.SceneDesc, width: int, height: int, max_depth: int = 4,
                 eye=(0.5, -0.5, 0.6), look=(0.5, 0.5, 0.0), up=(0.0, 0.0, 1.0), fov_deg: float = 60.0,
                 light=(0.3, 0.7, 0.9), light_power: float = 1.0, albedo: float = 0.6, background: float = 0.2,
                 seed: int = 1, device: str = "cuda", stream=None):
        import torch
        if desc.has_motion:
            raise ValueError("the wavefront stand-in does not shade motion-blurred objects")
        self.torch = torch
        self.scene, self.n = scene, width * height
        self.width, self.height, self.max_depth = width, height, max_depth
        self.device = device
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        f32 = dict(dtype=torch.float32, device=device)
        # geometry for the normals: each mesh once; per object (in meshIndex
        # order) its mesh's first triangle and the matrix that takes the mesh's
        # normals to world space (identity for plain objects, the inverse
        # transpose of the instance transform's 3x3 part for instances)
        verts, tris, tri_base, vbase, tbase = [], [], [], 0, 0
        for m in desc.meshes:
            verts.append(torch.from_numpy(np.ascontiguousarray(m.vertices, np.float32)))
            tris.append(torch.from_numpy(np.ascontiguousarray(m.triangles, np.int64)) + vbase)
            tri_base.append(tbase)
            vbase += m.vertices.shape[0]
            tbase += m.triangles.shape[0]
        self.verts = torch.cat(verts).to(device)
        self.tris = torch.cat(tris).to(device)
        nmat = np.tile(np.eye(3, dtype=np.float32), (len(desc.objects), 1, 1))
        for k, (_mi, m) in enumerate(desc.objects):
            if m is not None:
                nmat[k] = np.linalg.inv(np.asarray(m, np.float64).reshape(4, 4)[:3, :3]).T.astype(np.float32)
        self.obj_tri_base = torch.tensor([tri_base[mi] for mi, _m in desc.objects], dtype=torch.int64, device=device)
        self.obj_nmat = torch.from_numpy(nmat).to(device)
        # camera frame
        e = np.array(eye, np.float64)
        fwd = np.array(look, np.float64) - e
        fwd /= np.linalg.norm(fwd)
        right = np.cross(fwd, np.array(up, np.float64))
        right /= np.linalg.norm(right)
        upv = np.cross(right, fwd)
        th = math.tan(math.radians(fov_deg) * 0.5)
        self.cam = {k: torch.tensor(v, **f32) for k, v in
                    (("eye", e), ("fwd", fwd), ("right", right * th * width / height), ("up", upv * th))}
        self.light = torch.tensor(light, **f32)
        self.light_power, self.albedo, self.background = light_power, albedo, background
        # per-task state and the in-place ray / hit buffers (RayBuffer / RayHitBuffer)
        n = self.n
        self.rays = torch.zeros((n, RAY_WORDS), **f32)
        self.hits = torch.zeros((n, HIT_WORDS), **f32)
        self.state = torch.zeros(n, dtype=torch.int32, device=device)
        self.depth = torch.zeros(n, dtype=torch.int32, device=device)
        self.throughput = torch.ones(n, **f32)
        self.vertex = torch.zeros((n, 3), **f32)
        self.normal = torch.zeros((n, 3), **f32)
        self.film = torch.zeros(n, **f32)
        self.samples = torch.zeros(n, **f32)
        self.gen = torch.Generator(device=device)
        self.gen.manual_seed(seed)
        self.pixel = torch.arange(n, device=device)
        self.traced_dev = torch.zeros((), dtype=torch.int64, device=device)
        self.ex = torch.tensor([1.0, 0.0, 0.0], **f32)
        self.ey = torch.tensor([0.0, 1.0, 0.0], **f32)
        self._camera(torch.ones(n, dtype=torch.bool, device=device))

    # -- ray buffer helpers (dense: every update is a select, no host sync) ----
    def _select_rays(self, sel, o, d, mint, maxt, masked=None):
        """Rows of the ray buffer where `sel` holds become (o, d, mint, maxt)."""
        torch = self.torch
        r = self.rays
        new = torch.empty_like(r)
        new[:, 0:3] = o
        new[:, 3:6] = d
        new[:, 6] = mint
        new[:, 7] = maxt
        new[:, 8:] = 0.0
        flags = torch.zeros(self.n, dtype=torch.int32, device=self.device)
        if masked is not None:
            flags = torch.where(masked, torch.full_like(flags, W.RAY_FLAGS_MASKED), flags)
        new.view(torch.int32)[:, 9] = flags
        self.rays.copy_(torch.where(sel[:, None], new, r))

    def _camera(self, sel):
        torch = self.torch
        u = torch.rand((self.n, 2), generator=self.gen, device=self.device)
        px = ((self.pixel % self.width).float() + u[:, 0]) / self.width * 2.0 - 1.0
        py = 1.0 - ((self.pixel // self.width).float() + u[:, 1]) / self.height * 2.0
        d = self.cam["fwd"] + px[:, None] * self.cam["right"] + py[:, None] * self.cam["up"]
        d = d / d.norm(dim=1, keepdim=True)
        self._select_rays(sel, self.cam["eye"].expand_as(d), d, 1e-4, 1e30)
        self.state = torch.where(sel, torch.full_like(self.state, NEXT_VERTEX), self.state)
        self.depth = torch.where(sel, torch.zeros_like(self.depth), self.depth)
        self.throughput = torch.where(sel, torch.ones_like(self.throughput), self.throughput)

    # -- one iteration: trace the buffer, then advance every task -------------
    def trace(self):
        """EnqueueTraceRayBuffer: closest hit over the whole buffer, in place."""
        torch = self.torch
        self.traced_dev += ((self.rays.view(torch.int32)[:, 9] & W.RAY_FLAGS_MASKED) == 0).sum()
        self.scene.trace(self.rays.data_ptr(), self.hits.data_ptr(), self.n, lrx.LRX_TRACE_CLOSEST,
                         self.stream.cuda_stream)

    def advance(self):
        """AdvancePaths stand-in (element-wise torch on the device)."""
        torch = self.torch
        zero = torch.zeros_like(self.film)
        hits_i = self.hits.view(torch.int32)
        mesh = hits_i[:, 3]
        hit = mesh != -1  # NULL_INDEX
        masked = (self.rays.view(torch.int32)[:, 9] & W.RAY_FLAGS_MASKED) != 0
        nv = (self.state == NEXT_VERTEX) & ~masked
        dl = self.state == DIRECT_LIGHT
        # NEXT_VERTEX miss: background, restart
        miss_nv = nv & ~hit
        self.film += torch.where(miss_nv, self.throughput * self.background, zero)
        self.samples += miss_nv.float()
        # NEXT_VERTEX hit: store the vertex (geometric normal facing the ray)
        hv = nv & hit
        t = self.hits[:, 0]
        o = self.rays[:, 0:3] + self.rays[:, 3:6] * torch.where(hv, t, zero)[:, None]
        obj = mesh.clamp(min=0).long()
        tid = (self.obj_tri_base[obj] + hits_i[:, 4].long()).clamp(0, self.tris.shape[0] - 1)
        tri = self.tris[tid]
        p0, p1, p2 = self.verts[tri[:, 0]], self.verts[tri[:, 1]], self.verts[tri[:, 2]]
        nrm = torch.einsum("nij,nj->ni", self.obj_nmat[obj], torch.linalg.cross(p1 - p0, p2 - p0))
        nrm = nrm / nrm.norm(dim=1, keepdim=True).clamp(min=1e-30)
        nrm = torch.where(((nrm * self.rays[:, 3:6]).sum(1) > 0)[:, None], -nrm, nrm)
        self.vertex = torch.where(hv[:, None], o, self.vertex)
        self.normal = torch.where(hv[:, None], nrm, self.normal)
        to_l = self.light - self.vertex
        dist = to_l.norm(dim=1).clamp(min=1e-30)
        ldir = to_l / dist[:, None]
        cos_l = (ldir * self.normal).sum(1)
        # DIRECT_LIGHT done: add the light when the shadow ray reached it
        lit = dl & ~masked & ~hit
        contrib = self.throughput * self.albedo / math.pi * self.light_power * cos_l.clamp(min=0) / (dist * dist)
        self.film += torch.where(lit, contrib, zero)
        # DIRECT_LIGHT -> cosine-weighted bounce, or restart past the depth limit
        self.depth = self.depth + dl.int()
        cont = dl & (self.depth < self.max_depth)
        done = dl & ~cont
        self.samples += done.float()
        u = torch.rand((self.n, 2), generator=self.gen, device=self.device)
        r, phi = u[:, 0].sqrt(), 2.0 * math.pi * u[:, 1]
        lz = (1.0 - u[:, 0]).clamp(min=0).sqrt()
        n_b = self.normal
        a = torch.where(n_b[:, :1].abs() > 0.9, self.ey, self.ex)
        tt = torch.linalg.cross(n_b, a)
        tt = tt / tt.norm(dim=1, keepdim=True).clamp(min=1e-30)
        bb = torch.linalg.cross(n_b, tt)
        d = tt * (r * phi.cos())[:, None] + bb * (r * phi.sin())[:, None] + n_b * lz[:, None]
        d = d / d.norm(dim=1, keepdim=True).clamp(min=1e-30)
        self._select_rays(cont, self.vertex, d, 1e-4, 1e30)
        self.throughput = torch.where(cont, self.throughput * self.albedo, self.throughput)
        self.state = torch.where(cont, torch.full_like(self.state, NEXT_VERTEX), self.state)
        self._camera(done | miss_nv)
        # NEXT_VERTEX hit -> shadow ray; masked when the light is behind the surface
        self._select_rays(hv, self.vertex, ldir, 1e-4, dist * (1.0 - 1e-4), masked=cos_l <= 0)
        self.state = torch.where(hv, torch.full_like(self.state, DIRECT_LIGHT), self.state)

    def iterate(self, count: int = 1):
        for _ in range(count):
            self.trace()
            self.advance()

    def harvest(self, n_bounce: int, n_shadow: int, max_iterations: int = 64):
        """Runs iterations until it has seen n_bounce bounce rays (path rays
        past the camera vertex) and n_shadow shadow rays (unmasked direct-
        light rays), and returns the first of each as two (n, 12) float32
        ray tensors on the device -- the rays a PATHOCL wavefront hands the
        engine, for workloads that replay them.  Fewer come back if the
        scene yields fewer within max_iterations (a scene the camera barely
        sees)."""
        torch = self.torch
        bounce, shadow, nb, ns = [], [], 0, 0
        for _ in range(max_iterations):
            if nb >= n_bounce and ns >= n_shadow:
                break
            flags = self.rays.view(torch.int32)[:, 9]
            live = (flags & W.RAY_FLAGS_MASKED) == 0
            if nb < n_bounce:
                b = self.rays[live & (self.state == NEXT_VERTEX) & (self.depth > 0)]
                bounce.append(b.clone())
                nb += b.shape[0]
            if ns < n_shadow:
                sh = self.rays[live & (self.state == DIRECT_LIGHT)]
                shadow.append(sh.clone())
                ns += sh.shape[0]
            self.iterate()
        cat = lambda parts, n: (torch.cat(parts)[:n] if parts else torch.zeros((0, RAY_WORDS), device=self.device))
        return cat(bounce, n_bounce), cat(shadow, n_shadow)

    @property
    def traced(self) -> int:
        """Unmasked rays handed to the engine so far (reads the device)."""
        return int(self.traced_dev)

    def image(self) -> np.ndarray:
        """Mean radiance per pixel over the finished samples."""
        f = (self.film / self.samples.clamp(min=1)).cpu().numpy()
        return f.reshape(self.height, self.width)
