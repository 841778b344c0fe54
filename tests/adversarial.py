"""Adversarial ray sets for parity tests: axis-parallel and zero / negative
zero direction components, NaN fields, empty and inverted [mint, maxt]
intervals, masked rays, and rays that start on or aim exactly at triangle
vertices and edge midpoints (ties between neighbouring triangles)."""
import numpy as np

from luxcore_gb300 import workloads as W


def adversarial_rays(mesh: W.Mesh, seed: int, n_each: int = 64) -> np.ndarray:
    rng = np.random.default_rng(seed)
    v = mesh.vertices.astype(np.float32)
    t = mesh.triangles
    lo, hi = v.min(0), v.max(0)
    out = []

    def rnd_o(n):
        return (lo + (hi - lo) * rng.random((n, 3))).astype(np.float32)

    # axis-parallel directions, both signs, and signed zeros
    for ax in range(3):
        for sgn in (1.0, -1.0):
            d = np.zeros((n_each, 3), np.float32)
            d[:, ax] = sgn
            out.append(W.make_rays(rnd_o(n_each), d, 1e-4, 1e30))
    d = rng.normal(size=(n_each, 3)).astype(np.float32)
    d[:, 1] = -0.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[:, 1] = -0.0
    out.append(W.make_rays(rnd_o(n_each), d, 1e-4, 1e30))
    d = rng.normal(size=(n_each, 3)).astype(np.float32)
    d[:, 0] = 0.0
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out.append(W.make_rays(rnd_o(n_each), d, 1e-4, 1e30))

    # aim exactly at vertices and edge midpoints from outside (ties)
    tri = t[rng.integers(0, t.shape[0], n_each)]
    targets = np.concatenate([v[tri[:, 0]], 0.5 * (v[tri[:, 0]] + v[tri[:, 1]]),
                              (v[tri[:, 0]] + v[tri[:, 1]] + v[tri[:, 2]]) / 3.0]).astype(np.float32)
    off = rng.normal(size=targets.shape).astype(np.float32)
    off /= np.linalg.norm(off, axis=1, keepdims=True)
    o = (targets + 0.5 * off).astype(np.float32)
    d = (-off).astype(np.float32)
    out.append(W.make_rays(o, d, 1e-4, 1e30))
    # start on vertices / edges
    o = targets.copy()
    d = rng.normal(size=targets.shape).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out.append(W.make_rays(o, d, 0.0, 1e30))
    out.append(W.make_rays(o, d, 1e-4, 1e30))

    # NaN fields, inverted / empty intervals, negative bounds
    base = W.make_rays(rnd_o(n_each), W.uniform_sphere(W.Rng(seed, 99), n_each), 1e-4, 1e30)
    for field, val in (("o", np.nan), ("d", np.nan), ("maxt", np.nan), ("mint", np.nan)):
        r = base.copy()
        if field in ("o", "d"):
            r[field][:, rng.integers(0, 3)] = val
        else:
            r[field] = val
        out.append(r)
    r = base.copy(); r["mint"] = 1.0; r["maxt"] = 0.5; out.append(r)
    r = base.copy(); r["mint"] = 0.25; r["maxt"] = 0.25; out.append(r)
    r = base.copy(); r["mint"] = -1e30; r["maxt"] = 1e30; out.append(r)
    r = base.copy(); r["maxt"] = 1e-3; out.append(r)
    r = base.copy(); r["maxt"] = -1.0; out.append(r)
    r = base.copy(); r["maxt"] = np.inf; out.append(r)
    # masked rays (must not be written)
    r = base.copy(); r["flags"] = W.RAY_FLAGS_MASKED; out.append(r)
    return np.concatenate(out)
