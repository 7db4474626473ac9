"""Seeded synthetic workloads of the N-BVH ray-query path.

The reference benchmarks on glTF scenes whose mesh binaries and weights are not shipped; these
generators stand in for them with the shapes and sizes of the workload definitions:

* fbm_sphere: tetrahedron subdivided k times (4 * 4^k triangles: k = 7 -> 65,536, k = 8 ->
  262,144), vertices on the unit sphere displaced radially by 4-octave value-noise fBm (amplitude
  0.1), scaled into the unit cube.
* terrain: value-noise height field of nx * ny quads (1024 x 512 -> 1,048,576 triangles).
* soup: random triangles with edges of 1e-3..1e-2 in the unit cube (4,194,304 triangles).
* uniform_rays: origins uniform in the scene box scaled by 1.5 around its centre, directions
  uniform on the sphere (the training-ray distribution of the reference, used for query batches).
* camera / bounce rays: pinhole primary rays and one cosine-sampled bounce per hit.

Only +, -, *, /, sqrt and floor are used on the mesh coordinates (no libm transcendental), so a
seed gives the same FP32 mesh on x86-64 and aarch64.
"""

import numpy as np

FLT_MAX = np.float32(3.4028234663852886e38)


def _hash3(ix, iy, iz, seed):
    """32-bit integer hash of lattice coordinates (uint32 arithmetic, wraps)."""
    with np.errstate(over="ignore"):
        h = (ix.astype(np.uint32) * np.uint32(0x8DA6B343)) ^ (iy.astype(np.uint32) * np.uint32(0xD8163841)) ^ (
            iz.astype(np.uint32) * np.uint32(0xCB1AB31F)) ^ np.uint32(seed * 0x9E3779B1 & 0xFFFFFFFF)
        h ^= h >> np.uint32(15)
        h *= np.uint32(0x2C1B3C6D)
        h ^= h >> np.uint32(12)
        h *= np.uint32(0x297A2D39)
        h ^= h >> np.uint32(15)
    return h


def value_noise3(p, seed):
    """Trilinear value noise in [-1, 1] with smoothstep weights, p: (n, 3) float64."""
    fl = np.floor(p)
    f = p - fl
    i = fl.astype(np.int64)
    w = f * f * (3.0 - 2.0 * f)
    out = np.zeros(len(p))
    for c in range(8):
        dx, dy, dz = c & 1, (c >> 1) & 1, (c >> 2) & 1
        h = _hash3(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz, seed)
        val = h.astype(np.float64) * (2.0 / 4294967295.0) - 1.0
        wx = w[:, 0] if dx else 1.0 - w[:, 0]
        wy = w[:, 1] if dy else 1.0 - w[:, 1]
        wz = w[:, 2] if dz else 1.0 - w[:, 2]
        out += wx * wy * wz * val
    return out


def fbm(p, seed, octaves=4, base_freq=2.0):
    total = np.zeros(len(p))
    amp, freq, norm = 1.0, base_freq, 0.0
    for o in range(octaves):
        total += amp * value_noise3(p * freq, seed + 101 * o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return total / norm


def _to_unit_cube(v):
    lo = v.min(axis=0)
    hi = v.max(axis=0)
    return ((v - lo) / (hi - lo).max()).astype(np.float32)


def subdivided_tetrahedron(k):
    """Unit-sphere tetrahedron subdivided k times: 4 * 4^k triangles (float64 vertices)."""
    v = np.array([[1, 1, 1], [-1, -1, 1], [-1, 1, -1], [1, -1, -1]], np.float64) / np.sqrt(3.0)
    f = np.array([[0, 1, 2], [0, 3, 1], [0, 2, 3], [1, 3, 2]], np.int64)
    for _ in range(k):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.sqrt((mid * mid).sum(axis=1))[:, None]
        m = inv.reshape(3, -1).T + len(v)
        v = np.concatenate([v, mid])
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1), np.stack([ca, bc, c], 1),
                            np.stack([ab, bc, ca], 1)])
    return v, f


def fbm_sphere(subdiv=7, seed=0, amplitude=0.1, octaves=4):
    """Returns (vertices float32 [n,3], indices uint32 [m,3]) in the unit cube."""
    v, f = subdivided_tetrahedron(subdiv)
    r = 1.0 + amplitude * fbm(v, seed, octaves)
    return _to_unit_cube(v * r[:, None]), f.astype(np.uint32)


def terrain(nx=1024, ny=512, seed=0, amplitude=0.25):
    xs = np.arange(nx + 1, dtype=np.float64) / nx
    zs = np.arange(ny + 1, dtype=np.float64) / ny * (ny / nx)
    X, Z = np.meshgrid(xs, zs)
    p = np.stack([X.ravel() * 4.0, np.zeros(X.size), Z.ravel() * 4.0], 1)
    h = amplitude * fbm(p, seed, 6, 1.0)
    v = np.stack([X.ravel(), h, Z.ravel()], 1)
    idx = np.arange((nx + 1) * (ny + 1)).reshape(ny + 1, nx + 1)
    a, b, c, d = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel(), idx[1:, :-1].ravel(), idx[1:, 1:].ravel()
    f = np.concatenate([np.stack([a, c, b], 1), np.stack([b, c, d], 1)])
    return _to_unit_cube(v), f.astype(np.uint32)


def soup(n=4194304, seed=0, min_edge=1e-3, max_edge=1e-2):
    rng = np.random.default_rng(seed)
    c = rng.random((n, 3))
    e1 = rng.standard_normal((n, 3))
    e1 /= np.sqrt((e1 * e1).sum(1))[:, None]
    e2 = rng.standard_normal((n, 3))
    e2 /= np.sqrt((e2 * e2).sum(1))[:, None]
    l1 = rng.uniform(min_edge, max_edge, n)[:, None]
    l2 = rng.uniform(min_edge, max_edge, n)[:, None]
    v = np.stack([c, c + e1 * l1, c + e2 * l2], 1).reshape(-1, 3)
    f = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    return _to_unit_cube(v), f


def palette_albedo(n_triangles, seed=0, n_colors=8):
    """Per-triangle albedo from a seeded palette, constant over runs of 64 triangles."""
    rng = np.random.default_rng(seed + 7)
    pal = rng.uniform(0.1, 0.9, (n_colors, 3)).astype(np.float32)
    sel = (np.arange(n_triangles) // 64) % n_colors
    return pal[sel]


def make_rays(o, d, tmin=1e-4, tmax=FLT_MAX):
    """(n, 8) float32 ray records {o, tmin, d, tmax}."""
    n = len(o)
    r = np.empty((n, 8), np.float32)
    r[:, 0:3] = o
    r[:, 3] = tmin
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r


def uniform_rays(n, bbox_min, bbox_max, seed=0, scaling=1.5):
    rng = np.random.default_rng(seed)
    lo = np.asarray(bbox_min, np.float64)
    hi = np.asarray(bbox_max, np.float64)
    u = rng.random((n, 3)) * scaling - (scaling - 1.0) * 0.5
    o = lo + u * (hi - lo)
    d = rng.standard_normal((n, 3))
    d /= np.sqrt((d * d).sum(1))[:, None]
    return make_rays(o.astype(np.float32), d.astype(np.float32))


def orbit_camera(bbox_min, bbox_max, seed=0, distance=1.6):
    """Seeded orbit position looking at the box centre: (origin, target, up)."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(bbox_min, np.float64)
    hi = np.asarray(bbox_max, np.float64)
    c = 0.5 * (lo + hi)
    r = distance * float((hi - lo).max())
    d = rng.standard_normal(3)
    d[1] = abs(d[1]) * 0.5
    d /= np.linalg.norm(d)
    return (c + r * d).astype(np.float32), c.astype(np.float32), np.array([0.0, 1.0, 0.0], np.float32)


def camera_rays(width, height, origin, target, up, yfov_degrees=45.0, seed=0):
    """Pinhole rays through jittered pixel positions (row-major, y down)."""
    rng = np.random.default_rng(seed + 11)
    o = np.asarray(origin, np.float64)
    fwd = np.asarray(target, np.float64) - o
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, np.asarray(up, np.float64))
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    h = 2.0 * np.tan(np.radians(0.5 * yfov_degrees))
    w = h * width / height
    px, py = np.meshgrid(np.arange(width), np.arange(height))
    x = (px.ravel() + rng.random(width * height)) / width - 0.5
    y = 0.5 - (py.ravel() + rng.random(width * height)) / height
    d = fwd[None, :] + x[:, None] * w * right[None, :] + y[:, None] * h * upv[None, :]
    d /= np.sqrt((d * d).sum(1))[:, None]
    return make_rays(np.broadcast_to(o, d.shape).astype(np.float32), d.astype(np.float32))


def bounce_rays(rays, hits, vertices, indices, seed=0):
    """One cosine-sampled bounce per valid hit of (rays [n,8], hits {t,u,v,prim}) about the
    geometric normal facing the incoming ray; returns the bounce rays (float32 [m, 8])."""
    rng = np.random.default_rng(seed + 23)
    hits = np.asarray(hits)
    prim = hits[:, 3].view(np.uint32)
    t = hits[:, 0].view(np.float32)
    ok = prim != 0xFFFFFFFF
    r = rays[ok].astype(np.float64)
    p = r[:, 0:3] + t[ok, None].astype(np.float64) * r[:, 4:7]
    tri = indices[prim[ok]]
    v0, v1, v2 = (vertices[tri[:, k]].astype(np.float64) for k in range(3))
    n = np.cross(v1 - v0, v2 - v0)
    n /= np.maximum(np.sqrt((n * n).sum(1)), 1e-30)[:, None]
    flip = (n * r[:, 4:7]).sum(1) > 0
    n[flip] *= -1
    a = np.where(np.abs(n[:, 0:1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    tng = np.cross(a, n)
    tng /= np.sqrt((tng * tng).sum(1))[:, None]
    btg = np.cross(n, tng)
    u1 = rng.random(len(n))
    u2 = rng.random(len(n))
    rad = np.sqrt(u1)
    phi = 2.0 * np.pi * u2
    d = (rad * np.cos(phi))[:, None] * tng + (rad * np.sin(phi))[:, None] * btg + np.sqrt(1.0 - u1)[:, None] * n
    d /= np.sqrt((d * d).sum(1))[:, None]
    return make_rays(p.astype(np.float32), d.astype(np.float32))


def scene_bbox(vertices):
    return vertices.min(axis=0), vertices.max(axis=0)
