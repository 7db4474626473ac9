"""Independent pure-Python restatement of reference functions on the N-BVH ray-query path, used
only to generate the golden vectors in golden.npz (make_golden.py) that pin the C oracle.

Every FP32 operation is a numpy float32 scalar operation (IEEE single, rounded per operation, no
contraction); fused multiply-adds are evaluated in double and rounded to float32. Citations are
file:line in the reference project.
"""

import math

import numpy as np

F = np.float32
FLT_MAX = F(3.4028234663852886e38)
M32 = 0xFFFFFFFF


# ---- include/cuda/utils/lcg_rng.cuh:12-72 ----
def murmur_mix(h, k):
    k = (k * 0xCC9E2D51) & M32
    k = ((k << 15) | (k >> 17)) & M32
    k = (k * 0x1B873593) & M32
    h ^= k
    h = ((((h << 13) | (h >> 19)) & M32) * 5 + 0xE6546B64) & M32
    return h


def murmur_finalize(h):
    h ^= h >> 16
    h = (h * 0x85EBCA6B) & M32
    h ^= h >> 13
    h = (h * 0xC2B2AE35) & M32
    h ^= h >> 16
    return h


def lcg_seed(index, frame, linear):
    s = murmur_mix(0, linear)
    s = murmur_mix(s, (512 * frame + index) & M32)
    return murmur_finalize(s)


class Rng:
    def __init__(self, state):
        self.state = state

    def f(self):
        self.state = (self.state * 1664525 + 1013904223) & M32
        return F(F(self.state) * F(2.0 ** -32))


def fma(a, b, c):
    return F(float(a) * float(b) + float(c))


def sincos_turns(u):
    y = F(F(u) * F(8.0))
    o = F(np.floor(y))
    f = F(y - o)
    oct_ = int(o) & 7
    g = F(F(1.0) - f) if (oct_ & 1) else f
    x = F(g * F(0.785398163397448310))
    x2 = F(x * x)
    ps = fma(x2, F(-2.50521084e-08), F(2.75573192e-06))
    ps = fma(x2, ps, F(-1.98412698e-04))
    ps = fma(x2, ps, F(8.33333333e-03))
    ps = fma(x2, ps, F(-1.66666667e-01))
    ps = fma(x2, ps, F(1.0))
    sn = F(x * ps)
    pc = fma(x2, F(2.08767570e-09), F(-2.75573192e-07))
    pc = fma(x2, pc, F(2.48015873e-05))
    pc = fma(x2, pc, F(-1.38888889e-03))
    pc = fma(x2, pc, F(4.16666667e-02))
    pc = fma(x2, pc, F(-0.5))
    cs = fma(x2, pc, F(1.0))
    table = {0: (sn, cs), 1: (cs, sn), 2: (cs, -sn), 3: (sn, -cs), 4: (-sn, -cs), 5: (-cs, -sn), 6: (-cs, sn),
             7: (-sn, cs)}
    s, c = table[oct_]
    return F(s), F(c)


# ---- glm-order vector helpers ----
def sub(a, b):
    return [F(a[i] - b[i]) for i in range(3)]


def add(a, b):
    return [F(a[i] + b[i]) for i in range(3)]


def div(a, b):
    with np.errstate(all="ignore"):
        return [F(a[i] / b[i]) for i in range(3)]


def scale(a, s):
    return [F(a[i] * s) for i in range(3)]


def dot(a, b):
    return F(F(F(a[0] * b[0]) + F(a[1] * b[1])) + F(a[2] * b[2]))


def cross(a, b):
    return [F(F(a[1] * b[2]) - F(b[1] * a[2])), F(F(a[2] * b[0]) - F(b[2] * a[0])), F(F(a[0] * b[1]) - F(b[0] * a[1]))]


def gmin(a, b):
    return b if b < a else a


def gmax(a, b):
    return b if a < b else a


def cmax(v):
    return gmax(gmax(v[0], v[1]), v[2])


def cmin(v):
    return gmin(gmin(v[0], v[1]), v[2])


def node_box(nodes, i):
    f = nodes[i].view(np.float32)
    return [F(f[0]), F(f[1]), F(f[2])], int(nodes[i][3]), [F(f[4]), F(f[5]), F(f[6])], int(nodes[i][7])


# ---- include/base/accel/bvh.h:121-133, include/cuda/accel/bvh.cuh:98-136, bvh2.cuh:12-88 ----
def box_entry(bmin, bmax, o, d, rmint, rmaxt):
    t0 = div(sub(bmin, o), d)
    t1 = div(sub(bmax, o), d)
    mint = gmax(rmint, cmax([gmin(t0[i], t1[i]) for i in range(3)]))
    maxt = gmin(rmaxt, cmin([gmax(t0[i], t1[i]) for i in range(3)]))
    return mint if mint <= maxt else FLT_MAX


def tri_intersect(verts, idx, prim, o, d, rmint, rmaxt):
    ix = idx[prim]
    v0 = [F(x) for x in verts[ix[0]]]
    v1 = [F(x) for x in verts[ix[1]]]
    v2 = [F(x) for x in verts[ix[2]]]
    e1, e2 = sub(v1, v0), sub(v2, v0)
    pvec = cross(d, e2)
    det = dot(e1, pvec)
    if F(-1e-8) < det < F(1e-8):
        return None
    inv = F(F(1.0) / det)
    tvec = sub(o, v0)
    u = F(dot(tvec, pvec) * inv)
    if u < 0 or u > 1:
        return None
    qvec = cross(tvec, e1)
    v = F(dot(d, qvec) * inv)
    if v < 0 or F(u + v) > 1:
        return None
    t = F(dot(e2, qvec) * inv)
    if t < rmint or t >= rmaxt:
        return None
    return t, u, v


def classic_intersect(nodes, prims, verts, idx, ray, any_hit=False):
    o = [F(x) for x in ray[0:3]]
    d = [F(x) for x in ray[4:7]]
    rmint, rmaxt = F(ray[3]), F(ray[7])
    best = (FLT_MAX, F(0), F(0), M32)
    stack = []
    ni = 0
    while True:
        mn, cnt, mx, off = node_box(nodes, ni)
        if cnt > 0:
            done = False
            for pid in range(off, off + cnt):
                r = tri_intersect(verts, idx, int(prims[pid]), o, d, rmint, rmaxt)
                if r is not None and r[0] < rmaxt:
                    best = (r[0], r[1], r[2], int(prims[pid]))
                    if any_hit:
                        done = True
                        break
                    rmaxt = r[0]
            if done or not stack:
                return best
            ni = stack.pop()
            continue
        c1, c2 = off, off + 1
        m1, _, x1, _ = node_box(nodes, c1)
        m2, _, x2, _ = node_box(nodes, c2)
        d1 = box_entry(m1, x1, o, d, rmint, rmaxt)
        d2 = box_entry(m2, x2, o, d, rmint, rmaxt)
        if d1 > d2:
            d1, d2, c1, c2 = d2, d1, c2, c1
        if d1 == FLT_MAX:
            if not stack:
                return best
            ni = stack.pop()
        else:
            ni = c1
            if d2 != FLT_MAX:
                stack.append(c2)


# ---- include/cuda/neural/accel/neural_bvh2.cuh:80-86, 170-292 ----
def dilated(nodes, i, dil):
    mn, cnt, mx, off = node_box(nodes, i)
    if dil != 0:
        ext = sub(mx, mn)
        c = add(mn, scale(ext, F(0.5)))
        ne = scale(ext, F(F(1.0) + dil))
        return sub(c, scale(ne, F(0.5))), add(c, scale(ne, F(0.5))), cnt, off
    return mn, mx, cnt, off


def next_segment(nodes, o, d, stack, rmaxt, dil, mint_eps, maxt_eps, lod=0, stack_size=24):
    """Resumes the traversal from `stack` up to the next accepted leaf, with the traversal's current
    depth rmaxt: (mint, maxt, node), or None once the stack is exhausted."""
    rmint = -FLT_MAX
    while stack:
        ni = stack.pop()
        while True:
            bmin, bmax, cnt, off = dilated(nodes, ni, dil)
            if (0 < cnt <= 2 + lod) or off == M32:
                t0 = div(sub(bmin, o), d)
                t1 = div(sub(bmax, o), d)
                mint = cmax([gmin(t0[i], t1[i]) for i in range(3)])
                maxt = cmin([gmax(t0[i], t1[i]) for i in range(3)])
                if mint <= maxt:
                    valid = mint < rmaxt
                    valid = valid and (maxt > maxt_eps if mint < 0 else mint > mint_eps)
                    if valid:
                        return mint, maxt, ni
                break
            c1, c2 = off, off + 1
            b1 = dilated(nodes, c1, dil)
            b2 = dilated(nodes, c2, dil)
            d1 = box_entry(b1[0], b1[1], o, d, rmint, rmaxt)
            d2 = box_entry(b2[0], b2[1], o, d, rmint, rmaxt)
            if d1 > d2:
                d1, d2, c1, c2 = d2, d1, c2, c1
            if d1 == FLT_MAX:
                break
            ni = c1
            if d2 != FLT_MAX:
                stack.append(c2)
                assert len(stack) < stack_size
    return None


def neural_segments(nodes, ray, dil, mint_eps, maxt_eps, lod=0, stack_size=24):
    """Every leaf the traversal enters, in traversal order, with no depth found yet."""
    o = [F(x) for x in ray[0:3]]
    d = [F(x) for x in ray[4:7]]
    stack = [0]
    out = []
    while True:
        seg = next_segment(nodes, o, d, stack, FLT_MAX, dil, mint_eps, maxt_eps, lod, stack_size)
        if seg is None:
            return out
        out.append(seg)


# ---- hash-grid level (tcnn HashGrid behaviour, coherent prime hash) ----
# grid: [entries][features]; returns the level's features (as many as the grid's columns), each
# accumulated corner after corner.
def encode_level(grid, offset, size, res, scale_l, p):
    pos = [fma(F(p[i]), F(scale_l), F(0.5)) for i in range(3)]
    g = [int(np.floor(x)) for x in pos]
    fr = [F(pos[i] - F(np.floor(pos[i]))) for i in range(3)]
    acc = [F(0)] * grid.shape[1]
    dense = res ** 3 <= size
    for c in range(8):
        x, y, z = (g[0] + (c & 1)) & M32, (g[1] + ((c >> 1) & 1)) & M32, (g[2] + ((c >> 2) & 1)) & M32
        if dense:
            idx = (x + y * res + z * res * res) & M32
        else:
            idx = x ^ ((y * 2654435761) & M32) ^ ((z * 805459861) & M32)
        idx %= size
        w = F(F((fr[0] if c & 1 else F(F(1) - fr[0])) * (fr[1] if c & 2 else F(F(1) - fr[1]))) *
              (fr[2] if c & 4 else F(F(1) - fr[2])))
        for k in range(len(acc)):
            acc[k] = fma(w, grid[offset + idx, k], acc[k])
    return tuple(acc)


# ---- tcnn FullyFusedMLP as configured at src/cuda/neural/neural_bvh_module.cu:232-238 ----
# No biases, ReLU hidden layers, Sigmoid output padded to 16 rows. Matrices in network-first
# parameter order, each [rows][cols] row-major: W0 [n_neurons][n_inputs], then n_hidden_layers - 1
# times [n_neurons][n_neurons], then [16][n_neurons]. The layer inputs are FP16 values (the features
# rounded once, every hidden activation rounded to FP32 and then to FP16); the products are summed
# in double, input after input.
def mlp_forward(weights, n_inputs, n_hidden_layers, x, n_neurons=64):
    shapes = [(n_neurons, n_inputs)] + [(n_neurons, n_neurons)] * (n_hidden_layers - 1) + [(16, n_neurons)]
    a = [float(np.float16(v)) for v in x]
    off = 0
    out = None
    for m, (rows, cols) in enumerate(shapes):
        w = weights[off:off + rows * cols].astype(np.float64).reshape(rows, cols)
        off += rows * cols
        nxt = []
        for r in range(rows):
            acc = 0.0
            for k in range(cols):
                acc += float(w[r, k]) * a[k]
            nxt.append(acc)
        if m == len(shapes) - 1:
            out = [F(1.0 / (1.0 + math.exp(-v))) for v in nxt]
        else:
            a = [float(np.float16(F(v) if v > 0.0 else F(0))) for v in nxt]
    return out


# ---- Adam with ExponentialDecay (optimizer configured at src/cuda/neural/neural_bvh_module.cu:146-168) ----
# Bias-corrected Adam (Kingma and Ba, Algorithm 1) with the L2 term added to the gradient; the
# learning rate lr * base^floor((step - start) / interval) from step `start` on, folded with the
# bias corrections into one step size in double, then FP32 arithmetic per parameter.
def adam_step(params, m, v, grad, step, lr, beta1, beta2, eps, l2_reg, decay_start, decay_interval, decay_base):
    lr_s = float(lr)
    if step >= decay_start and decay_interval > 0:
        lr_s *= math.pow(float(decay_base), float((step - decay_start) // decay_interval))
    t = float(step) + 1.0
    lr_t = F(lr_s * math.sqrt(1.0 - math.pow(float(beta2), t)) / (1.0 - math.pow(float(beta1), t)))
    b1, b2, e, l2 = F(beta1), F(beta2), F(eps), F(l2_reg)
    omb1, omb2 = F(F(1) - b1), F(F(1) - b2)
    for i in range(len(params)):
        w = F(params[i])
        g = F(F(grad[i]) + F(l2 * w))
        mi = F(F(b1 * F(m[i])) + F(omb1 * g))
        vi = F(F(b2 * F(v[i])) + F(omb2 * F(g * g)))
        m[i], v[i] = mi, vi
        params[i] = F(w - F(lr_t * F(mi / F(F(np.sqrt(vi)) + e))))


# ---- the neural closest-hit query of one ray ----
# Traversal: neural_bvh2.cuh:170-292, resumed after every network step with the current depth
# (neural_bvh_module_common.cuh:496-550). Network input: encode_segment_from_world_po_pi and
# encode_bvh_network_input_data (neural_bvh_module_kernels.cu:10-97, 266-303): the segment ends
# swapped for a negative mint, mapped into the dilated scene box, points at equidistant interior
# (distribution 0) or exterior (1) positions. Output: neural_node_traversal and
# process_neural_bvh_traversal_step (neural_bvh_module_common.cuh:160-206,
# path_inference_kernels.cu:61-131) without depth interpolation: visible when the first output is
# above the threshold, LocalT depth, the hit kept when it is nearer, normal = normalize(2 n - 1).
# The ray's tmax is the query's current depth. Returns the 12-word record: t, normal, albedo,
# visibility, flags (bit 0 hit, bit 2 step cap), segments evaluated, 0xFFFFFFFF, 0.
def neural_query(nodes, ray, scene_min, scene_max, grid, levels, weights, n_hidden_layers, c):
    o = [F(x) for x in ray[0:3]]
    d = [F(x) for x in ray[4:7]]
    best_t = F(ray[7])
    valid, flags, segments = False, 0, 0
    normal, albedo, vis = [F(0)] * 3, [F(0)] * 3, F(0)
    dilation = F(F(F(1) + F(c["node_extent_dilation"])) + F(c["fixed_node_dilation"]))
    ext = [F(F(F(scene_max[i]) - F(scene_min[i])) * dilation) for i in range(3)]
    center = [F(F(F(scene_max[i]) + F(scene_min[i])) * F(0.5)) for i in range(3)]
    P = c["points"]
    if c["distribution"] == 1:
        delta, offset = (F(1) if P == 1 else F(F(1) / F(P - 1))), F(0)
    else:
        delta, offset = F(F(1) / F(P)), F(0.5)
    seg_args = (F(c["fixed_node_dilation"]), F(c["mint_eps"]), F(c["maxt_eps"]))
    stack = [0]
    seg = next_segment(nodes, o, d, stack, FLT_MAX, *seg_args)
    thr = F(c["threshold"])
    step = 0
    while seg is not None:
        if step > c["max_steps"]:
            flags |= 4
            break
        step += 1
        mint, maxt, _ = seg
        a, b = (maxt, mint) if mint < 0 else (mint, maxt)
        epo = [F(F(F(F(o[i] + F(d[i] * a)) - center[i]) / ext[i]) + F(0.5)) for i in range(3)]
        epi = [F(F(F(F(o[i] + F(d[i] * b)) - center[i]) / ext[i]) + F(0.5)) for i in range(3)]
        x = []
        for k in range(P):
            t = F(delta * F(F(k) + offset))
            omt = F(F(1) - t)
            pt = [F(F(epo[i] * omt) + F(epi[i] * t)) for i in range(3)]
            for (off, size, res, scl) in levels:
                x.extend(encode_level(grid, off, size, res, scl, pt))
        out = mlp_forward(weights, len(x), n_hidden_layers, x)
        segments += 1
        new_depth = best_t
        if out[0] > thr:
            de = decode_local_t(out[1], mint, maxt, mint < 0, F(c["depth_epsilon"]), F(c["fixed_depth_epsilon"]))
            if de != FLT_MAX and de < best_t:
                valid, best_t, new_depth, vis = True, de, de, out[0]
                n = [F(F(out[2 + i] * F(2)) - F(1)) for i in range(3)]
                inv = F(F(1) / F(np.sqrt(F(F(F(n[0] * n[0]) + F(n[1] * n[1])) + F(n[2] * n[2])))))
                normal = [F(n[i] * inv) for i in range(3)]
                albedo = [out[5], out[6], out[7]]
        if not stack:
            break
        seg = next_segment(nodes, o, d, stack, new_depth, *seg_args)
    words = [F(best_t if valid else FLT_MAX)] + normal + albedo + [F(vis if valid else 0)]
    rec = [int(np.float32(w).view(np.uint32)) for w in words]
    return rec + [(1 if valid else 0) | flags, segments, M32, 0]


# ---- training rays: granular_sample_bvh_network_input_data (neural_bvh_module_kernels.cu:119-264)
# with one sample per thread (no bounce continues), stack_based_sample_uniform_bvh_density and
# sample_bbox_position (neural_bvh_module_common.cuh:635-780), labels from
# generate_single_bvh_network_output_reference (:782-858) with LocalT depth, the geometric normal
# (compute_its_data, include/cuda/accel/bvh.cuh:55-95) and a per-triangle albedo (0.9 without one).
# Vector constructors draw their random components x first. Returns (points [P][3], targets [8],
# sampled node).
def _normalize(v):
    inv = F(F(1) / F(np.sqrt(dot(v, v))))
    return scale(v, inv)


def _uniform_sphere(sx, sy):
    sp, cp = sincos_turns(sx)
    cos_t = F(F(sy * F(2)) - F(1))
    sin_t = F(np.sqrt(F(F(1) - F(cos_t * cos_t))))
    return [F(sin_t * cp), F(sin_t * sp), cos_t]


def _cube_pos_on_face(face, u, v):
    return [[F(1), u, v], [F(0), u, v], [u, F(1), v], [u, F(0), v], [u, v, F(1)], [u, v, F(0)]][face]


def training_sample(i, training_step, batch_size, cut, scene_min, scene_max, bvh, prims, verts, idx, albedo, c,
                    learned_lod=6, n_lods=7):
    rng = Rng(lcg_seed((training_step * batch_size) & M32, 0, i))
    direction = _uniform_sphere(rng.f(), rng.f())
    n_learned = n_lods - learned_lod
    lod = learned_lod + min(int(F(rng.f() * F(n_learned))), n_learned - 1)
    dil = F(F(c["fixed_node_dilation"]) + F(rng.f() * F(c["node_extent_dilation"])))
    sbs = F(c["sampling_bbox_scaling"])
    ext = sub([F(x) for x in scene_max], [F(x) for x in scene_min])
    seg, stack, o = None, [], None
    while seg is None:
        if not stack:  # the ray escaped: a new origin, the same direction, the traversal from the root
            stack = [0]
            ps = [rng.f(), rng.f(), rng.f()]
            local = [F(F(sbs * ps[k]) - F(F(sbs - F(1)) * F(0.5))) for k in range(3)]
            o = [F(F(local[k] * ext[k]) + F(scene_min[k])) for k in range(3)]
        seg = next_segment(cut, o, direction, stack, FLT_MAX, dil, F(c["learning_mint_eps"]),
                           F(c["learning_maxt_eps"]), lod)
    mint, maxt, node = seg
    d = direction
    ratio = F(c["leaf_boundary_sampling_ratio"])
    if ratio != 0 and rng.f() <= ratio:
        f1 = min(int(F(rng.f() * F(6))), 5)
        while True:
            f2 = min(int(F(rng.f() * F(6))), 5)
            if f2 != f1:
                break
        lp1 = _cube_pos_on_face(f1, rng.f(), rng.f())
        lp2 = _cube_pos_on_face(f2, rng.f(), rng.f())
        bmn, _, bmx, _ = node_box(cut, node)
        nex = sub(bmx, bmn)
        center = add(bmn, scale(nex, F(0.5)))
        nex = scale(nex, F(F(1) + dil))
        nmin = sub(center, scale(nex, F(0.5)))
        entry = [F(nmin[k] + F(lp1[k] * nex[k])) for k in range(3)]
        exitp = [F(nmin[k] + F(lp2[k] * nex[k])) for k in range(3)]
        o, d = entry, _normalize(sub(exitp, entry))
        span = sub(exitp, entry)
        mint, maxt = F(0), F(np.sqrt(dot(span, span)))
    # segment points (no swap for a negative mint on this path)
    dilation = F(F(F(1) + F(c["node_extent_dilation"])) + F(c["fixed_node_dilation"]))
    sext = [F(F(F(scene_max[k]) - F(scene_min[k])) * dilation) for k in range(3)]
    center = [F(F(F(scene_max[k]) + F(scene_min[k])) * F(0.5)) for k in range(3)]
    epo = [F(F(F(F(o[k] + F(d[k] * mint)) - center[k]) / sext[k]) + F(0.5)) for k in range(3)]
    epi = [F(F(F(F(o[k] + F(d[k] * maxt)) - center[k]) / sext[k]) + F(0.5)) for k in range(3)]
    P = c["points"]
    if c["distribution"] == 1:
        delta, offset = (F(1) if P == 1 else F(F(1) / F(P - 1))), F(0)
    else:
        delta, offset = F(F(1) / F(P)), F(0.5)
    pts = []
    for k in range(P):
        t = rng.f() if c["distribution"] == 2 else F(delta * F(F(k) + offset))
        omt = F(F(1) - t)
        pts.append([F(F(epo[j] * omt) + F(epi[j] * t)) for j in range(3)])
    # labels from the classic BLAS on [mint, maxt]
    t, _, _, prim = classic_intersect(bvh, prims, verts, idx, o + [mint] + d + [maxt])
    if t == FLT_MAX:
        return pts, [F(0)] * 8, node
    depth = F((float(F(t - mint))) / (float(F(maxt - mint)) + 1e-3))
    ix = idx[prim]
    v0, v1, v2 = ([F(x) for x in verts[ix[k]]] for k in range(3))
    n = _normalize(cross(sub(v1, v0), sub(v2, v0)))
    nn = [F(F(n[k] + F(1)) * F(0.5)) for k in range(3)]
    alb = [F(x) for x in albedo[prim]] if albedo is not None else [F(0.9)] * 3
    return pts, [F(1), depth] + nn + alb, node


# ---- the library's hybrid path tracer (k_path.cu; the Lambertian case of the reference's scatter,
# path_inference_kernels.cu:224-429): camera rays with a per-sample jitter, one neural query per
# bounce, an analytic ground plane and sky, cosine-weighted bounces about the normal in the
# orthonormal basis of Duff et al. (JCGT 6(1), 2017), throughput times albedo, radiance from the
# sky. Returns the RGB image [width * height][3] and the rays traced.
def _cosine_sample(n, rng):
    u1, u2 = rng.f(), rng.f()
    sp, cp = sincos_turns(u2)
    r, z = F(np.sqrt(u1)), F(np.sqrt(gmax(F(0), F(F(1) - u1))))
    sign = F(1) if n[2] >= 0 else F(-1)
    a = F(F(-1) / F(sign + n[2]))
    c = F(F(n[0] * n[1]) * a)
    t = [F(F(1) + F(F(F(sign * n[0]) * n[0]) * a)), F(sign * c), F(-F(sign * n[0]))]
    b = [c, F(sign + F(F(n[1] * n[1]) * a)), F(-n[1])]
    rc, rs = F(r * cp), F(r * sp)
    return [F(F(F(rc * t[k]) + F(rs * b[k])) + F(z * n[k])) for k in range(3)]


def path_trace(nodes, scene_min, scene_max, grid, levels, weights, n_hidden_layers, c, p):
    W, Hh, spp = p["width"], p["height"], p["spp"]
    du, dv, tl, org = ([F(x) for x in p[k]] for k in ("du", "dv", "tl", "origin"))
    rays, ids, thr = [], [], []
    n = W * Hh * spp
    rad = [[F(0)] * 3 for _ in range(n)]
    for i in range(n):
        px, smp = i // spp, i % spp
        x, y = px % W, px // W
        rng = Rng(lcg_seed((p["sample_base"] + smp) & M32, p["sample_offset"], px))
        jx, jy = rng.f(), rng.f()
        xf, yf = F(F(F(x) + jx) / F(W)), F(F(F(y) + jy) / F(Hh))
        d = _normalize(add(add(scale(du, xf), scale(dv, yf)), tl))
        rays.append(org + [F(1e-4)] + d + [FLT_MAX])
        ids.append(i)
        thr.append([F(1), F(1), F(1), rng.state ^ ((p["seed"] * 0x9E3779B9) & M32)])
    traced = 0
    zen, hor, galb = ([F(x) for x in p[k]] for k in ("sky_zenith", "sky_horizon", "ground_albedo"))
    for bounce in range(p["max_bounces"] + 1):
        if not rays:
            break
        traced += len(rays)
        nxt, nxt_ids = [], []
        for ray, pid in zip(rays, ids):
            h = neural_query(nodes, ray, scene_min, scene_max, grid, levels, weights, n_hidden_layers, c)
            ro, d = ray[0:3], ray[4:7]
            words = np.array(h[:7], np.uint32).view(np.float32)
            t = F(words[0]) if h[8] & 1 else FLT_MAX
            nrm, alb = [F(v) for v in words[1:4]], [F(v) for v in words[4:7]]
            if p["has_ground"] and d[1] != 0:
                tp = F(F(F(p["ground_y"]) - ro[1]) / d[1])
                if tp > F(1e-4) and tp < t:
                    t, nrm, alb = tp, [F(0), F(1), F(0)], galb
            th = thr[pid]
            if t == FLT_MAX:
                w = gmax(d[1], F(0))
                for k in range(3):
                    rad[pid][k] = F(rad[pid][k] + F(th[k] * F(hor[k] + F(F(zen[k] - hor[k]) * w))))
            elif bounce < p["max_bounces"]:
                ln = F(np.sqrt(F(F(F(nrm[0] * nrm[0]) + F(nrm[1] * nrm[1])) + F(nrm[2] * nrm[2]))))
                nrm = [F(v / ln) for v in nrm] if ln > 0 else [F(-v) for v in d]
                if F(F(F(nrm[0] * d[0]) + F(nrm[1] * d[1])) + F(nrm[2] * d[2])) > 0:
                    nrm = [F(-v) for v in nrm]
                rng = Rng(th[3])
                nd = _cosine_sample(nrm, rng)
                for k in range(3):
                    th[k] = F(th[k] * alb[k])
                th[3] = rng.state
                o = [F(F(ro[k] + F(t * d[k])) + F(F(1e-3) * nrm[k])) for k in range(3)]
                if F(F(th[0] + th[1]) + th[2]) > 0:
                    nxt.append(o + [F(1e-4)] + nd + [FLT_MAX])
                    nxt_ids.append(pid)
        rays, ids = nxt, nxt_ids
    inv = F(F(1) / F(spp))
    img = []
    for px in range(W * Hh):
        acc = [F(0)] * 3
        for smp in range(spp):
            for k in range(3):
                acc[k] = F(acc[k] + rad[px * spp + smp][k])
        img.append([F(v * inv) for v in acc])
    return np.array(img, np.float32), traced


# ---- include/cuda/neural/neural_bvh_module_common.cuh:23-58 (LocalT) ----
def decode_local_t(out_depth, mint, maxt, inside, depth_epsilon=F(0.2), fixed_depth_epsilon=F(1e-5)):
    seg_len = F(F(maxt) - F(mint))
    u = gmin(gmax(F(out_depth), F(0)), F(1))
    if inside:
        if depth_epsilon != 1:
            inward = F(float(u) * (float(seg_len) + 1e-3))
            if inward < F(F(F(maxt) - F(seg_len * depth_epsilon)) - fixed_depth_epsilon):
                return F(F(maxt) - inward)
        return FLT_MAX
    return F(float(u) * (float(seg_len) + 1e-3) + float(mint))


# ---- include/cuda/neural/utils/loss_gradient.cuh:25-94 ----
def loss_and_gradient(kind, target, pred):
    target, pred = F(target), F(pred)
    if kind == "L1":
        diff = F(pred - target)
        return F(abs(diff)), F(np.copysign(F(1), diff))
    if kind == "L2":
        diff = F(pred - target)
        return F(diff * diff), F(F(2) * diff)
    if kind == "RelativeL2":
        diff = F(pred - target)
        den = F(F(pred * pred) + F(1e-2))
        return F(F(diff * diff) / den), F(F(F(2) * diff) / den)
    if kind == "BinaryCrossEntropy":
        p = min(max(pred, F(1e-5)), F(F(1) - F(1e-5)))
        loss = -(float(target) * np.log(float(p)) + (1 - float(target)) * np.log(1 - float(p)))
        grad = F(-F(target - p) / F(p - F(p * p)))
        return F(loss), grad
    raise KeyError(kind)
