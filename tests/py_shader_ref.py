"""A second, independent restatement of the reference's frame, in Python on
numpy float32 scalars (test infrastructure): written from the GLSL of
pimpale/vulkan-voxel-restir-gi's shaders and its Rust stage wiring, not from
oracle/vrg_oracle.cpp, so that a slip in either restatement shows as a
mismatch between them.

Covered, per pixel (file:line in src/render_system/):
  raygen                         shader/raygen.rs:80-111
  raytrace (shading, scatter)    shader/raytrace.rs:390-578, with
    traverseBvh / nodeImportance shader/raytrace.rs:181-281
    samplers, frame              shader/raytrace.rs:286-345
  nee_pdf (any-hit sum)          shader/nee_pdf.rs:281-337, with
    reverseTraverseBvh           shader/nee_pdf.rs:154-228
    computeNeePdf                shader/nee_pdf.rs:230-279
  outgoing_radiance              shader/outgoing_radiance.rs:58-94
  initial sample copies          interactive_rendering.rs:1359-1414
  temporal resampling            shader/restir_temporal_resampling.rs:256-301
  spatial resampling             shader/restir_spatial_resampling.rs:316-406
  finalize                       shader/restir_finalize.rs:121-141
  postprocess (scale 1, and srcscale > 1 in postprocess_scaled)
                                 shader/postprocess.rs:39-88
and the chunk mesh order of game_system/chunk.rs:158-292, the light BLAS of
scene.rs:547-571 (upload_object, for chunk meshes and for uploaded triangle
meshes alike), the light TL of scene.rs:248-287 over instances placed by
translations or full isometries (Aabb::transform, bvh/aabb.rs:75-92; built
with the independent builder restatement of tests/py_build_ref.py), and the
per-instance transform of triangles and light-BVH nodes (triangleTransform,
raytrace.rs:155-159; nodeImportance, raytrace.rs:181-208).

Four things have no reference definition and follow this project's
documented choices: which triangle a ray hits (the ray query is the
driver's; the hit of each bounce is taken from the frame under test, its
barycentrics recomputed: from the face geometry for a voxel face, by the
watertight test of tests/py_tri_ref.py for a mesh triangle), the arithmetic
of an isometry (the 3x4 matrix form ((r0 x + r1 y) + r2 z) + t, or p + t for
a translation), and sin/cos(2*pi*u) (the quarter-turn reduction with Taylor
polynomials).  GLSL built-ins evaluate left to right:
dot = (x*x' + y*y') + z*z', normalize(v) = v / length(v).
"""
import numpy as np

import py_build_ref
import py_tri_ref

F = np.float32
M32 = 0xFFFFFFFF
ZERO3 = (F(0), F(0), F(0))
PI = F(3.1415926535897932384626433832795)
EPS_TRACE = F(0.001)  # raytrace.rs EPSILON_BLOCK
EPS_NEE = F(0.0001)   # nee_pdf.rs EPSILON_BLOCK
FACE_PAD = F(1.0 / 4096.0)


# ---- vec3 in GLSL order ----------------------------------------------------
def v3(x, y, z):
    return (F(x), F(y), F(z))


def add(a, b):
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def sub(a, b):
    return (a[0] - b[0], a[1] - b[1], a[2] - b[2])


def vs(a, s):  # vec3 * float
    return (a[0] * s, a[1] * s, a[2] * s)


def sv(s, a):  # float * vec3
    return (s * a[0], s * a[1], s * a[2])


def vv(a, b):  # vec3 * vec3
    return (a[0] * b[0], a[1] * b[1], a[2] * b[2])


def dot(a, b):
    return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]


def cross(a, b):
    return (a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1])


def length(a):
    return F(np.sqrt(dot(a, a)))


def normalize(a):
    n = length(a)
    return (a[0] / n, a[1] / n, a[2] / n)


def is_zero(a):
    return a[0] == 0 and a[1] == 0 and a[2] == 0


def luminance(c):  # restir_*.rs luminance()
    return (F(0.2126) * c[0] + F(0.7152) * c[1]) + F(0.0722) * c[2]


# ---- instance transforms ---------------------------------------------------
def xform(m=None, translation=None):
    """(3x4 row-major matrix as float32 scalars, translation only)."""
    if m is None:
        t = [F(x) for x in (translation or (0, 0, 0))]
        return ((F(1), F(0), F(0), t[0], F(0), F(1), F(0), t[1], F(0), F(0), F(1), t[2]), True)
    m = tuple(F(x) for x in m)
    tonly = m[0] == 1 and m[5] == 1 and m[10] == 1 and all(m[k] == 0 for k in (1, 2, 4, 6, 8, 9))
    return (m, bool(tonly))


IDENT = xform()


def xf_point(X, p):
    m, tonly = X
    if tonly:
        return (p[0] + m[3], p[1] + m[7], p[2] + m[11])
    return (((m[0] * p[0] + m[1] * p[1]) + m[2] * p[2]) + m[3],
            ((m[4] * p[0] + m[5] * p[1]) + m[6] * p[2]) + m[7],
            ((m[8] * p[0] + m[9] * p[1]) + m[10] * p[2]) + m[11])


def aabb_transform(mn, mx, X):
    """Aabb::transform (bvh/aabb.rs:75-92): the AABB of the 8 transformed corners."""
    c = [xf_point(X, (mx[0] if k & 4 else mn[0], mx[1] if k & 2 else mn[1], mx[2] if k & 1 else mn[2]))
         for k in range(8)]
    a = py_build_ref.Aabb.from_points(c)
    return [*a.mn, *a.mx]


# ---- murmur3 chaining (raygen.rs:37-78) ------------------------------------
def combine(h, k):
    k = (k * 0x1B873593) & M32
    h ^= k
    h = ((h << 13) | (h >> 19)) & M32
    return (h * 5 + 0xE6546B64) & M32


def finalize(h):
    h ^= h >> 16
    h = (h * 0x85EBCA6B) & M32
    h ^= h >> 13
    h = (h * 0xC2B2AE35) & M32
    h ^= h >> 16
    return h


def float_construct(m):
    return np.array([(m & 0x007FFFFF) | 0x3F800000], np.uint32).view(np.float32)[0] - F(1.0)


def finalizef(h):
    return float_construct(finalize(h))


def sincos_2pi(x):
    """sin and cos of 2*pi*x for x in [0, 1): the quarter-turn reduction and
    Taylor polynomials this project uses for GLSL's sin/cos."""
    q = F(np.rint(x * F(4.0)))
    r = x - q * F(0.25)
    a = r * F(6.283185307179586476925286766559)
    a2 = a * a
    ps = (((F(2.75573192e-6) * a2 - F(1.98412698e-4)) * a2 + F(8.33333333e-3)) * a2 - F(1.66666667e-1)) * a2
    sn = a + a * ps
    pc = ((((F(-2.75573192e-7) * a2 + F(2.48015873e-5)) * a2 - F(1.38888889e-3)) * a2 + F(4.16666667e-2)) * a2
          - F(0.5)) * a2
    cs = F(1.0) + pc
    k = int(q) & 3
    return [(sn, cs), (cs, -sn), (-sn, -cs), (-cs, sn)][k]


# ---- chunk meshing (chunk.rs:158-292) ---------------------------------------
# per face (left, right, down, up, back, front): six vertices as (a, b, c)
# corner offsets of v{abc} and their uvs, in the order gen_mesh pushes them
FACES = [
    [((0, 0, 1), (0, 1)), ((0, 1, 0), (1, 0)), ((0, 0, 0), (1, 1)), ((0, 1, 1), (0, 0)), ((0, 1, 0), (1, 0)),
     ((0, 0, 1), (0, 1))],
    [((1, 1, 0), (0, 0)), ((1, 0, 1), (1, 1)), ((1, 0, 0), (0, 1)), ((1, 1, 0), (0, 0)), ((1, 1, 1), (1, 0)),
     ((1, 0, 1), (1, 1))],
    [((0, 0, 0), (0, 0)), ((1, 0, 0), (1, 0)), ((0, 0, 1), (0, 1)), ((1, 0, 0), (1, 0)), ((1, 0, 1), (1, 1)),
     ((0, 0, 1), (0, 1))],
    [((0, 1, 1), (1, 1)), ((1, 1, 0), (0, 0)), ((0, 1, 0), (1, 0)), ((0, 1, 1), (1, 1)), ((1, 1, 1), (0, 1)),
     ((1, 1, 0), (0, 0))],
    [((0, 1, 0), (0, 0)), ((1, 0, 0), (1, 1)), ((0, 0, 0), (0, 1)), ((0, 1, 0), (0, 0)), ((1, 1, 0), (1, 0)),
     ((1, 0, 0), (1, 1))],
    [((0, 0, 1), (1, 1)), ((1, 0, 1), (0, 1)), ((0, 1, 1), (1, 0)), ((1, 0, 1), (0, 1)), ((1, 1, 1), (0, 0)),
     ((0, 1, 1), (1, 0))],
]
NEIGHBOUR = [(-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)]


class Chunk:
    """gen_mesh of one chunk (triangle k -> block x, y, z, face, half, texture
    slot) and the light BLAS that upload_object builds from it."""

    def __init__(self, blocks, neighbour_blocks, mats, n_slots):
        n_types = n_slots // 6  # six texture slots per block type (block.rs:116-119)
        air = n_types  # completely_transparent (block.rs:121-123)
        see_through = [(int(mats[6 * b].flags) & 1) != 0 for b in range(n_types)] + [True]
        blk = np.asarray(blocks, np.uint8).reshape(32, 32, 32)
        nbs = [None if a is None else np.asarray(a, np.uint8).reshape(32, 32, 32) for a in neighbour_blocks]

        def at(x, y, z, f):  # chunk.rs:170-205: outside the chunk, the neighbour's far plane
            if 0 <= x < 32 and 0 <= y < 32 and 0 <= z < 32:
                return int(blk[x, y, z])
            return air if nbs[f] is None else int(nbs[f][x % 32, y % 32, z % 32])

        self.mesh = False
        self.tris = []
        for x in range(32):
            for y in range(32):
                for z in range(32):
                    b = int(blk[x, y, z])
                    if b == air:
                        continue
                    for f, (dx, dy, dz) in enumerate(NEIGHBOUR):
                        if see_through[at(x + dx, y + dy, z + dz, f)]:
                            t = 6 * b + f  # get_material_offset (block.rs:116-119)
                            self.tris.append((x, y, z, f, 0, t))
                            self.tris.append((x, y, z, f, 1, t))
        # upload_object (scene.rs:555-571): luminous triangles, power = luminance * area
        lum, ltri, lid = [], [], []
        for k, tri in enumerate(self.tris):
            L = F(mats[tri[5]].luminance)
            if L > 0:
                a, b, c = self.local_vertices(k)
                area = length(cross(sub(b, a), sub(c, a))) / F(2.0)
                lum.append(L * area)
                ltri.append([*a, *b, *c])
                lid.append(k)
        self.n_light = len(lum)
        self.light_nodes = None
        if self.n_light:
            self.light_nodes, _ = py_build_ref.build_bl_bvh(np.array(ltri, np.float32), np.array(lum, np.float32),
                                                           np.array(lid, np.uint32))

    def local_vertices(self, k):
        x, y, z, f, h, _ = self.tris[k]
        out = []
        for j in range(3):
            (a, b, c), _ = FACES[f][3 * h + j]
            out.append(v3(F(x) + F(a), F(y) + F(b), F(z) + F(c)))
        return out

    def uvs(self, k):
        _, _, _, f, h, _ = self.tris[k]
        return [FACES[f][3 * h + j][1] for j in range(3)]

    def slot(self, k):
        return self.tris[k][5]


class Mesh:
    """upload_object of a Vec<Vertex3D> (scene.rs:547-571): triangle k is
    vertices 3k..3k+2, its texture slot that of its first vertex; luminous
    triangles (luminance of that slot > 0) make the light BLAS, power =
    luminance * area, ids = triangle index."""

    def __init__(self, vertices, mats):
        pos = np.asarray(vertices["position"], np.float32).reshape(-1, 3, 3)
        slots = np.asarray(vertices["t"], np.uint32)[0::3]
        self.mesh = True
        self.pos = [[tuple(F(x) for x in pos[k, j]) for j in range(3)] for k in range(len(pos))]
        self.slots = [int(t) for t in slots]
        self.uv = np.asarray(vertices["uv"], np.float32).reshape(-1, 3, 2)
        lum, ltri, lid = [], [], []
        for k, tri in enumerate(self.pos):
            L = F(mats[self.slots[k]].luminance)
            if L > 0:
                a, b, c = tri
                lum.append(L * (length(cross(sub(b, a), sub(c, a))) / F(2.0)))
                ltri.append([*a, *b, *c])
                lid.append(k)
        self.n_light = len(lum)
        self.light_nodes = None
        if self.n_light:
            self.light_nodes, _ = py_build_ref.build_bl_bvh(np.array(ltri, np.float32), np.array(lum, np.float32),
                                                           np.array(lid, np.uint32))

    def local_vertices(self, k):
        return self.pos[k]

    def uvs(self, k):
        return [tuple(self.uv[k, j]) for j in range(3)]

    def slot(self, k):
        return self.slots[k]


class World:
    """Instances in key order (scene.rs:245-260), each an object (Chunk or
    Mesh) and its transform (xform()); the light TL over the instances with
    lights (scene.rs:248-287): a translated instance's light AABB goes to the
    builder with its translation, any other's is transformed first
    (Aabb::transform) and goes with translation 0."""

    def __init__(self, instances, mats, atlas=None):
        self.mats = mats
        # texture atlas: (slots, 3 maps, h, w, RGBA8 sRGB) and the sRGB EOTF
        # of a texel byte (the maps are sampled as sRGB textures)
        self.atlas = None if atlas is None else np.asarray(atlas, np.uint8)
        self.srgb = [F(c / 12.92 if c <= 0.04045 else ((c + 0.055) / 1.055) ** 2.4)
                     for c in (i / 255.0 for i in range(256))]
        self.inst = []
        for c, x in instances:
            if isinstance(x, tuple) and len(x) == 2 and isinstance(x[1], bool):
                self.inst.append((c, x))
            else:
                self.inst.append((c, xform(translation=x)))
        aabbs, pw, ids, tr = [], [], [], []
        for i, (c, X) in enumerate(self.inst):
            if not c.n_light:
                continue
            # build_bl_bvh's light_aabb and power are its root's (build.rs:362-371)
            root = c.light_nodes[0]
            if X[1]:
                aabbs.append([*root["min"], *root["max"]])
                tr.append((X[0][3], X[0][7], X[0][11]))
            else:
                aabbs.append(aabb_transform(root["min"], root["max"], X))
                tr.append((F(0), F(0), F(0)))
            pw.append(root["power"])
            ids.append(i)
        self.tl_idx = {}
        if aabbs:
            self.light_tl, _ = py_build_ref.build_tl_bvh(np.array(aabbs, np.float32), np.array(pw, np.float32),
                                                         np.array(ids, np.uint32), np.array(tr, np.float32))
            for j, n in enumerate(self.light_tl):
                if n["left"] == 0xFFFFFFFF:
                    self.tl_idx[int(n["right"])] = j
        else:
            self.light_tl = None

    def world_vertices(self, inst, tri):
        c, X = self.inst[inst]
        return [xf_point(X, p) for p in c.local_vertices(tri)]


# ---- light BVH (raytrace.rs:181-281, nee_pdf.rs:119-228) --------------------
def node_importance(nee, point, normal, X, node):
    """nodeImportance: v000 and v111 are the instance transform X applied to
    the node's min and max (the corners are the box they span); raytrace.rs
    counts visible corners as uint (EPS 1e-3), nee_pdf.rs sums 0.125 per
    visible corner as float (EPS 1e-4)."""
    v000 = xf_point(X, v3(*node["min"]))
    v111 = xf_point(X, v3(*node["max"]))
    corners = [v000, (v000[0], v000[1], v111[2]), (v000[0], v111[1], v000[2]), (v000[0], v111[1], v111[2]),
               (v111[0], v000[1], v000[2]), (v111[0], v000[1], v111[2]), (v111[0], v111[1], v000[2]), v111]
    eps = EPS_NEE if nee else EPS_TRACE
    if nee:
        visible = F(0)
        for c in corners:
            visible += F(0.125) * (F(1.0) if dot(sub(c, point), normal) >= eps else F(0.0))
    else:
        count = sum(1 for c in corners if dot(sub(c, point), normal) >= eps)
    e = sub(v111, v000)
    m = sub(sv(F(0.5), add(v000, v111)), point)
    distance_sq = max(dot(e, e), dot(m, m))
    if nee:
        return F(node["power"]) / distance_sq * visible
    return F(node["power"]) / distance_sq * (F(count) / F(8.0))


def traverse_bvh(W, point, normal, seed):
    """traverseBvh: (success, instance, light BLAS leaf, importance)."""
    if W.light_tl is None:
        return False, 0, 0, F(0)
    root = W.light_tl
    node = root[0]
    importance = F(0)
    X = IDENT
    inst, idx, top = 0xFFFFFFFF, 0, True
    while True:
        if top and node["left"] == 0xFFFFFFFF:
            inst = int(node["right"])
            c, X = W.inst[inst]
            top = False
            root = c.light_nodes
            node = root[0]
            idx = 0
            if importance == 0:
                importance = node_importance(False, point, normal, X, node)
        if not top and node["left"] == 0xFFFFFFFF:
            return True, inst, idx, importance
        li, ri = int(node["left"]), int(node["right"])
        lI = node_importance(False, point, normal, X, root[li])
        rI = node_importance(False, point, normal, X, root[ri])
        total = lI + rI
        ln = lI / total
        if finalizef(seed) < ln:
            node, idx, importance = root[li], li, lI
        else:
            node, idx, importance = root[ri], ri, rI
        seed = combine(seed, 0)


def reverse_traverse(W, point, normal, inst, leaf):
    c, X = W.inst[inst]
    root = c.light_nodes
    prob = F(1.0)
    top = False
    node, idx = root[leaf], leaf
    while True:
        old = idx
        if node["parent"] == 0xFFFFFFFF:
            if top:
                return prob
            top = True
            root = W.light_tl
            old = W.tl_idx[inst]
            tl_leaf = root[old]
            if tl_leaf["parent"] == 0xFFFFFFFF:
                return prob
            idx = int(tl_leaf["parent"])
            node = root[idx]
            X = IDENT
        else:
            idx = int(node["parent"])
            node = root[idx]
        lI = node_importance(True, point, normal, X, root[int(node["left"])])
        rI = node_importance(True, point, normal, X, root[int(node["right"])])
        total = lI + rI
        prob = prob * (lI / total if old == int(node["left"]) else rI / total)


def compute_nee_pdf(W, point, normal, direction, inst, leaf, b1, b2):
    c, _ = W.inst[inst]
    tri = int(c.light_nodes[leaf]["right"])
    t = W.world_vertices(inst, tri)
    # pointOnTriangle (nee_pdf.rs:230-232): x * v0 + y * v1 + (1 - x - y) * v2
    p = add(add(sv(b1, t[0]), sv(b2, t[1])), sv((F(1.0) - b1) - b2, t[2]))
    light_distance = length(sub(p, point))
    light_area = F(0.5) * length(cross(sub(t[0], t[1]), sub(t[2], t[1])))
    cos_theta = dot(normal, direction)
    ppp = light_distance * light_distance / (cos_theta * light_area)
    return reverse_traverse(W, point, normal, inst, leaf) * ppp


# ---- the voxel face test (this project's restatement of the ray query) ----
def face_hit(W, inst, tri, o, d, tmin, tmax):
    """(t, b1, b2) of the ray on triangle `tri` of instance `inst` — the plane
    hit of its face, the point inside the closed face square padded by 2^-12,
    on this triangle's side of the face diagonal — or None."""
    c, X = W.inst[inst]
    off = (X[0][3], X[0][7], X[0][11])  # chunks are placed by translations
    x, y, z, f, h, _ = c.tris[tri]
    axis = f >> 1
    u_ax = 0 if axis != 0 else 1
    v_ax = 2 if axis != 2 else 1
    corner = [F(x) + off[0], F(y) + off[1], F(z) + off[2]]
    plane = corner[axis] + F(f & 1)
    t = (plane - o[axis]) * (F(1.0) / d[axis])
    if not (tmin <= t <= tmax):
        return None
    lu = (o[u_ax] + t * d[u_ax]) - corner[u_ax]
    lv = (o[v_ax] + t * d[v_ax]) - corner[v_ax]
    if not (-FACE_PAD <= lu <= F(1.0) + FACE_PAD and -FACE_PAD <= lv <= F(1.0) + FACE_PAD):
        return None
    half = 0 if (F(1.0) - lu) - lv >= 0 else 1
    if half != h:
        return None

    def weight(cu, cv):  # barycentric weight of the triangle's corner (cu, cv)
        if h == 0:
            if cu == 0 and cv == 0:
                return (F(1.0) - lu) - lv
            return lu if cu == 1 else lv
        if cu == 1 and cv == 1:
            return (lu + lv) - F(1.0)
        return F(1.0) - lv if cu == 1 else F(1.0) - lu

    bary = []
    for j in (1, 2):
        (a, b, cc), _ = FACES[f][3 * h + j]
        bits = (a, b, cc)
        bary.append(weight(bits[u_ax], bits[v_ax]))
    return t, bary[0], bary[1]


def hit_of(W, inst, tri, o, d, tmin, tmax):
    """(t, b1, b2) of the ray on triangle `tri` of instance `inst`, or None: a
    voxel face by face_hit, a mesh triangle by the watertight test on its
    world-space vertices."""
    c, _ = W.inst[inst]
    if c.mesh:
        t = W.world_vertices(inst, tri)
        return py_tri_ref.tri_test([*t[0], *t[1], *t[2]], o, d, tmin, tmax)
    return face_hit(W, inst, tri, o, d, tmin, tmax)


# ---- the frame ---------------------------------------------------------------
class Frame:
    """Per-pixel state of one frame in the reference's SoA layout."""


def render(W, cam, params, hits, frame_index, history):
    """Renders one frame; `hits` gives, per bounce and pixel, the (instance,
    triangle) the ray query returned (None = miss); `history` is the temporal
    reservoir ring (3 slots, interactive_rendering.rs frame_count % 3), updated
    in place.  Returns the per-bounce arrays, the reservoirs and the image."""
    Wd, Hd, nb = cam.width, cam.height, params.num_bounces
    P = Wd * Hd
    eye, front, right, up = (v3(*cam.eye), v3(*cam.front), v3(*cam.right), v3(*cam.up))
    o = [[None] * P for _ in range(nb + 1)]
    dr = [[None] * P for _ in range(nb + 1)]
    nrm = [[None] * P for _ in range(nb)]
    emis = [[None] * P for _ in range(nb)]
    refl = [[None] * P for _ in range(nb)]
    mis = [[F(0)] * P for _ in range(nb)]
    pdf = [[F(1)] * P for _ in range(nb)]
    nee = [[F(0)] * P for _ in range(nb)]
    # raygen (raygen.rs:84-111): jitter is multiplied by 0.00
    aspect = F(Wd) / F(Hd)
    for p in range(P):
        x, y = p % Wd, p // Wd
        u = F(2.0) * F(x) / F(Wd) - F(1.0)
        v = F(2.0) * F(y) / F(Hd) - F(1.0)
        o[0][p] = eye
        dr[0][p] = normalize(add(add(vs(sv(u, right), aspect), sv(v, up)), front))
    for b in range(nb):
        inv_seed = (frame_index * nb + b) & M32  # interactive_rendering.rs:1189
        for p in range(P):
            seed = combine(inv_seed, p)
            origin, direction = o[b][p], dr[b][p]
            if is_zero(direction):  # raytrace.rs:406-416
                o[b + 1][p], dr[b + 1][p] = origin, ZERO3
                nrm[b][p] = emis[b][p] = refl[b][p] = ZERO3
                continue
            hit = hits[b][p]
            if hit is None:  # miss (raytrace.rs:421-430)
                o[b + 1][p] = add(origin, vs(direction, F(5000.0)))
                dr[b + 1][p] = ZERO3
                nrm[b][p] = ZERO3
                sky = F(50.0) if dot(direction, v3(0, 1, 0)) > F(0.9) else F(0.0)
                emis[b][p] = (sky, sky, sky)
                refl[b][p] = ZERO3
                continue
            inst, tri = hit
            th = hit_of(W, inst, tri, origin, direction, EPS_TRACE, F(1000.0))
            assert th is not None, (b, p, hit)
            _, b1, b2 = th
            b0 = (F(1.0) - b1) - b2
            t3 = W.world_vertices(inst, tri)
            # localCoordinateSystem (raytrace.rs:319-331)
            e1, e2 = sub(t3[1], t3[0]), sub(t3[2], t3[0])
            n_raw = cross(e1, e2)
            n, tangent, bitangent = normalize(n_raw), normalize(e1), normalize(cross(n_raw, e1))
            slot = W.inst[inst][0].slot(tri)
            m = W.mats[slot]
            new_o = add(add(vs(t3[0], b0), vs(t3[1], b1)), vs(t3[2], b2))
            R = v3(*m.reflectivity)
            alpha = F(m.alpha)
            ndd = -dot(direction, n)
            E = vs(v3(*m.emission), ndd)
            metal = F(m.metallic)
            if W.atlas is not None:
                # raytrace.rs:457-480: uv = v0.uv*b0 + v1.uv*b1 + v2.uv*b2, the three
                # maps of slot t sampled there (nearest texel, clamped to the edge)
                uvs = [tuple(F(x) for x in q) for q in W.inst[inst][0].uvs(tri)]
                u = ((uvs[0][0] * b0) + (uvs[1][0] * b1)) + (uvs[2][0] * b2)
                v = ((uvs[0][1] * b0) + (uvs[1][1] * b1)) + (uvs[2][1] * b2)
                ah, aw = W.atlas.shape[2], W.atlas.shape[3]
                ix = min(max(int(np.floor(u * F(aw))), 0), aw - 1)
                iy = min(max(int(np.floor(v * F(ah))), 0), ah - 1)
                t0, t1, t2 = (W.atlas[slot, k, iy, ix] for k in range(3))
                lin = W.srgb
                R = (lin[t0[0]], lin[t0[1]], lin[t0[2]])
                alpha = F(int(t0[3])) / F(255.0)
                E = ((F(1000.0) * lin[t1[0]]) * ndd, (F(1000.0) * lin[t1[1]]) * ndd, (F(1000.0) * lin[t1[2]]) * ndd)
                metal = lin[t2[0]]
            r0 = finalizef(combine(seed, 0))
            w_mis = F(0.0)
            if r0 < metal:
                bsdf_pdf = F(1.0)
                new_d = sub(direction, sv(F(2.0) * dot(n, direction), n))
            elif r0 < metal + (F(1.0) - alpha):
                new_d = direction
                R = v3(1, 1, 1)
                bsdf_pdf = F(1.0)
            else:
                new_o = add(new_o, sv(EPS_TRACE * F(1.5), n))
                R = (R[0] / PI, R[1] / PI, R[2] / PI)
                ok, l_inst, l_leaf, imp = False, 0, 0, F(0)
                if params.nee_type == 1 or (params.nee_type == 2 and b == 1):
                    ok, l_inst, l_leaf, imp = traverse_bvh(W, new_o, n, combine(seed, 2))
                if ok and imp > 0:
                    w_mis = F(0.3)
                ux, uy = finalizef(combine(seed, 4)), finalizef(combine(seed, 5))
                if finalizef(combine(seed, 3)) < w_mis:
                    c, _ = W.inst[l_inst]
                    lt = W.world_vertices(l_inst, int(c.light_nodes[l_leaf]["right"]))
                    if ux + uy > F(1.0):  # triangleSample
                        ux, uy = F(1.0) - ux, F(1.0) - uy
                    bx = (F(1.0) - ux) - uy
                    sp = add(add(sv(bx, lt[0]), sv(ux, lt[1])), sv(uy, lt[2]))
                    new_d = normalize(sub(sp, new_o))
                else:
                    s, cs = sincos_2pi(ux)
                    vv_ = F(np.sqrt(max(F(0.0), F(1.0) - uy * uy)))
                    hs = (vv_ * cs, uy, vv_ * s)
                    new_d = normalize(add(add(sv(hs[0], tangent), sv(hs[1], n)), sv(hs[2], bitangent)))
                bsdf_pdf = dot(new_d, n) / PI
            o[b + 1][p], dr[b + 1][p] = new_o, new_d
            nrm[b][p], emis[b][p], refl[b][p] = n, E, R
            mis[b][p], pdf[b][p] = w_mis, bsdf_pdf
    # nee_pdf (nee_pdf.rs:281-337) for b < nb - 1: every light triangle the
    # chosen direction crosses in [1e-4, 1000], summed in (instance, leaf) order
    for b in range(nb - 1):
        for p in range(P):
            d = dr[b + 1][p]
            if length(d) == 0 or mis[b][p] == 0:
                continue
            org, n = o[b + 1][p], nrm[b][p]
            hits_l = []
            for i, (c, _) in enumerate(W.inst):
                if not c.n_light:
                    continue
                for leaf, node in enumerate(c.light_nodes):
                    if node["left"] != 0xFFFFFFFF:
                        continue
                    th = hit_of(W, i, int(node["right"]), org, d, EPS_NEE, F(1000.0))
                    if th is not None:
                        hits_l.append(((i << 32) | leaf, compute_nee_pdf(W, org, n, d, i, leaf, th[1], th[2])))
            total = F(0.0)
            for _, val in sorted(hits_l):
                total += val
            nee[b][p] = total
    # outgoing_radiance (outgoing_radiance.rs:58-94), bounce nb-1 down to 0
    Lo = [[None] * P for _ in range(nb)]
    q = [[None] * P for _ in range(nb)]
    inv2pi = F(1.0) / (F(2.0) * PI)
    for p in range(P):
        L = ZERO3
        for b in range(nb - 1, -1, -1):
            valid = F(0.0) if is_zero(dr[b][p]) else F(1.0)
            qo = nee[b][p] * mis[b][p] + (F(1.0) - mis[b][p]) * inv2pi
            w = pdf[b][p] / qo
            L = add(emis[b][p], vs(vs(vv(refl[b][p], L), w), valid))
            Lo[b][p], q[b][p] = L, qo
    out = dict(origin=o, direction=dr, normal=nrm, emissivity=emis, reflectivity=refl, mis=mis, bsdf_pdf=pdf,
               nee_pdf=nee, radiance=Lo, q=q)
    if nb < 2:
        return out
    # initial sample (interactive_rendering.rs:1359-1414); the seed is never written.
    # The ring of temporal reservoirs has params.history_slots slots (3 in the
    # reference, frame % 3); CONFIG mode may cap the history's m (m_cap), scaling
    # w_sum by m_cap / m after the reset test (this project's extension)
    slots = params.history_slots if params.history_slots else 3
    ring = history[frame_index % slots]
    radius = F(params.spatial_radius)  # spatialSearchRadius, 15 in the reference
    temporal = []
    for p in range(P):
        S = dict(x_v=o[1][p], n_v=nrm[0][p], x_s=o[2][p], n_s=nrm[1][p], l=Lo[1][p], p_omega=q[0][p], seed=0)
        R = ring[p]
        ps = combine(params.temporal_seed, p)
        if finalizef(combine(ps, 0)) < F(0.4):
            R["w_sum"], R["m"] = F(0.0), 0
        if params.mode == 1 and params.m_cap and R["m"] > params.m_cap:
            R["w_sum"] = R["w_sum"] * (F(params.m_cap) / F(R["m"]))
            R["m"] = params.m_cap
        w = luminance(S["l"]) / S["p_omega"]
        R["w_sum"] = R["w_sum"] + w
        R["m"] += 1
        if float_construct(finalize(combine(ps, 1))) < w / R["w_sum"]:
            R["z"] = dict(S)
        ph = luminance(R["z"]["l"])
        R["ucw"] = R["w_sum"] / (F(R["m"]) * ph) if ph > 0 else F(0.0)
        temporal.append(dict(R, z=dict(R["z"])))
    spatial, final = [], []
    cos25 = F(0.906307787036649963)
    for p in range(P):
        qx, qy = p % Wd, p // Wd
        ps = combine(params.spatial_seed, p)
        Rs = dict(temporal[p], z=dict(temporal[p]["z"]))
        S = Rs["z"]
        Z = Rs["m"] if luminance(Rs["z"]["l"]) > 0 else 0
        for s in range(params.spatial_iterations):
            it = combine(ps, s)
            jx = radius * (finalizef(combine(it, 0)) - F(0.5))
            jy = radius * (finalizef(combine(it, 1)) - F(0.5))
            nx = min(max(int((F(qx) + F(0.5)) + jx), 0), Wd - 1)
            ny = min(max(int((F(qy) + F(0.5)) + jy), 0), Hd - 1)
            Rn = temporal[nx + ny * Wd]
            if is_zero(S["n_v"]) or is_zero(Rn["z"]["n_v"]) or dot(S["n_v"], Rn["z"]["n_v"]) < cos25:
                continue
            qz = Rn["z"]
            if is_zero(qz["n_s"]):
                J = F(1.0)
            else:
                qv = sub(qz["x_v"], qz["x_s"])
                rv = sub(S["x_v"], qz["x_s"])
                cq = abs(dot(normalize(qv), qz["n_s"]))
                cr = abs(dot(normalize(rv), qz["n_s"]))
                J = (cr / cq) * (length(qv) / length(rv))
            J = min(max(J, F(0.1)), F(10.0))
            p_adj = luminance(qz["l"]) / J
            m0 = Rs["m"]
            wn = (p_adj * Rn["ucw"]) * F(Rn["m"])
            Rs["w_sum"] = Rs["w_sum"] + wn
            Rs["m"] += 1
            if float_construct(finalize(combine(it, 2))) < wn / Rs["w_sum"]:
                Rs["z"] = dict(qz)
            Rs["m"] = m0 + Rn["m"]
            if luminance(qz["l"]) > 0:
                Z += Rn["m"]
        ph = luminance(Rs["z"]["l"])
        Rs["ucw"] = F(0.0) if ph == 0 else Rs["w_sum"] / (F(Z) * ph)
        spatial.append(Rs)
        # restir_finalize.rs:121-141
        dvec = normalize(sub(Rs["z"]["x_s"], o[1][p]))
        bp = dot(dvec, Rs["z"]["n_v"]) / PI
        final.append(add(emis[0][p], vs(vs(vv(refl[0][p], Rs["z"]["l"]), Rs["ucw"]), bp)))
    out.update(temporal=temporal, spatial=spatial, final=final)
    # postprocess (postprocess.rs:39-88) at srcscale 1: view 0 the path's
    # radiance, 1 the ReSTIR target, 2 the spatial ucw / 10 (restir_finalize.rs:140)
    image = np.zeros((P, 4), np.uint8)
    for p in range(P):
        if params.debug_view == 0:
            c = Lo[0][p]
        elif params.debug_view == 1:
            c = final[p]
        else:
            d = spatial[p]["ucw"] / F(10.0)
            c = (d, d, d)
        c = (c[0] / F(1.0), c[1] / F(1.0), c[2] / F(1.0))
        image[p] = (to_u8(c[2]), to_u8(c[1]), to_u8(c[0]), 255)
    out.update(image=image.reshape(Hd, Wd, 4))
    return out


def to_u8(x):
    """u8(x * 255) as this project defines the conversion GLSL leaves open
    outside 0..255: saturating, NaN to 0, truncating inside."""
    v = x * F(255.0)
    if not v > 0:
        return 0
    return 255 if v >= 255 else int(v)


def empty_history(P, slots=3):
    z = dict(x_v=ZERO3, n_v=ZERO3, x_s=ZERO3, n_s=ZERO3, l=ZERO3, p_omega=F(0), seed=0)
    return [[dict(z=dict(z), ucw=F(0), m=0, w_sum=F(0)) for _ in range(P)] for _ in range(slots)]


def reservoir_row(R):
    """The 20-float layout of the frame readback: x_v, n_v, x_s, n_s, l_o_hat,
    p_omega, seed, ucw, m, w_sum (seed and m as u32 bits)."""
    z = R["z"]
    a = np.zeros(20, np.float32)
    a[0:3], a[3:6], a[6:9], a[9:12], a[12:15] = z["x_v"], z["n_v"], z["x_s"], z["n_s"], z["l"]
    a[15] = z["p_omega"]
    a[16] = np.array([z["seed"]], np.uint32).view(np.float32)[0]
    a[17] = R["ucw"]
    a[18] = np.array([R["m"]], np.uint32).view(np.float32)[0]
    a[19] = R["w_sum"]
    return a


def atlas_luminances(atlas):
    """get_texture_luminances (utils.rs:223-235): per slot, the float sum over
    the emissivity map's texels of (r + g) + b, in texel order, divided by the
    texel count."""
    atlas = np.asarray(atlas, np.uint8)
    n, _, h, w, _ = atlas.shape
    out = []
    for t in range(n):
        e = atlas[t, 1].reshape(-1, 4)
        L = F(0.0)
        for r, g, b, _a in e:
            L = L + ((F(int(r)) + F(int(g))) + F(int(b)))
        out.append(L / F(w * h))
    return out


def postprocess_scaled(view, scale):
    """postprocess.rs:39-88 with srcscale = scale, dstscale = 1: each output
    pixel the sum of its scale x scale source samples (rows outer, columns
    inner, from vec3(0.0)) divided by float(scale*scale), then u8(bgr*255)."""
    view = np.asarray(view, np.float32)
    H, W = view.shape[:2]
    oh, ow = H // scale, W // scale
    img = np.zeros((oh, ow, 4), np.uint8)
    out = np.zeros((oh, ow, 3), np.float32)
    n = F(scale * scale)
    for oy in range(oh):
        for ox in range(ow):
            c = ZERO3
            for sy in range(scale):
                for sx in range(scale):
                    c = add(c, tuple(view[oy * scale + sy, ox * scale + sx]))
            c = (c[0] / n, c[1] / n, c[2] / n)
            out[oy, ox] = c
            img[oy, ox] = (to_u8(c[2]), to_u8(c[1]), to_u8(c[0]), 255)
    return img, out
