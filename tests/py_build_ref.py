"""A second, independent restatement of src/render_system/bvh/build.rs and
bvh/aabb.rs in plain Python with numpy float32 scalars (small inputs only).
It follows the Rust recursion literally (recursive subdivide, Vec push order,
reverse-order power sums) and is used to cross-check the C++ oracle.

partition::partition (crate 0.1.2, source not available) is restated as the
two-pointer in-place partition: the k-th false element from the left is
swapped with the k-th true element from the right; the split is the number of
true elements.
"""
import numpy as np

f32 = np.float32
F32_MAX = f32(np.finfo(np.float32).max)
INVALID = 0xFFFFFFFF


def fmin(a, b):  # f32::min: ignores NaN
    if np.isnan(a):
        return b
    if np.isnan(b):
        return a
    return a if a < b else b


def fmax(a, b):
    if np.isnan(a):
        return b
    if np.isnan(b):
        return a
    return a if a > b else b


class Aabb:
    __slots__ = ("empty", "mn", "mx")

    def __init__(self, mn=None, mx=None):
        self.empty = mn is None
        self.mn = mn
        self.mx = mx

    @staticmethod
    def from_points(pts):  # aabb.rs:10-22
        mn = list(pts[0])
        mx = list(pts[0])
        for p in pts:
            mn = [fmin(mn[k], p[k]) for k in range(3)]
            mx = [fmax(mx[k], p[k]) for k in range(3)]
        return Aabb(mn, mx)

    @staticmethod
    def union(a, b):  # aabb.rs:24-42
        if a.empty:
            return b
        if b.empty:
            return a
        return Aabb([fmin(a.mn[k], b.mn[k]) for k in range(3)], [fmax(a.mx[k], b.mx[k]) for k in range(3)])

    def area(self):  # aabb.rs:44-52
        if self.empty:
            return f32(0.0)
        dx, dy, dz = (f32(self.mx[k] - self.mn[k]) for k in range(3))
        return f32(f32(2.0) * f32(f32(f32(dx * dy) + f32(dx * dz)) + f32(dy * dz)))

    def transform_translate(self, t):  # aabb.rs:75-92 for a pure translation
        if self.empty:
            return self
        lo = [f32(self.mn[k] + t[k]) for k in range(3)]
        hi = [f32(self.mx[k] + t[k]) for k in range(3)]
        corners = [[(hi if (c >> (2 - k)) & 1 else lo)[k] for k in range(3)] for c in range(8)]
        return Aabb.from_points(corners)


def bin_index(v):  # `as usize` saturating, then min(BINS-1)
    if np.isnan(v) or v <= 0:
        return 0
    if v >= 31:
        return 31
    return int(v)


def find_best_plane(first, count, idxs, cen, aabbs):  # build.rs:45-128
    BINS = 32
    best_cost = F32_MAX
    best_dim = 0
    best_split = f32(0.0)
    for d in range(3):
        bmin, bmax = F32_MAX, f32(-F32_MAX)
        for i in range(first, first + count):
            c = cen[idxs[i]][d]
            bmin = fmin(bmin, c)
            bmax = fmax(bmax, c)
        bb = [Aabb() for _ in range(BINS)]
        bc = [0] * BINS
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            scale = f32(f32(BINS) / f32(bmax - bmin))
            for i in range(first, first + count):
                p = idxs[i]
                b = min(BINS - 1, bin_index(f32(f32(cen[p][d] - bmin) * scale)))
                bc[b] += 1
                bb[b] = Aabb.union(bb[b], aabbs[p])
        pl, pr, cl, cr = [None] * 31, [None] * 31, [0] * 31, [0] * 31
        al, ar, nl, nr = Aabb(), Aabb(), 0, 0
        for plane in range(BINS - 1):
            nl += bc[plane]
            cl[plane] = nl
            al = Aabb.union(al, bb[plane])
            pl[plane] = al
            nr += bc[BINS - 1 - plane]
            cr[BINS - 2 - plane] = nr
            ar = Aabb.union(ar, bb[BINS - 1 - plane])
            pr[BINS - 2 - plane] = ar
        scale2 = f32(f32(bmax - bmin) / f32(BINS))
        for plane in range(BINS - 1):
            cost = f32(f32(pl[plane].area() * f32(cl[plane])) + f32(pr[plane].area() * f32(cr[plane])))
            if cost < best_cost:
                best_cost = cost
                best_dim = d
                best_split = f32(bmin + f32(f32(f32(plane) + f32(1.0)) * scale2))
    return best_dim, best_split


def partition(data, lo, n, pred):
    """in-place two-pointer partition of data[lo:lo+n]; returns the true count"""
    if n == 0:
        return 0
    l, r = 0, n - 1
    while True:
        while l < n and pred(data[lo + l]):
            l += 1
        while r > 0 and not pred(data[lo + r]):
            r -= 1
        if l >= r:
            return l
        data[lo + l], data[lo + r] = data[lo + r], data[lo + l]


class Node:
    __slots__ = ("aabb", "leaf", "parent", "first", "count", "left", "right")


def _insert(nodes, parent, first, count, idxs, aabbs):  # insert_blas_leaf_node, build.rs:235-247
    n = Node()
    b = Aabb()
    for i in range(first, first + count):
        b = Aabb.union(b, aabbs[idxs[i]])
    n.aabb, n.leaf, n.parent, n.first, n.count = b, True, parent, first, count
    nodes.append(n)
    return len(nodes) - 1


def subdivide(ni, idxs, aabbs, cen, nodes):  # build.rs:130-233
    nd = nodes[ni]
    if not nd.leaf:
        return
    if nd.count > 2:
        d, split = find_best_plane(nd.first, nd.count, idxs, cen, aabbs)
        nl = partition(idxs, nd.first, nd.count, lambda p: cen[p][d] < split)
        if nl == 0 or nl == nd.count:
            nl = nd.count // 2
        li = _insert(nodes, ni, nd.first, nl, idxs, aabbs)
        ri = _insert(nodes, ni, nd.first + nl, nd.count - nl, idxs, aabbs)
        subdivide(li, idxs, aabbs, cen, nodes)
        subdivide(ri, idxs, aabbs, cen, nodes)
        nd.leaf, nd.left, nd.right = False, li, ri
    elif nd.count == 2:
        li = _insert(nodes, ni, nd.first, 1, idxs, aabbs)
        ri = _insert(nodes, ni, nd.first + 1, 1, idxs, aabbs)
        nd.leaf, nd.left, nd.right = False, li, ri


def _flatten(nodes, idxs, aabbs, power, ids):
    out = []
    pad = f32(0.0001)
    for nd in nodes:
        if nd.leaf:
            assert nd.count == 1
            p = idxs[nd.first]
            a = aabbs[p]
            out.append([INVALID, int(ids[p]), list(a.mn), f32(power[p]), list(a.mx), nd.parent])
        else:
            out.append([nd.left, nd.right, [f32(v - pad) for v in nd.aabb.mn], f32(0.0),
                        [f32(v + pad) for v in nd.aabb.mx], nd.parent])
    for i in range(len(out) - 1, -1, -1):
        if out[i][0] != INVALID:
            p = f32(out[i][3])
            p = f32(p + out[out[i][0]][3])
            p = f32(p + out[out[i][1]][3])
            out[i][3] = p
    arr = np.zeros(len(out), dtype=[("left", "<u4"), ("right", "<u4"), ("min", "<f4", 3), ("power", "<f4"),
                                    ("max", "<f4", 3), ("parent", "<u4")])
    for i, o in enumerate(out):
        arr[i] = (o[0], o[1], o[2], o[3], o[4], o[5])
    return arr


def build_tl_bvh(aabbs6, power, ids, translations=None):  # build.rs:374-480
    n = len(aabbs6)
    t = np.zeros((n, 3), np.float32) if translations is None else np.asarray(translations, np.float32)
    aabbs = [Aabb([f32(v) for v in a[:3]], [f32(v) for v in a[3:]]).transform_translate(
        [f32(x) for x in t[i]]) for i, a in enumerate(aabbs6)]
    cen = [[f32(f32(a.mn[k] + a.mx[k]) / f32(2.0)) for k in range(3)] for a in aabbs]
    idxs = list(range(n))
    nodes = []
    _insert(nodes, INVALID, 0, n, idxs, aabbs)
    subdivide(0, idxs, aabbs, cen, nodes)
    return _flatten(nodes, idxs, aabbs, np.asarray(power, np.float32), ids), np.array(idxs, np.uint32)


def build_bl_bvh(tris9, lum, ids):  # build.rs:249-372
    n = len(tris9)
    pts = [[[f32(v) for v in t[3 * j:3 * j + 3]] for j in range(3)] for t in tris9]
    aabbs = [Aabb.from_points(p) for p in pts]
    cen = [[f32(f32(f32(p[0][k] + p[1][k]) + p[2][k]) / f32(3.0)) for k in range(3)] for p in pts]
    idxs = list(range(n))
    nodes = []
    _insert(nodes, INVALID, 0, n, idxs, aabbs)
    subdivide(0, idxs, aabbs, cen, nodes)
    return _flatten(nodes, idxs, aabbs, np.asarray(lum, np.float32), ids), np.array(idxs, np.uint32)
