"""Seeded synthetic scenes and a host ECM builder.

The reference builds its scene in ``Environment`` (ECMGenerator/Environment.cpp:188-229)
and its Explicit Corridor Map with Boost.Polygon's segment Voronoi diagram
(ECMGenerator/ECMGenerator.cpp:60-256).  Boost is not available, so this module
builds the ECM from a point-sampled Voronoi diagram (scipy / Qhull):

* every obstacle segment (walkable-area border and box sides) is sampled at
  spacing ``h``; every segment interior and every corner is one *feature*;
* a Voronoi ridge is kept when its two sites belong to different features that
  are not a segment and its own end point (those ridges are the "secondary"
  edges that ECMGenerator.cpp:157 skips with ``is_primary()``), and both of its
  vertices lie in free space (ECMGenerator.cpp:107-130);
* chains of ridges that separate the same pair of features are merged into one
  ECM edge, split again where the chain leaves its chord by more than ``tol``;
* each half-edge stores the closest obstacle points at its source vertex, left
  and right of its direction, as ECMGenerator.cpp:173-195 does
  (``closest_left/right`` of half-edge 0 at vertex0, of half-edge 1 at vertex1).

The graph is returned as flat arrays in the layout of ``ECMGraph``
(ECMGenerator/ECM.h:20-116): half-edge ``2e+h`` of edge ``e``.  Construction is
host work, once per scene; it has no counterpart on the device.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

F32 = np.float32


@dataclass
class Ecm:
    v_pos: np.ndarray        # (V,2) f32  ECMVertex::position
    v_clear: np.ndarray      # (V,)  f32  ECMVertex::clearance
    v_idx: np.ndarray        # (V,)  i32  ECMVertex::idx
    v_halfedge: np.ndarray   # (V,)  i32  ECMVertex::half_edge_idx
    he_target: np.ndarray    # (2E,) i32
    he_next: np.ndarray      # (2E,) i32
    he_left: np.ndarray      # (2E,2) f32 closest_left
    he_right: np.ndarray     # (2E,2) f32 closest_right

    @property
    def n_vertices(self) -> int:
        return int(self.v_pos.shape[0])

    @property
    def n_edges(self) -> int:
        return int(self.he_target.shape[0] // 2)


@dataclass
class Scene:
    width: float
    height: float
    obst_off: np.ndarray     # (O+1,) i32 ring offsets
    obst_xy: np.ndarray      # (NV,2) f32 CCW rings (Simulator::AddObstacleArea order)
    obst_next: np.ndarray    # (NV,) i32
    obst_prev: np.ndarray    # (NV,) i32
    obst_convex: np.ndarray  # (NV,) u8  Obstacle::Initialize convexity
    walk: np.ndarray         # (4,4) f32 walkable-area segments
    boxes: np.ndarray        # (O,4) f64 cx, cy, hx, hy
    ecm: Ecm | None = None
    meta: dict = field(default_factory=dict)

    @property
    def n_obstacles(self) -> int:
        return int(self.obst_off.shape[0] - 1)


# --------------------------------------------------------------------------
# obstacles
# --------------------------------------------------------------------------

def box_ring(cx: float, cy: float, hx: float, hy: float) -> np.ndarray:
    """Vertex order of Simulator::AddObstacleArea (Simulator.cpp:404-407)."""
    return np.array([[cx + hx, cy + hy], [cx - hx, cy + hy],
                     [cx - hx, cy - hy], [cx + hx, cy - hy]], dtype=F32)


def ring_links(off: np.ndarray, xy: np.ndarray):
    """prev/next/convex exactly as Obstacle::Initialize (ECMDataTypes.cpp:23-61)."""
    nv = xy.shape[0]
    nxt = np.empty(nv, np.int32)
    prv = np.empty(nv, np.int32)
    cvx = np.empty(nv, np.uint8)
    for o in range(off.shape[0] - 1):
        a, b = int(off[o]), int(off[o + 1])
        n = b - a
        for i in range(n):
            prv[a + i] = a + (n - 1 if i == 0 else i - 1)
            nxt[a + i] = a + (1 if i == 0 else (i + 1) % n)
        for i in range(n):
            g = a + i
            if n == 2:
                cvx[g] = 1
                continue
            p, pp, pn = xy[g], xy[prv[g]], xy[nxt[g]]
            ax, ay = F32(pp[0] - pn[0]), F32(pp[1] - pn[1])
            bx, by = F32(p[0] - pp[0]), F32(p[1] - pp[1])
            det = F32(F32(ax * by) - F32(ay * bx))
            cvx[g] = 1 if det >= F32(0.0) else 0
    return nxt, prv, cvx


def gen_boxes(rng: np.random.Generator, w: float, h: float, n: int, side_lo: float, side_hi: float,
              gap: float = 2.0, wall_gap: float = 2.0, max_tries: int = 200000) -> np.ndarray:
    """Axis-aligned boxes, sides U[side_lo, side_hi], centres uniform; a box is
    rejected when its gap to another box (or to the border) is below ``gap``."""
    boxes = []
    cell = side_hi + gap
    grid: dict[tuple[int, int], list[int]] = {}
    tries = 0
    while len(boxes) < n and tries < max_tries:
        tries += 1
        sx, sy = rng.uniform(side_lo, side_hi, 2)
        hx, hy = 0.5 * sx, 0.5 * sy
        cx = rng.uniform(wall_gap + hx, w - wall_gap - hx)
        cy = rng.uniform(wall_gap + hy, h - wall_gap - hy)
        gx, gy = int(cx // cell), int(cy // cell)
        ok = True
        for ix in range(gx - 1, gx + 2):
            for iy in range(gy - 1, gy + 2):
                for j in grid.get((ix, iy), ()):
                    bx, by, bhx, bhy = boxes[j]
                    dx = abs(cx - bx) - hx - bhx
                    dy = abs(cy - by) - hy - bhy
                    d = math.hypot(max(dx, 0.0), max(dy, 0.0))
                    if d < gap:
                        ok = False
                        break
                if not ok:
                    break
            if not ok:
                break
        if ok:
            grid.setdefault((gx, gy), []).append(len(boxes))
            boxes.append((cx, cy, hx, hy))
    return np.array(boxes, dtype=np.float64).reshape(-1, 4)


def make_scene(w: float, h: float, boxes: np.ndarray) -> Scene:
    rings = [box_ring(*b) for b in boxes]
    off = np.zeros(len(rings) + 1, np.int32)
    for i, r in enumerate(rings):
        off[i + 1] = off[i] + r.shape[0]
    xy = np.concatenate(rings, 0) if rings else np.zeros((0, 2), F32)
    nxt, prv, cvx = ring_links(off, xy)
    walk = np.array([[0, 0, w, 0], [w, 0, w, h], [0, h, w, h], [0, h, 0, 0]], dtype=F32)
    return Scene(float(w), float(h), off, xy.astype(F32), nxt, prv, cvx, walk, boxes)


# --------------------------------------------------------------------------
# free-space queries (float64 geometry, scene setup only)
# --------------------------------------------------------------------------

class BoxIndex:
    """Uniform-grid index over boxes for distance-to-obstacle queries."""

    def __init__(self, scene: Scene, cell: float = 16.0):
        self.s = scene
        self.cell = cell
        self.map: dict[tuple[int, int], list[int]] = {}
        for i, (cx, cy, hx, hy) in enumerate(scene.boxes):
            for ix in range(int((cx - hx) // cell), int((cx + hx) // cell) + 1):
                for iy in range(int((cy - hy) // cell), int((cy + hy) // cell) + 1):
                    self.map.setdefault((ix, iy), []).append(i)

    def clearance(self, x: np.ndarray, y: np.ndarray, reach: float = 16.0) -> np.ndarray:
        """Distance to the nearest box side or border, capped at ``reach``;
        negative inside a box."""
        s = self.s
        d = np.minimum.reduce([x, y, s.width - x, s.height - y]).astype(np.float64)
        d = np.minimum(d, reach)
        if s.boxes.shape[0] == 0:
            return d
        b = s.boxes
        r = int(math.ceil(reach / self.cell))
        gx = np.floor(x / self.cell).astype(np.int64)
        gy = np.floor(y / self.cell).astype(np.int64)
        keys = {}
        for i in range(x.shape[0]):
            keys.setdefault((int(gx[i]), int(gy[i])), []).append(i)
        for (kx, ky), idx in keys.items():
            cand = set()
            for ix in range(kx - r, kx + r + 1):
                for iy in range(ky - r, ky + r + 1):
                    cand.update(self.map.get((ix, iy), ()))
            if not cand:
                continue
            c = np.fromiter(cand, np.int64)
            idx = np.asarray(idx)
            dx = np.abs(x[idx, None] - b[None, c, 0]) - b[None, c, 2]
            dy = np.abs(y[idx, None] - b[None, c, 1]) - b[None, c, 3]
            out = np.hypot(np.maximum(dx, 0), np.maximum(dy, 0))
            inside = (dx < 0) & (dy < 0)
            out = np.where(inside, np.maximum(dx, dy), out)
            d[idx] = np.minimum(d[idx], out.min(1))
        return d


def sample_free(rng, scene: Scene, n: int, radius: np.ndarray | float, bidx: BoxIndex,
                region=None, no_overlap: bool = True, margin: float = 0.0, max_rounds: int = 400):
    """Uniform points whose disk lies in free space; optionally without
    disk-disk overlap (rejection sampling on a hash grid)."""
    if region is None:
        region = (0.0, 0.0, scene.width, scene.height)
    x0, y0, x1, y1 = region
    rad = np.broadcast_to(np.asarray(radius, np.float64), (n,)).copy()
    out = np.zeros((n, 2), np.float64)
    done = np.zeros(n, bool)
    cell = 1.0
    occ: dict[tuple[int, int], list[int]] = {}
    rmax = float(rad.max()) if n else 0.0
    for _ in range(max_rounds):
        todo = np.nonzero(~done)[0]
        if todo.size == 0:
            break
        px = rng.uniform(x0, x1, todo.size)
        py = rng.uniform(y0, y1, todo.size)
        clr = bidx.clearance(px, py, reach=rmax + margin + 1.0)
        good = clr >= rad[todo] + margin
        if not no_overlap:
            sel = todo[good]
            out[sel, 0], out[sel, 1] = px[good], py[good]
            done[sel] = True
            continue
        for j in np.nonzero(good)[0]:
            i = int(todo[j])
            if no_overlap:
                kx, ky = int(px[j] // cell), int(py[j] // cell)
                hit = False
                span = int(math.ceil(2 * rmax / cell))
                for ix in range(kx - span, kx + span + 1):
                    for iy in range(ky - span, ky + span + 1):
                        for q in occ.get((ix, iy), ()):
                            if (out[q, 0] - px[j]) ** 2 + (out[q, 1] - py[j]) ** 2 < (rad[q] + rad[i]) ** 2:
                                hit = True
                                break
                        if hit:
                            break
                    if hit:
                        break
                if hit:
                    continue
                occ.setdefault((kx, ky), []).append(i)
            out[i] = (px[j], py[j])
            done[i] = True
    if not done.all():
        raise RuntimeError(f"could only place {int(done.sum())} of {n} points")
    return out


# --------------------------------------------------------------------------
# ECM builder
# --------------------------------------------------------------------------

def _segments(scene: Scene):
    """Obstacle union of Environment::AddWalkableArea/AddObstacle
    (Environment.cpp:188-229): border segments then every ring edge."""
    segs = [tuple(map(float, s)) for s in scene.walk]
    for o in range(scene.n_obstacles):
        a, b = int(scene.obst_off[o]), int(scene.obst_off[o + 1])
        for i in range(a, b):
            j = a + (i - a + 1) % (b - a)
            segs.append((float(scene.obst_xy[i, 0]), float(scene.obst_xy[i, 1]),
                         float(scene.obst_xy[j, 0]), float(scene.obst_xy[j, 1])))
    return np.array(segs, np.float64)


def _closest_on_seg(p, a, b):
    d = b - a
    L = float(d @ d)
    if L == 0.0:
        return a.copy()
    t = float((p - a) @ d) / L
    t = min(1.0, max(0.0, t))
    return a + t * d


def build_ecm(scene: Scene, h: float = 0.2, tol: float = 0.3) -> Ecm:
    from scipy.spatial import Voronoi

    segs = _segments(scene)
    S = segs.shape[0]
    # corner features: unique segment end points
    ends = np.concatenate([segs[:, 0:2], segs[:, 2:4]], 0)
    key = np.round(ends * 1e4).astype(np.int64)
    uniq, inv = np.unique(key, axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    corner_pt = np.zeros((uniq.shape[0], 2))
    corner_pt[inv] = ends
    seg_c0 = inv[:S]
    seg_c1 = inv[S:]
    C = uniq.shape[0]
    # sites
    pts = [corner_pt]
    feat = [S + np.arange(C)]
    for s in range(S):
        a, b = segs[s, 0:2], segs[s, 2:4]
        L = float(np.hypot(*(b - a)))
        m = max(1, int(math.ceil(L / h)))
        t = (np.arange(1, m) / m)[:, None]
        if t.size:
            pts.append(a + t * (b - a))
            feat.append(np.full(t.shape[0], s))
    P = np.concatenate(pts, 0)
    Fe = np.concatenate(feat, 0).astype(np.int64)
    vor = Voronoi(P)
    V = vor.vertices
    rp = vor.ridge_points
    rv = np.array(vor.ridge_vertices, dtype=np.int64)
    fa, fb = Fe[rp[:, 0]], Fe[rp[:, 1]]
    keep = (rv[:, 0] >= 0) & (rv[:, 1] >= 0) & (fa != fb)
    # secondary ridges: a segment and its own end point
    def is_secondary(f1, f2):
        seg_f = np.where(f1 < S, f1, f2)
        cor_f = np.where(f1 < S, f2, f1) - S
        one_seg = (f1 < S) != (f2 < S)
        segc = np.clip(seg_f, 0, S - 1)
        return one_seg & ((seg_c0[segc] == cor_f) | (seg_c1[segc] == cor_f))
    keep &= ~is_secondary(fa, fb)
    # free-space test of Voronoi vertices
    bidx = BoxIndex(scene)
    vfree = np.zeros(V.shape[0], bool)
    used = np.unique(rv[keep].reshape(-1))
    cl = bidx.clearance(V[used, 0], V[used, 1], reach=4.0)
    vfree[used] = cl > 1e-6
    keep &= vfree[rv[:, 0]] & vfree[rv[:, 1]]
    rv, fa, fb, rp = rv[keep], fa[keep], fb[keep], rp[keep]
    # orient each ridge: left site of v0 -> v1
    d = V[rv[:, 1]] - V[rv[:, 0]]
    s0 = P[rp[:, 0]] - V[rv[:, 0]]
    left_is_a = (d[:, 0] * s0[:, 1] - d[:, 1] * s0[:, 0]) > 0
    fl = np.where(left_is_a, fa, fb)
    fr = np.where(left_is_a, fb, fa)
    # adjacency
    R = rv.shape[0]
    adj: dict[int, list[int]] = {}
    for r in range(R):
        adj.setdefault(int(rv[r, 0]), []).append(r)
        adj.setdefault(int(rv[r, 1]), []).append(r)

    def pair(r):
        return (min(fl[r], fr[r]), max(fl[r], fr[r]))

    junction = set()
    for v, rs in adj.items():
        if len(rs) != 2 or pair(rs[0]) != pair(rs[1]):
            junction.add(v)
    visited = np.zeros(R, bool)
    chains = []  # (vertex list, left feature, right feature)

    def walk(v_start, r0):
        verts = [v_start]
        r = r0
        v = v_start
        # orientation of the first ridge relative to the walk
        if rv[r, 0] == v:
            left, right = fl[r], fr[r]
        else:
            left, right = fr[r], fl[r]
        while True:
            visited[r] = True
            nv = int(rv[r, 1] if rv[r, 0] == v else rv[r, 0])
            verts.append(nv)
            v = nv
            if v in junction:
                break
            nr = [q for q in adj[v] if not visited[q]]
            if not nr:
                break
            r = nr[0]
        return verts, left, right

    for v in sorted(junction):
        for r in adj[v]:
            if not visited[r]:
                chains.append(walk(v, r))
    for r in range(R):  # closed loops without junctions
        if not visited[r]:
            v = int(rv[r, 0])
            junction.add(v)
            chains.append(walk(v, r))

    # split chains that bend away from their chord (Douglas-Peucker)
    def split(vs):
        out_, stack = [], [vs]
        while stack:
            cur = stack.pop()
            if len(cur) <= 2:
                out_.append(cur)
                continue
            pts_ = V[cur]
            a, b = pts_[0], pts_[-1]
            ab = b - a
            L = math.hypot(*ab)
            if L == 0:
                dist = np.hypot(*(pts_ - a).T)
            else:
                dist = np.abs(ab[0] * (pts_[:, 1] - a[1]) - ab[1] * (pts_[:, 0] - a[0])) / L
            i = int(np.argmax(dist))
            if dist[i] <= tol or i == 0 or i == len(cur) - 1:
                out_.append(cur)
                continue
            stack.append(cur[i:])
            stack.append(cur[: i + 1])
        return out_

    edges = []
    for vs, l, r in chains:
        for piece in split(vs):
            if piece[0] != piece[-1]:
                edges.append((piece[0], piece[-1], l, r))
    # compact vertex ids, spatially ordered (Morton-like) for locality
    vids = sorted({e[0] for e in edges} | {e[1] for e in edges})
    vpos64 = V[vids]
    order = np.lexsort((vpos64[:, 0], np.floor(vpos64[:, 1] / 8.0)))
    remap = {vids[o]: i for i, o in enumerate(order)}
    vpos = vpos64[order]
    nV = vpos.shape[0]
    edges = [(remap[a], remap[b], l, r) for a, b, l, r in edges]
    mid = np.array([(vpos[a] + vpos[b]) * 0.5 for a, b, _, _ in edges]).reshape(-1, 2)
    eorder = np.lexsort((mid[:, 0], np.floor(mid[:, 1] / 8.0))) if len(edges) else np.zeros(0, np.int64)
    edges = [edges[i] for i in eorder]
    E = len(edges)

    # A vertex where a corner's wedge meets the cell of one of that corner's
    # own segments lies, in the exact diagram, on the segment's normal through
    # the corner.  The sampled diagram puts it within ~h of that line; moving
    # it onto the line makes the spoke to the corner perpendicular to the
    # segment, so the corner triangle and the segment quad share one spoke and
    # retraction rays (perpendicular to the segment) stay inside the quad.
    vfeat: dict[int, set] = {}
    for a_, b_, l_, r_ in edges:
        for v_ in (a_, b_):
            vfeat.setdefault(v_, set()).update((l_, r_))
    for v_, fs in vfeat.items():
        for f in fs:
            if f < S:
                continue
            c = corner_pt[f - S]
            for sg in fs:
                if sg >= S or (seg_c0[sg] != f - S and seg_c1[sg] != f - S):
                    continue
                d = segs[sg, 2:4] - segs[sg, 0:2]
                L2 = float(d @ d)
                if L2 == 0.0:
                    continue
                t = float((vpos[v_] - c) @ d) / L2
                if abs(t) * math.sqrt(L2) < 2.0 * h:
                    vpos[v_] = vpos[v_] - t * d
                break

    def feat_point(f, p):
        if f >= S:
            return corner_pt[f - S].copy()
        a, b = segs[f, 0:2], segs[f, 2:4]
        q = _closest_on_seg(p, a, b)
        # snap onto the segment's end point when the foot is within reach of it:
        # keeps the corner wedge and the segment cell sharing one spoke
        for c in (a, b):
            if math.hypot(*(q - c)) < 1.5 * h:
                return c.copy()
        return q

    he_target = np.zeros(2 * E, np.int32)
    he_left = np.zeros((2 * E, 2), np.float64)
    he_right = np.zeros((2 * E, 2), np.float64)
    vclear = np.full(nV, np.inf)
    for e, (a, b, l, r) in enumerate(edges):
        pa, pb = vpos[a], vpos[b]
        la, ra = feat_point(l, pa), feat_point(r, pa)
        lb, rb = feat_point(l, pb), feat_point(r, pb)
        he_target[2 * e] = b
        he_left[2 * e], he_right[2 * e] = la, ra
        he_target[2 * e + 1] = a
        he_left[2 * e + 1], he_right[2 * e + 1] = rb, lb
        vclear[a] = min(vclear[a], math.hypot(*(pa - la)), math.hypot(*(pa - ra)))
        vclear[b] = min(vclear[b], math.hypot(*(pb - lb)), math.hypot(*(pb - rb)))
    # rotation order of outgoing half-edges (ECMGenerator.cpp:211-255)
    out: dict[int, list[int]] = {}
    for e, (a, b, _, _) in enumerate(edges):
        out.setdefault(a, []).append(2 * e)      # half-edge 0 leaves vertex a
        out.setdefault(b, []).append(2 * e + 1)  # half-edge 1 leaves vertex b
    he_next = np.zeros(2 * E, np.int32)
    v_he = np.full(nV, -1, np.int32)
    for v, hes in out.items():
        ang = []
        for q in hes:
            t = he_target[q]
            dd = vpos[t] - vpos[v]
            ang.append(math.atan2(dd[1], dd[0]))
        hs = [hes[i] for i in np.argsort(ang)]
        for i, q in enumerate(hs):
            he_next[q] = hs[(i + 1) % len(hs)]
        v_he[v] = hs[0]
    return Ecm(v_pos=vpos.astype(F32), v_clear=vclear.astype(F32), v_idx=np.arange(nV, dtype=np.int32),
               v_halfedge=v_he, he_target=he_target, he_next=he_next,
               he_left=he_left.astype(F32), he_right=he_right.astype(F32))
