"""Seeded synthetic scenes and the host ECM builders.

The reference builds its scene in ``Environment`` (ECMGenerator/Environment.cpp:188-229)
and its Explicit Corridor Map with Boost.Polygon's segment Voronoi diagram
(ECMGenerator/ECMGenerator.cpp:60-256).  Boost is not available; both builders
here start from a point-sampled Voronoi diagram (scipy / Qhull):

* every obstacle segment (walkable-area border and box sides) is sampled at
  spacing ``h``; every segment interior and every corner is one *feature*;
* a Voronoi ridge is kept when its two sites belong to different features that
  are not a segment and its own end point (those ridges are the "secondary"
  edges that ECMGenerator.cpp:157 skips with ``is_primary()``), and both of its
  vertices lie in free space (ECMGenerator.cpp:107-130);
* chains of ridges that separate the same pair of features, from junction to
  junction, are the diagram's edges.

``build_ecm_exact`` (``cfg["ecm"] = "exact"``) turns every chain into one
straight edge between exact Voronoi vertices, each solved as the point
equidistant from the features that meet there -- the graph the reference builds
from Boost's diagram.  ``build_ecm`` (the workloads' default) keeps the
sampled vertices and splits chains where they leave their chord by more than
``tol``, so that a curved bisector is followed to within ``tol``.  Each half-edge
stores the closest obstacle points at its source vertex, left and right of its
direction, as ECMGenerator.cpp:173-195 does (``closest_left/right`` of
half-edge 0 at vertex0, of half-edge 1 at vertex1).

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
    meta: dict = field(default_factory=dict)

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


class _Diagram:
    """The point-sampled Voronoi diagram of an obstacle union, reduced to
    chains: maximal runs of kept ridges that separate the same two features
    (segment interiors 0..S-1, corner points S..S+C-1), from junction to
    junction."""

    def __init__(self, scene: Scene, h: float, segs: np.ndarray, end_eps: float = 0.0):
        """segs: the obstacle union; h: sample spacing; end_eps > 0 adds a
        sample that far from each end of every segment, so that the boundary
        between a corner's cell and its own segment's cell (the segment's
        normal through the corner) is placed to within end_eps / 2"""
        from scipy.spatial import Voronoi

        self.segs = segs
        S = self.S = segs.shape[0]
        # corner features: unique segment end points
        ends = np.concatenate([segs[:, 0:2], segs[:, 2:4]], 0)
        key = np.round(ends * 1e4).astype(np.int64)
        uniq, inv = np.unique(key, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        corner_pt = np.zeros((uniq.shape[0], 2))
        corner_pt[inv] = ends
        self.corner_pt = corner_pt
        self.seg_c0 = seg_c0 = inv[:S]
        self.seg_c1 = seg_c1 = inv[S:]
        C = uniq.shape[0]
        # sites
        pts = [corner_pt]
        feat = [S + np.arange(C)]
        for s in range(S):
            a, b = segs[s, 0:2], segs[s, 2:4]
            L = float(np.hypot(*(b - a)))
            m = max(1, int(math.ceil(L / h)))
            t = np.arange(1, m) / m
            if end_eps > 0.0 and L > 4.0 * end_eps:
                t = np.concatenate([[end_eps / L], t, [1.0 - end_eps / L]])
            t = t[:, None]
            if t.size:
                pts.append(a + t * (b - a))
                feat.append(np.full(t.shape[0], s))
        P = np.concatenate(pts, 0)
        Fe = np.concatenate(feat, 0).astype(np.int64)
        vor = Voronoi(P)
        self.V = V = vor.vertices
        rp = vor.ridge_points
        rv = np.array(vor.ridge_vertices, dtype=np.int64)
        fa, fb = Fe[rp[:, 0]], Fe[rp[:, 1]]
        finite = (rv[:, 0] >= 0) & (rv[:, 1] >= 0)
        # the features whose sites generate each Voronoi vertex (every ridge
        # around it, kept or not)
        gv = np.concatenate([rv[:, 0], rv[:, 0], rv[:, 1], rv[:, 1]])
        gf = np.concatenate([fa, fb, fa, fb])
        self._gen_v, self._gen_f = gv[gv >= 0], gf[gv >= 0]
        keep = finite & (fa != fb)
        keep &= ~self.is_secondary(fa, fb)
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
        self.chains = self._chains(rv, fl, fr)

    def is_secondary(self, f1, f2):
        """a segment and its own end point (ECMGenerator.cpp:157 skips these
        edges with is_primary())"""
        S = self.S
        seg_f = np.where(f1 < S, f1, f2)
        cor_f = np.where(f1 < S, f2, f1) - S
        one_seg = (f1 < S) != (f2 < S)
        segc = np.clip(seg_f, 0, S - 1)
        return one_seg & ((self.seg_c0[segc] == cor_f) | (self.seg_c1[segc] == cor_f))

    def generators(self, v: int) -> list[int]:
        """distinct features of the sites around sampled vertex v"""
        if not hasattr(self, "_gen"):
            order = np.argsort(self._gen_v, kind="stable")
            gv, gf = self._gen_v[order], self._gen_f[order]
            b = np.searchsorted(gv, np.arange(self.V.shape[0] + 1))
            self._gen = (gf, b)
        gf, b = self._gen
        return sorted(set(int(f) for f in gf[b[v]:b[v + 1]]))

    @staticmethod
    def _chains(rv, fl, fr):
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
            return verts, int(left), int(right)

        for v in sorted(junction):
            for r in adj[v]:
                if not visited[r]:
                    chains.append(walk(v, r))
        for r in range(R):  # closed loops without junctions
            if not visited[r]:
                v = int(rv[r, 0])
                junction.add(v)
                chains.append(walk(v, r))
        return chains


def build_ecm(scene: Scene, h: float = 0.2, tol: float = 0.3) -> Ecm:
    segs = _segments(scene)
    D = _Diagram(scene, h, segs)
    S, V, corner_pt, seg_c0, seg_c1, chains = D.S, D.V, D.corner_pt, D.seg_c0, D.seg_c1, D.chains

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
    def snap(vpos, edges):
        # A vertex where a corner's wedge meets the cell of one of that
        # corner's own segments lies, in the exact diagram, on the segment's
        # normal through the corner.  The sampled diagram puts it within ~h of
        # that line; moving it onto the line makes the spoke to the corner
        # perpendicular to the segment, so the corner triangle and the segment
        # quad share one spoke and retraction rays (perpendicular to the
        # segment) stay inside the quad.
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

    return _assemble(V, edges, feat_point, snap)


def _solve_vertex(D: _Diagram, feats: list, x0: np.ndarray, h: float):
    """The point equidistant from the features `feats` (segment interiors as
    lines, corners as points) nearest the sampled vertex x0 (Newton on the
    differences of the distances, least squares beyond three features).
    Returns (point, ok)."""
    S, segs = D.S, D.segs
    # a corner together with two of its own segments: the corner itself (a
    # walkable-area corner, where the border's two bisected sides meet)
    for f in feats:
        if f >= S:
            c = f - S
            own = [g for g in feats if g < S and (D.seg_c0[g] == c or D.seg_c1[g] == c)]
            if len(own) >= 2:
                return D.corner_pt[c].copy(), True
    lines = {}
    for f in feats:
        if f < S:
            a, b = segs[f, 0:2], segs[f, 2:4]
            t = b - a
            n = np.array([-t[1], t[0]]) / math.hypot(t[0], t[1])
            if float(n @ (x0 - a)) < 0.0:
                n = -n
            lines[f] = (a, n)
    x = np.array(x0, np.float64)
    ok = False
    for _ in range(60):
        ds, gs = [], []
        for f in feats:
            if f >= S:
                d = x - D.corner_pt[f - S]
                r = math.hypot(d[0], d[1])
                ds.append(r)
                gs.append(d / r if r > 0.0 else np.zeros(2))
            else:
                a, n = lines[f]
                ds.append(float(n @ (x - a)))
                gs.append(n)
        A = np.array([gs[i] - gs[0] for i in range(1, len(feats))])
        res = np.array([ds[i] - ds[0] for i in range(1, len(feats))])
        dx = np.linalg.lstsq(A, -res, rcond=None)[0]
        x = x + dx
        if math.hypot(dx[0], dx[1]) <= 1e-12 * max(1.0, math.hypot(x[0], x[1])):
            ok = True
            break
    if ok:
        ds = [math.hypot(*(x - D.corner_pt[f - S])) if f >= S else float(lines[f][1] @ (x - lines[f][0]))
              for f in feats]
        ok = min(ds) > 0.0 and max(ds) - min(ds) <= 1e-9 * max(1.0, max(ds)) and math.hypot(*(x - x0)) < 4.0 * h
    return x, ok


def build_ecm_exact(scene: Scene, h: float = 0.2, int_sites: bool = False) -> Ecm:
    """The ECM of the exact segment Voronoi diagram of the obstacle union, the
    graph ECMGenerator::ConstructECMGraph (ECMGenerator.cpp:60-232) builds
    from Boost.Polygon's diagram: one straight edge per primary Voronoi edge
    in free space, between its two Voronoi vertices, curved edges included.

    The topology comes from the point-sampled diagram (`_Diagram`: which
    features meet at which vertex, which two features each edge separates);
    every vertex is then solved exactly as the point equidistant from its
    generating features, so vertex positions and clearances are those of the
    segment diagram (to double precision) rather than of the samples, and a
    bisector between two features is one edge however curved.  The samples
    must be dense enough to separate the vertices (spacing h well below the
    shortest Voronoi edge that matters).  With int_sites the diagram is built
    on the coordinates truncated to integers, as construct_voronoi sees them
    through the reference's int point_traits (ECMGenerator.cpp:37-44); closest
    points and the free-space test use the scene's own coordinates
    (ECMGenerator.cpp:84-105, 259-277)."""
    segs = _segments(scene)
    site = np.trunc(segs) if int_sites else segs
    D = _Diagram(scene, h, site, end_eps=1e-4)
    S = D.S
    cache: dict[int, np.ndarray | None] = {}

    def vert(v):
        if v not in cache:
            feats = D.generators(v)
            x = None
            if len(feats) >= 3:
                x, ok = _solve_vertex(D, feats, D.V[v], h)
                if not ok:
                    x = None
            cache[v] = x
        return cache[v]

    pts: list[np.ndarray] = []
    ids: dict[tuple[int, int], int] = {}

    def vid(x):
        k = (int(round(x[0] * 1e6)), int(round(x[1] * 1e6)))  # one micrometre
        if k not in ids:
            ids[k] = len(pts)
            pts.append(x)
        return ids[k]

    bidx = BoxIndex(scene)
    edges, seen = [], set()
    dropped = 0
    for vs, l, r in D.chains:
        xa, xb = vert(vs[0]), vert(vs[-1])
        if xa is None or xb is None:
            dropped += 1
            continue
        a, b = vid(xa), vid(xb)
        if a == b or (a, b, l, r) in seen or (b, a, r, l) in seen:
            continue
        seen.add((a, b, l, r))
        edges.append((a, b, l, r))
    P = np.array(pts, np.float64).reshape(-1, 2)
    # vertices strictly inside an obstacle are not ECM vertices
    # (ECMGenerator.cpp:84-87); corners of the walkable area are
    inside = np.zeros(P.shape[0], bool)
    if P.shape[0] and scene.boxes.shape[0]:
        b = scene.boxes
        for i in range(P.shape[0]):
            dx = np.abs(P[i, 0] - b[:, 0]) - b[:, 2]
            dy = np.abs(P[i, 1] - b[:, 1]) - b[:, 3]
            inside[i] = bool(np.any((dx < 0) & (dy < 0)))
    edges = [e for e in edges if not inside[e[0]] and not inside[e[1]]]
    # a corner's own point: the corner of the scene's segment it belongs to
    corner_src = np.zeros((D.corner_pt.shape[0], 2))
    corner_src[D.seg_c1] = segs[:, 2:4]
    corner_src[D.seg_c0] = segs[:, 0:2]

    def feat_point(f, p):
        """GetClosestPointsToSource (ECMGenerator.cpp:259-277)"""
        if f >= S:
            return corner_src[f - S].copy()
        return _closest_on_seg(p, segs[f, 0:2], segs[f, 2:4])

    e = _assemble(P, edges, feat_point)
    e.meta = dict(builder="exact segment Voronoi", h=h, int_sites=int_sites, unresolved_chains=dropped)
    return e


def _assemble(V: np.ndarray, edges: list, feat_point, adjust=None) -> Ecm:
    """ECM arrays from straight edges (a, b, left feature, right feature)
    between rows of V: vertices and edges in a spatial order, half-edge 2e
    from a to b and 2e+1 back, each with the closest obstacle points left and
    right of its direction at its source vertex (ECMGenerator.cpp:173-195),
    and the rotation order of the half-edges around every vertex
    (ECMGenerator.cpp:211-255).  adjust(vpos, edges) may move vertices after
    the renumbering."""
    # compact vertex ids, spatially ordered (Morton-like) for locality
    vids = sorted({e[0] for e in edges} | {e[1] for e in edges})
    vpos64 = V[vids] if vids else np.zeros((0, 2))
    order = np.lexsort((vpos64[:, 0], np.floor(vpos64[:, 1] / 8.0)))
    remap = {vids[o]: i for i, o in enumerate(order)}
    vpos = vpos64[order].copy()
    nV = vpos.shape[0]
    edges = [(remap[a], remap[b], l, r) for a, b, l, r in edges]
    mid = np.array([(vpos[a] + vpos[b]) * 0.5 for a, b, _, _ in edges]).reshape(-1, 2)
    eorder = np.lexsort((mid[:, 0], np.floor(mid[:, 1] / 8.0))) if len(edges) else np.zeros(0, np.int64)
    edges = [edges[i] for i in eorder]
    E = len(edges)
    if adjust is not None:
        adjust(vpos, edges)

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
