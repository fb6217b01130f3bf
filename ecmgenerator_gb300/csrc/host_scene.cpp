/*
 * host_scene.cpp -- host side of the static scene: obstacle rings, ECM
 * point-location grid, obstacle candidate grid and the path planner.
 * Compiled with -ffp-contract=off so that the shared geometry in
 * ecmg_geom.cuh rounds as on the device.
 */
#include "host_scene.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <queue>

namespace ecmg {

EcmView HostScene::ecm_view() const
{
    EcmView e{};
    e.v_pos = v_pos.data();
    e.v_idx = v_idx.data();
    e.he_target = he_target.data();
    e.he_left = he_left.data();
    e.he_right = he_right.data();
    e.n_edges = (int)(he_target.size() / 2);
    e.gx0 = ecm_grid.x0;
    e.gy0 = ecm_grid.y0;
    e.ginv = ecm_grid.inv;
    e.gw = ecm_grid.gw;
    e.gh = ecm_grid.gh;
    e.g_start = ecm_grid.start.data();
    e.g_items = ecm_grid.items.data();
    e.special_y = special_y.data();
    e.n_special = (int)special_y.size();
    e.sp_start = sp_start.data();
    e.sp_items = sp_items.data();
    e.sp_bloom = sp_bloom.empty() ? nullptr : sp_bloom.data();
    return e;
}

ObstView HostScene::obst_view(const GridCSR* g) const
{
    ObstView o{};
    o.p = ob_p.data();
    o.next = ob_next.data();
    o.prev = ob_prev.data();
    o.convex = ob_convex.data();
    o.n_verts = (int)ob_p.size();
    if (g && g->gw > 0) {
        o.gx0 = g->x0;
        o.gy0 = g->y0;
        o.ginv = g->inv;
        o.gw = g->gw;
        o.gh = g->gh;
        o.reach = g->reach;
        o.g_start = g->start.data();
        o.g_items = g->items.data();
    }
    return o;
}

void set_obstacles(HostScene& s, int n_obst, const int* off, const float* xy)
{
    int nv = n_obst > 0 ? off[n_obst] : 0;
    s.ob_p.resize(nv);
    s.ob_next.resize(nv);
    s.ob_prev.resize(nv);
    s.ob_convex.resize(nv);
    s.ob_ring_off.assign(off, off + n_obst + 1);
    for (int i = 0; i < nv; i++) s.ob_p[i] = mk(xy[2 * i], xy[2 * i + 1]);
    for (int o = 0; o < n_obst; o++) {
        int a = off[o], n = off[o + 1] - a;
        for (int i = 0; i < n; i++) {
            int g = a + i;
            /* Obstacle::Initialize: i == 0 links to verts[n-1] and verts[1] */
            s.ob_prev[g] = a + (i == 0 ? n - 1 : i - 1);
            s.ob_next[g] = a + (i == 0 ? 1 % n : (i + 1) % n);
        }
        for (int i = 0; i < n; i++) {
            int g = a + i;
            if (n == 2) { s.ob_convex[g] = 1; continue; }
            V2 p = s.ob_p[g], pp = s.ob_p[s.ob_prev[g]], pn = s.ob_p[s.ob_next[g]];
            s.ob_convex[g] = det(pp - pn, p - pp) >= 0.0f ? 1 : 0;
        }
    }
}

static void bbox_grow(float& x0, float& y0, float& x1, float& y1, V2 p)
{
    x0 = std::min(x0, p.x);
    y0 = std::min(y0, p.y);
    x1 = std::max(x1, p.x);
    y1 = std::max(y1, p.y);
}

/* Landmarks for the planner's A* (the ALT bound): graph distances from a
   few vertices spread over the ECM (each the vertex farthest, by graph
   distance, from those chosen before).  For every vertex pair,
   |d(L, v) - d(L, t)| <= d(v, t), a lower bound of the remaining route that
   is much closer to it than the straight line when obstacles force
   detours.  Edge lengths are the search's own. */
static void build_landmarks(HostScene& s)
{
    const int V = (int)s.v_pos.size();
    s.n_land = 0;
    s.land_d.clear();
    if (V == 0) return;
    const int L = std::min(8, V);
    const float INF = std::numeric_limits<float>::infinity();
    std::vector<float> best(V, INF); /* distance to the nearest chosen landmark */
    std::vector<double> d(V);
    s.land_d.assign((size_t)V * L, INF);
    auto elen = [&](int v, int w) {
        V2 a = s.v_pos[v], b = s.v_pos[w];
        return std::sqrt((a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y));
    };
    /* the first landmark: the vertex farthest from the ECM's centroid */
    double cx = 0, cy = 0;
    for (auto& p : s.v_pos) { cx += p.x; cy += p.y; }
    cx /= V; cy /= V;
    int next = 0;
    double far = -1;
    for (int v = 0; v < V; v++) {
        double dd = (s.v_pos[v].x - cx) * (s.v_pos[v].x - cx) + (s.v_pos[v].y - cy) * (s.v_pos[v].y - cy);
        if (dd > far) { far = dd; next = v; }
    }
    typedef std::pair<double, int> QE;
    for (int l = 0; l < L; l++) {
        std::fill(d.begin(), d.end(), std::numeric_limits<double>::infinity());
        std::priority_queue<QE, std::vector<QE>, std::greater<QE>> q;
        d[next] = 0;
        q.push(QE(0.0, next));
        while (!q.empty()) {
            QE e = q.top();
            q.pop();
            int v = e.second;
            if (e.first > d[v]) continue;
            int h0 = s.v_halfedge[v];
            if (h0 < 0) continue;
            int h = h0, guard = 0;
            do {
                int w = s.he_target[h];
                double nd = d[v] + elen(v, w);
                if (nd < d[w]) {
                    d[w] = nd;
                    q.push(QE(nd, w));
                }
                h = s.he_next[h];
            } while (h != h0 && ++guard < 1024);
        }
        for (int v = 0; v < V; v++) {
            s.land_d[(size_t)v * L + l] = std::isfinite(d[v]) ? (float)d[v] : INF;
            if (std::isfinite(d[v])) best[v] = std::min(best[v], (float)d[v]);
        }
        /* the next one: the connected vertex farthest from all chosen */
        float bf = -1;
        for (int v = 0; v < V; v++)
            if (std::isfinite(best[v]) && best[v] > bf) { bf = best[v]; next = v; }
    }
    s.n_land = L;
}

void build_ecm_grid(HostScene& s)
{
    build_landmarks(s);
    int E = (int)(s.he_target.size() / 2);
    int C = 2 * E;
    EcmView ev = s.ecm_view();
    std::vector<V2> q(4 * (size_t)C);
    float x0 = std::numeric_limits<float>::max(), y0 = x0, x1 = -x0, y1 = -x0;
    std::vector<float> ys;
    ys.reserve(4 * (size_t)C);
    for (int c = 0; c < C; c++) {
        cell_quad(ev, c, &q[4 * (size_t)c]);
        for (int k = 0; k < 4; k++) {
            bbox_grow(x0, y0, x1, y1, q[4 * (size_t)c + k]);
            ys.push_back(q[4 * (size_t)c + k].y);
        }
    }
    std::sort(ys.begin(), ys.end());
    ys.erase(std::unique(ys.begin(), ys.end()), ys.end());
    s.special_y = ys;
    s.sp_bloom.assign(2048, 0u);
    for (float y : ys) {
        unsigned h = sp_hash(y);
        s.sp_bloom[h >> 5] |= 1u << (h & 31u);
    }
    /* per special height, the quads with a corner there (ascending) */
    {
        std::vector<int> cnt(ys.size() + 1, 0);
        std::vector<int> idx(4 * (size_t)C);
        for (int c = 0; c < C; c++) {
            for (int k = 0; k < 4; k++) {
                float y = q[4 * (size_t)c + k].y;
                int si = (int)(std::lower_bound(ys.begin(), ys.end(), y) - ys.begin());
                bool dup = false;
                for (int k2 = 0; k2 < k; k2++) dup |= idx[4 * (size_t)c + k2] == si;
                idx[4 * (size_t)c + k] = dup ? -1 : si;
                if (!dup) cnt[si + 1]++;
            }
        }
        for (size_t i = 1; i < cnt.size(); i++) cnt[i] += cnt[i - 1];
        s.sp_start = cnt;
        s.sp_items.assign(std::max(1, cnt.back()), 0);
        std::vector<int> fill(cnt.begin(), cnt.end() - 1);
        for (int c = 0; c < C; c++)
            for (int k = 0; k < 4; k++) {
                int si = idx[4 * (size_t)c + k];
                if (si >= 0) s.sp_items[fill[si]++] = c;
            }
    }
    if (C == 0) {
        s.ecm_grid = GridCSR();
        s.ecm_grid.start.assign(2, 0);
        s.ecm_grid.gw = s.ecm_grid.gh = 1;
        return;
    }
    float maxc = std::max(std::max(std::fabs(x0), std::fabs(x1)), std::max(std::fabs(y0), std::fabs(y1)));
    /* margin covers the rounding of the x-intersection in the ray-cast test and
       of the query's cell index (coordinates stay far below 1e5) */
    float margin = 0.01f + 1e-6f * maxc;
    float area = (x1 - x0) * (y1 - y0);
    float cell = std::sqrt(std::max(area, 1.0f) / (float)C) * 1.5f;
    cell = std::min(std::max(cell, 0.5f), 64.0f);
    GridCSR& g = s.ecm_grid;
    g.x0 = x0 - 2 * margin;
    g.y0 = y0 - 2 * margin;
    g.cell = cell;
    g.inv = 1.0f / cell;
    g.gw = std::max(1, (int)std::ceil((x1 - g.x0 + 2 * margin) / cell) + 1);
    g.gh = std::max(1, (int)std::ceil((y1 - g.y0 + 2 * margin) / cell) + 1);
    size_t ng = (size_t)g.gw * g.gh;
    std::vector<int> cnt(ng + 1, 0);
    auto range = [&](int c, int& ix0, int& iy0, int& ix1, int& iy1) {
        float a0 = std::numeric_limits<float>::max(), b0 = a0, a1 = -a0, b1 = -a0;
        for (int k = 0; k < 4; k++) bbox_grow(a0, b0, a1, b1, q[4 * (size_t)c + k]);
        ix0 = std::max(0, (int)std::floor((a0 - margin - g.x0) * g.inv));
        iy0 = std::max(0, (int)std::floor((b0 - margin - g.y0) * g.inv));
        ix1 = std::min(g.gw - 1, (int)std::floor((a1 + margin - g.x0) * g.inv));
        iy1 = std::min(g.gh - 1, (int)std::floor((b1 + margin - g.y0) * g.inv));
    };
    for (int c = 0; c < C; c++) {
        int ix0, iy0, ix1, iy1;
        range(c, ix0, iy0, ix1, iy1);
        for (int y = iy0; y <= iy1; y++)
            for (int x = ix0; x <= ix1; x++) cnt[(size_t)y * g.gw + x]++;
    }
    g.start.assign(ng + 1, 0);
    for (size_t i = 0; i < ng; i++) g.start[i + 1] = g.start[i] + cnt[i];
    g.items.assign((size_t)g.start[ng], 0);
    std::vector<int> cur(g.start.begin(), g.start.end() - 1);
    for (int c = 0; c < C; c++) { /* ascending c -> ascending lists */
        int ix0, iy0, ix1, iy1;
        range(c, ix0, iy0, ix1, iy1);
        for (int y = iy0; y <= iy1; y++)
            for (int x = ix0; x <= ix1; x++) g.items[(size_t)cur[(size_t)y * g.gw + x]++] = c;
    }
}

static double seg_rect_dist(V2 a, V2 b, double rx0, double ry0, double rx1, double ry1)
{
    /* distance between segment ab and an axis-aligned rectangle (double) */
    auto inside = [&](double x, double y) { return x >= rx0 && x <= rx1 && y >= ry0 && y <= ry1; };
    if (inside(a.x, a.y) || inside(b.x, b.y)) return 0.0;
    auto pt_seg = [](double px, double py, double ax, double ay, double bx, double by) {
        double dx = bx - ax, dy = by - ay, L = dx * dx + dy * dy;
        double t = L > 0 ? ((px - ax) * dx + (py - ay) * dy) / L : 0.0;
        t = std::min(1.0, std::max(0.0, t));
        double qx = ax + t * dx - px, qy = ay + t * dy - py;
        return std::sqrt(qx * qx + qy * qy);
    };
    auto seg_seg_cross = [](double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy) {
        auto orient = [](double px, double py, double qx, double qy, double rx, double ry) {
            return (qx - px) * (ry - py) - (qy - py) * (rx - px);
        };
        double o1 = orient(ax, ay, bx, by, cx, cy), o2 = orient(ax, ay, bx, by, dx, dy);
        double o3 = orient(cx, cy, dx, dy, ax, ay), o4 = orient(cx, cy, dx, dy, bx, by);
        return ((o1 > 0) != (o2 > 0)) && ((o3 > 0) != (o4 > 0));
    };
    double cs[4][2] = {{rx0, ry0}, {rx1, ry0}, {rx1, ry1}, {rx0, ry1}};
    double d = std::numeric_limits<double>::max();
    for (int k = 0; k < 4; k++) {
        const double* p = cs[k];
        const double* q = cs[(k + 1) & 3];
        if (seg_seg_cross(a.x, a.y, b.x, b.y, p[0], p[1], q[0], q[1])) return 0.0;
        d = std::min(d, pt_seg(p[0], p[1], a.x, a.y, b.x, b.y));
    }
    d = std::min(d, pt_seg(a.x, a.y, rx0, ry0, rx1, ry0));
    d = std::min(d, pt_seg(a.x, a.y, rx1, ry0, rx1, ry1));
    d = std::min(d, pt_seg(a.x, a.y, rx1, ry1, rx0, ry1));
    d = std::min(d, pt_seg(a.x, a.y, rx0, ry1, rx0, ry0));
    d = std::min(d, pt_seg(b.x, b.y, rx0, ry0, rx1, ry0));
    d = std::min(d, pt_seg(b.x, b.y, rx1, ry0, rx1, ry1));
    d = std::min(d, pt_seg(b.x, b.y, rx1, ry1, rx0, ry1));
    d = std::min(d, pt_seg(b.x, b.y, rx0, ry1, rx0, ry0));
    return d;
}

void build_obst_grid(const HostScene& s, float reach, float cell, GridCSR& g)
{
    int nv = (int)s.ob_p.size();
    float x0 = s.bx0, y0 = s.by0, x1 = s.bx1, y1 = s.by1;
    for (int i = 0; i < nv; i++) bbox_grow(x0, y0, x1, y1, s.ob_p[i]);
    float pad = reach + cell;
    g.reach = reach;
    g.cell = cell;
    g.inv = 1.0f / cell;
    g.x0 = x0 - pad;
    g.y0 = y0 - pad;
    g.gw = std::max(1, (int)std::ceil((x1 + pad - g.x0) / cell));
    g.gh = std::max(1, (int)std::ceil((y1 + pad - g.y0) / cell));
    size_t ng = (size_t)g.gw * g.gh;
    const double margin = 0.05; /* float rounding of the exact in-range test */
    std::vector<std::vector<int>> lists(ng);
    for (int i = 0; i < nv; i++) { /* ascending vertex id -> ascending lists */
        V2 a = s.ob_p[i], b = s.ob_p[s.ob_next[i]];
        double r = (double)reach + margin;
        int ix0 = std::max(0, (int)std::floor((std::min(a.x, b.x) - r - g.x0) / cell));
        int iy0 = std::max(0, (int)std::floor((std::min(a.y, b.y) - r - g.y0) / cell));
        int ix1 = std::min(g.gw - 1, (int)std::floor((std::max(a.x, b.x) + r - g.x0) / cell));
        int iy1 = std::min(g.gh - 1, (int)std::floor((std::max(a.y, b.y) + r - g.y0) / cell));
        for (int y = iy0; y <= iy1; y++)
            for (int x = ix0; x <= ix1; x++) {
                double rx0 = (double)g.x0 + (double)x * cell, ry0 = (double)g.y0 + (double)y * cell;
                if (seg_rect_dist(a, b, rx0, ry0, rx0 + cell, ry0 + cell) <= r) lists[(size_t)y * g.gw + x].push_back(i);
            }
    }
    g.start.assign(ng + 1, 0);
    for (size_t i = 0; i < ng; i++) g.start[i + 1] = g.start[i] + (int)lists[i].size();
    g.items.clear();
    g.items.reserve((size_t)g.start[ng]);
    for (auto& l : lists) g.items.insert(g.items.end(), l.begin(), l.end());
}

/* ---------------------------------------------------------------------- */
static double pt_seg_d(V2 p, V2 a, V2 b)
{
    double dx = (double)b.x - a.x, dy = (double)b.y - a.y, L = dx * dx + dy * dy;
    double t = L > 0 ? (((double)p.x - a.x) * dx + ((double)p.y - a.y) * dy) / L : 0.0;
    t = std::min(1.0, std::max(0.0, t));
    double qx = a.x + t * dx - p.x, qy = a.y + t * dy - p.y;
    return std::sqrt(qx * qx + qy * qy);
}

static bool segs_cross(V2 a, V2 b, V2 c, V2 d)
{
    auto orient = [](V2 p, V2 q, V2 r) {
        return ((double)q.x - p.x) * ((double)r.y - p.y) - ((double)q.y - p.y) * ((double)r.x - p.x);
    };
    double o1 = orient(a, b, c), o2 = orient(a, b, d), o3 = orient(c, d, a), o4 = orient(c, d, b);
    return ((o1 > 0) != (o2 > 0)) && ((o3 > 0) != (o4 > 0));
}

/* straight piece a->b keeps `clr` from every obstacle edge near it; each
   edge is tested once per call (it may be listed in several cells) */
static bool clear_line(const HostScene& s, const GridCSR& g, V2 a, V2 b, double clr, PlanScratch& scr)
{
    if (g.gw == 0) return true;
    if (scr.ob_stamp.size() != s.ob_p.size()) {
        scr.ob_stamp.assign(s.ob_p.size(), 0);
        scr.ob_gen = 0;
    }
    const unsigned gen = ++scr.ob_gen;
    if (gen == 0) std::fill(scr.ob_stamp.begin(), scr.ob_stamp.end(), 0u);
    /* an edge whose bounding box is farther than clr (plus a rounding
       margin) from the segment's on either axis neither crosses it nor comes
       closer than clr: skipping it leaves the result unchanged */
    const double sx0 = std::min(a.x, b.x), sx1 = std::max(a.x, b.x);
    const double sy0 = std::min(a.y, b.y), sy1 = std::max(a.y, b.y);
    const double far = clr + 1e-6 + 1e-9 * std::max(std::max(std::fabs(sx0), std::fabs(sx1)),
                                                     std::max(std::fabs(sy0), std::fabs(sy1)));
    double pad = clr + 0.01;
    int iy0 = std::max(0, (int)std::floor((std::min(a.y, b.y) - pad - g.y0) * g.inv));
    int iy1 = std::min(g.gh - 1, (int)std::floor((std::max(a.y, b.y) + pad - g.y0) * g.inv));
    const double ax = a.x, ay = a.y, bx = b.x, by = b.y;
    const double cell = 1.0 / g.inv;
    /* only the cells within pad of the segment: per grid row, the x-range of
       the part of the segment whose y lies within pad of the row (a superset
       of the cells closer than pad, so every obstacle edge closer than clr is
       tested; the bounding box of a long diagonal would hold far more) */
    for (int y = iy0; y <= iy1; y++) {
        const double ylo = g.y0 + y * cell - pad, yhi = g.y0 + (y + 1) * cell + pad;
        double t0 = 0.0, t1 = 1.0;
        if (by != ay) {
            double ta = (ylo - ay) / (by - ay), tb = (yhi - ay) / (by - ay);
            if (ta > tb) std::swap(ta, tb);
            t0 = std::max(t0, ta);
            t1 = std::min(t1, tb);
            if (t0 > t1) continue;
        } else if (ay < ylo || ay > yhi) {
            continue;
        }
        const double xa = ax + (bx - ax) * t0, xb = ax + (bx - ax) * t1;
        int ix0 = std::max(0, (int)std::floor((std::min(xa, xb) - pad - g.x0) * g.inv) - 1);
        int ix1 = std::min(g.gw - 1, (int)std::floor((std::max(xa, xb) + pad - g.x0) * g.inv) + 1);
        for (int x = ix0; x <= ix1; x++) {
            size_t c = (size_t)y * g.gw + x;
            for (int q = g.start[c]; q < g.start[c + 1]; q++) {
                int i = g.items[(size_t)q];
                if (scr.ob_stamp[i] == gen) continue;
                scr.ob_stamp[i] = gen;
                V2 c0 = s.ob_p[i], c1 = s.ob_p[s.ob_next[i]];
                const double cx0 = std::min(c0.x, c1.x), cx1 = std::max(c0.x, c1.x);
                const double cy0 = std::min(c0.y, c1.y), cy1 = std::max(c0.y, c1.y);
                if (cx0 - sx1 >= far || sx0 - cx1 >= far || cy0 - sy1 >= far || sy0 - cy1 >= far) continue;
                if (segs_cross(a, b, c0, c1)) return false;
                double d = std::min(std::min(pt_seg_d(a, c0, c1), pt_seg_d(b, c0, c1)),
                                    std::min(pt_seg_d(c0, a, b), pt_seg_d(c1, a, b)));
                if (d < clr) return false;
            }
        }
    }
    /* the walkable rectangle's border */
    double lo = std::min(std::min(a.x - s.bx0, b.x - s.bx0), std::min(a.y - s.by0, b.y - s.by0));
    double hi = std::min(std::min(s.bx1 - a.x, s.bx1 - b.x), std::min(s.by1 - a.y, s.by1 - b.y));
    return std::min(lo, hi) >= clr;
}

bool plan_path(const HostScene& s, const GridCSR& vis, V2 start, V2 goal, float clearance,
               std::vector<V2>& out, PlanScratch& scr, int* astar_fail_edge)
{
    out.clear();
    if (astar_fail_edge) *astar_fail_edge = -1;
    if (!s.has_ecm) return false;
    EcmView ev = s.ecm_view();
    V2 rs, rg;
    int es, eg;
    if (!retract(ev, start, &rs, &es)) return false;
    if (!retract(ev, goal, &rg, &eg)) return false;
    if (es == eg) { /* ECMPathPlanner.cpp:74-80 */
        out.push_back(start);
        out.push_back(goal);
        return true;
    }
    int V = (int)s.v_pos.size();
    if ((int)scr.g.size() != V) {
        scr.g.assign(V, 0.0f);
        scr.parent.assign(V, -1);
        scr.stamp.assign(V, 0);
        scr.closed.assign(V, 0);
        scr.gen = 0;
    }
    int gen = ++scr.gen;
    auto touch = [&](int v) {
        if (scr.stamp[v] != gen) {
            scr.stamp[v] = gen;
            scr.g[v] = std::numeric_limits<float>::max();
            scr.parent[v] = -1;
            scr.closed[v] = 0;
        }
    };
    auto dist = [](V2 a, V2 b) { return std::sqrt((a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y)); };
    /* Heuristic: the search ends at a vertex t of the goal's edge, with
       f = g(t) + |t - goal|, so the remaining cost from v is at least
       min over t of (d(v, t) + |t - goal|) >= |v - goal|.  d(v, t) is bounded
       below by |v - t| and by the landmark bound (scaled down by 1e-5 for
       float rounding); both bounds are consistent, so A* stays optimal. */
    const int nl = s.n_land;
    float tl[2][8];
    V2 tp[2];
    float tg[2];
    int tv[2];
    auto h_of = [&](int v) -> float {
        float h = dist(s.v_pos[v], goal);
        if (nl == 0) return h;
        const float* dv = s.land_d.data() + (size_t)v * nl;
        float hm = std::numeric_limits<float>::infinity();
        for (int t = 0; t < 2; t++) {
            float lb = dist(s.v_pos[v], tp[t]);
            for (int l = 0; l < nl; l++) {
                const float a = dv[l], b = tl[t][l];
                if (std::isfinite(a) && std::isfinite(b)) lb = std::max(lb, std::fabs(a - b) * 0.99999f);
            }
            hm = std::min(hm, lb + tg[t]);
        }
        return std::max(h, hm);
    };
    typedef std::pair<float, int> QE;
    /* min-heap on (f, vertex): a total order, so the pops are those of any
       other min-heap; the storage is reused from search to search */
    std::vector<QE>& open = scr.open;
    open.clear();
    const std::greater<QE> later;
    auto push = [&](QE e) {
        open.push_back(e);
        std::push_heap(open.begin(), open.end(), later);
    };
    int sa = s.he_target[2 * es], sb = s.he_target[2 * es + 1];
    int ga = s.he_target[2 * eg], gb = s.he_target[2 * eg + 1];
    tv[0] = ga;
    tv[1] = gb;
    for (int t = 0; t < 2; t++) {
        tp[t] = s.v_pos[tv[t]];
        tg[t] = dist(tp[t], goal);
        for (int l = 0; l < nl; l++) tl[t][l] = s.land_d[(size_t)tv[t] * nl + l];
    }
    for (int v : {sa, sb}) {
        touch(v);
        float g0 = dist(start, s.v_pos[v]);
        if (g0 < scr.g[v]) {
            scr.g[v] = g0;
            push(QE(g0 + h_of(v), v));
        }
    }
    int found = -1;
    while (!open.empty()) {
        std::pop_heap(open.begin(), open.end(), later);
        QE top = open.back();
        open.pop_back();
        int v = top.second;
        if (scr.closed[v]) continue;
        scr.closed[v] = 1;
        if (s.v_clear[v] < clearance) continue; /* AStar.cpp:103 */
        if (v == ga || v == gb) { found = v; break; }
        int h0 = s.v_halfedge[v];
        if (h0 < 0) continue;
        int h = h0, guard = 0;
        do {
            int w = s.he_target[h];
            touch(w);
            if (!scr.closed[w]) {
                float ng = scr.g[v] + dist(s.v_pos[v], s.v_pos[w]);
                if (ng < scr.g[w]) {
                    scr.g[w] = ng;
                    scr.parent[w] = v;
                    push(QE(ng + h_of(w), w));
                }
            }
            h = s.he_next[h];
        } while (h != h0 && ++guard < 1024);
    }
    if (found < 0) {
        if (astar_fail_edge) *astar_fail_edge = es;
        return false;
    }
    std::vector<V2> pts;
    pts.push_back(goal);
    for (int v = found; v >= 0; v = scr.parent[v]) pts.push_back(s.v_pos[v]);
    pts.push_back(start);
    std::reverse(pts.begin(), pts.end());
    /* greedy shortening */
    double clr = (double)clearance;
    out.push_back(pts[0]);
    size_t i = 0;
    while (i + 1 < pts.size()) {
        size_t j = i + 1;
        while (j + 1 < pts.size() && clear_line(s, vis, pts[i], pts[j + 1], clr, scr)) j++;
        out.push_back(pts[j]);
        i = j;
    }
    return true;
}

}  // namespace ecmg
