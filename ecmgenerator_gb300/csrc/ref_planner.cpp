/*
 * ref_planner.cpp -- the reference's path planner, restated on the host:
 * ECMPathPlanner::FindPath (ECMGenerator/ECMPathPlanner.cpp:22-136) with
 * AStar::FindPath (AStar.cpp:44-160), CreateCorridor / ShrinkCorridor
 * (ECMPathPlanner.cpp:146-214), TriangulateCorridor / SampleCorridorArc /
 * FitPortalRange (ECMPathPlanner.cpp:216-318) and Funnel
 * (ECMPathPlanner.cpp:321-411), so that re-plans and spawns get the paths the
 * reference computes.  Every float expression keeps the reference's operand
 * order (this file is compiled with -ffp-contract=off).
 *
 * The reference's A* keeps pointers to its nodes in a std::priority_queue and
 * changes a node's cost after pushing it, so the order of the pops is that
 * of the heap algorithm run on keys that move.  The open list here is the
 * same binary heap -- sift-up on push; on pop the last element moves to the
 * root, the hole descends to a leaf along the child that compares first, and
 * the element sifts up from there (the algorithm of the C++ library the
 * reference is built with here) -- on node indices whose cost is read at
 * every comparison.
 */
#include "host_scene.h"

#include <algorithm>
#include <cmath>
#include <limits>

namespace ecmg {

namespace {

constexpr float kEpsR = 0.0001f; /* Utility::EPSILON (Configuration.h:14) */
constexpr float kMaxF = std::numeric_limits<float>::max();

/* MathUtility::Distance(p1, p2) (UtilityFunctions.cpp:15-22): p2 - p1 */
inline float r_dist(V2 p1, V2 p2)
{
    const float dx = p2.x - p1.x, dy = p2.y - p1.y;
    return std::sqrt(dx * dx + dy * dy);
}
/* a.Approximate(b) (ECMDataTypes.cpp:97-100) */
inline bool r_approx(V2 a, V2 b)
{
    return a.x < (b.x + kEpsR) && a.x > (b.x - kEpsR) && a.y < (b.y + kEpsR) && a.y > (b.y - kEpsR);
}
/* Point::operator== (ECMDataTypes.h:99-103): approximate */
inline bool r_eq(V2 a, V2 b)
{
    return a.x > b.x - kEpsR && a.x < b.x + kEpsR && a.y > b.y - kEpsR && a.y < b.y + kEpsR;
}
/* MathUtility::TriangleArea (UtilityFunctions.cpp:203-210) */
inline float r_area(V2 p1, V2 p2, V2 p3)
{
    const float ax = p2.x - p1.x, ay = p2.y - p1.y;
    const float bx = p3.x - p1.x, by = p3.y - p1.y;
    return bx * ay - ax * by;
}
/* MathUtility::IsLeftOfSegment (UtilityFunctions.cpp:193-196) */
inline bool r_left(V2 s0, V2 s1, V2 p) { return (s1.x - s0.x) * (p.y - s0.y) - (s1.y - s0.y) * (p.x - s0.x) > 0; }
/* Vec2::Normalize (ECMDataTypes.h:45-52): unchanged when the length is 0 */
inline V2 r_norm(V2 v)
{
    const float l = std::sqrt(v.x * v.x + v.y * v.y);
    if (l == 0.0f) return v;
    return mk(v.x / l, v.y / l);
}

struct Portal {
    V2 p0, p1;
};

/* the open list: a binary heap of node indices ordered by the nodes'
   current f costs ("a before b" when f[b] > f[a] is false for a > b ...):
   cmp(a, b) = f[a] > f[b], as AStarCompare (AStar.h) */
struct OpenList {
    std::vector<int>& h;
    const std::vector<float>& f;
    bool cmp(int a, int b) const { return f[a] > f[b]; }
    void sift_up(long hole, long top, int value)
    {
        long parent = (hole - 1) / 2;
        while (hole > top && cmp(h[parent], value)) {
            h[hole] = h[parent];
            hole = parent;
            parent = (hole - 1) / 2;
        }
        h[hole] = value;
    }
    void push(int v)
    {
        h.push_back(v);
        sift_up((long)h.size() - 1, 0, v);
    }
    int top() const { return h.front(); }
    void pop()
    {
        const long len = (long)h.size();
        if (len > 1) {
            const long n = len - 1; /* heap [0, n) after the move */
            const int value = h[n];
            h[n] = h[0];
            long hole = 0, child = 0;
            while (child < (n - 1) / 2) {
                child = 2 * (child + 1);
                if (cmp(h[child], h[child - 1])) child--;
                h[hole] = h[child];
                hole = child;
            }
            if ((n & 1) == 0 && child == (n - 2) / 2) {
                child = 2 * (child + 1);
                h[hole] = h[child - 1];
                hole = child - 1;
            }
            sift_up(hole, 0, value);
        }
        h.pop_back();
    }
};

/* AStar::FindPath (AStar.cpp:44-160) from the start edge's two vertices to
   either vertex of the goal edge; outPath as ConstructPath (AStar.cpp:183-210) */
bool ref_astar(const HostScene& s, RefPlanScratch& r, V2 startLoc, V2 goalLoc, int startEdge, int goalEdge,
               float clearance, std::vector<int>& out)
{
    const int V = (int)s.v_pos.size();
    const int INVALID = V;
    if ((int)r.g.size() != V) {
        r.g.assign(V, kMaxF);
        r.f.assign(V, kMaxF);
        r.parent.assign(V, INVALID);
        r.visited.assign(V, 0);
        r.touched.clear();
    }
    /* CleanRequestData (AStar.cpp:162-175) resets every node; resetting the
       nodes this search wrote (g, f or parent set, or visited) leaves the
       same state */
    auto clean = [&]() {
        for (int v : r.touched) {
            r.g[v] = kMaxF;
            r.f[v] = kMaxF;
            r.parent[v] = INVALID;
            r.visited[v] = 0;
        }
        r.touched.clear();
    };
    OpenList open{r.heap, r.f};
    r.heap.clear();
    const int sa = s.he_target[2 * startEdge], sb = s.he_target[2 * startEdge + 1];
    r.touched.push_back(sa);
    r.touched.push_back(sb);
    r.g[sa] = r_dist(startLoc, s.v_pos[sa]);
    r.f[sa] = r.g[sa] + r_dist(s.v_pos[sa], goalLoc);
    r.g[sb] = r_dist(startLoc, s.v_pos[sb]);
    r.f[sb] = r.g[sb] + r_dist(s.v_pos[sb], goalLoc);
    open.push(sa);
    open.push(sb);
    const int ga = s.he_target[2 * goalEdge], gb = s.he_target[2 * goalEdge + 1];
    while (!r.heap.empty()) {
        while (!r.heap.empty() && r.visited[open.top()]) open.pop();
        if (r.heap.empty()) {
            clean();
            return false;
        }
        const int cur = open.top();
        open.pop();
        r.visited[cur] = 1;
        if (s.v_clear[cur] < clearance) continue;
        if (cur == ga || cur == gb) {
            /* ConstructPath: the other goal vertex, the reached one, its
               ancestors; reversed */
            std::vector<int> rev;
            if (cur == ga) {
                rev.push_back(gb);
                rev.push_back(ga);
            } else {
                rev.push_back(ga);
                rev.push_back(gb);
            }
            for (int nx = r.parent[cur]; nx < INVALID; nx = r.parent[nx]) rev.push_back(nx);
            out.assign(rev.rbegin(), rev.rend());
            clean();
            return true;
        }
        /* the neighbours in the order of the outgoing half-edges, from the
           first one until its target comes round again */
        int he = s.v_halfedge[cur];
        if (he < 0) continue;
        const int first = s.he_target[he];
        int nb = first, guard = 0;
        do {
            if (!r.visited[nb]) {
                open.push(nb);
                const V2 cp = s.v_pos[cur], np = s.v_pos[nb];
                const float ng = r.g[cur] + r_dist(cp, np);
                if (ng < r.g[nb]) {
                    if (r.g[nb] == kMaxF) r.touched.push_back(nb);
                    r.parent[nb] = cur;
                    r.f[nb] = ng + r_dist(np, goalLoc);
                    r.g[nb] = ng;
                }
            }
            he = s.he_next[he];
            nb = s.he_target[he];
        } while (nb != first && ++guard < 4096);
    }
    clean();
    return false;
}

/* SampleCorridorArc (ECMPathPlanner.cpp:255-276) */
void sample_arc(V2 p1, V2 p2, V2 o1, V2 o2, V2 c, float radius, bool leftArc, std::vector<Portal>& portals)
{
    const float maxLen = 10.0f;
    if (leftArc) portals.push_back({p1, o1});
    else portals.push_back({o1, p1});
    const V2 d = mk(p2.x - p1.x, p2.y - p1.y);
    const float edgeLength = std::sqrt(d.x * d.x + d.y * d.y);
    const int numSamples = (int)std::ceil(edgeLength / maxLen);
    const float sampleLength = edgeLength / (float)numSamples;
    const V2 dir = mk(d.x / edgeLength, d.y / edgeLength);
    for (int i = 0; i < numSamples; i++) {
        const V2 step = mk(dir.x * sampleLength, dir.y * sampleLength);
        const float fi = (float)i;
        V2 p = mk(p1.x + step.x * fi, p1.y + step.y * fi);
        const V2 a = r_norm(mk(p.x - c.x, p.y - c.y));
        p = mk(c.x + a.x * radius, c.y + a.y * radius);
        if (leftArc) portals.push_back({p, o2});
        else portals.push_back({o2, p});
    }
}

/* Funnel (ECMPathPlanner.cpp:321-411), the simple stupid funnel algorithm */
void funnel(const std::vector<Portal>& portals, V2 start, V2 goal, std::vector<V2>& out)
{
    V2 apex = start, pl = start, pr = start;
    int leftIdx = 0, rightIdx = 0, apexIdx = 0;
    out.push_back(start);
    for (int i = 0; i < (int)portals.size(); i++) {
        const V2 left = portals[i].p0, right = portals[i].p1;
        if (r_area(apex, pr, right) <= 0.0f) {
            if (r_approx(apex, pr) || r_area(apex, pl, right) > 0.0f) {
                pr = right;
                rightIdx = i;
            } else {
                out.push_back(pl);
                apex = pl;
                apexIdx = leftIdx;
                pl = apex;
                pr = apex;
                leftIdx = apexIdx;
                rightIdx = apexIdx;
                i = apexIdx;
                continue;
            }
        }
        if (r_area(apex, pl, left) >= 0.0f) {
            if (r_approx(apex, pl) || r_area(apex, pr, left) < 0.0f) {
                pl = left;
                leftIdx = i;
            } else {
                out.push_back(pr);
                apex = pr;
                apexIdx = rightIdx;
                pl = apex;
                pr = apex;
                leftIdx = apexIdx;
                rightIdx = apexIdx;
                i = apexIdx;
                continue;
            }
        }
    }
    if (!r_approx(out.back(), goal)) out.push_back(goal);
}

}  // namespace

bool plan_path_reference(const HostScene& s, V2 start, V2 goal, float clearance, std::vector<V2>& out,
                         RefPlanScratch& r, int* astar_fail_edge)
{
    out.clear();
    if (astar_fail_edge) *astar_fail_edge = -1;
    if (!s.has_ecm) return false;
    const EcmView ev = s.ecm_view();
    /* 1. ECMGraph::FindCell (ECM.cpp:191-194) for start and goal */
    if (point_location(ev, start) < 0 || point_location(ev, goal) < 0) return false;
    /* 2. ECM::RetractPoint */
    V2 rs, rg;
    int es, eg;
    if (!retract(ev, start, &rs, &es)) return false;
    if (!retract(ev, goal, &rg, &eg)) return false;
    if (es == eg) {
        out.push_back(start);
        out.push_back(goal);
        return true;
    }
    /* 3. A* on the medial axis */
    std::vector<int> ap;
    if (!ref_astar(s, r, rs, rg, es, eg, clearance, ap)) {
        if (astar_fail_edge) *astar_fail_edge = es;
        return false;
    }
    /* the half-edges between consecutive vertices of the A* path */
    std::vector<int> hp;
    for (size_t i = 0; i + 1 < ap.size(); i++) {
        const int a = ap[i], b = ap[i + 1];
        const int h0 = s.v_halfedge[a];
        if (h0 < 0) continue;
        int h = h0, guard = 0;
        do {
            if (s.he_target[h] == b) {
                hp.push_back(h);
                break;
            }
            h = s.he_next[h];
        } while (h != h0 && ++guard < 4096);
    }
    if (hp.empty()) return false; /* the reference would read an empty corridor */
    /* 4. CreateCorridor + ShrinkCorridor (ECMPathPlanner.cpp:146-214) */
    const size_t n = hp.size();
    std::vector<V2> centers(n), lb(n), rb(n), lcb(n), rcb(n);
    std::vector<float> radii(n);
    std::vector<int> curve(n > 0 ? n - 1 : 0);
    for (size_t i = 0; i < n; i++) {
        const int h = hp[i];
        const int src = s.he_target[h ^ 1]; /* ECMGraph::GetSource: the twin's target */
        centers[i] = s.v_pos[src];
        radii[i] = s.v_clear[src];
        lb[i] = s.he_left[h];
        rb[i] = s.he_right[h];
    }
    auto shrink = [&](size_t i) {
        if (radii[i] < clearance) {
            lcb[i] = centers[i];
            rcb[i] = centers[i];
        } else {
            const V2 ml = r_norm(mk(centers[i].x - lb[i].x, centers[i].y - lb[i].y));
            const V2 mr = r_norm(mk(centers[i].x - rb[i].x, centers[i].y - rb[i].y));
            lcb[i] = mk(lb[i].x + ml.x * clearance, lb[i].y + ml.y * clearance);
            rcb[i] = mk(rb[i].x + mr.x * clearance, rb[i].y + mr.y * clearance);
        }
    };
    for (size_t i = 0; i + 1 < n; i++) {
        shrink(i);
        if (r_eq(lb[i], lb[i + 1])) curve[i] = 1;      /* LEFT_ARC */
        else if (r_eq(rb[i], rb[i + 1])) curve[i] = 2; /* RIGHT_ARC */
        else curve[i] = 0;                             /* LINEAR */
    }
    shrink(n - 1);
    /* 5. TriangulateCorridor (ECMPathPlanner.cpp:216-253) */
    std::vector<Portal> portals;
    for (size_t i = 0; i + 1 < n; i++) {
        if (curve[i] == 0) {
            portals.push_back({lcb[i], rcb[i]});
            portals.push_back({lcb[i + 1], rcb[i]});
        } else if (curve[i] == 1) {
            sample_arc(lcb[i], lcb[i + 1], rcb[i], rcb[i + 1], lb[i], clearance, true, portals);
        } else {
            sample_arc(rcb[i], rcb[i + 1], lcb[i], lcb[i + 1], rb[i], clearance, false, portals);
        }
    }
    portals.push_back({lcb[n - 1], rcb[n - 1]});
    /* FitPortalRange (ECMPathPlanner.cpp:278-318) */
    int first = 0;
    for (int i = 0; i < (int)portals.size(); i++)
        if (!r_left(portals[i].p0, portals[i].p1, start)) {
            first = i;
            break;
        }
    portals.erase(portals.begin(), portals.begin() + first);
    int last = (int)portals.size() - 1;
    for (int i = (int)portals.size() - 1; i >= 0; i--)
        if (r_left(portals[i].p0, portals[i].p1, goal)) {
            last = i;
            break;
        }
    const int toRemove = (int)portals.size() - last;
    for (int i = 0; i < toRemove; i++) portals.pop_back();
    portals.push_back({goal, goal});
    /* 7. Funnel */
    funnel(portals, start, goal, out);
    return true;
}

}  // namespace ecmg
