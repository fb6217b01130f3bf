/*
 * ecmg_geom.cuh -- per-agent geometry of the crowd tick, compiled for the
 * device (tick kernels) and for the host (planner, setup).
 *
 * Every function restates one reference function with the same sequence of
 * binary32 operations, so that the tick computes what the reference computes
 * on the same inputs; the source location is given above each function.
 * Translation units that include this header are built without fused
 * multiply-add (-fmad=false for nvcc, -ffp-contract=off for g++).
 */
#ifndef ECMG_GEOM_CUH
#define ECMG_GEOM_CUH

#include "ecmg_tmath.h"

#include <math.h>

#if defined(__CUDACC__)
#define EG_HD __host__ __device__ __forceinline__
#define EG_NI static __host__ __device__ __noinline__
#else
#include <cmath>
#define EG_HD inline
#define EG_NI inline
#ifndef __align__
#define __align__(n) __attribute__((aligned(n)))
#endif
#endif

namespace ecmg {

constexpr float kEps = 0.0001f; /* Utility::EPSILON, ECMGenerator/Configuration.h:14 */

struct __align__(8) V2 {
    float x, y;
};

EG_HD V2 mk(float x, float y) { V2 r; r.x = x; r.y = y; return r; }
/* Vec2/Point operators, ECMGenerator/ECMDataTypes.h:20-98 */
EG_HD V2 operator+(V2 a, V2 b) { return mk(a.x + b.x, a.y + b.y); }
EG_HD V2 operator-(V2 a, V2 b) { return mk(a.x - b.x, a.y - b.y); }
EG_HD V2 operator*(V2 a, float s) { return mk(a.x * s, a.y * s); }
EG_HD V2 operator/(V2 a, float s) { return mk(a.x / s, a.y / s); }
/* MathUtility, ECMGenerator/UtilityFunctions.cpp:170-262 */
EG_HD float dot(V2 a, V2 b) { return a.x * b.x + a.y * b.y; }
EG_HD float det(V2 a, V2 b) { return a.x * b.y - a.y * b.x; }
EG_HD float len2(V2 a) { return a.x * a.x + a.y * a.y; }
EG_HD float len(V2 a) { return sqrtf(a.x * a.x + a.y * a.y); }
EG_HD V2 right(V2 a) { return mk(a.y, -a.x); }
EG_HD V2 left(V2 a) { return mk(-a.y, a.x); }
/* Vec2::Normalize (ECMDataTypes.h:45-52) */
EG_HD V2 normalize(V2 a)
{
    float l = len(a);
    if (l == 0.0f) return a;
    a.x /= l;
    a.y /= l;
    return a;
}
/* Vec2::Normalized (ECMDataTypes.h:54-60); zero vector -> (0,0) */
EG_HD V2 normalized(V2 a)
{
    float l = len(a);
    if (l == 0.0f) return mk(0.0f, 0.0f);
    return mk(a.x / l, a.y / l);
}
/* Point::Approximate (ECMDataTypes.cpp:97-100) */
EG_HD bool approx(V2 p, V2 a)
{
    return p.x < (a.x + kEps) && p.x > (a.x - kEps) && p.y < (a.y + kEps) && p.y > (a.y - kEps);
}
/* MathUtility::SquareDistance(Point, Point) (UtilityFunctions.cpp:32-39) */
EG_HD float sqdist(V2 p1, V2 p2)
{
    float dx = p2.x - p1.x, dy = p2.y - p1.y;
    return dx * dx + dy * dy;
}
/* MathUtility::GetClosestPointOnSegment (UtilityFunctions.cpp:287-306) */
EG_HD V2 closest_on_segment(V2 point, V2 s1, V2 s2)
{
    if (approx(s1, s2)) return s1;
    V2 seg = s2 - s1;
    V2 pts = point - s1;
    float tsq = sqdist(s1, s2);
    float d = (pts.x * seg.x + pts.y * seg.y) / tsq;
    if (d > 1.0f) d = 1.0f;
    if (d < 0.0f) d = 0.0f;
    return mk(s1.x + d * seg.x, s1.y + d * seg.y);
}
/* MathUtility::RotateVector (UtilityFunctions.cpp:233-242) with the
   deterministic sin/cos of ecmg_tmath.h */
EG_HD V2 rotate(V2 v, float rad)
{
    float sn, cs;
    ecmg_sincosf(rad, &sn, &cs);
    return mk(v.x * cs - v.y * sn, v.x * sn + v.y * cs);
}

/* ------------------------------------------------------------------------
 * ECM (ECMGenerator/ECM.h), flattened.  Cell c: edge c>>1, left (even) or
 * right (odd) side (ECMCellCollection::Construct, ECMCellCollection.cpp:10-49).
 * ---------------------------------------------------------------------- */
struct EcmView {
    const V2* v_pos;
    const int* v_idx;
    const int* he_target;
    const V2* he_left;
    const V2* he_right;
    int n_edges;
    /* point-location grid over the cell quads: cell g lists, in ascending
       order, every ECM cell whose bounding box (grown by a margin) meets g */
    float gx0, gy0, ginv;
    int gw, gh;
    const int* g_start;   /* gw*gh + 1 */
    const int* g_items;
    /* sorted distinct y of all quad corners.  At such a height the ray-cast
       test can report a hit left of a quad's bounding box, but only for the
       quads with a corner at that height: sp_items[sp_start[s] ..
       sp_start[s+1]) lists them (ascending) for special_y[s]. */
    const float* special_y;
    int n_special;
    const int* sp_start;
    const int* sp_items;
    /* 65536-bit filter of the special heights (bit sp_hash(y) set for each):
       a clear bit proves that y is not special (null: no filter) */
    const unsigned* sp_bloom;
};

/* bit index of a height in the filter; -0 and +0 hash alike (they compare equal) */
EG_HD unsigned sp_hash(float y)
{
    union {
        float f;
        unsigned u;
    } b;
    b.f = (y == 0.0f) ? 0.0f : y;
    return (b.u * 2654435769u) >> 16;
}

/* quad of PointLocationQueryLinear (ECMCellCollection.cpp:67-80):
   [v(he1.target), boundary.p0, boundary.p1, v(he0.target)] */
EG_HD void cell_quad(const EcmView& e, int c, V2* q)
{
    int ed = c >> 1;
    int h0 = 2 * ed, h1 = 2 * ed + 1;
    V2 b0, b1;
    if ((c & 1) == 0) { b0 = e.he_left[h0]; b1 = e.he_right[h1]; }
    else { b0 = e.he_right[h0]; b1 = e.he_left[h1]; }
    q[0] = e.v_pos[e.he_target[h1]];
    q[1] = b0;
    q[2] = b1;
    q[3] = e.v_pos[e.he_target[h0]];
}

/* MathUtility::Contains(Point, vector<Segment>) (UtilityFunctions.cpp:54-86) */
EG_HD bool contains_quad(V2 p, const V2* q)
{
    bool inside = false;
#pragma unroll
    for (int s = 0; s < 4; s++) {
        V2 a = q[s], b = q[(s + 1) & 3];
        if (approx(p, a)) return false;
        if (approx(p, b)) return false;
        if (p.y > fminf(a.y, b.y)) {
            if (p.y < fmaxf(a.y, b.y)) {
                if (p.x < fmaxf(a.x, b.x)) {
                    float xi = (p.y - a.y) * (b.x - a.x) / (b.y - a.y) + a.x;
                    if (a.x == b.x || p.x < xi) inside = !inside;
                }
            }
        }
    }
    return inside;
}

/* index s with special_y[s] == y, or -1 */
EG_HD int special_index(const EcmView& e, float y)
{
    if (e.sp_bloom) {
        const unsigned h = sp_hash(y);
        if (!((e.sp_bloom[h >> 5] >> (h & 31u)) & 1u)) return -1;
    }
    int lo = 0, hi = e.n_special;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        float v = e.special_y[mid];
        if (v < y) lo = mid + 1;
        else hi = mid;
    }
    return (lo < e.n_special && e.special_y[lo] == y) ? lo : -1;
}

/* ECMCellCollection::PointLocationQueryLinear (ECMCellCollection.cpp:57-90):
   the first cell, in cell order, whose quad contains p.  Every quad that can
   contain p is listed in p's grid cell or, when p.y is the height of a quad
   corner, in that height's list; both lists are ascending, so the smaller of
   their first hits is the linear scan's first hit. */
EG_HD int point_location_inl(const EcmView& e, V2 p)
{
    V2 q[4];
    int best = -1;
    const int s = e.n_special > 0 ? special_index(e, p.y) : -1;
    if (s >= 0) {
        for (int i = e.sp_start[s], en = e.sp_start[s + 1]; i < en; i++) {
            int c = e.sp_items[i];
            cell_quad(e, c, q);
            if (contains_quad(p, q)) { best = c; break; }
        }
    }
    float fx = (p.x - e.gx0) * e.ginv, fy = (p.y - e.gy0) * e.ginv;
    if (!(fx >= 0.0f && fy >= 0.0f && fx < (float)e.gw && fy < (float)e.gh)) return best;
    int g = (int)fy * e.gw + (int)fx;
    int b = e.g_start[g], en = e.g_start[g + 1];
    for (int i = b; i < en; i++) {
        int c = e.g_items[i];
        if (best >= 0 && c >= best) break;
        cell_quad(e, c, q);
        if (contains_quad(p, q)) return c;
    }
    return best;
}

/* the out-of-line copy of point_location_inl for the callers that only
   need it now and then */
EG_NI int point_location(const EcmView& e, V2 p) { return point_location_inl(e, p); }

/* MathUtility::GetRayToLineSegmentIntersection (UtilityFunctions.cpp:323-349) */
EG_HD bool ray_segment(V2 o, V2 d, V2 p1, V2 p2, V2* out)
{
    V2 v1 = o - p1;
    V2 v2 = p2 - p1;
    V2 v3 = mk(-d.y, d.x);
    float dt = dot(v2, v3);
    if ((double)fabsf(dt) < 0.000001) return false;
    float t1 = det(v2, v1) / dt;
    float t2 = dot(v1, v3) / dt;
    if (t1 >= 0.0f && (t2 >= 0.0f && t2 <= 1.0f)) {
        out->x = o.x + d.x * t1;
        out->y = o.y + d.y * t1;
        return true;
    }
    return false;
}

/* ECM::RetractPoint (ECMGenerator/ECM.cpp:20-96) */
/* cell: loc's point location when the caller has it already (-2: look it up) */
EG_HD bool retract(const EcmView& e, V2 loc, V2* out, int* out_edge, int cell = -2)
{
    int c = cell == -2 ? point_location(e, loc) : cell;
    if (c < 0) return false;
    int ed = c >> 1;
    int ip1 = e.he_target[2 * ed + 1], ip2 = e.he_target[2 * ed];
    V2 p1 = e.v_pos[ip1], p2 = e.v_pos[ip2];
    int toP2 = e.he_target[2 * ed] == e.v_idx[ip2] ? 0 : 1;
    int toP1 = (toP2 + 1) % 2;
    V2 o1, o2, rd;
    bool isLeft = (p2.x - p1.x) * (loc.y - p1.y) - (p2.y - p1.y) * (loc.x - p1.x) > 0; /* IsLeftOfSegment */
    if (isLeft) {
        o1 = e.he_left[2 * ed + toP2];
        o2 = e.he_right[2 * ed + toP1];
        if (approx(o1, o2)) rd = (p1 - o1) + (p2 - o1);
        else { V2 v = o2 - o1; rd = mk(v.y, -v.x); }
    } else {
        o1 = e.he_right[2 * ed + toP2];
        o2 = e.he_left[2 * ed + toP1];
        if (approx(o1, o2)) rd = (p1 - o1) + (p2 - o1);
        else { V2 v = o2 - o1; rd = mk(-v.y, v.x); }
    }
    rd = normalize(rd);
    *out_edge = ed;
    return ray_segment(loc, rd, p1, p2, out);
}

/* IRMPathFollower::FindAttractionPoint (IRMPathFollower.cpp:14-115).
   *out is written only where the reference writes outPoint; *no_retract is
   set when the failure is the retraction of pos itself. */
EG_NI bool irm(const EcmView& e, V2 pos, const V2* path, int n, V2* out, bool* no_retract = nullptr,
               int* edge = nullptr, int cell = -2)
{
    V2 r;
    int ed;
    if (!retract(e, pos, &r, &ed, cell)) {
        if (no_retract) *no_retract = true;
        return false;
    }
    if (edge) *edge = ed;
    V2 co = closest_on_segment(r, e.he_left[2 * ed], e.he_right[2 * ed + 1]);
    float clr = len(r - co);
    float rcs = clr * clr;
    V2 goal = path[n - 1];
    if (len2(goal - r) < rcs) { *out = goal; return true; }
    bool success = false;
    for (int i = 0; i < n - 1; i++) {
        V2 p1 = path[i] - r;
        V2 p2 = path[i + 1] - r;
        V2 ed2 = p2 - p1;
        float els = len2(ed2);
        float dd = det(p1, p2);
        float disc = rcs * els - dd * dd;
        if (disc < kEps) continue;
        success = true;
        float dySign = ed2.y < 0.0f ? -1.0f : 1.0f;
        float sd = sqrtf(disc);
        V2 i1 = mk((dd * ed2.y + dySign * ed2.x * sd) / els, (-dd * ed2.x + fabsf(ed2.y) * sd) / els);
        V2 i2 = mk((dd * ed2.y - dySign * ed2.x * sd) / els, (-dd * ed2.x - fabsf(ed2.y) * sd) / els);
        V2 g1 = p1 + r, g2 = p2 + r;
        V2 gi1 = i1 + r, gi2 = i2 + r;
        V2 edge = g2 - g1;
        float t1 = dot(gi1 - g1, edge) / els;
        float t2 = dot(gi2 - g1, edge) / els;
        float maxT = -1.0f;
        if (t1 >= 0.0f && t1 <= 1.0f) { *out = gi1; maxT = t1; }
        if (t2 >= 0.0f && t2 <= 1.0f) {
            if (t2 > maxT) *out = gi2;
        }
    }
    return success;
}

/* ------------------------------------------------------------------------
 * Obstacles
 * ---------------------------------------------------------------------- */
struct ObstView {
    const V2* p;
    const int* next;
    const int* prev;
    const unsigned char* convex;
    int n_verts;
    /* candidate grid: cell g lists, ascending, every obstacle edge (vertex id)
       within `reach` metres of the cell */
    float gx0, gy0, ginv;
    int gw, gh;
    float reach;
    const int* g_start;
    const int* g_items;
};

/* one edge of Simulator::FindNearestObstacles (Simulator.cpp:268-290) */
EG_HD bool obstacle_in_range(const ObstView& o, int i, V2 pos, float rangeSq)
{
    V2 a = o.p[i];
    V2 b = o.p[o.next[i]];
    float sld = det(a - pos, b - a); /* LineLeftDistance */
    float sq = (sld * sld) / sqdist(a, b); /* std::powf(sld, 2.0f) */
    if (sq < rangeSq) {
        if (sld < 0.0f) {
            V2 c = closest_on_segment(pos, a, b);
            if (sqdist(c, pos) < rangeSq) return true;
        }
    }
    return false;
}

/* ------------------------------------------------------------------------
 * ORCA (ECMAgentSimulator/ORCA.cpp)
 * ---------------------------------------------------------------------- */
struct Con {
    V2 p; /* Constraint::PointOnLine */
    V2 n; /* Constraint::Normal      */
};

/* obstacle part of ORCA::GenerateConstraints (ORCA.cpp:70-333) for one
   candidate edge L; returns true and fills *c when a constraint is emitted.
   Inline for the plain tick's kernel; obstacle_constraint is the out-of-line
   copy for the larger kernels. */
EG_HD bool obstacle_constraint_inl(const ObstView& o, int L, V2 position, V2 velocity, float clr,
                                   float tau_obst, Con* c)
{
    int R = o.next[L];
    V2 pL = o.p[L], pR = o.p[R];
    V2 rp1 = pL - position;
    V2 rp2 = pR - position;
    V2 seg = pR - pL;
    const float s = dot(rp1 * -1.0f, seg) / len2(seg);
    const float distSqLine = len2(rp1 * -1.0f - seg * s);
    const float distSq1 = len2(rp1);
    const float distSq2 = len2(rp2);
    seg = normalize(seg);
    const float radiusSq = clr * clr;
    const V2 zero = mk(0.0f, 0.0f);
    bool cL = o.convex[L] != 0, cR = o.convex[R] != 0;

    if (s < 0.0f && distSq1 <= radiusSq) {
        if (cL) { c->p = zero; c->n = normalized(rp1 * -1.0f); return true; }
        return false;
    } else if (s > 1.0f && distSq2 <= radiusSq) {
        V2 rnd = normalize(o.p[o.next[R]] - pR);
        if (cR && det(rp2, rnd) >= 0.0f) { c->p = zero; c->n = normalized(rp2 * -1.0f); return true; }
        return false;
    } else if (s >= 0.0f && s < 1.0f && distSqLine <= radiusSq) {
        c->p = zero;
        c->n = right(seg);
        return true;
    }

    V2 leftLeg, rightLeg;
    if (s < 0.0f && distSqLine <= radiusSq) {
        if (!cL) return false;
        R = L;
        pR = pL;
        cR = cL;
        const float leg1 = sqrtf(distSq1 - radiusSq);
        leftLeg = mk(rp1.x * leg1 - rp1.y * clr, rp1.x * clr + rp1.y * leg1) / distSq1;
        rightLeg = mk(rp1.x * leg1 + rp1.y * clr, -rp1.x * clr + rp1.y * leg1) / distSq1;
    } else if (s > 1.0f && distSqLine <= radiusSq) {
        if (!cR) return false;
        L = R;
        pL = pR;
        cL = cR;
        const float leg2 = sqrtf(distSq2 - radiusSq);
        leftLeg = mk(rp2.x * leg2 - rp2.y * clr, rp2.x * clr + rp2.y * leg2) / distSq2;
        rightLeg = mk(rp2.x * leg2 + rp2.y * clr, -rp2.x * clr + rp2.y * leg2) / distSq2;
    } else {
        if (cL) {
            const float leg1 = sqrtf(distSq1 - radiusSq);
            leftLeg = mk(rp1.x * leg1 - rp1.y * clr, rp1.x * clr + rp1.y * leg1) / distSq1;
        } else {
            leftLeg = seg * -1.0f;
        }
        if (cR) {
            const float leg2 = sqrtf(distSq2 - radiusSq);
            rightLeg = mk(rp2.x * leg2 + rp2.y * clr, -rp2.x * clr + rp2.y * leg2) / distSq2;
        } else {
            rightLeg = seg;
        }
    }

    bool isLeftForeign = false, isRightForeign = false;
    V2 lnd = normalize(pL - o.p[o.prev[L]]);
    if (cL && det(leftLeg, lnd * -1.0f) >= 0.0f) {
        leftLeg = lnd * -1.0f;
        isLeftForeign = true;
    }
    V2 rnd = normalize(o.p[o.next[R]] - pR);
    if (cR && det(rightLeg, rnd) <= 0.0f) {
        rightLeg = rnd;
        isRightForeign = true;
    }

    float invT = 1.0f / tau_obst;
    const V2 leftCutoff = (pL - position) * invT;
    const V2 rightCutoff = (pR - position) * invT;
    const V2 cutoffVec = rightCutoff - leftCutoff;
    const bool same = (L == R);
    const float t = (same ? 0.5f : dot(velocity - leftCutoff, cutoffVec) / len2(cutoffVec));
    const float tLeft = dot(velocity - leftCutoff, leftLeg);
    const float tRight = dot(velocity - rightCutoff, rightLeg);

    if ((t < 0.0f && tLeft < 0.0f) || (same && tLeft < 0.0f && tRight < 0.0f)) {
        V2 unitW = normalized(velocity - leftCutoff);
        c->p = leftCutoff + (unitW * invT) * clr;
        c->n = unitW;
        return true;
    } else if (t > 1.0f && tRight < 0.0f) {
        V2 unitW = normalized(velocity - rightCutoff);
        c->p = rightCutoff + (unitW * invT) * clr;
        c->n = unitW;
        return true;
    }

    const float inf = INFINITY;
    const float distSqCutoff = ((t < 0.0f || t > 1.0f || same) ? inf : len2(velocity - (leftCutoff + cutoffVec * t)));
    const float distSqLeft = ((tLeft < 0.0f) ? inf : len2(velocity - (leftCutoff + leftLeg * tLeft)));
    const float distSqRight = ((tRight < 0.0f) ? inf : len2(velocity - (rightCutoff + rightLeg * tRight)));

    if (distSqCutoff <= distSqLeft && distSqCutoff <= distSqRight) {
        V2 normal = left(seg * -1.0f);
        c->p = leftCutoff + (normal * invT) * clr;
        c->n = normal;
        return true;
    } else if (distSqLeft <= distSqRight) {
        if (isLeftForeign) return false;
        V2 normal = left(leftLeg);
        c->p = leftCutoff + (normal * clr) * invT;
        c->n = normal;
        return true;
    } else {
        if (isRightForeign) return false;
        V2 normal = right(rightLeg);
        c->p = rightCutoff + (normal * clr) * invT;
        c->n = normal;
        return true;
    }
}

EG_NI bool obstacle_constraint(const ObstView& o, int L, V2 position, V2 velocity, float clr,
                               float tau_obst, Con* c)
{
    return obstacle_constraint_inl(o, L, position, velocity, clr, tau_obst, c);
}

/* agent part of ORCA::GenerateConstraints (ORCA.cpp:339-423) for one
   neighbour.  inv_tau != 0 must be 1/tau for a power-of-two tau: x / tau and
   x * (1/tau) are then the same correctly rounded value (the quotient is an
   exact scaling), and the multiplication is cheaper. */
EG_HD Con agent_constraint(V2 position, V2 velocity, float clr, V2 np, V2 nv, float nclr, float tau, float dt,
                           float inv_tau = 0.0f)
{
    Con c;
    const float rx = np.x - position.x, ry = np.y - position.y;
    V2 VOPos = inv_tau != 0.0f ? mk(rx * inv_tau, ry * inv_tau) : mk(rx / tau, ry / tau);
    V2 relPos = mk(rx, ry);
    float relPosLength = len(relPos);
    /* with a power-of-two 1/tau every step of the length scales exactly
       while all squares and sums stay normal numbers -- each component zero
       or within [1e-12, 1e12] m and 1/tau within [2^-20, 2^20] -- so
       |VOPos| = |relPos| / tau bit for bit and needs no second square root */
    const float ax = fabsf(rx), ay = fabsf(ry);
    const bool scaled = inv_tau >= 9.5367431640625e-07f && inv_tau <= 1048576.0f &&
                        (ax == 0.0f || (ax >= 1e-12f && ax <= 1e12f)) && (ay == 0.0f || (ay >= 1e-12f && ay <= 1e12f));
    float VOPosLength = scaled ? relPosLength * inv_tau : len(VOPos);
    float combinedRadius = nclr + clr;
    float VORadius = inv_tau != 0.0f ? combinedRadius * inv_tau : combinedRadius / tau;
    V2 relVel = mk(velocity.x - nv.x, velocity.y - nv.y);
    if (relPosLength < combinedRadius) {
        V2 w = relVel - relPos / dt;
        float wLength = len(w);
        V2 unitW = w / wLength;
        V2 U = unitW * (combinedRadius / dt - wLength);
        c.p = velocity + U * 0.5f;
        c.n = unitW;
        return c;
    }
    float tanAngleFactor = VORadius / VOPosLength;
    float tanHalfAngle = ecmg_atanf(tanAngleFactor);
    /* RotateVector(VOPos, +/-tanHalfAngle): ecmg_sincosf is odd / even
       symmetric bit for bit on the nonzero angles of [-pi/2, pi/2] (the
       range of the atan), so the rotation by -angle takes (-sin, cos) of the
       same call; a zero or NaN angle (where the sign of a zero or of a NaN
       could differ) calls it again */
    float sn, cs, sn2, cs2;
    ecmg_sincosf(tanHalfAngle, &sn, &cs);
    if (tanHalfAngle != 0.0f && tanHalfAngle == tanHalfAngle) {
        sn2 = -sn;
        cs2 = cs;
    } else {
        ecmg_sincosf(-tanHalfAngle, &sn2, &cs2);
    }
    V2 VOLeftLeg = mk(VOPos.x * cs - VOPos.y * sn, VOPos.x * sn + VOPos.y * cs);
    V2 VORightLeg = mk(VOPos.x * cs2 - VOPos.y * sn2, VOPos.x * sn2 + VOPos.y * cs2);
    float sqDistFromCircleCentre = sqdist(VOPos, relVel);
    V2 bse = VOLeftLeg - VOPos, chk = relVel - VOPos;
    bool liesBelow = bse.x * chk.y - bse.y * chk.x > 0; /* IsLeftOfVector */
    if (liesBelow) {
        float distToEdge = VORadius - sqrtf(sqDistFromCircleCentre);
        V2 lineNormal = normalize(relVel - VOPos);
        c.p = velocity + (lineNormal * distToEdge) * 0.5f;
        c.n = lineNormal;
    } else {
        V2 leftPerp = left(VOPos) / VOPosLength;
        if (dot(leftPerp, relVel) >= 0) {
            V2 lln = normalized(VOLeftLeg);
            float l = dot(relVel, lln); /* GetClosestPointOnLineThroughOrigin */
            V2 U = (lln * l) - relVel;
            c.p = velocity + U * 0.5f;
            c.n = left(lln);
        } else {
            V2 rln = normalized(VORightLeg);
            float l = dot(relVel, rln);
            V2 U = (rln * l) - relVel;
            c.p = velocity + U * 0.5f;
            c.n = right(rln);
        }
    }
    return c;
}

/* Which update produced an LP result: the last constraint whose line the
   solution was moved onto (-1: none) and what fixed the position on it. */
struct LpTrace {
    int h = -1;
    int src = 0; /* 0 projection of opt, 1 circle bound, 2 bound from constraint j */
    int j = -1;
};

/* the starting point of ORCA::RandomizedLP (ORCA.cpp:438-453) */
EG_HD V2 lp2d_start(V2 opt, float maxSpeed, bool useDirOpt)
{
    if (useDirOpt) return opt * maxSpeed;
    if (len(opt) > maxSpeed) return normalized(opt) * maxSpeed;
    return opt;
}

/* step i of ORCA::RandomizedLP (ORCA.cpp:459-583): half-plane h (the
   constraint at index i) against the solution *out of the steps before it;
   the earlier constraints are fetched through get(j), j < i.  Returns false
   when the LP fails at i (*out is then the solution before the step).  With
   TRACE the update is recorded in *tr (bookkeeping only). */
template <class Get, bool TRACE = false>
EG_HD bool lp2d_step(const Get& get, int i, const Con& h, V2 opt, float maxSpeed, bool useDirOpt, V2* out,
                     LpTrace* tr = nullptr)
{
    if (det(right(h.n), h.p - *out) <= 0.0f) return true; /* Constraint::Contains */
    V2 dir = right(h.n);
    float dirPointDot = dot(dir, h.p);
    float disc = dirPointDot * dirPointDot + maxSpeed * maxSpeed - dot(h.p, h.p);
    if (disc <= 0.0f) return false;
    /* a NaN discriminant takes neither branch of ORCA.cpp:498-506: the
       constraint is passed over */
    if (!(disc > 0.0f)) return true;
    float sq = sqrtf(disc);
    float lo = -dirPointDot - sq;
    float hi = -dirPointDot + sq;
    int lo_src = -1, hi_src = -1;
    for (int j = 0; j < i; j++) {
        Con g = get(j);
        float den = det(right(h.n), right(g.n));
        float num = det(right(g.n), h.p - g.p);
        if (fabsf(den) <= kEps) {
            if (num < 0.0f) return false;
            continue;
        }
        const float t = num / den;
        if (den >= 0.0f) { /* std::min(right, t) */
            if (TRACE && t < hi) hi_src = j;
            hi = (t < hi) ? t : hi;
        } else { /* std::max(left, t) */
            if (TRACE && lo < t) lo_src = j;
            lo = (lo < t) ? t : lo;
        }
        if (lo > hi) return false;
    }
    if (useDirOpt) {
        if (dot(opt, right(h.n)) > 0) *out = h.p + right(h.n) * hi;
        else *out = h.p + right(h.n) * lo;
    } else {
        float t = dot(right(h.n), opt - h.p);
        if (t < lo) {
            *out = h.p + right(h.n) * lo;
            if (TRACE) { tr->h = i; tr->src = lo_src < 0 ? 1 : 2; tr->j = lo_src; }
        } else if (t > hi) {
            *out = h.p + right(h.n) * hi;
            if (TRACE) { tr->h = i; tr->src = hi_src < 0 ? 1 : 2; tr->j = hi_src; }
        } else {
            *out = h.p + right(h.n) * t;
            if (TRACE) { tr->h = i; tr->src = 0; tr->j = -1; }
        }
    }
    return true;
}

/* ORCA::RandomizedLP (ORCA.cpp:428-587): its steps over the constraints
   0 .. n-1 in order; returns the failing index or n.  The constraint at index
   i is fetched through get(i) so that callers may keep constraints in
   registers, shared or local memory. */
template <class Get, bool TRACE = false>
EG_HD int lp2d(const Get& get, int n, V2 opt, float maxSpeed, bool useDirOpt, V2* out, LpTrace* tr = nullptr)
{
    *out = lp2d_start(opt, maxSpeed, useDirOpt);
    for (int i = 0; i < n; i++)
        if (!lp2d_step<Get, TRACE>(get, i, get(i), opt, maxSpeed, useDirOpt, out, tr)) return i;
    return n;
}

/* the projected lines of RandomizedLP3D: the obstacle constraints (read in
   place), then the bisectors in proj */
template <class Get>
struct Lp3dProj {
    const Get* get;
    const Con* proj;
    int nObst;
    EG_HD Con operator()(int q) const { return q < nObst ? (*get)(q) : proj[q - nObst]; }
};

/* ORCA::RandomizedLP3D (ORCA.cpp:592-669).  proj must hold n - nObst
   constraints.  With fp64 the bisector lines are intersected in double
   precision (the reference computes them in float). */
template <class Get>
EG_HD void lp3d(const Get& get, int n, int nObst, float maxSpeed, int failed, V2* out, Con* proj, bool fp64)
{
    float maxPen = 0.0f;
    for (int i = failed; i < n; i++) {
        Con ci = get(i);
        V2 dir = right(ci.n);
        if (det(dir, ci.p - *out) <= maxPen) continue;
        /* RandomizedLP over the projected lines -- the obstacle constraints,
           then the bisectors in order -- taking each bisector as soon as it
           is built: the same steps as building them all first, and the
           bisectors after a failing line are never read */
        const V2 temp = *out;
        Lp3dProj<Get> pg{&get, proj, nObst};
        *out = lp2d_start(ci.n, maxSpeed, true);
        bool ok = true;
        for (int q = 0; q < nObst && ok; q++) ok = lp2d_step(pg, q, get(q), ci.n, maxSpeed, true, out);
        int m = 0;
        for (int j = nObst; j < i && ok; j++) {
            Con cj = get(j);
            float dt = det(right(ci.n), right(cj.n));
            V2 np_;
            if (fabsf(dt) <= kEps) {
                if (dot(ci.n, cj.n) > 0) continue;
                np_ = (ci.p + cj.p) * 0.5f;
            } else if (!fp64) {
                float t = det(right(cj.n), ci.p - cj.p) / dt;
                np_ = ci.p + right(ci.n) * t;
            } else {
                double ax = (double)cj.n.y, ay = -(double)cj.n.x;             /* Right(cj.N) */
                double bx = (double)ci.p.x - (double)cj.p.x, by = (double)ci.p.y - (double)cj.p.y;
                double rx = (double)ci.n.y, ry = -(double)ci.n.x;             /* Right(ci.N) */
                double dd = rx * ay - ry * ax;
                double t = (ax * by - ay * bx) / dd;
                np_ = mk((float)((double)ci.p.x + rx * t), (float)((double)ci.p.y + ry * t));
            }
            Con nc;
            nc.p = np_;
            nc.n = normalized(cj.n - ci.n);
            proj[m] = nc;
            ok = lp2d_step(pg, nObst + m, nc, ci.n, maxSpeed, true, out);
            m++;
        }
        if (!ok) *out = temp; /* ORCA.cpp:658-664 */
        maxPen = det(dir, ci.p - *out);
    }
}

} /* namespace ecmg */

#endif
