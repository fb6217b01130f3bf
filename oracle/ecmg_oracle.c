/*
 * ecmg_oracle.c -- CPU oracle (test infrastructure, see ecmg_oracle.h).
 *
 * Each function restates one reference function; the comment above it gives
 * the file:line it follows.  Operand order of every arithmetic expression is
 * the reference's; build with -ffp-contract=off.
 */
#define _POSIX_C_SOURCE 200809L
#include "ecmg_oracle.h"
#include "../ecmgenerator_gb300/csrc/ecmg_tmath.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#ifdef OG_REAL_DOUBLE
#define og_sqrt sqrt
#define og_fabs fabs
#define og_fmax fmax
#define og_fmin fmin
#define og_atan atan
#define og_sin sin
#define og_cos cos
#define og_pow pow
#define og_ceil ceil
#define OG_REAL_MAX DBL_MAX
#else
#define og_sqrt sqrtf
#define og_fabs fabsf
#define og_fmax fmaxf
#define og_fmin fminf
#define og_atan atanf
#define og_sin sinf
#define og_cos cosf
#define og_pow powf
#define og_ceil ceilf
#define OG_REAL_MAX FLT_MAX
#endif

#define OG_EPS 0.0001f /* Utility::EPSILON, ECMGenerator/Configuration.h:14 */

/* ---------------------------------------------------------------------------
 * Vec2 / Point algebra, ECMGenerator/ECMDataTypes.h:13-104 and
 * MathUtility, ECMGenerator/UtilityFunctions.cpp:15-349
 * ------------------------------------------------------------------------- */
static inline og_v2 v2(og_real x, og_real y) { og_v2 r; r.x = x; r.y = y; return r; }
static inline og_v2 vadd(og_v2 a, og_v2 b) { return v2(a.x + b.x, a.y + b.y); }
static inline og_v2 vsub(og_v2 a, og_v2 b) { return v2(a.x - b.x, a.y - b.y); }
static inline og_v2 vmul(og_v2 a, og_real s) { return v2(a.x * s, a.y * s); }
static inline og_v2 vdiv(og_v2 a, og_real s) { return v2(a.x / s, a.y / s); }
static inline og_real vlen(og_v2 a) { return og_sqrt(a.x * a.x + a.y * a.y); }
static inline og_real vlen2(og_v2 a) { return a.x * a.x + a.y * a.y; }
static inline og_real vdot(og_v2 a, og_v2 b) { return a.x * b.x + a.y * b.y; }
static inline og_real vdet(og_v2 a, og_v2 b) { return a.x * b.y - a.y * b.x; }
static inline og_v2 vright(og_v2 a) { return v2(a.y, -a.x); }
static inline og_v2 vleft(og_v2 a) { return v2(-a.y, a.x); }
/* Vec2::Normalize (ECMDataTypes.h:45-52) */
static inline og_v2 vnormalize(og_v2 a)
{
    og_real l = vlen(a);
    if (l == 0.0f) return a;
    a.x /= l;
    a.y /= l;
    return a;
}
/* Vec2::Normalized (ECMDataTypes.h:54-60); the reference returns an
   uninitialised Vec2 for a zero vector, this returns (0,0). */
static inline og_v2 vnormalized(og_v2 a)
{
    og_real l = vlen(a);
    if (l == 0.0f) return v2(0.0f, 0.0f);
    return v2(a.x / l, a.y / l);
}
/* Point::Approximate (ECMDataTypes.cpp:97-100) */
static inline int vapprox(og_v2 p, og_v2 a)
{
    return p.x < (a.x + OG_EPS) && p.x > (a.x - OG_EPS) && p.y < (a.y + OG_EPS) && p.y > (a.y - OG_EPS);
}
/* MathUtility::SquareDistance(Point,Point) (UtilityFunctions.cpp:32-39): p2 - p1 */
static inline og_real vsqdist(og_v2 p1, og_v2 p2)
{
    og_real dx = p2.x - p1.x, dy = p2.y - p1.y;
    return dx * dx + dy * dy;
}
/* MathUtility::GetClosestPointOnSegment (UtilityFunctions.cpp:287-306) */
static og_v2 closest_on_segment(og_v2 point, og_v2 s1, og_v2 s2)
{
    if (vapprox(s1, s2)) return s1;
    og_v2 seg = vsub(s2, s1);
    og_v2 pts = vsub(point, s1);
    og_real tsq = vsqdist(s1, s2);
    og_real d = (pts.x * seg.x + pts.y * seg.y) / tsq;
    if (d > 1.0f) d = 1.0f;
    if (d < 0.0f) d = 0.0f;
    return v2(s1.x + d * seg.x, s1.y + d * seg.y);
}
/* MathUtility::RotateVector (UtilityFunctions.cpp:233-242) */
static og_v2 rotate(og_v2 v, og_real rad, int libm)
{
    og_real cs, sn;
    if (libm) {
        cs = og_cos(rad);
        sn = og_sin(rad);
    } else {
        float s32, c32;
        ecmg_sincosf((float)rad, &s32, &c32);
        sn = s32;
        cs = c32;
    }
    og_real px = v.x * cs - v.y * sn;
    og_real py = v.x * sn + v.y * cs;
    return v2(px, py);
}

/* ---------------------------------------------------------------------------
 * kNN
 * ------------------------------------------------------------------------- */

/* Exact k nearest neighbours, ordered by (d2, id).  This is the neighbour
   definition the GPU grid query must reproduce bit for bit; the reference's
   kd-tree (below) is a different, approximate query.  d2 is computed exactly
   as KDTree.cpp:107-108 computes it, self and coincident agents are excluded
   by the same d2 > EPSILON test (KDTree.cpp:112). */
int og_knn_exact(const og_state* s, int agent, int k, og_real r2, int* out_ids, og_real* out_d2)
{
    og_v2 t = s->pos[agent];
    int n = 0;
    for (int j = 0; j <= s->last_idx; j++) {
        if (!s->active[j]) continue;
        og_real dx = s->pos[j].x - t.x;
        og_real dy = s->pos[j].y - t.y;
        og_real d2 = dx * dx + dy * dy;
        if (!(d2 > OG_EPS) || !(d2 < r2)) continue;
        /* insertion into the sorted top-k list */
        if (n == k && !(d2 < out_d2[k - 1])) continue; /* ties: ids arrive ascending */
        int pos = n < k ? n : k - 1;
        while (pos > 0 && d2 < out_d2[pos - 1]) {
            out_d2[pos] = out_d2[pos - 1];
            out_ids[pos] = out_ids[pos - 1];
            pos--;
        }
        out_d2[pos] = d2;
        out_ids[pos] = j;
        if (n < k) n++;
    }
    return n;
}

struct og_kdtree {
    int k;
    int* tree;
    int tree_cap;
    int tree_size;
    int max_depth;
    int* cache;   /* ORCA::m_NeighborCache, persists across agents and ticks */
    og_real* dist;  /* nearestSqDistances (fresh per query)                   */
    int* idx;
    int idx_cap;
    const og_v2* sort_pos;
};

og_kdtree* og_kdtree_create(int k)
{
    og_kdtree* t = (og_kdtree*)calloc(1, sizeof(og_kdtree));
    t->k = k;
    t->cache = (int*)calloc((size_t)k, sizeof(int)); /* std::vector<int>::resize -> 0 */
    t->dist = (og_real*)malloc(sizeof(og_real) * (size_t)k);
    return t;
}

void og_kdtree_destroy(og_kdtree* t)
{
    if (!t) return;
    free(t->tree);
    free(t->cache);
    free(t->dist);
    free(t->idx);
    free(t);
}

/* stable merge sort of ids by one coordinate (std::sort in the reference;
   identical result whenever the coordinates are distinct) */
static void msort(int* a, int* tmp, int n, const og_v2* pos, int axis)
{
    if (n < 2) return;
    int h = n / 2;
    msort(a, tmp, h, pos, axis);
    msort(a + h, tmp, n - h, pos, axis);
    int i = 0, j = h, o = 0;
    while (i < h && j < n) {
        og_real ka = axis ? pos[a[i]].y : pos[a[i]].x;
        og_real kb = axis ? pos[a[j]].y : pos[a[j]].x;
        if (kb < ka) tmp[o++] = a[j++];
        else tmp[o++] = a[i++];
    }
    while (i < h) tmp[o++] = a[i++];
    while (j < n) tmp[o++] = a[j++];
    memcpy(a, tmp, sizeof(int) * (size_t)n);
}

/* KDTree::ConstructRecursive (KDTree.cpp:59-83) */
static void kd_rec(og_kdtree* t, int index, int lo, int hi, int depth, int* ids, int* tmp)
{
    if (lo >= hi) return;
    msort(ids + lo, tmp, hi - lo, t->sort_pos, depth % 2);
    int mid = lo + (hi - 1 - lo) / 2;
    t->tree[index] = ids[mid];
    kd_rec(t, index * 2 + 1, lo, mid, depth + 1, ids, tmp);
    kd_rec(t, index * 2 + 2, mid + 1, hi, depth + 1, ids, tmp);
}

/* KDTree::Construct (KDTree.cpp:22-57) */
void og_kdtree_build(og_kdtree* t, const og_state* s)
{
    int size = s->num_agents;
    if (size == 0) return; /* the reference keeps the previous tree */
    if (t->idx_cap < size) {
        free(t->idx);
        t->idx = (int*)malloc(sizeof(int) * (size_t)size * 2);
        t->idx_cap = size;
    }
    int c = 0;
    for (int i = 0; i <= s->last_idx; i++)
        if (s->active[i]) t->idx[c++] = i;
    t->max_depth = (int)ceil(log2((double)size + 1.0) - 1.0);
    int tsize = (int)pow(2.0, (double)(t->max_depth + 1)) - 1;
    if (t->tree_cap < tsize) {
        free(t->tree);
        t->tree = (int*)malloc(sizeof(int) * (size_t)tsize);
        t->tree_cap = tsize;
    }
    t->tree_size = tsize;
    for (int i = 0; i < tsize; i++) t->tree[i] = -1;
    t->sort_pos = s->pos;
    kd_rec(t, 0, 0, size, 0, t->idx, t->idx + t->idx_cap);
}

/* KDTree::KNearestAgents_R (KDTree.cpp:98-202), quirks included */
static void kd_knn_rec(og_kdtree* t, const og_v2* pos, og_v2 target, int cur, int k, int* kfound, int depth)
{
    if (depth > t->max_depth) return;
    if (t->tree[cur] == -1) return;
    og_v2 cp = pos[t->tree[cur]];
    og_real dx = cp.x - target.x, dy = cp.y - target.y;
    og_real d = dx * dx + dy * dy;
    int* ni = t->cache;
    og_real* nd = t->dist;
    if (*kfound < k && d > OG_EPS) {
        ni[*kfound] = t->tree[cur];
        nd[*kfound] = d;
        (*kfound)++;
        if (*kfound == k) {
            og_real largest = d;
            int li = k - 1;
            for (int i = 0; i < k - 1; i++)
                if (nd[i] > largest) { largest = nd[i]; li = i; }
            nd[0] = largest;
            ni[0] = ni[li];
            nd[li] = d;
            ni[li] = t->tree[cur];
        }
    } else {
        *kfound = k;
        if (d < nd[0] && d > OG_EPS) {
            nd[0] = d;
            ni[0] = t->tree[cur];
            og_real largest = d;
            int li = 0;
            for (int i = 1; i < k; i++)
                if (nd[i] > largest) { largest = nd[i]; li = i; }
            nd[0] = largest;
            ni[0] = ni[li];
            nd[li] = d;
            ni[li] = t->tree[cur];
        }
    }
    og_real cv = depth % 2 == 0 ? cp.x : cp.y;
    og_real tv = depth % 2 == 0 ? target.x : target.y;
    if (tv < cv) {
        kd_knn_rec(t, pos, target, cur * 2 + 1, k, kfound, depth + 1);
        og_real db = tv - cv;
        if (db * db < nd[k - 1]) kd_knn_rec(t, pos, target, cur * 2 + 2, k, kfound, depth + 1);
    } else {
        kd_knn_rec(t, pos, target, cur * 2 + 2, k, kfound, depth + 1);
        og_real db = tv - cv;
        if (db * db < nd[k - 1]) kd_knn_rec(t, pos, target, cur * 2 + 1, k, kfound, depth + 1);
    }
}

/* KDTree::KNearestAgents (KDTree.cpp:85-96): returns kFound, list in the cache */
int og_kdtree_query(og_kdtree* t, const og_state* s, int agent, int* out_ids)
{
    int k = t->k;
    for (int i = 0; i < k; i++) t->dist[i] = OG_REAL_MAX;
    int kfound = 0;
    kd_knn_rec(t, s->pos, s->pos[agent], 0, k, &kfound, 0);
    if (out_ids)
        for (int i = 0; i < k; i++) out_ids[i] = t->cache[i];
    return kfound;
}

/* ---------------------------------------------------------------------------
 * Simulator::FindNearestObstacles (ECMAgentSimulator/Simulator.cpp:259-292)
 * ------------------------------------------------------------------------- */
int og_find_obstacles(const og_obstacles* o, og_v2 pos, og_real range_sq, int* out, int cap, int libm)
{
    int n = 0;
    for (int i = 0; i < o->n_verts; i++) {
        og_v2 a = o->p[i];
        og_v2 b = o->p[o->next[i]];
        /* LineLeftDistance (UtilityFunctions.cpp:28-31): Det(v1 - p, v2 - v1) */
        og_real sld = vdet(vsub(a, pos), vsub(b, a));
        og_real num = libm ? og_pow(sld, 2.0f) : sld * sld;
        og_real sq = num / vsqdist(a, b);
        if (sq < range_sq) {
            if (sld < 0.0f) {
                og_v2 c = closest_on_segment(pos, a, b);
                if (vsqdist(c, pos) < range_sq) {
                    if (n < cap) out[n] = i;
                    n++;
                }
            }
        }
    }
    return n;
}

/* ---------------------------------------------------------------------------
 * ORCA::GenerateConstraints (ECMAgentSimulator/ORCA.cpp:60-424)
 * A constraint is stored as 4 floats: point.x, point.y, normal.x, normal.y
 * (Constraint::Init, ORCA.h:29-47; slope/intercepts are unused by the LP).
 * ------------------------------------------------------------------------- */
static inline int push_con(og_real* c, int n, int cap, og_v2 p, og_v2 nrm)
{
    if (n < cap) {
        c[4 * n + 0] = p.x;
        c[4 * n + 1] = p.y;
        c[4 * n + 2] = nrm.x;
        c[4 * n + 3] = nrm.y;
    }
    return n + 1;
}

int og_generate_constraints(const og_obstacles* o, const og_state* s, const og_params* p, int agent,
                            const int* nbrs, int n_nbrs, const int* obst, int n_obst_cand,
                            og_real* cons, int cap, int* out_n_obst)
{
    og_v2 position = s->pos[agent];
    og_v2 velocity = s->vel[agent];
    og_real clr = s->clear[agent];
    int n = 0;
    const og_v2 zero = v2(0.0f, 0.0f);
    const og_real inf = INFINITY;

    for (int i = 0; i < n_obst_cand; i++) {
        int L = obst[i];
        int R = o->next[L];
        og_v2 rp1 = vsub(o->p[L], position);
        og_v2 rp2 = vsub(o->p[R], position);
        og_v2 seg = vsub(o->p[R], o->p[L]);
        const og_real sparam = vdot(vmul(rp1, -1.0f), seg) / vlen2(seg);
        const og_real distSqLine = vlen2(vsub(vmul(rp1, -1.0f), vmul(seg, sparam)));
        const og_real distSq1 = vlen2(rp1);
        const og_real distSq2 = vlen2(rp2);
        seg = vnormalize(seg);
        const og_real radiusSq = clr * clr;

        if (sparam < 0.0f && distSq1 <= radiusSq) { /* ORCA.cpp:92-105 */
            if (o->convex[L]) n = push_con(cons, n, cap, zero, vnormalized(vmul(rp1, -1.0f)));
            continue;
        } else if (sparam > 1.0f && distSq2 <= radiusSq) { /* ORCA.cpp:108-121 */
            og_v2 rnd = vnormalize(vsub(o->p[o->next[R]], o->p[R]));
            if (o->convex[R] && vdet(rp2, rnd) >= 0.0f)
                n = push_con(cons, n, cap, zero, vnormalized(vmul(rp2, -1.0f)));
            continue;
        } else if (sparam >= 0.0f && sparam < 1.0f && distSqLine <= radiusSq) { /* ORCA.cpp:124-135 */
            n = push_con(cons, n, cap, zero, vright(seg));
            continue;
        }

        og_v2 leftLeg, rightLeg;
        if (sparam < 0.0f && distSqLine <= radiusSq) { /* ORCA.cpp:146-169 */
            if (!o->convex[L]) continue;
            R = L;
            const og_real leg1 = og_sqrt(distSq1 - radiusSq);
            leftLeg = vdiv(v2(rp1.x * leg1 - rp1.y * clr, rp1.x * clr + rp1.y * leg1), distSq1);
            rightLeg = vdiv(v2(rp1.x * leg1 + rp1.y * clr, -rp1.x * clr + rp1.y * leg1), distSq1);
        } else if (sparam > 1.0f && distSqLine <= radiusSq) { /* ORCA.cpp:171-183 */
            if (!o->convex[R]) continue;
            L = R;
            const og_real leg2 = og_sqrt(distSq2 - radiusSq);
            leftLeg = vdiv(v2(rp2.x * leg2 - rp2.y * clr, rp2.x * clr + rp2.y * leg2), distSq2);
            rightLeg = vdiv(v2(rp2.x * leg2 + rp2.y * clr, -rp2.x * clr + rp2.y * leg2), distSq2);
        } else { /* ORCA.cpp:186-212 */
            if (o->convex[L]) {
                const og_real leg1 = og_sqrt(distSq1 - radiusSq);
                leftLeg = vdiv(v2(rp1.x * leg1 - rp1.y * clr, rp1.x * clr + rp1.y * leg1), distSq1);
            } else {
                leftLeg = vmul(seg, -1.0f);
            }
            if (o->convex[R]) {
                const og_real leg2 = og_sqrt(distSq2 - radiusSq);
                rightLeg = vdiv(v2(rp2.x * leg2 + rp2.y * clr, -rp2.x * clr + rp2.y * leg2), distSq2);
            } else {
                rightLeg = seg;
            }
        }

        /* foreign legs, ORCA.cpp:218-239 */
        int leftNeighbor = o->prev[L];
        int isLeftForeign = 0, isRightForeign = 0;
        og_v2 lnd = vnormalize(vsub(o->p[L], o->p[leftNeighbor]));
        if (o->convex[L] && vdet(leftLeg, vmul(lnd, -1.0f)) >= 0.0f) {
            leftLeg = vmul(lnd, -1.0f);
            isLeftForeign = 1;
        }
        og_v2 rnd = vnormalize(vsub(o->p[o->next[R]], o->p[R]));
        if (o->convex[R] && vdet(rightLeg, rnd) <= 0.0f) {
            rightLeg = rnd;
            isRightForeign = 1;
        }

        /* cut-off, ORCA.cpp:241-332 */
        og_real invT = 1.0f / p->tau_obst;
        const og_v2 leftCutoff = vmul(vsub(o->p[L], position), invT);
        const og_v2 rightCutoff = vmul(vsub(o->p[R], position), invT);
        const og_v2 cutoffVec = vsub(rightCutoff, leftCutoff);
        const og_real t = (L == R ? 0.5f : vdot(vsub(velocity, leftCutoff), cutoffVec) / vlen2(cutoffVec));
        const og_real tLeft = vdot(vsub(velocity, leftCutoff), leftLeg);
        const og_real tRight = vdot(vsub(velocity, rightCutoff), rightLeg);

        if ((t < 0.0f && tLeft < 0.0f) || (L == R && tLeft < 0.0f && tRight < 0.0f)) {
            og_v2 unitW = vnormalized(vsub(velocity, leftCutoff));
            og_v2 pc = vadd(leftCutoff, vmul(vmul(unitW, invT), clr));
            n = push_con(cons, n, cap, pc, unitW);
            continue;
        } else if (t > 1.0f && tRight < 0.0f) {
            og_v2 unitW = vnormalized(vsub(velocity, rightCutoff));
            og_v2 pc = vadd(rightCutoff, vmul(vmul(unitW, invT), clr));
            n = push_con(cons, n, cap, pc, unitW);
            continue;
        }

        const og_real distSqCutoff = ((t < 0.0f || t > 1.0f || L == R) ? inf
                                    : vlen2(vsub(velocity, vadd(leftCutoff, vmul(cutoffVec, t)))));
        const og_real distSqLeft = ((tLeft < 0.0f) ? inf : vlen2(vsub(velocity, vadd(leftCutoff, vmul(leftLeg, tLeft)))));
        const og_real distSqRight = ((tRight < 0.0f) ? inf : vlen2(vsub(velocity, vadd(rightCutoff, vmul(rightLeg, tRight)))));

        if (distSqCutoff <= distSqLeft && distSqCutoff <= distSqRight) {
            og_v2 normal = vleft(vmul(seg, -1.0f));
            og_v2 pc = vadd(leftCutoff, vmul(vmul(normal, invT), clr));
            n = push_con(cons, n, cap, pc, normal);
            continue;
        } else if (distSqLeft <= distSqRight) {
            if (isLeftForeign) continue;
            og_v2 normal = vleft(leftLeg);
            og_v2 pc = vadd(leftCutoff, vmul(vmul(normal, clr), invT));
            n = push_con(cons, n, cap, pc, normal);
            continue;
        } else {
            if (isRightForeign) continue;
            og_v2 normal = vright(rightLeg);
            og_v2 pc = vadd(rightCutoff, vmul(vmul(normal, clr), invT));
            n = push_con(cons, n, cap, pc, normal);
            continue;
        }
    }
    *out_n_obst = n;

    /* agent constraints, ORCA.cpp:339-423 */
    const og_real ta = p->tau_agent;
    for (int i = 0; i < n_nbrs; i++) {
        int nb = nbrs[i];
        og_v2 np = s->pos[nb];
        og_v2 nv = s->vel[nb];
        og_real nc = s->clear[nb];
        og_v2 VOPos = v2((np.x - position.x) / ta, (np.y - position.y) / ta);
        og_real VOPosLength = vlen(VOPos);
        og_real combinedRadius = nc + clr;
        og_real VORadius = combinedRadius / ta;
        og_v2 relVel = v2(velocity.x - nv.x, velocity.y - nv.y);
        og_v2 relPos = v2(np.x - position.x, np.y - position.y);
        og_real relPosLength = vlen(relPos);

        if (relPosLength < combinedRadius) { /* ORCA.cpp:356-372 */
            og_v2 w = vsub(relVel, vdiv(relPos, p->dt));
            og_real wLength = vlen(w);
            og_v2 unitW = vdiv(w, wLength);
            og_v2 U = vmul(unitW, (combinedRadius / p->dt - wLength));
            n = push_con(cons, n, cap, vadd(velocity, vmul(U, 0.5f)), unitW);
            continue;
        }

        og_real tanAngleFactor = VORadius / VOPosLength;
        og_real tanHalfAngle = p->libm ? og_atan(tanAngleFactor) : ecmg_atanf(tanAngleFactor);
        og_v2 VOLeftLeg = rotate(VOPos, tanHalfAngle, p->libm);
        og_v2 VORightLeg = rotate(VOPos, -tanHalfAngle, p->libm);
        og_real sqDistFromCircleCentre = vsqdist(VOPos, relVel);
        og_v2 bse = vsub(VOLeftLeg, VOPos), chk = vsub(relVel, VOPos);
        int liesBelow = bse.x * chk.y - bse.y * chk.x > 0; /* IsLeftOfVector */

        if (liesBelow) {
            og_real distToEdge = VORadius - og_sqrt(sqDistFromCircleCentre);
            og_v2 lineNormal = vnormalize(vsub(relVel, VOPos));
            og_v2 pointOnLine = vadd(velocity, vmul(vmul(lineNormal, distToEdge), 0.5f));
            n = push_con(cons, n, cap, pointOnLine, lineNormal);
        } else {
            og_v2 leftPerp = vdiv(vleft(VOPos), VOPosLength);
            int closerToLeft = vdot(leftPerp, relVel) >= 0;
            if (closerToLeft) {
                og_v2 lln = vnormalized(VOLeftLeg);
                og_real len = vdot(relVel, lln); /* GetClosestPointOnLineThroughOrigin */
                og_v2 U = vsub(vmul(lln, len), relVel);
                n = push_con(cons, n, cap, vadd(velocity, vmul(U, 0.5f)), vleft(lln));
            } else {
                og_v2 rln = vnormalized(VORightLeg);
                og_real len = vdot(relVel, rln);
                og_v2 U = vsub(vmul(rln, len), relVel);
                n = push_con(cons, n, cap, vadd(velocity, vmul(U, 0.5f)), vright(rln));
            }
        }
    }
    return n;
}

/* ---------------------------------------------------------------------------
 * ORCA::RandomizedLP (ECMAgentSimulator/ORCA.cpp:428-587)
 * ------------------------------------------------------------------------- */
int og_lp(const og_real* cons, int n, og_v2 opt, og_real maxSpeed, int useDirOpt, og_v2* out)
{
    if (useDirOpt) {
        *out = vmul(opt, maxSpeed);
    } else if (vlen(opt) > maxSpeed) {
        *out = vmul(vnormalized(opt), maxSpeed);
    } else {
        *out = opt;
    }
    if (n == 0) return n;

    for (int i = 0; i < n; i++) {
        og_v2 P = v2(cons[4 * i], cons[4 * i + 1]);
        og_v2 N = v2(cons[4 * i + 2], cons[4 * i + 3]);
        /* Constraint::Contains (ORCA.h:49-60): Det(Right(N), P - out) <= 0 */
        if (vdet(vright(N), vsub(P, *out)) <= 0.0f) continue;

        og_v2 dir = vright(N);
        og_real dirPointDot = vdot(dir, P);
        og_real discriminant = dirPointDot * dirPointDot + maxSpeed * maxSpeed - vdot(P, P);
        if (discriminant <= 0.0f) return i;
        /* a NaN discriminant takes neither branch (ORCA.cpp:498-506): the
           constraint is passed over */
        if (!(discriminant > 0.0f)) continue;

        og_real sq = og_sqrt(discriminant);
        og_real left = -dirPointDot - sq;
        og_real right = -dirPointDot + sq;
        for (int j = 0; j < i; j++) {
            og_v2 Pj = v2(cons[4 * j], cons[4 * j + 1]);
            og_v2 Nj = v2(cons[4 * j + 2], cons[4 * j + 3]);
            og_real den = vdet(vright(N), vright(Nj));
            og_real num = vdet(vright(Nj), vsub(P, Pj));
            if (og_fabs(den) <= OG_EPS) {
                if (num < 0.0f) return i;
                continue;
            }
            const og_real t = num / den;
            if (den >= 0.0f) right = (t < right) ? t : right; /* std::min(right, t) */
            else left = (left < t) ? t : left;                 /* std::max(left, t)  */
            if (left > right) return i;
        }
        if (useDirOpt) {
            if (vdot(opt, vright(N)) > 0) *out = vadd(P, vmul(vright(N), right));
            else *out = vadd(P, vmul(vright(N), left));
        } else {
            og_real t = vdot(vright(N), vsub(opt, P));
            if (t < left) *out = vadd(P, vmul(vright(N), left));
            else if (t > right) *out = vadd(P, vmul(vright(N), right));
            else *out = vadd(P, vmul(vright(N), t));
        }
    }
    return n;
}

/* ---------------------------------------------------------------------------
 * ORCA::RandomizedLP3D (ECMAgentSimulator/ORCA.cpp:592-669)
 * ------------------------------------------------------------------------- */
/* fp64 != 0: the bisector of two non-parallel lines is intersected in
   double precision and rounded to og_real, as the GPU tick's lp3d_fp64 mode
   does (the reference computes it in float) */
static void lp3d_impl(const og_real* cons, int n, int nObst, og_real maxSpeed, int failed, og_v2* out, int fp64);
void og_lp3d(const og_real* cons, int n, int nObst, og_real maxSpeed, int failed, og_v2* out)
{
    lp3d_impl(cons, n, nObst, maxSpeed, failed, out, 0);
}
static void lp3d_impl(const og_real* cons, int n, int nObst, og_real maxSpeed, int failed, og_v2* out, int fp64)
{
    og_real maxPen = 0.0f;
    og_real* proj = (og_real*)malloc(sizeof(og_real) * 4 * (size_t)(n + 1));
    for (int i = failed; i < n; i++) {
        og_v2 Pi = v2(cons[4 * i], cons[4 * i + 1]);
        og_v2 Ni = v2(cons[4 * i + 2], cons[4 * i + 3]);
        og_v2 dir = vright(Ni);
        if (vdet(dir, vsub(Pi, *out)) <= maxPen) continue;

        int m = 0;
        for (int k = 0; k < nObst; k++, m++) memcpy(proj + 4 * m, cons + 4 * k, sizeof(og_real) * 4);
        for (int j = nObst; j < i; j++) {
            og_v2 Pj = v2(cons[4 * j], cons[4 * j + 1]);
            og_v2 Nj = v2(cons[4 * j + 2], cons[4 * j + 3]);
            og_real det = vdet(vright(Ni), vright(Nj));
            og_v2 newP;
            if (og_fabs(det) <= OG_EPS) {
                if (vdot(Ni, Nj) > 0) continue;
                newP = vmul(vadd(Pi, Pj), 0.5f);
            } else if (!fp64) {
                og_real t = vdet(vright(Nj), vsub(Pi, Pj)) / det;
                newP = vadd(Pi, vmul(vright(Ni), t));
            } else {
                const double ax = (double)Nj.y, ay = -(double)Nj.x; /* Right(Nj) */
                const double bx = (double)Pi.x - (double)Pj.x, by = (double)Pi.y - (double)Pj.y;
                const double rx = (double)Ni.y, ry = -(double)Ni.x; /* Right(Ni) */
                const double dd = rx * ay - ry * ax;
                const double t = (ax * by - ay * bx) / dd;
                newP = v2((og_real)((double)Pi.x + rx * t), (og_real)((double)Pi.y + ry * t));
            }
            og_v2 nn = vnormalized(vsub(Nj, Ni));
            proj[4 * m + 0] = newP.x;
            proj[4 * m + 1] = newP.y;
            proj[4 * m + 2] = nn.x;
            proj[4 * m + 3] = nn.y;
            m++;
        }
        og_v2 temp = *out;
        if (og_lp(proj, m, Ni, maxSpeed, 1, out) < m) *out = temp;
        maxPen = vdet(dir, vsub(Pi, *out));
    }
    free(proj);
}

/* ORCA::GetVelocity (ECMAgentSimulator/ORCA.cpp:14-57), neighbours given */
int og_orca_velocity(const og_obstacles* o, const og_state* s, const og_params* p,
                     int agent, const int* nbrs, int n_nbrs, og_v2 pref_vel,
                     og_v2* out_vel, int* out_n_obst, int* out_fail)
{
    og_real maxSpeed = p->max_speed > 0.0f ? p->max_speed : s->pref_speed[agent];
    og_real range = p->tau_obst * maxSpeed + s->clear[agent];
    int cap_o = 64;
    int* ob = (int*)malloc(sizeof(int) * (size_t)cap_o);
    int no = og_find_obstacles(o, s->pos[agent], range * range, ob, cap_o, p->libm);
    if (no > cap_o) {
        free(ob);
        cap_o = no;
        ob = (int*)malloc(sizeof(int) * (size_t)cap_o);
        no = og_find_obstacles(o, s->pos[agent], range * range, ob, cap_o, p->libm);
    }
    int cap = no + n_nbrs + 1;
    og_real* cons = (og_real*)malloc(sizeof(og_real) * 4 * (size_t)cap);
    int nob = 0;
    int m = og_generate_constraints(o, s, p, agent, nbrs, n_nbrs, ob, no, cons, cap, &nob);
    int failed = og_lp(cons, m, pref_vel, maxSpeed, 0, out_vel);
    if (failed < m) lp3d_impl(cons, m, nob, maxSpeed, failed, out_vel, p->lp3d_fp64);
    if (out_n_obst) *out_n_obst = nob;
    if (out_fail) *out_fail = failed;
    free(cons);
    free(ob);
    return m;
}

/* ---------------------------------------------------------------------------
 * ECM queries
 * ------------------------------------------------------------------------- */

/* MathUtility::Contains(Point, vector<Segment>) (UtilityFunctions.cpp:54-86) */
static int contains_poly(og_v2 p, const og_v2* q, int nq)
{
    int inside = 0;
    for (int s = 0; s < nq; s++) {
        og_v2 a = q[s], b = q[(s + 1) % nq];
        if (vapprox(p, a)) return 0;
        if (vapprox(p, b)) return 0;
        if (p.y > og_fmin(a.y, b.y)) {
            if (p.y < og_fmax(a.y, b.y)) {
                if (p.x < og_fmax(a.x, b.x)) {
                    og_real xi = (p.y - a.y) * (b.x - a.x) / (b.y - a.y) + a.x;
                    if (a.x == b.x || p.x < xi) inside = !inside;
                }
            }
        }
    }
    return inside;
}

/* cell c of ECMCellCollection::Construct (ECMCellCollection.cpp:10-49):
   cell 2e = left, 2e+1 = right; polygon of PointLocationQueryLinear
   (ECMCellCollection.cpp:67-80): [v(he1.target), b.p0, b.p1, v(he0.target)] */
static void cell_quad(const og_ecm* e, int c, og_v2* q)
{
    int ed = c >> 1;
    const int h0 = 2 * ed, h1 = 2 * ed + 1;
    og_v2 b0, b1;
    if ((c & 1) == 0) { b0 = e->he_left[h0]; b1 = e->he_right[h1]; }
    else { b0 = e->he_right[h0]; b1 = e->he_left[h1]; }
    q[0] = e->v_pos[e->he_target[h1]];
    q[1] = b0;
    q[2] = b1;
    q[3] = e->v_pos[e->he_target[h0]];
}

/* ECMCellCollection::PointLocationQueryLinear (ECMCellCollection.cpp:57-90) */
int og_point_location(const og_ecm* e, og_v2 p)
{
    og_v2 q[4];
    for (int c = 0; c < 2 * e->n_edges; c++) {
        cell_quad(e, c, q);
        if (contains_poly(p, q, 4)) return c;
    }
    return -1;
}

/* MathUtility::GetRayToLineSegmentIntersection (UtilityFunctions.cpp:323-349) */
static int ray_segment(og_v2 o, og_v2 d, og_v2 p1, og_v2 p2, og_v2* out)
{
    og_v2 v1 = vsub(o, p1);
    og_v2 v2_ = vsub(p2, p1);
    og_v2 v3 = v2(-d.y, d.x);
    og_real dot = vdot(v2_, v3);
    if (og_fabs(dot) < 0.000001) return 0;
    og_real t1 = vdet(v2_, v1) / dot; /* Cross(v2, v1) */
    og_real t2 = vdot(v1, v3) / dot;
    if (t1 >= 0.0 && (t2 >= 0.0 && t2 <= 1.0)) {
        out->x = o.x + d.x * t1;
        out->y = o.y + d.y * t1;
        return 1;
    }
    return 0;
}

/* ECM::RetractPoint (ECMGenerator/ECM.cpp:20-96) */
int og_retract(const og_ecm* e, og_v2 loc, og_v2* out, int* out_edge)
{
    int c = og_point_location(e, loc);
    if (c < 0) return 0;
    int ed = c >> 1;
    const int h0 = 2 * ed, h1 = 2 * ed + 1;
    int ip1 = e->he_target[h1], ip2 = e->he_target[h0];
    og_v2 p1 = e->v_pos[ip1], p2 = e->v_pos[ip2];
    int toP2 = e->he_target[h0] == e->v_idx[ip2] ? 0 : 1;
    int toP1 = (toP2 + 1) % 2;
    og_v2 o1, o2, rd;
    /* IsLeftOfSegment (UtilityFunctions.cpp:193-196) */
    int left = (p2.x - p1.x) * (loc.y - p1.y) - (p2.y - p1.y) * (loc.x - p1.x) > 0;
    if (left) {
        o1 = e->he_left[2 * ed + toP2];
        o2 = e->he_right[2 * ed + toP1];
        if (vapprox(o1, o2)) rd = vadd(vsub(p1, o1), vsub(p2, o1));
        else { og_v2 v = vsub(o2, o1); rd = v2(v.y, -v.x); }
        rd = vnormalize(rd);
    } else {
        o1 = e->he_right[2 * ed + toP2];
        o2 = e->he_left[2 * ed + toP1];
        if (vapprox(o1, o2)) rd = vadd(vsub(p1, o1), vsub(p2, o1));
        else { og_v2 v = vsub(o2, o1); rd = v2(-v.y, v.x); }
        rd = vnormalize(rd);
    }
    if (out_edge) *out_edge = ed;
    return ray_segment(loc, rd, p1, p2, out);
}

/* IRMPathFollower::FindAttractionPoint (ECMAgentSimulator/IRMPathFollower.cpp:14-115)
   *out is only written on the paths where the reference writes outPoint. */
int og_irm(const og_ecm* e, og_v2 pos, const og_v2* path, int n, og_v2* out)
{
    og_v2 r;
    int ed;
    if (!og_retract(e, pos, &r, &ed)) return 0;
    og_v2 oa = e->he_left[2 * ed];
    og_v2 ob = e->he_right[2 * ed + 1];
    og_v2 co = closest_on_segment(r, oa, ob);
    og_real clearance = vlen(vsub(r, co));
    og_real rcs = clearance * clearance;
    og_v2 goal = path[n - 1];
    og_v2 ptg = vsub(goal, r);
    if (vlen2(ptg) < rcs) { *out = goal; return 1; }
    int success = 0;
    for (int i = 0; i < n - 1; i++) {
        og_v2 p1 = vsub(path[i], r);
        og_v2 p2 = vsub(path[i + 1], r);
        og_v2 ed2 = vsub(p2, p1);
        og_real els = vlen2(ed2);
        og_real det = vdet(p1, p2);
        og_real disc = rcs * els - det * det;
        if (disc < OG_EPS) continue;
        success = 1;
        int dySign = ed2.y < 0.0f ? -1 : 1;
        og_real sd = og_sqrt(disc);
        og_v2 i1 = v2((det * ed2.y + (og_real)dySign * ed2.x * sd) / els, (-det * ed2.x + og_fabs(ed2.y) * sd) / els);
        og_v2 i2 = v2((det * ed2.y - (og_real)dySign * ed2.x * sd) / els, (-det * ed2.x - og_fabs(ed2.y) * sd) / els);
        og_v2 g1 = vadd(p1, r), g2 = vadd(p2, r);
        og_v2 gi1 = vadd(i1, r), gi2 = vadd(i2, r);
        og_v2 edge = vsub(g2, g1);
        og_real t1 = vdot(vsub(gi1, g1), edge) / els;
        og_real t2 = vdot(vsub(gi2, g1), edge) / els;
        og_real maxT = -1.0f;
        if (t1 >= 0.0f && t1 <= 1.0f) { *out = gi1; maxT = t1; }
        if (t2 >= 0.0f && t2 <= 1.0f) {
            if (t2 > maxT) *out = gi2;
        }
    }
    return success;
}

/* ---------------------------------------------------------------------------
 * Simulator::Update (ECMAgentSimulator/Simulator.cpp:314-323)
 * ------------------------------------------------------------------------- */
typedef struct {
    const og_obstacles* o;
    const og_state* s;
    const og_params* p;
    const unsigned char* alive;   /* active after the attraction stage */
    const og_state* snap;         /* neighbour set: active at tick start */
    og_v2* vorca;
    og_tick_out* out;
    int lo, hi;
    int n_lp3d;
} og_job;

static void orca_range(og_job* j)
{
    const og_params* p = j->p;
    int k = p->k;
    int* ids = (int*)malloc(sizeof(int) * (size_t)(k > 0 ? k : 1));
    og_real* d2 = (og_real*)malloc(sizeof(og_real) * (size_t)(k > 0 ? k : 1));
    og_real r2 = p->neighbor_dist * p->neighbor_dist;
    for (int i = j->lo; i < j->hi; i++) {
        if (!j->alive[i]) continue;
        int nn = og_knn_exact(j->snap, i, k, r2, ids, d2);
        int nob = 0, fail = 0;
        og_v2 v;
        int m = og_orca_velocity(j->o, j->s, p, i, ids, nn, j->s->pref_vel[i], &v, &nob, &fail);
        j->vorca[i] = v;
        if (fail < m) j->n_lp3d++;
        og_tick_out* out = j->out;
        if (out) {
            if (out->nbr_ids) {
                for (int q = 0; q < k; q++) out->nbr_ids[(size_t)i * k + q] = q < nn ? ids[q] : -1;
            }
            if (out->nbr_count) out->nbr_count[i] = nn;
            if (out->n_constraints) out->n_constraints[i] = m;
            if (out->n_obst_constraints) out->n_obst_constraints[i] = nob;
            if (out->lp_fail) out->lp_fail[i] = fail;
        }
    }
    free(ids);
    free(d2);
}

static void* orca_thread(void* arg)
{
    orca_range((og_job*)arg);
    return NULL;
}

/* one agent of UpdateAttractionPointSystem (Simulator.cpp:538-590): writes
   the attraction point to *attr (left as it is when the IRM query fails);
   returns 0, 1 when the agent is to be destroyed, 2 when it needs a replan */
static int attract_one(const og_ecm* e, const og_state* s, const og_params* p, int i, og_v2* attr)
{
    const og_real delSq = p->delete_radius * p->delete_radius;
    const og_real arrSq = p->arrival_radius * p->arrival_radius;
    const og_v2* path = s->path_xy + s->path_off[i];
    int np = s->path_len[i];
    og_v2 pos = s->pos[i];
    og_v2 g = path[np - 1];
    og_real dx = pos.x - g.x, dy = pos.y - g.y; /* SquareDistance(x0,y0,x1,y1) */
    og_real dist = dx * dx + dy * dy;
    if (dist < arrSq) {
        *attr = g;
        return dist < delSq ? 1 : 0;
    }
    og_v2 ap = v2(0.0f, 0.0f); /* Point attractionPoint; */
    if (og_irm(e, pos, path, np, &ap)) {
        *attr = ap;
        return 0;
    }
    return 2;
}

int og_tick(const og_obstacles* o, const og_ecm* e, og_state* s, const og_params* p,
            og_kdtree* kd, og_tick_out* out)
{
    /* UpdateMaxAgentIndex (Simulator.cpp:481-492) */
    int empty = 0;
    for (int i = s->last_idx; i >= 0; i--) {
        if (s->active[i]) break;
        empty++;
    }
    s->last_idx = s->last_idx - empty;
    int last = s->last_idx;
    int n = s->n_slots;

    /* tick-start snapshot: the neighbour structure is built before any agent
       is destroyed (Simulator.cpp:319 before 320) */
    unsigned char* act0 = (unsigned char*)malloc((size_t)(n > 0 ? n : 1));
    memcpy(act0, s->active, (size_t)n);
    og_state snap = *s;
    snap.active = act0;
    if (p->knn_mode == 1 && kd) og_kdtree_build(kd, s);

    if (out) { out->n_destroyed = 0; out->n_replan = 0; out->n_lp3d = 0; }

    /* UpdateAttractionPointSystem (Simulator.cpp:538-590) */
    for (int i = 0; i <= last; i++) {
        if (!s->active[i]) continue;
        int r = attract_one(e, s, p, i, &s->attr[i]);
        if (r == 1) { /* DestroyAgent (Simulator.cpp:202-208) */
            s->num_agents--;
            s->active[i] = 0;
            if (out) {
                if (out->destroyed) out->destroyed[out->n_destroyed] = i;
                out->n_destroyed++;
            }
        } else if (r == 2 && out) {
            if (out->replan) out->replan[out->n_replan] = i;
            if (out->replan_pos) out->replan_pos[out->n_replan] = s->pos[i];
            out->n_replan++;
        }
    }

    /* ApplySteeringForce (Simulator.cpp:638-657) */
    for (int i = 0; i <= last; i++) {
        if (!s->active[i]) continue;
        og_v2 d = vsub(s->attr[i], s->pos[i]);
        d = vnormalize(d);
        d = vmul(d, s->pref_speed[i]);
        s->pref_vel[i] = d;
    }

    /* ApplyObstacleAvoidanceForce (Simulator.cpp:659-686) */
    og_v2* vorca = (og_v2*)malloc(sizeof(og_v2) * (size_t)(n > 0 ? n : 1));
    int n_lp3d = 0;
    if (p->knn_mode == 1) {
        int k = p->k;
        int* ids = (int*)malloc(sizeof(int) * (size_t)k);
        for (int i = 0; i <= last; i++) {
            if (!s->active[i]) continue;
            int nn = og_kdtree_query(kd, &snap, i, ids);
            int nob = 0, fail = 0;
            og_v2 v;
            int m = og_orca_velocity(o, s, p, i, ids, nn, s->pref_vel[i], &v, &nob, &fail);
            vorca[i] = v;
            if (fail < m) n_lp3d++;
            if (out) {
                if (out->nbr_ids)
                    for (int q = 0; q < k; q++) out->nbr_ids[(size_t)i * k + q] = q < nn ? ids[q] : -1;
                if (out->nbr_count) out->nbr_count[i] = nn;
                if (out->n_constraints) out->n_constraints[i] = m;
                if (out->n_obst_constraints) out->n_obst_constraints[i] = nob;
                if (out->lp_fail) out->lp_fail[i] = fail;
            }
        }
        free(ids);
    } else {
        int th = p->threads > 1 ? p->threads : 1;
        og_job* jobs = (og_job*)calloc((size_t)th, sizeof(og_job));
        pthread_t* tid = (pthread_t*)calloc((size_t)th, sizeof(pthread_t));
        int span = (last + 1 + th - 1) / th;
        for (int t = 0; t < th; t++) {
            jobs[t].o = o; jobs[t].s = s; jobs[t].p = p; jobs[t].alive = s->active;
            jobs[t].snap = &snap; jobs[t].vorca = vorca; jobs[t].out = out;
            jobs[t].lo = t * span;
            jobs[t].hi = (t + 1) * span < last + 1 ? (t + 1) * span : last + 1;
            if (th > 1) pthread_create(&tid[t], NULL, orca_thread, &jobs[t]);
            else orca_range(&jobs[t]);
        }
        for (int t = 0; t < th; t++) {
            if (th > 1) pthread_join(tid[t], NULL);
            n_lp3d += jobs[t].n_lp3d;
        }
        free(jobs);
        free(tid);
    }
    if (out) {
        out->n_lp3d = n_lp3d;
        if (out->v_orca)
            for (int i = 0; i <= last; i++)
                if (s->active[i]) out->v_orca[i] = vorca[i];
    }

    /* UpdateVelocitySystem (Simulator.cpp:619-635): force = vOrca - v
       (Simulator.cpp:676-677), v += F * (1/m) * dt */
    const og_real massRecip = 1.0f / p->mass;
    for (int i = 0; i <= last; i++) {
        if (!s->active[i]) continue;
        og_real fx = vorca[i].x - s->vel[i].x;
        og_real fy = vorca[i].y - s->vel[i].y;
        s->vel[i].x += fx * massRecip * p->dt;
        s->vel[i].y += fy * massRecip * p->dt;
    }
    /* UpdatePositionSystem (Simulator.cpp:592-606) */
    for (int i = 0; i <= last; i++) {
        if (!s->active[i]) continue;
        s->pos[i].x += (s->vel[i].x * p->dt);
        s->pos[i].y += (s->vel[i].y * p->dt);
    }
    free(vorca);
    free(act0);
    return 0;
}

/* ---------------------------------------------------------------------------
 * CPU-baseline timing (see ecmg_oracle.h)
 * ------------------------------------------------------------------------- */
#include <time.h>

static double og_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

typedef struct {
    const og_obstacles* o;
    const og_ecm* e;
    const og_state* s;
    const og_params* p;
    og_kdtree kd; /* shares the tree, owns its neighbour cache */
    const int* sample;
    int lo, hi;
    double sink;
} og_sjob;

static void* sample_thread(void* arg)
{
    og_sjob* j = (og_sjob*)arg;
    const og_state* s = j->s;
    const og_params* p = j->p;
    int k = p->k;
    int* ids = (int*)malloc(sizeof(int) * (size_t)k);
    const og_real arrSq = p->arrival_radius * p->arrival_radius;
    for (int q = j->lo; q < j->hi; q++) {
        int i = j->sample[q];
        const og_v2* path = s->path_xy + s->path_off[i];
        int np = s->path_len[i];
        og_v2 pos = s->pos[i];
        og_v2 g = path[np - 1];
        og_real dx = pos.x - g.x, dy = pos.y - g.y;
        og_v2 attr = s->attr[i];
        if (dx * dx + dy * dy < arrSq) attr = g;
        else {
            og_v2 ap = v2(0.0f, 0.0f);
            if (og_irm(j->e, pos, path, np, &ap)) attr = ap;
        }
        og_v2 pv = vmul(vnormalize(vsub(attr, pos)), s->pref_speed[i]);
        int nn = og_kdtree_query(&j->kd, s, i, ids);
        og_v2 v;
        int nob, fail;
        og_orca_velocity(j->o, s, p, i, ids, nn, pv, &v, &nob, &fail);
        j->sink += v.x + v.y;
    }
    free(ids);
    return NULL;
}

int og_time_sample(const og_obstacles* o, const og_ecm* e, const og_state* s, const og_params* p,
                   const int* sample, int n_sample, int threads, double* t_build, double* t_agents)
{
    og_kdtree* kd = og_kdtree_create(p->k);
    double t0 = og_now();
    og_kdtree_build(kd, s);
    double t1 = og_now();
    int th = threads > 1 ? threads : 1;
    og_sjob* jobs = (og_sjob*)calloc((size_t)th, sizeof(og_sjob));
    pthread_t* tid = (pthread_t*)calloc((size_t)th, sizeof(pthread_t));
    int span = (n_sample + th - 1) / th;
    for (int t = 0; t < th; t++) {
        jobs[t].o = o; jobs[t].e = e; jobs[t].s = s; jobs[t].p = p;
        jobs[t].kd = *kd;
        jobs[t].kd.cache = (int*)calloc((size_t)p->k, sizeof(int));
        jobs[t].kd.dist = (og_real*)malloc(sizeof(og_real) * (size_t)p->k);
        jobs[t].sample = sample;
        jobs[t].lo = t * span < n_sample ? t * span : n_sample;
        jobs[t].hi = (t + 1) * span < n_sample ? (t + 1) * span : n_sample;
    }
    double t2 = og_now();
    for (int t = 1; t < th; t++) pthread_create(&tid[t], NULL, sample_thread, &jobs[t]);
    sample_thread(&jobs[0]);
    for (int t = 1; t < th; t++) pthread_join(tid[t], NULL);
    double t3 = og_now();
    for (int t = 0; t < th; t++) { free(jobs[t].kd.cache); free(jobs[t].kd.dist); }
    free(jobs);
    free(tid);
    og_kdtree_destroy(kd);
    if (t_build) *t_build = t1 - t0;
    if (t_agents) *t_agents = t3 - t2;
    return 0;
}

/* the shared transcendentals, exported for their accuracy tests */
float og_test_atanf(float x) { return ecmg_atanf(x); }
void og_test_sincosf(float a, float* s, float* c) { ecmg_sincosf(a, s, c); }
/* number of a in (0, pi/2] (every step-th binary32 value) where
   ecmg_sincosf(-a) is not (-sin a, cos a) bit for bit */
long og_test_sincos_symmetry(unsigned step)
{
    const float top = 1.57079637050628662109375f;
    unsigned top_bits;
    memcpy(&top_bits, &top, 4);
    long bad = 0;
    for (unsigned u = 1; u <= top_bits; u += step) {
        float a, s1, c1, s2, c2;
        memcpy(&a, &u, 4);
        ecmg_sincosf(a, &s1, &c1);
        ecmg_sincosf(-a, &s2, &c2);
        float ns1 = -s1;
        if (memcmp(&ns1, &s2, 4) != 0 || memcmp(&c1, &c2, 4) != 0) bad++;
    }
    return bad;
}

/* ---------------------------------------------------------------------------
 * One tick for a sample of agents (see ecmg_oracle.h)
 * ------------------------------------------------------------------------- */
typedef struct {
    const og_obstacles* o;
    const og_ecm* e;
    const og_state* s;
    const og_params* p;
    const int* sample;
    og_sample_out* out;
    int lo, hi;
} og_tjob;

static void* tick_sample_thread(void* arg)
{
    og_tjob* j = (og_tjob*)arg;
    const og_state* s = j->s;
    const og_params* p = j->p;
    og_sample_out* out = j->out;
    int k = p->k;
    int* ids = (int*)malloc(sizeof(int) * (size_t)(k > 0 ? k : 1));
    og_real* d2 = (og_real*)malloc(sizeof(og_real) * (size_t)(k > 0 ? k : 1));
    const og_real r2 = p->neighbor_dist * p->neighbor_dist;
    const og_real massRecip = 1.0f / p->mass;
    for (int q = j->lo; q < j->hi; q++) {
        int i = j->sample[q];
        for (int c = 0; c < k; c++) out->nbr_ids[(size_t)q * k + c] = -1;
        out->nbr_count[q] = 0;
        if (i < 0 || i > s->last_idx || !s->active[i]) {
            out->status[q] = 3;
            continue;
        }
        og_v2 attr = s->attr[i];
        int r = attract_one(j->e, s, p, i, &attr);
        out->attr[q] = attr;
        out->status[q] = (unsigned char)r;
        if (r == 1) continue;
        /* ApplySteeringForce (Simulator.cpp:638-657) */
        og_v2 pv = vmul(vnormalize(vsub(attr, s->pos[i])), s->pref_speed[i]);
        /* ApplyObstacleAvoidanceForce: neighbours among the agents active at
           the start of the tick */
        int nn = og_knn_exact(s, i, k, r2, ids, d2);
        og_v2 v;
        int nob = 0, fail = 0;
        og_orca_velocity(j->o, s, p, i, ids, nn, pv, &v, &nob, &fail);
        for (int c = 0; c < nn; c++) out->nbr_ids[(size_t)q * k + c] = ids[c];
        out->nbr_count[q] = nn;
        out->v_orca[q] = v;
        /* UpdateVelocitySystem, UpdatePositionSystem */
        og_v2 vel = s->vel[i];
        og_real fx = v.x - vel.x;
        og_real fy = v.y - vel.y;
        vel.x += fx * massRecip * p->dt;
        vel.y += fy * massRecip * p->dt;
        og_v2 pos = s->pos[i];
        pos.x += (vel.x * p->dt);
        pos.y += (vel.y * p->dt);
        out->vel[q] = vel;
        out->pos[q] = pos;
    }
    free(ids);
    free(d2);
    return NULL;
}

int og_tick_sample(const og_obstacles* o, const og_ecm* e, const og_state* s, const og_params* p,
                   const int* sample, int n_sample, int threads, og_sample_out* out)
{
    int th = threads > 1 ? threads : 1;
    og_tjob* jobs = (og_tjob*)calloc((size_t)th, sizeof(og_tjob));
    pthread_t* tid = (pthread_t*)calloc((size_t)th, sizeof(pthread_t));
    int span = (n_sample + th - 1) / th;
    for (int t = 0; t < th; t++) {
        jobs[t].o = o; jobs[t].e = e; jobs[t].s = s; jobs[t].p = p;
        jobs[t].sample = sample;
        jobs[t].out = out;
        jobs[t].lo = t * span < n_sample ? t * span : n_sample;
        jobs[t].hi = (t + 1) * span < n_sample ? (t + 1) * span : n_sample;
    }
    for (int t = 1; t < th; t++) pthread_create(&tid[t], NULL, tick_sample_thread, &jobs[t]);
    tick_sample_thread(&jobs[0]);
    for (int t = 1; t < th; t++) pthread_join(tid[t], NULL);
    free(jobs);
    free(tid);
    return 0;
}

/* ---------------------------------------------------------------------------
 * Path planning: ECMPathPlanner::FindPath (ECMGenerator/ECMPathPlanner.cpp:22-136)
 * ------------------------------------------------------------------------- */

/* a growable array of fixed-size elements */
typedef struct { void* p; int n, cap, esz; } og_vec;
static void* vec_push(og_vec* v)
{
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 64;
        v->p = realloc(v->p, (size_t)v->cap * (size_t)v->esz);
    }
    return (char*)v->p + (size_t)v->n++ * (size_t)v->esz;
}
#define VEC_AT(v, T, i) (((T*)(v).p)[i])

typedef struct { og_v2 p0, p1; } og_seg;

struct og_planner {
    const og_ecm* e;
    /* AStar::m_Nodes (AStar.h:59-63): per vertex index g and f cost, parent,
       visited flag; reset after every request (CleanRequestData) */
    og_real* g;
    og_real* f;
    unsigned* parent;
    unsigned char* visited;
    og_vec heap, apath, rpath, hpath, centers, radii, lb, rb, lcb, rcb, curve, portals;
};

og_planner* og_planner_create(const og_ecm* e)
{
    og_planner* pl = (og_planner*)calloc(1, sizeof(og_planner));
    const int V = e->n_vertices > 0 ? e->n_vertices : 1;
    pl->e = e;
    pl->g = (og_real*)malloc(sizeof(og_real) * (size_t)V);
    pl->f = (og_real*)malloc(sizeof(og_real) * (size_t)V);
    pl->parent = (unsigned*)malloc(sizeof(unsigned) * (size_t)V);
    pl->visited = (unsigned char*)calloc((size_t)V, 1);
    /* AStar::Initialize (AStar.cpp:9-31) */
    for (int i = 0; i < V; i++) {
        pl->g[i] = OG_REAL_MAX;
        pl->f[i] = OG_REAL_MAX;
        pl->parent[i] = (unsigned)e->n_vertices;
    }
    pl->heap.esz = pl->apath.esz = pl->rpath.esz = pl->hpath.esz = pl->curve.esz = sizeof(int);
    pl->centers.esz = pl->lb.esz = pl->rb.esz = pl->lcb.esz = pl->rcb.esz = sizeof(og_v2);
    pl->radii.esz = sizeof(og_real);
    pl->portals.esz = sizeof(og_seg);
    return pl;
}

void og_planner_destroy(og_planner* pl)
{
    if (!pl) return;
    free(pl->g); free(pl->f); free(pl->parent); free(pl->visited);
    og_vec* v[] = {&pl->heap, &pl->apath, &pl->rpath, &pl->hpath, &pl->centers, &pl->radii, &pl->lb, &pl->rb,
                   &pl->lcb, &pl->rcb, &pl->curve, &pl->portals};
    for (size_t i = 0; i < sizeof(v) / sizeof(v[0]); i++) free(v[i]->p);
    free(pl);
}

/* MathUtility::Distance(p1, p2) (UtilityFunctions.cpp:15-22) */
static og_real pl_dist(og_v2 p1, og_v2 p2)
{
    og_real dx = p2.x - p1.x, dy = p2.y - p1.y;
    return og_sqrt(dx * dx + dy * dy);
}
/* Point::operator== (ECMDataTypes.h:99-103) */
static int pl_eq(og_v2 a, og_v2 b)
{
    return a.x > b.x - OG_EPS && a.x < b.x + OG_EPS && a.y > b.y - OG_EPS && a.y < b.y + OG_EPS;
}
/* MathUtility::TriangleArea (UtilityFunctions.cpp:203-210) */
static og_real pl_area(og_v2 p1, og_v2 p2, og_v2 p3)
{
    og_real ax = p2.x - p1.x, ay = p2.y - p1.y, bx = p3.x - p1.x, by = p3.y - p1.y;
    return bx * ay - ax * by;
}
/* MathUtility::IsLeftOfSegment (UtilityFunctions.cpp:193-196) */
static int pl_left(og_seg s, og_v2 p)
{
    return (s.p1.x - s.p0.x) * (p.y - s.p0.y) - (s.p1.y - s.p0.y) * (p.x - s.p0.x) > 0;
}

/* The open list of AStar::FindPath is a std::priority_queue of node pointers
   ordered by AStarCompare (a->fCost > b->fCost, AStar.h:26-33) whose costs
   change after they are pushed, so its pop order is that of the binary-heap
   algorithm itself, restated here on vertex indices with the current f read
   at every comparison: push = append + sift up; pop = move the last element
   out, walk the hole from the root to a leaf along the child that does not
   compare before its sibling, then sift the moved element up from there. */
static int heap_before(const og_planner* pl, int a, int b) { return pl->f[a] > pl->f[b]; }
static void heap_sift_up(og_planner* pl, long hole, long top, int value)
{
    int* h = (int*)pl->heap.p;
    long parent = (hole - 1) / 2;
    while (hole > top && heap_before(pl, h[parent], value)) {
        h[hole] = h[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    h[hole] = value;
}
static void heap_push(og_planner* pl, int v)
{
    *(int*)vec_push(&pl->heap) = v;
    heap_sift_up(pl, pl->heap.n - 1, 0, v);
}
static void heap_pop(og_planner* pl)
{
    int* h = (int*)pl->heap.p;
    const long size = pl->heap.n;
    if (size > 1) {
        const long len = size - 1;
        const int value = h[len];
        h[len] = h[0];
        long hole = 0, child = 0;
        while (child < (len - 1) / 2) {
            child = 2 * (child + 1);
            if (heap_before(pl, h[child], h[child - 1])) child--;
            h[hole] = h[child];
            hole = child;
        }
        if ((len & 1) == 0 && child == (len - 2) / 2) {
            child = 2 * (child + 1);
            h[hole] = h[child - 1];
            hole = child - 1;
        }
        heap_sift_up(pl, hole, 0, value);
    }
    pl->heap.n--;
}

/* AStar::CleanRequestData (AStar.cpp:162-175) */
static void astar_clean(og_planner* pl)
{
    const int V = pl->e->n_vertices;
    for (int i = 0; i < V; i++) {
        pl->f[i] = OG_REAL_MAX;
        pl->g[i] = OG_REAL_MAX;
        pl->parent[i] = (unsigned)V;
        pl->visited[i] = 0;
    }
}

/* AStar::FindPath (AStar.cpp:44-160) with ConstructPath (AStar.cpp:183-210):
   vertex indices into pl->apath */
static int astar(og_planner* pl, og_v2 startLoc, og_v2 goalLoc, int startEdge, int goalEdge, og_real clearance)
{
    const og_ecm* e = pl->e;
    const unsigned INVALID = (unsigned)e->n_vertices;
    pl->heap.n = 0;
    pl->apath.n = 0;
    const int a = e->v_idx[e->he_target[2 * startEdge]], b = e->v_idx[e->he_target[2 * startEdge + 1]];
    pl->g[a] = pl_dist(startLoc, e->v_pos[e->he_target[2 * startEdge]]);
    pl->f[a] = pl->g[a] + pl_dist(e->v_pos[e->he_target[2 * startEdge]], goalLoc);
    pl->g[b] = pl_dist(startLoc, e->v_pos[e->he_target[2 * startEdge + 1]]);
    pl->f[b] = pl->g[b] + pl_dist(e->v_pos[e->he_target[2 * startEdge + 1]], goalLoc);
    heap_push(pl, a);
    heap_push(pl, b);
    const int ga = e->he_target[2 * goalEdge], gb = e->he_target[2 * goalEdge + 1];
    while (pl->heap.n > 0) {
        while (pl->heap.n > 0 && pl->visited[VEC_AT(pl->heap, int, 0)]) heap_pop(pl);
        if (pl->heap.n == 0) {
            astar_clean(pl);
            return 0;
        }
        const int cur = VEC_AT(pl->heap, int, 0);
        heap_pop(pl);
        pl->visited[cur] = 1;
        if (e->v_clear[cur] < clearance) continue;
        if (cur == ga || cur == gb) {
            pl->rpath.n = 0;
            *(int*)vec_push(&pl->rpath) = cur == ga ? gb : ga;
            *(int*)vec_push(&pl->rpath) = cur == ga ? ga : gb;
            for (unsigned nx = pl->parent[cur]; nx < INVALID; nx = pl->parent[nx]) *(int*)vec_push(&pl->rpath) = (int)nx;
            for (int i = pl->rpath.n - 1; i >= 0; i--) *(int*)vec_push(&pl->apath) = VEC_AT(pl->rpath, int, i);
            astar_clean(pl);
            return 1;
        }
        /* neighbours: the targets of the half-edges from the vertex's first
           outgoing one, following next_idx until the first target recurs */
        int he = e->v_halfedge[cur];
        if (he < 0) continue; /* an isolated vertex (the reference would read out of bounds) */
        const int first = e->he_target[he];
        int nb = first, guard = 0;
        do {
            if (!pl->visited[nb]) {
                heap_push(pl, nb);
                const og_v2 cp = e->v_pos[cur], np = e->v_pos[nb];
                const og_real ng = pl->g[cur] + pl_dist(cp, np);
                if (ng < pl->g[nb]) {
                    const og_real nf = ng + pl_dist(np, goalLoc);
                    pl->parent[nb] = (unsigned)cur;
                    pl->f[nb] = nf;
                    pl->g[nb] = ng;
                }
            }
            he = e->he_next[he];
            nb = e->he_target[he];
        } while (nb != first && ++guard < 65536);
    }
    astar_clean(pl);
    return 0;
}

/* SampleCorridorArc (ECMPathPlanner.cpp:255-276) */
static void sample_arc(og_planner* pl, og_v2 p1, og_v2 p2, og_v2 o1, og_v2 o2, og_v2 c, og_real radius, int leftArc)
{
    const og_real maxLen = 10.0f;
    og_seg* s = (og_seg*)vec_push(&pl->portals);
    if (leftArc) { s->p0 = p1; s->p1 = o1; }
    else { s->p0 = o1; s->p1 = p1; }
    const og_v2 d = vsub(p2, p1);
    const og_real edgeLength = og_sqrt(d.x * d.x + d.y * d.y);
    const int numSamples = (int)og_ceil(edgeLength / maxLen);
    const og_real sampleLength = edgeLength / (og_real)numSamples;
    const og_v2 dir = vdiv(d, edgeLength);
    for (int i = 0; i < numSamples; i++) {
        og_v2 step = vmul(vmul(dir, sampleLength), (og_real)i);
        og_v2 p = v2(p1.x + step.x, p1.y + step.y);
        og_v2 a = vnormalize(vsub(p, c));
        p = v2(c.x + a.x * radius, c.y + a.y * radius);
        s = (og_seg*)vec_push(&pl->portals);
        if (leftArc) { s->p0 = p; s->p1 = o2; }
        else { s->p0 = o2; s->p1 = p; }
    }
}

/* ECMPathPlanner::Funnel (ECMPathPlanner.cpp:321-411): the simple stupid
   funnel algorithm; returns the number of points written (-2: more than cap) */
static int funnel(const og_seg* portals, int np, og_v2 start, og_v2 goal, og_v2* out, int cap)
{
    og_v2 apex = start, pleft = start, pright = start;
    int leftIdx = 0, rightIdx = 0, apexIdx = 0, n = 0;
#define PL_EMIT(q) do { if (n >= cap) return -2; out[n++] = (q); } while (0)
    PL_EMIT(start);
    for (int i = 0; i < np; i++) {
        const og_v2 left = portals[i].p0, right = portals[i].p1;
        if (pl_area(apex, pright, right) <= 0.0f) {
            if (vapprox(apex, pright) || pl_area(apex, pleft, right) > 0.0f) {
                pright = right;
                rightIdx = i;
            } else {
                PL_EMIT(pleft);
                apex = pleft;
                apexIdx = leftIdx;
                pleft = apex;
                pright = apex;
                leftIdx = apexIdx;
                rightIdx = apexIdx;
                i = apexIdx;
                continue;
            }
        }
        if (pl_area(apex, pleft, left) >= 0.0f) {
            if (vapprox(apex, pleft) || pl_area(apex, pright, left) < 0.0f) {
                pleft = left;
                leftIdx = i;
            } else {
                PL_EMIT(pright);
                apex = pright;
                apexIdx = rightIdx;
                pleft = apex;
                pright = apex;
                leftIdx = apexIdx;
                rightIdx = apexIdx;
                i = apexIdx;
                continue;
            }
        }
    }
    if (!vapprox(out[n - 1], goal)) PL_EMIT(goal);
#undef PL_EMIT
    return n;
}

int og_find_path(og_planner* pl, og_v2 start, og_v2 goal, og_real clearance, og_v2* out, int cap)
{
    const og_ecm* e = pl->e;
    if (cap < 2) return -2;
    /* clearance += preferredAdditionalClearance (0, Simulator.cpp:108) */
    /* 1. FindCell of start and goal (ECM.cpp:191-194: the linear query) */
    if (og_point_location(e, start) < 0 || og_point_location(e, goal) < 0) return -1;
    /* 2. ECM::RetractPoint */
    og_v2 rs, rg;
    int es, eg;
    if (!og_retract(e, start, &rs, &es)) return -1;
    if (!og_retract(e, goal, &rg, &eg)) return -1;
    if (es == eg) {
        out[0] = start;
        out[1] = goal;
        return 2;
    }
    /* 3. A* on the medial axis */
    if (!astar(pl, rs, rg, es, eg, clearance)) return -1;
    /* the half-edge between consecutive vertices of the A* path */
    pl->hpath.n = 0;
    for (int i = 0; i + 1 < pl->apath.n; i++) {
        const int a = VEC_AT(pl->apath, int, i), b = VEC_AT(pl->apath, int, i + 1);
        const int h0 = e->v_halfedge[a];
        if (h0 < 0) continue;
        int h = h0, guard = 0;
        do {
            if (e->he_target[h] == b) {
                *(int*)vec_push(&pl->hpath) = h;
                break;
            }
            h = e->he_next[h];
        } while (h != h0 && ++guard < 65536);
    }
    const int n = pl->hpath.n;
    if (n == 0) return -1; /* the reference would read an empty corridor */
    /* 4. CreateCorridor (ECMPathPlanner.cpp:144-156): the source vertex of
       each half-edge (GetSource: the twin's target, ECM.h:71-84) */
    pl->centers.n = pl->radii.n = pl->lb.n = pl->rb.n = pl->lcb.n = pl->rcb.n = pl->curve.n = 0;
    for (int i = 0; i < n; i++) {
        const int h = VEC_AT(pl->hpath, int, i);
        const int src = e->he_target[h ^ 1];
        *(og_v2*)vec_push(&pl->centers) = e->v_pos[src];
        *(og_real*)vec_push(&pl->radii) = e->v_clear[src];
        *(og_v2*)vec_push(&pl->lb) = e->he_left[h];
        *(og_v2*)vec_push(&pl->rb) = e->he_right[h];
    }
    /* ShrinkCorridor (ECMPathPlanner.cpp:158-214) */
    for (int i = 0; i < n; i++) {
        const og_v2 c = VEC_AT(pl->centers, og_v2, i), l = VEC_AT(pl->lb, og_v2, i), r = VEC_AT(pl->rb, og_v2, i);
        og_v2 lc, rc;
        if (VEC_AT(pl->radii, og_real, i) < clearance) {
            lc = c;
            rc = c;
        } else {
            const og_v2 ml = vnormalize(vsub(c, l)), mr = vnormalize(vsub(c, r));
            lc = v2(l.x + ml.x * clearance, l.y + ml.y * clearance);
            rc = v2(r.x + mr.x * clearance, r.y + mr.y * clearance);
        }
        *(og_v2*)vec_push(&pl->lcb) = lc;
        *(og_v2*)vec_push(&pl->rcb) = rc;
        if (i + 1 < n) { /* CorridorBoundCurve: 0 LINEAR, 1 LEFT_ARC, 2 RIGHT_ARC */
            int t = 0;
            if (pl_eq(l, VEC_AT(pl->lb, og_v2, i + 1))) t = 1;
            else if (pl_eq(r, VEC_AT(pl->rb, og_v2, i + 1))) t = 2;
            *(int*)vec_push(&pl->curve) = t;
        }
    }
    /* 5. TriangulateCorridor (ECMPathPlanner.cpp:216-253) */
    pl->portals.n = 0;
    const og_v2* L = (const og_v2*)pl->lcb.p;
    const og_v2* R = (const og_v2*)pl->rcb.p;
    for (int i = 0; i + 1 < n; i++) {
        const int t = VEC_AT(pl->curve, int, i);
        if (t == 0) {
            og_seg* s = (og_seg*)vec_push(&pl->portals);
            s->p0 = L[i]; s->p1 = R[i];
            s = (og_seg*)vec_push(&pl->portals);
            s->p0 = L[i + 1]; s->p1 = R[i];
        } else if (t == 1) {
            sample_arc(pl, L[i], L[i + 1], R[i], R[i + 1], VEC_AT(pl->lb, og_v2, i), clearance, 1);
        } else {
            sample_arc(pl, R[i], R[i + 1], L[i], L[i + 1], VEC_AT(pl->rb, og_v2, i), clearance, 0);
        }
    }
    og_seg* last = (og_seg*)vec_push(&pl->portals);
    last->p0 = L[n - 1];
    last->p1 = R[n - 1];
    /* FitPortalRange (ECMPathPlanner.cpp:278-318) */
    og_seg* P = (og_seg*)pl->portals.p;
    int np = pl->portals.n, first = 0;
    for (int i = 0; i < np; i++)
        if (!pl_left(P[i], start)) {
            first = i;
            break;
        }
    memmove(P, P + first, sizeof(og_seg) * (size_t)(np - first));
    np -= first;
    int lastIdx = np - 1;
    for (int i = np - 1; i >= 0; i--)
        if (pl_left(P[i], goal)) {
            lastIdx = i;
            break;
        }
    np -= np - lastIdx;
    pl->portals.n = np;
    og_seg* gs = (og_seg*)vec_push(&pl->portals);
    gs->p0 = goal;
    gs->p1 = goal;
    /* 7. Funnel */
    return funnel((const og_seg*)pl->portals.p, pl->portals.n, start, goal, out, cap);
}

typedef struct {
    const og_ecm* e;
    const og_v2 *starts, *goals;
    const og_real* clr;
    og_v2* out;
    int* out_n;
    int cap, lo, hi;
} og_pjob;

static void* plan_thread(void* arg)
{
    og_pjob* j = (og_pjob*)arg;
    og_planner* pl = og_planner_create(j->e);
    for (int i = j->lo; i < j->hi; i++)
        j->out_n[i] = og_find_path(pl, j->starts[i], j->goals[i], j->clr[i], j->out + (size_t)i * j->cap, j->cap);
    og_planner_destroy(pl);
    return NULL;
}

int og_find_paths(const og_ecm* e, int n, const og_v2* starts, const og_v2* goals, const og_real* clr, int threads,
                  int cap, og_v2* out, int* out_n)
{
    int th = threads > 1 ? threads : 1;
    if (th > n) th = n > 0 ? n : 1;
    og_pjob* jobs = (og_pjob*)calloc((size_t)th, sizeof(og_pjob));
    pthread_t* tid = (pthread_t*)calloc((size_t)th, sizeof(pthread_t));
    for (int t = 0; t < th; t++) {
        jobs[t].e = e; jobs[t].starts = starts; jobs[t].goals = goals; jobs[t].clr = clr;
        jobs[t].out = out; jobs[t].out_n = out_n; jobs[t].cap = cap;
        jobs[t].lo = (int)((long long)n * t / th);
        jobs[t].hi = (int)((long long)n * (t + 1) / th);
    }
    for (int t = 1; t < th; t++) pthread_create(&tid[t], NULL, plan_thread, &jobs[t]);
    plan_thread(&jobs[0]);
    for (int t = 1; t < th; t++) pthread_join(tid[t], NULL);
    free(jobs);
    free(tid);
    return 0;
}

/* ---------------------------------------------------------------------------
 * Whole tick on host threads (see ecmg_oracle.h)
 * ------------------------------------------------------------------------- */
typedef struct {
    const og_obstacles* o;
    const og_ecm* e;
    og_state* s;
    const og_state* snap;
    const og_params* p;
    og_kdtree kd;            /* shares the tree, owns its neighbour cache */
    unsigned char* res;      /* attraction stage result per slot */
    og_v2* vorca;
    int stage, lo, hi, n_lp3d;
} og_mjob;

static void* mt_thread(void* arg)
{
    og_mjob* j = (og_mjob*)arg;
    og_state* s = j->s;
    const og_params* p = j->p;
    if (j->stage == 0) {
        /* UpdateAttractionPointSystem (Simulator.cpp:538-590), per slot */
        for (int i = j->lo; i < j->hi; i++)
            j->res[i] = s->active[i] ? (unsigned char)attract_one(j->e, s, p, i, &s->attr[i]) : 0;
    } else if (j->stage == 1) {
        /* ApplySteeringForce + ApplyObstacleAvoidanceForce (Simulator.cpp:638-686) */
        int* ids = (int*)malloc(sizeof(int) * (size_t)(p->k > 0 ? p->k : 1));
        for (int i = j->lo; i < j->hi; i++) {
            if (!s->active[i]) continue;
            s->pref_vel[i] = vmul(vnormalize(vsub(s->attr[i], s->pos[i])), s->pref_speed[i]);
            int nn = og_kdtree_query(&j->kd, j->snap, i, ids);
            int nob = 0, fail = 0;
            int m = og_orca_velocity(j->o, s, p, i, ids, nn, s->pref_vel[i], &j->vorca[i], &nob, &fail);
            if (fail < m) j->n_lp3d++;
        }
        free(ids);
    } else {
        /* UpdateVelocitySystem, UpdatePositionSystem (Simulator.cpp:592-635) */
        const og_real massRecip = 1.0f / p->mass;
        for (int i = j->lo; i < j->hi; i++) {
            if (!s->active[i]) continue;
            og_real fx = j->vorca[i].x - s->vel[i].x;
            og_real fy = j->vorca[i].y - s->vel[i].y;
            s->vel[i].x += fx * massRecip * p->dt;
            s->vel[i].y += fy * massRecip * p->dt;
            s->pos[i].x += (s->vel[i].x * p->dt);
            s->pos[i].y += (s->vel[i].y * p->dt);
        }
    }
    return NULL;
}

int og_tick_mt(const og_obstacles* o, const og_ecm* e, og_state* s, const og_params* p, og_kdtree* kd, int threads,
               og_tick_out* out)
{
    /* UpdateMaxAgentIndex (Simulator.cpp:481-492) */
    int empty = 0;
    for (int i = s->last_idx; i >= 0; i--) {
        if (s->active[i]) break;
        empty++;
    }
    s->last_idx -= empty;
    const int last = s->last_idx, n = s->n_slots;
    unsigned char* act0 = (unsigned char*)malloc((size_t)(n > 0 ? n : 1));
    memcpy(act0, s->active, (size_t)n);
    og_state snap = *s;
    snap.active = act0;
    /* KDTree::Construct (KDTree.cpp:22-83) over the tick-start agents */
    og_kdtree_build(kd, s);
    const int th = threads > 1 ? threads : 1;
    og_mjob* jobs = (og_mjob*)calloc((size_t)th, sizeof(og_mjob));
    pthread_t* tid = (pthread_t*)calloc((size_t)th, sizeof(pthread_t));
    unsigned char* res = (unsigned char*)calloc((size_t)(n > 0 ? n : 1), 1);
    og_v2* vorca = (og_v2*)calloc((size_t)(n > 0 ? n : 1), sizeof(og_v2));
    for (int t = 0; t < th; t++) {
        jobs[t].o = o; jobs[t].e = e; jobs[t].s = s; jobs[t].snap = &snap; jobs[t].p = p;
        jobs[t].kd = *kd;
        jobs[t].kd.cache = (int*)calloc((size_t)p->k, sizeof(int));
        jobs[t].kd.dist = (og_real*)malloc(sizeof(og_real) * (size_t)p->k);
        jobs[t].res = res; jobs[t].vorca = vorca;
        jobs[t].lo = (int)((long long)(last + 1) * t / th);
        jobs[t].hi = (int)((long long)(last + 1) * (t + 1) / th);
    }
    for (int stage = 0; stage < 3; stage++) {
        for (int t = 0; t < th; t++) jobs[t].stage = stage;
        for (int t = 1; t < th; t++) pthread_create(&tid[t], NULL, mt_thread, &jobs[t]);
        mt_thread(&jobs[0]);
        for (int t = 1; t < th; t++) pthread_join(tid[t], NULL);
        if (stage == 0) {
            /* DestroyAgent (Simulator.cpp:202-208) and re-plan requests, in slot order */
            if (out) { out->n_destroyed = 0; out->n_replan = 0; }
            for (int i = 0; i <= last; i++) {
                if (res[i] == 1) {
                    s->num_agents--;
                    s->active[i] = 0;
                    if (out) {
                        if (out->destroyed) out->destroyed[out->n_destroyed] = i;
                        out->n_destroyed++;
                    }
                } else if (res[i] == 2 && out) {
                    if (out->replan) out->replan[out->n_replan] = i;
                    if (out->replan_pos) out->replan_pos[out->n_replan] = s->pos[i];
                    out->n_replan++;
                }
            }
        }
    }
    int n_lp3d = 0;
    for (int t = 0; t < th; t++) {
        n_lp3d += jobs[t].n_lp3d;
        free(jobs[t].kd.cache);
        free(jobs[t].kd.dist);
    }
    if (out) out->n_lp3d = n_lp3d;
    free(jobs); free(tid); free(res); free(vorca); free(act0);
    return 0;
}
