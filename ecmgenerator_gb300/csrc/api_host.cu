/*
 * api_host.cu -- C ABI entry points that need no simulation context: the
 * host-only ECM planner (ecmg_planner_*) and the stand-alone device kNN
 * (ecmg_knn, ecmg_knn_scratch_bytes).
 */
#include "../../include/ecmg.h"
#include "ecmg_internal.h"
#include "host_scene.h"

#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

using namespace ecmg;

extern "C" {

struct ecmg_planner {
    HostScene scene;
    GridCSR vis;
    int mode = ECMG_PLANNER_REFERENCE;
};

ecmg_status ecmg_planner_create(const ecmg_obstacles* o, const ecmg_ecm* e, ecmg_planner** out)
{
    if (!o || !e || !out) return ECMG_ERR_INVALID_ARG;
    *out = nullptr;
    if (o->n_obstacles < 0 || e->n_vertices < 0 || e->n_edges < 0) return ECMG_ERR_INVALID_ARG;
    for (int r = 0; r < o->n_obstacles; r++)
        if (o->ring_offsets[r + 1] - o->ring_offsets[r] < 2) return ECMG_ERR_INVALID_ARG;
    for (int h = 0; h < 2 * e->n_edges; h++)
        if (e->he_target[h] < 0 || e->he_target[h] >= e->n_vertices) return ECMG_ERR_INVALID_ARG;
    ecmg_planner* p = new ecmg_planner();
    HostScene& s = p->scene;
    set_obstacles(s, o->n_obstacles, o->ring_offsets, o->xy);
    int V = e->n_vertices, E = e->n_edges;
    s.v_pos.resize(V); s.v_clear.resize(V); s.v_idx.resize(V); s.v_halfedge.resize(V);
    s.he_target.assign(e->he_target, e->he_target + 2 * (size_t)E);
    s.he_next.assign(e->he_next, e->he_next + 2 * (size_t)E);
    s.he_left.resize(2 * (size_t)E); s.he_right.resize(2 * (size_t)E);
    for (int i = 0; i < V; i++) {
        s.v_pos[i] = mk(e->v_pos[2 * i], e->v_pos[2 * i + 1]);
        s.v_clear[i] = e->v_clear[i];
        s.v_idx[i] = e->v_idx ? e->v_idx[i] : i;
        s.v_halfedge[i] = e->v_halfedge[i];
    }
    for (int h = 0; h < 2 * E; h++) {
        s.he_left[h] = mk(e->he_left[2 * h], e->he_left[2 * h + 1]);
        s.he_right[h] = mk(e->he_right[2 * h], e->he_right[2 * h + 1]);
    }
    s.has_ecm = true;
    float x0 = 1e30f, y0 = 1e30f, x1 = -1e30f, y1 = -1e30f;
    auto grow = [&](V2 q) { x0 = std::min(x0, q.x); y0 = std::min(y0, q.y); x1 = std::max(x1, q.x); y1 = std::max(y1, q.y); };
    for (auto& q : s.ob_p) grow(q);
    for (auto& q : s.v_pos) grow(q);
    for (auto& q : s.he_left) grow(q);
    for (auto& q : s.he_right) grow(q);
    if (x0 > x1) { x0 = y0 = 0; x1 = y1 = 1; }
    s.bx0 = x0; s.by0 = y0; s.bx1 = x1; s.by1 = y1;
    build_ecm_grid(s);
    build_obst_grid(s, 0.0f, 4.0f, p->vis);
    *out = p;
    return ECMG_OK;
}

ecmg_status ecmg_planner_destroy(ecmg_planner* p)
{
    if (!p) return ECMG_ERR_INVALID_ARG;
    delete p;
    return ECMG_OK;
}

ecmg_status ecmg_planner_find_paths(ecmg_planner* pl, int n, const float* starts, const float* goals,
                                    const float* clearances, int threads, int cap, float* out_xy, int* out_n)
{
    if (!pl || n < 0 || cap < 1 || (n > 0 && (!starts || !goals || !clearances || !out_xy || !out_n)))
        return ECMG_ERR_INVALID_ARG;
    if (threads < 1) threads = (int)std::max(1u, std::thread::hardware_concurrency());
    threads = std::min(threads, std::max(1, n));
    auto work = [&](int t) {
        PlanScratch scr;
        std::vector<V2> p;
        for (int i = t; i < n; i += threads) {
            const V2 a = mk(starts[2 * i], starts[2 * i + 1]), b = mk(goals[2 * i], goals[2 * i + 1]);
            bool ok = pl->mode == ECMG_PLANNER_REFERENCE ? plan_path_reference(pl->scene, a, b, clearances[i], p, scr.ref)
                                                         : plan_path(pl->scene, pl->vis, a, b, clearances[i], p, scr);
            if (!ok) { out_n[i] = -1; continue; }
            if ((int)p.size() > cap) { out_n[i] = -2; continue; }
            out_n[i] = (int)p.size();
            for (size_t q = 0; q < p.size(); q++) {
                out_xy[2 * ((size_t)i * cap + q)] = p[q].x;
                out_xy[2 * ((size_t)i * cap + q) + 1] = p[q].y;
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < threads; t++) th.emplace_back(work, t);
    work(0);
    for (auto& x : th) x.join();
    return ECMG_OK;
}

ecmg_status ecmg_planner_set_mode(ecmg_planner* pl, int mode)
{
    if (!pl || (mode != ECMG_PLANNER_FAST && mode != ECMG_PLANNER_REFERENCE)) return ECMG_ERR_INVALID_ARG;
    pl->mode = mode;
    return ECMG_OK;
}

ecmg_status ecmg_planner_locate(ecmg_planner* pl, int n, const float* xy, int* out)
{
    if (!pl || n < 0 || (n > 0 && (!xy || !out))) return ECMG_ERR_INVALID_ARG;
    EcmView ev = pl->scene.ecm_view();
    for (int i = 0; i < n; i++) out[i] = point_location(ev, mk(xy[2 * i], xy[2 * i + 1]));
    return ECMG_OK;
}

/* Simulator::ValidSpawnLocation (Simulator.cpp:295-311) on the device state */

}  // extern "C"

/* ---------------------------------------------------------------------- */
/* The grid of the stand-alone kNN: cells of `cell` metres over the box with
   one spare ring and one overflow bucket.  Sizes are computed in double and
   refused (false) when the box or the cell is not finite or the grid would
   exceed kKnnMaxCells cells, so that no int below overflows. */
bool ecmg::knn_grid_of(float x0, float y0, float x1, float y1, float cell, AgentGrid* out)
{
    if (!std::isfinite(x0) || !std::isfinite(y0) || !std::isfinite(x1) || !std::isfinite(y1)) return false;
    if (!(cell > 0.0f) || !std::isfinite(cell) || !(x1 >= x0) || !(y1 >= y0)) return false;
    const double gw = std::ceil(((double)x1 - (double)x0) / (double)cell) + 3.0;
    const double gh = std::ceil(((double)y1 - (double)y0) / (double)cell) + 3.0;
    if (!(gw * gh <= (double)kKnnMaxCells)) return false;
    AgentGrid g;
    g.cell = cell;
    g.inv = 1.0f / cell;
    g.x0 = x0 - cell;
    g.y0 = y0 - cell;
    g.gw = (int)gw;
    g.gh = (int)gh;
    g.ncells = g.gw * g.gh;
    *out = g;
    return true;
}

extern "C" {

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t ecmg_knn_scratch_bytes(int n, float min_x, float min_y, float max_x, float max_y, float cell)
{
    AgentGrid g;
    if (n < 0 || !knn_grid_of(min_x, min_y, max_x, max_y, cell, &g)) return 0;
    size_t nb = (size_t)g.ncells + 1;
    size_t b = 0;
    b += align256(sizeof(int) * (size_t)std::max(1, n)) * 3; /* key, rank, s_slot */
    b += align256(sizeof(V2) * (size_t)std::max(1, n));      /* s_pos */
    b += align256(sizeof(int) * (nb + 1 + kCounters));      /* cell_count + counters */
    b += align256(sizeof(int) * (nb + 1));                  /* cell_start */
    b += align256(sizeof(int) * (size_t)scan_tmp_ints((int)nb));
    return b;
}

ecmg_status ecmg_knn(const float* dev_pos, const unsigned char* dev_active, int n, int k, float radius, float min_x,
                     float min_y, float max_x, float max_y, float cell, int* dev_out_ids, int* dev_out_count,
                     void* dev_scratch, size_t scratch_bytes, void* stream)
{
    if (n < 0 || k < 1 || k > kMaxK || !(radius > 0.0f) || !(cell > 0.0f)) return ECMG_ERR_INVALID_ARG;
    if (n == 0) return ECMG_OK;
    if (!dev_pos || !dev_active || !dev_out_ids || !dev_out_count || !dev_scratch) return ECMG_ERR_INVALID_ARG;
    size_t need = ecmg_knn_scratch_bytes(n, min_x, min_y, max_x, max_y, cell);
    if (need == 0 || scratch_bytes < need) return ECMG_ERR_INVALID_ARG;
    AgentGrid g;
    if (!knn_grid_of(min_x, min_y, max_x, max_y, cell, &g)) return ECMG_ERR_INVALID_ARG;
    size_t nb = (size_t)g.ncells + 1;
    char* p = (char*)dev_scratch;
    auto take = [&](size_t bytes) { char* r = p; p += align256(bytes); return r; };
    int* key = (int*)take(sizeof(int) * n);
    int* rank = (int*)take(sizeof(int) * n);
    int* s_slot = (int*)take(sizeof(int) * n);
    V2* s_pos = (V2*)take(sizeof(V2) * n);
    int* cell_count = (int*)take(sizeof(int) * (nb + 1 + kCounters));
    int* cell_start = (int*)take(sizeof(int) * (nb + 1));
    int* scan_tmp = (int*)take(sizeof(int) * (size_t)scan_tmp_ints((int)nb));
    cudaError_t e = launch_knn((const V2*)dev_pos, dev_active, n, k, radius, g, key, rank, cell_count, cell_start,
                               s_slot, s_pos, scan_tmp, 0, dev_out_ids, dev_out_count, (cudaStream_t)stream);
    return e == cudaSuccess ? ECMG_OK : ECMG_ERR_CUDA;
}

}  // extern "C"
