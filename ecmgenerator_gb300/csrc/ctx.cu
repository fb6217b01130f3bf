/*
 * ctx.cu -- the C ABI of include/ecmg.h: context, device buffers, agent pool,
 * tick loop (optionally captured as a CUDA graph) and host re-planning.
 */
#include "../../include/ecmg.h"
#include "ecmg_internal.h"
#include "host_scene.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

using namespace ecmg;

namespace {

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t alloc(size_t count)
    {
        if (count <= n && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc((void**)&p, sizeof(T) * count);
        if (e == cudaSuccess) n = count;
        return e;
    }
    void free_()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

}  // namespace

struct ecmg_ctx {
    ecmg_params prm;
    int max_agents = 0;
    std::string err;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr, ev_a0 = nullptr, ev_a1 = nullptr;
    int sms = 1;

    /* host mirrors (Simulator bookkeeping, Simulator.h:164-171) */
    std::vector<unsigned char> active;
    std::vector<float> clear, speed;
    std::vector<std::vector<V2>> paths;
    std::vector<int> free_stack; /* back() = top */
    int num_agents = 0;
    int last_idx = -1;

    /* device agent state */
    DBuf<V2> pos, vel, attr, pref_vel, replan_pos;
    DBuf<float> d_clear, d_speed;
    DBuf<unsigned char> d_active;
    DBuf<int> path_off, path_len, key, rank, destroyed_list, replan_list;
    DBuf<V2> path_xy;
    size_t path_used = 0;
    /* snapshot */
    DBuf<int> s_slot;
    DBuf<V2> s_pos, s_vel;
    DBuf<float> s_clear;
    /* grid */
    AgentGrid grid{};
    bool grid_ready = false;
    int grid_agents = 0;
    DBuf<int> cell_count, cell_start, scan_tmp, counters;
    /* scene */
    HostScene scene;
    bool has_obst = false;
    GridCSR ob_grid;     /* device candidate grid */
    GridCSR vis_grid;    /* planner visibility grid */
    float ob_reach_needed = 0.0f;
    bool ob_dirty = true;
    DBuf<V2> d_ob_p, d_v_pos, d_he_left, d_he_right;
    DBuf<int> d_ob_next, d_ob_prev, d_v_idx, d_he_target, d_ob_gstart, d_ob_gitems, d_ecm_gstart, d_ecm_gitems;
    DBuf<unsigned char> d_ob_convex;
    DBuf<float> d_special_y;
    /* planner */
    ecmg_plan_fn plan_fn = nullptr;
    void* plan_user = nullptr;
    PlanScratch scratch;
    /* recording */
    bool record = false;
    DBuf<int> rec_nbr, rec_cnt, rec_fail, rec_ncons, rec_nobst;
    DBuf<V2> rec_vorca;
    /* pinned staging */
    int* h_counters = nullptr; /* [2 * kCounters]: in, out */
    /* graph */
    cudaGraphExec_t graph = nullptr;
    bool graph_dirty = true;
};

static ecmg_status fail(ecmg_ctx* c, ecmg_status s, const char* fmt, ...)
{
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return s;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return fail(c, ECMG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

static bool finite2(float a, float b) { return std::isfinite(a) && std::isfinite(b); }

extern "C" {

void ecmg_default_params(ecmg_params* p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->dt = 0.1f;
    p->tau_agent = 10.0f;
    p->tau_obst = 10.0f;
    p->neighbor_dist = 5.0f;
    p->max_speed = 0.0f;
    p->mass = 0.8f;
    p->arrival_radius = 20.0f;
    p->delete_radius = 2.0f;
    p->max_neighbors = 5;
    p->lp3d_fp64 = 0;
    p->use_graph = 1;
    p->block_size = 0;
    p->grid_cell = 0.0f;
}

const char* ecmg_last_error(const ecmg_ctx* c) { return c ? c->err.c_str() : "null context"; }

ecmg_status ecmg_get_params(const ecmg_ctx* c, ecmg_params* out)
{
    if (!c || !out) return ECMG_ERR_INVALID_ARG;
    *out = c->prm;
    return ECMG_OK;
}

static ecmg_status check_params(ecmg_ctx* c, const ecmg_params* p)
{
    if (!(p->dt > 0.0f) || !std::isfinite(p->dt)) return fail(c, ECMG_ERR_INVALID_ARG, "dt must be > 0");
    if (!(p->tau_agent > 0.0f) || !(p->tau_obst > 0.0f)) return fail(c, ECMG_ERR_INVALID_ARG, "time horizons must be > 0");
    if (!(p->neighbor_dist > 0.0f) || !std::isfinite(p->neighbor_dist))
        return fail(c, ECMG_ERR_INVALID_ARG, "neighbor_dist must be > 0");
    if (p->max_neighbors < 1 || p->max_neighbors > kMaxK)
        return fail(c, ECMG_ERR_INVALID_ARG, "max_neighbors must be in [1, %d]", kMaxK);
    if (!(p->mass > 0.0f)) return fail(c, ECMG_ERR_INVALID_ARG, "mass must be > 0");
    if (!std::isfinite(p->max_speed)) return fail(c, ECMG_ERR_INVALID_ARG, "max_speed must be finite");
    if (p->grid_cell < 0.0f || !std::isfinite(p->grid_cell)) return fail(c, ECMG_ERR_INVALID_ARG, "grid_cell must be >= 0");
    return ECMG_OK;
}

ecmg_status ecmg_create(const ecmg_params* p, int max_agents, ecmg_ctx** out)
{
    if (!out) return ECMG_ERR_INVALID_ARG;
    *out = nullptr;
    if (max_agents < 1) return ECMG_ERR_INVALID_ARG;
    ecmg_params prm;
    if (p) prm = *p;
    else ecmg_default_params(&prm);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return ECMG_ERR_NO_DEVICE;
    }
    ecmg_ctx* c = new ecmg_ctx();
    ecmg_status st = check_params(c, &prm);
    if (st != ECMG_OK) { delete c; return st; }
    c->prm = prm;
    c->max_agents = max_agents;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev);
#define CKC(x) do { if ((x) != cudaSuccess) { ecmg_destroy(c); return ECMG_ERR_CUDA; } } while (0)
    CKC(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CKC(cudaEventCreate(&c->ev_t0));
    CKC(cudaEventCreate(&c->ev_t1));
    CKC(cudaEventCreate(&c->ev_a0));
    CKC(cudaEventCreate(&c->ev_a1));
    size_t N = (size_t)max_agents;
    CKC(c->pos.alloc(N)); CKC(c->vel.alloc(N)); CKC(c->attr.alloc(N)); CKC(c->pref_vel.alloc(N));
    CKC(c->d_clear.alloc(N)); CKC(c->d_speed.alloc(N)); CKC(c->d_active.alloc(N));
    CKC(c->path_off.alloc(N)); CKC(c->path_len.alloc(N)); CKC(c->key.alloc(N)); CKC(c->rank.alloc(N));
    CKC(c->destroyed_list.alloc(N)); CKC(c->replan_list.alloc(N)); CKC(c->replan_pos.alloc(N));
    CKC(c->s_slot.alloc(N)); CKC(c->s_pos.alloc(N)); CKC(c->s_vel.alloc(N)); CKC(c->s_clear.alloc(N));
    CKC(c->counters.alloc(kCounters));
    CKC(c->path_xy.alloc(std::max<size_t>(1024, 4 * N)));
    CKC(cudaMemset(c->pos.p, 0, sizeof(V2) * N)); CKC(cudaMemset(c->vel.p, 0, sizeof(V2) * N));
    CKC(cudaMemset(c->attr.p, 0, sizeof(V2) * N)); CKC(cudaMemset(c->pref_vel.p, 0, sizeof(V2) * N));
    CKC(cudaMemset(c->d_active.p, 0, N)); CKC(cudaMemset(c->path_len.p, 0, sizeof(int) * N));
    CKC(cudaMemset(c->path_off.p, 0, sizeof(int) * N));
    CKC(cudaHostAlloc((void**)&c->h_counters, sizeof(int) * 2 * kCounters, cudaHostAllocDefault));
#undef CKC
    c->active.assign(N, 0);
    c->clear.assign(N, 0.0f);
    c->speed.assign(N, 0.0f);
    c->paths.assign(N, {});
    c->free_stack.reserve(N);
    for (int i = max_agents - 1; i >= 0; i--) c->free_stack.push_back(i); /* Simulator.h:66-69 */
    *out = c;
    return ECMG_OK;
}

ecmg_status ecmg_destroy(ecmg_ctx* c)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->graph) cudaGraphExecDestroy(c->graph);
    DBuf<V2>* v2s[] = {&c->pos, &c->vel, &c->attr, &c->pref_vel, &c->replan_pos, &c->path_xy, &c->s_pos, &c->s_vel,
                       &c->d_ob_p, &c->d_v_pos, &c->d_he_left, &c->d_he_right, &c->rec_vorca};
    for (auto* b : v2s) b->free_();
    DBuf<int>* is[] = {&c->path_off, &c->path_len, &c->key, &c->rank, &c->destroyed_list, &c->replan_list,
                       &c->s_slot, &c->cell_count, &c->cell_start, &c->scan_tmp, &c->counters, &c->d_ob_next,
                       &c->d_ob_prev, &c->d_v_idx, &c->d_he_target, &c->d_ob_gstart, &c->d_ob_gitems,
                       &c->d_ecm_gstart, &c->d_ecm_gitems, &c->rec_nbr, &c->rec_cnt, &c->rec_fail,
                       &c->rec_ncons, &c->rec_nobst};
    for (auto* b : is) b->free_();
    c->d_clear.free_();
    c->d_speed.free_();
    c->s_clear.free_();
    c->d_special_y.free_();
    c->d_active.free_();
    c->d_ob_convex.free_();
    if (c->h_counters) cudaFreeHost(c->h_counters);
    if (c->ev_t0) cudaEventDestroy(c->ev_t0);
    if (c->ev_t1) cudaEventDestroy(c->ev_t1);
    if (c->ev_a0) cudaEventDestroy(c->ev_a0);
    if (c->ev_a1) cudaEventDestroy(c->ev_a1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return ECMG_OK;
}

static void scene_bbox(ecmg_ctx* c)
{
    HostScene& s = c->scene;
    float x0 = 1e30f, y0 = 1e30f, x1 = -1e30f, y1 = -1e30f;
    auto grow = [&](V2 p) {
        x0 = std::min(x0, p.x); y0 = std::min(y0, p.y);
        x1 = std::max(x1, p.x); y1 = std::max(y1, p.y);
    };
    for (auto& p : s.ob_p) grow(p);
    for (auto& p : s.v_pos) grow(p);
    for (auto& p : s.he_left) grow(p);
    for (auto& p : s.he_right) grow(p);
    if (x0 > x1) { x0 = y0 = 0; x1 = y1 = 1; }
    s.bx0 = x0; s.by0 = y0; s.bx1 = x1; s.by1 = y1;
}

ecmg_status ecmg_set_obstacles(ecmg_ctx* c, const ecmg_obstacles* o)
{
    if (!c || !o) return fail(c, ECMG_ERR_INVALID_ARG, "null argument");
    if (o->n_obstacles < 0 || (o->n_obstacles > 0 && (!o->ring_offsets || !o->xy)))
        return fail(c, ECMG_ERR_INVALID_ARG, "bad obstacle arrays");
    for (int r = 0; r < o->n_obstacles; r++)
        if (o->ring_offsets[r + 1] - o->ring_offsets[r] < 2)
            return fail(c, ECMG_ERR_INVALID_ARG, "obstacle %d has fewer than 2 vertices (Environment.cpp:288)", r);
    int nv = o->n_obstacles > 0 ? o->ring_offsets[o->n_obstacles] : 0;
    for (int i = 0; i < nv; i++)
        if (!finite2(o->xy[2 * i], o->xy[2 * i + 1])) return fail(c, ECMG_ERR_INVALID_ARG, "non-finite obstacle vertex");
    set_obstacles(c->scene, o->n_obstacles, o->ring_offsets, o->xy);
    scene_bbox(c);
    HostScene& s = c->scene;
    size_t n = std::max<size_t>(1, s.ob_p.size());
    CK(c->d_ob_p.alloc(n)); CK(c->d_ob_next.alloc(n)); CK(c->d_ob_prev.alloc(n)); CK(c->d_ob_convex.alloc(n));
    if (nv > 0) {
        CK(cudaMemcpy(c->d_ob_p.p, s.ob_p.data(), sizeof(V2) * nv, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_ob_next.p, s.ob_next.data(), sizeof(int) * nv, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_ob_prev.p, s.ob_prev.data(), sizeof(int) * nv, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_ob_convex.p, s.ob_convex.data(), nv, cudaMemcpyHostToDevice));
    }
    build_obst_grid(s, 0.0f, 4.0f, c->vis_grid);
    c->has_obst = true;
    c->ob_dirty = true;
    c->grid_ready = false;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_set_ecm(ecmg_ctx* c, const ecmg_ecm* e)
{
    if (!c || !e) return fail(c, ECMG_ERR_INVALID_ARG, "null argument");
    if (e->n_vertices < 0 || e->n_edges < 0) return fail(c, ECMG_ERR_INVALID_ARG, "negative sizes");
    int V = e->n_vertices, E = e->n_edges;
    HostScene& s = c->scene;
    s.v_pos.resize(V); s.v_clear.resize(V); s.v_idx.resize(V); s.v_halfedge.resize(V);
    s.he_target.resize(2 * (size_t)E); s.he_next.resize(2 * (size_t)E);
    s.he_left.resize(2 * (size_t)E); s.he_right.resize(2 * (size_t)E);
    for (int i = 0; i < V; i++) {
        if (!finite2(e->v_pos[2 * i], e->v_pos[2 * i + 1])) return fail(c, ECMG_ERR_INVALID_ARG, "non-finite ECM vertex");
        s.v_pos[i] = mk(e->v_pos[2 * i], e->v_pos[2 * i + 1]);
        s.v_clear[i] = e->v_clear ? e->v_clear[i] : 0.0f;
        s.v_idx[i] = e->v_idx ? e->v_idx[i] : i;
        s.v_halfedge[i] = e->v_halfedge ? e->v_halfedge[i] : -1;
    }
    for (int h = 0; h < 2 * E; h++) {
        int t = e->he_target[h];
        if (t < 0 || t >= V) return fail(c, ECMG_ERR_INVALID_ARG, "half-edge %d targets vertex %d of %d", h, t, V);
        s.he_target[h] = t;
        s.he_next[h] = e->he_next ? e->he_next[h] : -1;
        s.he_left[h] = mk(e->he_left[2 * h], e->he_left[2 * h + 1]);
        s.he_right[h] = mk(e->he_right[2 * h], e->he_right[2 * h + 1]);
    }
    s.has_ecm = true;
    scene_bbox(c);
    build_ecm_grid(s);
    if (c->has_obst) build_obst_grid(s, 0.0f, 4.0f, c->vis_grid);
    size_t nV = std::max<size_t>(1, V), nH = std::max<size_t>(1, 2 * (size_t)E);
    CK(c->d_v_pos.alloc(nV)); CK(c->d_v_idx.alloc(nV)); CK(c->d_he_target.alloc(nH));
    CK(c->d_he_left.alloc(nH)); CK(c->d_he_right.alloc(nH));
    CK(c->d_ecm_gstart.alloc(s.ecm_grid.start.size()));
    CK(c->d_ecm_gitems.alloc(std::max<size_t>(1, s.ecm_grid.items.size())));
    CK(c->d_special_y.alloc(std::max<size_t>(1, s.special_y.size())));
    if (V) {
        CK(cudaMemcpy(c->d_v_pos.p, s.v_pos.data(), sizeof(V2) * V, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_v_idx.p, s.v_idx.data(), sizeof(int) * V, cudaMemcpyHostToDevice));
    }
    if (E) {
        CK(cudaMemcpy(c->d_he_target.p, s.he_target.data(), sizeof(int) * 2 * E, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_he_left.p, s.he_left.data(), sizeof(V2) * 2 * E, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_he_right.p, s.he_right.data(), sizeof(V2) * 2 * E, cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(c->d_ecm_gstart.p, s.ecm_grid.start.data(), sizeof(int) * s.ecm_grid.start.size(), cudaMemcpyHostToDevice));
    if (!s.ecm_grid.items.empty())
        CK(cudaMemcpy(c->d_ecm_gitems.p, s.ecm_grid.items.data(), sizeof(int) * s.ecm_grid.items.size(), cudaMemcpyHostToDevice));
    if (!s.special_y.empty())
        CK(cudaMemcpy(c->d_special_y.p, s.special_y.data(), sizeof(float) * s.special_y.size(), cudaMemcpyHostToDevice));
    c->grid_ready = false;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_set_planner(ecmg_ctx* c, ecmg_plan_fn fn, void* user)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    c->plan_fn = fn;
    c->plan_user = user;
    return ECMG_OK;
}

static ecmg_status upload_path(ecmg_ctx* c, int slot)
{
    const std::vector<V2>& p = c->paths[slot];
    size_t n = p.size();
    if (c->path_used + n > c->path_xy.n) {
        /* grow (x2) and compact: live paths only */
        size_t live = 0;
        for (int i = 0; i < c->max_agents; i++) live += c->paths[i].size();
        size_t cap = std::max(c->path_xy.n * 2, live * 2 + 1024);
        DBuf<V2> nb;
        CK(nb.alloc(cap));
        std::vector<V2> host;
        host.reserve(live);
        std::vector<int> off(c->max_agents, 0), len(c->max_agents, 0);
        for (int i = 0; i < c->max_agents; i++) {
            off[i] = (int)host.size();
            len[i] = (int)c->paths[i].size();
            host.insert(host.end(), c->paths[i].begin(), c->paths[i].end());
        }
        if (!host.empty()) CK(cudaMemcpy(nb.p, host.data(), sizeof(V2) * host.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->path_off.p, off.data(), sizeof(int) * c->max_agents, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->path_len.p, len.data(), sizeof(int) * c->max_agents, cudaMemcpyHostToDevice));
        c->path_xy.free_();
        c->path_xy = nb;
        c->path_used = host.size();
        c->graph_dirty = true;
        return ECMG_OK;
    }
    int off = (int)c->path_used, len = (int)n;
    if (n) CK(cudaMemcpy(c->path_xy.p + off, p.data(), sizeof(V2) * n, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->path_off.p + slot, &off, sizeof(int), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->path_len.p + slot, &len, sizeof(int), cudaMemcpyHostToDevice));
    c->path_used += n;
    return ECMG_OK;
}

static void note_range(ecmg_ctx* c, float clearance, float speed)
{
    float ms = c->prm.max_speed > 0.0f ? c->prm.max_speed : speed;
    float r = c->prm.tau_obst * ms + clearance;
    if (r > c->ob_reach_needed) {
        c->ob_reach_needed = r;
        if (r > c->ob_grid.reach) c->ob_dirty = true;
    }
}

ecmg_status ecmg_add_agents(ecmg_ctx* c, int n, const float* pos, const float* clearance, const float* pref_speed,
                            const int* path_off, const int* path_len, const float* path_xy, int* out_slots)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (n < 0 || (n > 0 && (!pos || !clearance || !pref_speed || !path_off || !path_len || !path_xy)))
        return fail(c, ECMG_ERR_INVALID_ARG, "null or negative argument");
    if ((size_t)n > c->free_stack.size()) return fail(c, ECMG_ERR_NO_SLOT, "%d agents requested, %zu slots free", n, c->free_stack.size());
    for (int i = 0; i < n; i++) {
        if (!finite2(pos[2 * i], pos[2 * i + 1]) || !std::isfinite(clearance[i]) || !std::isfinite(pref_speed[i]))
            return fail(c, ECMG_ERR_INVALID_ARG, "agent %d: non-finite input", i);
        if (!(clearance[i] >= 0.0f) || !(pref_speed[i] >= 0.0f))
            return fail(c, ECMG_ERR_INVALID_ARG, "agent %d: negative clearance or speed", i);
        if (path_len[i] < 1) return fail(c, ECMG_ERR_INVALID_ARG, "agent %d: empty path (Simulator.cpp:554 reads path.x[numPoints-1])", i);
        for (int q = 0; q < path_len[i]; q++)
            if (!finite2(path_xy[2 * (path_off[i] + q)], path_xy[2 * (path_off[i] + q) + 1]))
                return fail(c, ECMG_ERR_INVALID_ARG, "agent %d: non-finite path point", i);
    }
    std::vector<int> slots(n);
    for (int i = 0; i < n; i++) {
        int idx = c->free_stack.back();
        c->free_stack.pop_back();
        slots[i] = idx;
        c->num_agents++;
        c->last_idx = std::max(c->last_idx, idx);
        c->active[idx] = 1;
        c->clear[idx] = clearance[i];
        c->speed[idx] = pref_speed[i];
        c->paths[idx].assign((const V2*)(path_xy + 2 * (size_t)path_off[i]),
                             (const V2*)(path_xy + 2 * (size_t)(path_off[i] + path_len[i])));
        note_range(c, clearance[i], pref_speed[i]);
    }
    /* contiguous runs of slots are uploaded in one copy each */
    std::vector<V2> zero(1, mk(0, 0));
    for (int i = 0; i < n;) {
        int j = i;
        while (j + 1 < n && slots[j + 1] == slots[j] + 1) j++;
        int s0 = slots[i], cnt = j - i + 1;
        std::vector<V2> z((size_t)cnt, mk(0.0f, 0.0f));
        std::vector<unsigned char> one((size_t)cnt, 1);
        CK(cudaMemcpy(c->pos.p + s0, pos + 2 * (size_t)i, sizeof(V2) * cnt, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->vel.p + s0, z.data(), sizeof(V2) * cnt, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->pref_vel.p + s0, z.data(), sizeof(V2) * cnt, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_clear.p + s0, clearance + i, sizeof(float) * cnt, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_speed.p + s0, pref_speed + i, sizeof(float) * cnt, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->d_active.p + s0, one.data(), cnt, cudaMemcpyHostToDevice));
        i = j + 1;
    }
    /* paths: append all at once */
    size_t total = 0;
    for (int i = 0; i < n; i++) total += (size_t)path_len[i];
    if (c->path_used + total > c->path_xy.n) {
        for (int i = 0; i < n; i++) {
            ecmg_status st = upload_path(c, slots[i]);
            if (st != ECMG_OK) return st;
        }
    } else {
        std::vector<V2> buf;
        buf.reserve(total);
        std::vector<int> offs(n), lens(n);
        for (int i = 0; i < n; i++) {
            offs[i] = (int)(c->path_used + buf.size());
            lens[i] = path_len[i];
            buf.insert(buf.end(), c->paths[slots[i]].begin(), c->paths[slots[i]].end());
        }
        if (total) CK(cudaMemcpy(c->path_xy.p + c->path_used, buf.data(), sizeof(V2) * total, cudaMemcpyHostToDevice));
        c->path_used += total;
        for (int i = 0; i < n;) {
            int j = i;
            while (j + 1 < n && slots[j + 1] == slots[j] + 1) j++;
            CK(cudaMemcpy(c->path_off.p + slots[i], offs.data() + i, sizeof(int) * (j - i + 1), cudaMemcpyHostToDevice));
            CK(cudaMemcpy(c->path_len.p + slots[i], lens.data() + i, sizeof(int) * (j - i + 1), cudaMemcpyHostToDevice));
            i = j + 1;
        }
    }
    if (out_slots) std::memcpy(out_slots, slots.data(), sizeof(int) * n);
    if (c->grid_agents == 0 || c->num_agents > 2 * c->grid_agents) c->grid_ready = false;
    return ECMG_OK;
}

static ecmg_status plan(ecmg_ctx* c, V2 s, V2 g, float clr, std::vector<V2>& out)
{
    out.clear();
    if (c->plan_fn) {
        std::vector<float> buf(2 * 4096);
        int n = c->plan_fn(c->plan_user, s.x, s.y, g.x, g.y, clr, buf.data(), 4096);
        if (n < 0) return ECMG_ERR_NO_PATH;
        n = std::min(n, 4096);
        for (int i = 0; i < n; i++) out.push_back(mk(buf[2 * i], buf[2 * i + 1]));
        return n > 0 ? ECMG_OK : ECMG_ERR_NO_PATH;
    }
    if (!c->scene.has_ecm) return ECMG_ERR_STATE;
    return plan_path(c->scene, c->vis_grid, s, g, clr, out, c->scratch) ? ECMG_OK : ECMG_ERR_NO_PATH;
}

ecmg_status ecmg_find_path(ecmg_ctx* c, float sx, float sy, float gx, float gy, float clearance, float* out_xy,
                           int cap, int* out_n)
{
    if (!c || !out_n || (cap > 0 && !out_xy)) return ECMG_ERR_INVALID_ARG;
    std::vector<V2> p;
    ecmg_status st = plan(c, mk(sx, sy), mk(gx, gy), clearance, p);
    *out_n = st == ECMG_OK ? (int)p.size() : -1;
    for (int i = 0; i < (int)p.size() && i < cap; i++) { out_xy[2 * i] = p[i].x; out_xy[2 * i + 1] = p[i].y; }
    return st;
}

struct ecmg_planner {
    HostScene scene;
    GridCSR vis;
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
            bool ok = plan_path(pl->scene, pl->vis, mk(starts[2 * i], starts[2 * i + 1]),
                                mk(goals[2 * i], goals[2 * i + 1]), clearances[i], p, scr);
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

ecmg_status ecmg_planner_locate(ecmg_planner* pl, int n, const float* xy, int* out)
{
    if (!pl || n < 0 || (n > 0 && (!xy || !out))) return ECMG_ERR_INVALID_ARG;
    EcmView ev = pl->scene.ecm_view();
    for (int i = 0; i < n; i++) out[i] = point_location(ev, mk(xy[2 * i], xy[2 * i + 1]));
    return ECMG_OK;
}

/* Simulator::ValidSpawnLocation (Simulator.cpp:295-311) on the device state */
static ecmg_status valid_spawn(ecmg_ctx* c, V2 loc, float clearance, bool* ok)
{
    *ok = true;
    if (c->last_idx < 0) return ECMG_OK;
    std::vector<V2> p((size_t)c->last_idx + 1);
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(p.data(), c->pos.p, sizeof(V2) * p.size(), cudaMemcpyDeviceToHost));
    float cs = clearance * clearance;
    for (int i = 0; i <= c->last_idx; i++) {
        if (!c->active[i]) continue;
        float dx = loc.x - p[i].x, dy = loc.y - p[i].y;
        if (dx * dx + dy * dy < cs) { *ok = false; return ECMG_OK; }
    }
    return ECMG_OK;
}

ecmg_status ecmg_spawn_agent(ecmg_ctx* c, float sx, float sy, float gx, float gy, float clearance, float pref_speed,
                             int* out_slot)
{
    if (!c || !out_slot) return ECMG_ERR_INVALID_ARG;
    *out_slot = -1;
    if (!finite2(sx, sy) || !finite2(gx, gy) || !std::isfinite(clearance) || !std::isfinite(pref_speed))
        return fail(c, ECMG_ERR_INVALID_ARG, "non-finite spawn argument");
    if (c->free_stack.empty()) return fail(c, ECMG_ERR_NO_SLOT, "no free slot");
    bool ok;
    ecmg_status st = valid_spawn(c, mk(sx, sy), clearance, &ok);
    if (st != ECMG_OK) return st;
    if (!ok) return fail(c, ECMG_ERR_INVALID_SPAWN, "spawn location occupied");
    std::vector<V2> p;
    st = plan(c, mk(sx, sy), mk(gx, gy), clearance, p);
    if (st != ECMG_OK || p.empty()) return fail(c, ECMG_ERR_NO_PATH, "no path from (%g,%g) to (%g,%g)", sx, sy, gx, gy);
    std::vector<float> xy(2 * p.size());
    for (size_t i = 0; i < p.size(); i++) { xy[2 * i] = p[i].x; xy[2 * i + 1] = p[i].y; }
    int off = 0, len = (int)p.size();
    float pos[2] = {sx, sy};
    return ecmg_add_agents(c, 1, pos, &clearance, &pref_speed, &off, &len, xy.data(), out_slot);
}

ecmg_status ecmg_destroy_agent(ecmg_ctx* c, int slot)
{
    if (!c || slot < 0 || slot >= c->max_agents) return fail(c, ECMG_ERR_INVALID_ARG, "bad slot");
    if (!c->active[slot]) return fail(c, ECMG_ERR_INVALID_ARG, "slot %d is not active", slot);
    c->num_agents--;
    c->active[slot] = 0;
    c->free_stack.push_back(slot);
    unsigned char z = 0;
    CK(cudaMemcpy(c->d_active.p + slot, &z, 1, cudaMemcpyHostToDevice));
    return ECMG_OK;
}

ecmg_status ecmg_reset(ecmg_ctx* c)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    for (int i = 0; i <= c->last_idx; i++) /* Simulator.cpp:327-332 */
        if (c->active[i]) {
            c->num_agents--;
            c->active[i] = 0;
            c->free_stack.push_back(i);
        }
    if (c->last_idx >= 0) CK(cudaMemset(c->d_active.p, 0, (size_t)c->last_idx + 1));
    return ECMG_OK;
}

ecmg_status ecmg_set_path(ecmg_ctx* c, int slot, const float* xy, int n)
{
    if (!c || slot < 0 || slot >= c->max_agents || n < 1 || !xy) return fail(c, ECMG_ERR_INVALID_ARG, "bad path argument");
    for (int i = 0; i < n; i++)
        if (!finite2(xy[2 * i], xy[2 * i + 1])) return fail(c, ECMG_ERR_INVALID_ARG, "non-finite path point");
    c->paths[slot].assign((const V2*)xy, (const V2*)(xy + 2 * (size_t)n));
    return upload_path(c, slot);
}

ecmg_status ecmg_get_path(ecmg_ctx* c, int slot, float* out_xy, int cap, int* out_n)
{
    if (!c || slot < 0 || slot >= c->max_agents || !out_n) return ECMG_ERR_INVALID_ARG;
    const auto& p = c->paths[slot];
    *out_n = (int)p.size();
    for (int i = 0; i < (int)p.size() && i < cap; i++) { out_xy[2 * i] = p[i].x; out_xy[2 * i + 1] = p[i].y; }
    return ECMG_OK;
}

/* ---------------------------------------------------------------------- */
static ecmg_status ensure_grids(ecmg_ctx* c)
{
    HostScene& s = c->scene;
    if (c->ob_dirty) {
        float reach = std::max(c->ob_reach_needed, 1.0f) * 1.05f + 0.1f;
        build_obst_grid(s, reach, std::max(2.0f, std::min(reach, 8.0f)), c->ob_grid);
        CK(c->d_ob_gstart.alloc(c->ob_grid.start.size()));
        CK(c->d_ob_gitems.alloc(std::max<size_t>(1, c->ob_grid.items.size())));
        CK(cudaMemcpy(c->d_ob_gstart.p, c->ob_grid.start.data(), sizeof(int) * c->ob_grid.start.size(), cudaMemcpyHostToDevice));
        if (!c->ob_grid.items.empty())
            CK(cudaMemcpy(c->d_ob_gitems.p, c->ob_grid.items.data(), sizeof(int) * c->ob_grid.items.size(), cudaMemcpyHostToDevice));
        c->ob_dirty = false;
        c->graph_dirty = true;
    }
    if (!c->grid_ready) {
        float w = std::max(1.0f, s.bx1 - s.bx0), h = std::max(1.0f, s.by1 - s.by0);
        float cell = c->prm.grid_cell;
        if (!(cell > 0.0f)) {
            float dens = (float)std::max(1, c->num_agents) / (w * h);
            cell = std::sqrt((float)c->prm.max_neighbors / dens) * 0.6f;
            cell = std::min(std::max(cell, 0.5f), std::max(0.5f, c->prm.neighbor_dist));
        }
        /* at most 32M cells */
        while ((double)(w / cell + 3) * (double)(h / cell + 3) > 32.0e6) cell *= 1.5f;
        AgentGrid g;
        g.cell = cell;
        g.inv = 1.0f / cell;
        g.x0 = s.bx0 - cell;
        g.y0 = s.by0 - cell;
        g.gw = (int)std::ceil(w / cell) + 3;
        g.gh = (int)std::ceil(h / cell) + 3;
        g.ncells = g.gw * g.gh;
        c->grid = g;
        CK(c->cell_count.alloc((size_t)g.ncells + 2 + kCounters));
        CK(c->cell_start.alloc((size_t)g.ncells + 2));
        CK(c->scan_tmp.alloc((size_t)scan_tmp_ints(g.ncells + 1)));
        c->grid_ready = true;
        c->grid_agents = std::max(1, c->num_agents);
        c->graph_dirty = true;
    }
    if (c->record) {
        size_t N = (size_t)c->max_agents;
        int k = c->prm.max_neighbors;
        CK(c->rec_nbr.alloc(N * k)); CK(c->rec_cnt.alloc(N)); CK(c->rec_fail.alloc(N));
        CK(c->rec_ncons.alloc(N)); CK(c->rec_nobst.alloc(N)); CK(c->rec_vorca.alloc(N));
    }
    return ECMG_OK;
}

static void fill_args(ecmg_ctx* c, BinArgs& b, TickArgs& t)
{
    b = BinArgs{};
    b.pos = c->pos.p;
    b.vel = c->vel.p;
    b.clear = c->d_clear.p;
    b.active = c->d_active.p;
    b.key = c->key.p;
    b.rank = c->rank.p;
    b.cell_count = c->cell_count.p;
    b.s_slot = c->s_slot.p;
    b.s_pos = c->s_pos.p;
    b.s_vel = c->s_vel.p;
    b.s_clear = c->s_clear.p;
    b.cell_start = c->cell_start.p;
    b.counters = c->counters.p;
    b.grid = c->grid;

    t = TickArgs{};
    t.pos = c->pos.p;
    t.vel = c->vel.p;
    t.attr = c->attr.p;
    t.pref_vel = c->pref_vel.p;
    t.clear = c->d_clear.p;
    t.speed = c->d_speed.p;
    t.active = c->d_active.p;
    t.path_off = c->path_off.p;
    t.path_len = c->path_len.p;
    t.path_xy = c->path_xy.p;
    t.s_slot = c->s_slot.p;
    t.s_pos = c->s_pos.p;
    t.s_vel = c->s_vel.p;
    t.s_clear = c->s_clear.p;
    t.cell_start = c->cell_start.p;
    t.grid = c->grid;
    HostScene& s = c->scene;
    ObstView o{};
    o.p = c->d_ob_p.p;
    o.next = c->d_ob_next.p;
    o.prev = c->d_ob_prev.p;
    o.convex = c->d_ob_convex.p;
    o.n_verts = c->has_obst ? (int)s.ob_p.size() : 0;
    if (c->ob_grid.gw > 0) {
        o.gx0 = c->ob_grid.x0; o.gy0 = c->ob_grid.y0; o.ginv = c->ob_grid.inv;
        o.gw = c->ob_grid.gw; o.gh = c->ob_grid.gh; o.reach = c->ob_grid.reach;
        o.g_start = c->d_ob_gstart.p;
        o.g_items = c->d_ob_gitems.p;
    }
    t.ob = o;
    EcmView e{};
    e.v_pos = c->d_v_pos.p;
    e.v_idx = c->d_v_idx.p;
    e.he_target = c->d_he_target.p;
    e.he_left = c->d_he_left.p;
    e.he_right = c->d_he_right.p;
    e.n_edges = (int)(s.he_target.size() / 2);
    e.gx0 = s.ecm_grid.x0; e.gy0 = s.ecm_grid.y0; e.ginv = s.ecm_grid.inv;
    e.gw = s.ecm_grid.gw; e.gh = s.ecm_grid.gh;
    e.g_start = c->d_ecm_gstart.p;
    e.g_items = c->d_ecm_gitems.p;
    e.special_y = c->d_special_y.p;
    e.n_special = (int)s.special_y.size();
    t.ecm = e;
    const ecmg_params& p = c->prm;
    t.dt = p.dt;
    t.tau_a = p.tau_agent;
    t.tau_o = p.tau_obst;
    t.rnb = p.neighbor_dist;
    t.rnb2 = p.neighbor_dist * p.neighbor_dist;
    t.max_speed = p.max_speed;
    t.mass_recip = 1.0f / p.mass; /* Simulator.cpp:623 */
    t.arr_sq = p.arrival_radius * p.arrival_radius;
    t.del_sq = p.delete_radius * p.delete_radius;
    t.k = p.max_neighbors;
    t.lp3d_fp64 = p.lp3d_fp64;
    t.counters = c->counters.p;
    t.destroyed_list = c->destroyed_list.p;
    t.replan_list = c->replan_list.p;
    t.replan_pos = c->replan_pos.p;
    t.list_cap = c->max_agents;
    if (c->record) {
        t.rec_nbr = c->rec_nbr.p;
        t.rec_cnt = c->rec_cnt.p;
        t.rec_vorca = c->rec_vorca.p;
        t.rec_fail = c->rec_fail.p;
        t.rec_ncons = c->rec_ncons.p;
        t.rec_nobst = c->rec_nobst.p;
    }
}

/* the device work of one tick: counters in, kernels, counters out */
static cudaError_t enqueue_tick(ecmg_ctx* c)
{
    BinArgs b;
    TickArgs t;
    fill_args(c, b, t);
    cudaGetLastError(); /* launch errors below must not be confused with older ones */
    cudaError_t e = cudaMemcpyAsync(c->counters.p, c->h_counters, sizeof(int) * kCounters, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return e;
    e = launch_tick(b, t, c->max_agents, c->scan_tmp.p, 0, c->prm.block_size, c->sms, c->stream, c->ev_a0, c->ev_a1);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(c->h_counters + kCounters, c->counters.p, sizeof(int) * kCounters, cudaMemcpyDeviceToHost,
                           c->stream);
}

void* ecmg_stream(const ecmg_ctx* c) { return c ? (void*)c->stream : nullptr; }

int ecmg_kernels_per_tick(const ecmg_ctx* c)
{
    (void)c;
    return 6; /* k_bin, k_scan_local, k_scan_top, k_scan_add, k_scatter, k_agents */
}

ecmg_status ecmg_tick(ecmg_ctx* c, int n_ticks, ecmg_tick_stats* stats)
{
    if (!c || n_ticks < 0) return ECMG_ERR_INVALID_ARG;
    if (!c->scene.has_ecm) return fail(c, ECMG_ERR_STATE, "ecmg_set_ecm must be called before ecmg_tick");
    ecmg_tick_stats st{};
    ecmg_status result = ECMG_OK;
    for (int tk = 0; tk < n_ticks; tk++) {
        /* UpdateMaxAgentIndex (Simulator.cpp:481-492) */
        int empty = 0;
        for (int i = c->last_idx; i >= 0; i--) {
            if (c->active[i]) break;
            empty++;
        }
        c->last_idx -= empty;
        st.ticks++;
        if (c->last_idx < 0) continue;
        ecmg_status gs = ensure_grids(c);
        if (gs != ECMG_OK) return gs;
        std::memset(c->h_counters, 0, sizeof(int) * kCounters);
        c->h_counters[C_LAST] = c->last_idx;
        CK(cudaEventRecord(c->ev_t0, c->stream));
        if (c->prm.use_graph) {
            if (c->graph_dirty || !c->graph) {
                if (c->graph) cudaGraphExecDestroy(c->graph);
                c->graph = nullptr;
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = enqueue_tick(c);
                cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
                if (e != cudaSuccess) return fail(c, ECMG_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
                if (e2 != cudaSuccess) return fail(c, ECMG_ERR_CUDA, "end capture: %s", cudaGetErrorString(e2));
                CK(cudaGraphInstantiate(&c->graph, g, 0));
                cudaGraphDestroy(g);
                c->graph_dirty = false;
            }
            CK(cudaGraphLaunch(c->graph, c->stream));
        } else {
            CK(enqueue_tick(c));
        }
        CK(cudaEventRecord(c->ev_t1, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        float ms = 0, ams = 0;
        if (cudaEventElapsedTime(&ms, c->ev_t0, c->ev_t1) != cudaSuccess) ms = 0;
        if (cudaEventElapsedTime(&ams, c->ev_a0, c->ev_a1) != cudaSuccess) ams = 0;
        cudaGetLastError();
        st.device_ms += ms;
        st.agent_kernel_ms += ams;
        const int* out = c->h_counters + kCounters;
        int nd = out[C_DESTROYED], nr = out[C_REPLAN];
        st.agent_steps += out[C_NSORTED];
        st.lp3d += out[C_LP3D];
        st.destroyed += nd;
        st.replans += nr;
        if (out[C_ERROR]) {
            result = fail(c, ECMG_ERR_BOUND, "device bound exceeded (flags 0x%x): %s", out[C_ERROR],
                          (out[C_ERROR] & ECMG_DEV_ERR_CONSTRAINTS) ? "more than 64 half-planes for one agent"
                                                                    : "event list overflow");
        }
        if (nd > 0) {
            std::vector<int> d(std::min(nd, c->max_agents));
            CK(cudaMemcpy(d.data(), c->destroyed_list.p, sizeof(int) * d.size(), cudaMemcpyDeviceToHost));
            std::sort(d.begin(), d.end()); /* DestroyAgent order: slot order of the loop */
            for (int s : d) {
                c->num_agents--;
                c->active[s] = 0;
                c->free_stack.push_back(s);
            }
        }
        if (nr > 0) {
            int m = std::min(nr, c->max_agents);
            std::vector<int> r(m);
            std::vector<V2> rp(m);
            CK(cudaMemcpy(r.data(), c->replan_list.p, sizeof(int) * m, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(rp.data(), c->replan_pos.p, sizeof(V2) * m, cudaMemcpyDeviceToHost));
            std::vector<int> order(m);
            for (int i = 0; i < m; i++) order[i] = i;
            std::sort(order.begin(), order.end(), [&](int a, int b) { return r[a] < r[b]; });
            std::vector<V2> p;
            for (int q : order) {
                int s = r[q];
                V2 goal = c->paths[s].back();
                /* Simulator::UpdatePath (Simulator.cpp:97-124) from the tick-start position.
                   When no path is found the agent keeps its previous path (the
                   reference would keep an empty one and index path.x[-1]). */
                if (plan(c, rp[q], goal, c->clear[s], p) == ECMG_OK && !p.empty()) {
                    c->paths[s] = p;
                    ecmg_status ps = upload_path(c, s);
                    if (ps != ECMG_OK) return ps;
                } else {
                    st.replans_failed++;
                }
            }
        }
    }
    st.active_agents = c->num_agents;
    st.last_index = c->last_idx;
    if (stats) *stats = st;
    return result;
}

ecmg_status ecmg_get_state(ecmg_ctx* c, int field, void* dst)
{
    if (!c || !dst) return ECMG_ERR_INVALID_ARG;
    size_t N = (size_t)c->max_agents;
    CK(cudaStreamSynchronize(c->stream));
    switch (field) {
    case ECMG_FIELD_POSITION: CK(cudaMemcpy(dst, c->pos.p, sizeof(V2) * N, cudaMemcpyDeviceToHost)); break;
    case ECMG_FIELD_VELOCITY: CK(cudaMemcpy(dst, c->vel.p, sizeof(V2) * N, cudaMemcpyDeviceToHost)); break;
    case ECMG_FIELD_PREF_VELOCITY: CK(cudaMemcpy(dst, c->pref_vel.p, sizeof(V2) * N, cudaMemcpyDeviceToHost)); break;
    case ECMG_FIELD_ATTRACTION: CK(cudaMemcpy(dst, c->attr.p, sizeof(V2) * N, cudaMemcpyDeviceToHost)); break;
    case ECMG_FIELD_CLEARANCE: std::memcpy(dst, c->clear.data(), sizeof(float) * N); break;
    case ECMG_FIELD_SPEED: std::memcpy(dst, c->speed.data(), sizeof(float) * N); break;
    case ECMG_FIELD_ACTIVE: std::memcpy(dst, c->active.data(), N); break;
    default: return fail(c, ECMG_ERR_INVALID_ARG, "unknown field %d", field);
    }
    return ECMG_OK;
}

ecmg_status ecmg_set_state(ecmg_ctx* c, int field, const void* src)
{
    if (!c || !src) return ECMG_ERR_INVALID_ARG;
    size_t N = (size_t)c->max_agents;
    CK(cudaStreamSynchronize(c->stream));
    switch (field) {
    case ECMG_FIELD_POSITION: CK(cudaMemcpy(c->pos.p, src, sizeof(V2) * N, cudaMemcpyHostToDevice)); break;
    case ECMG_FIELD_VELOCITY: CK(cudaMemcpy(c->vel.p, src, sizeof(V2) * N, cudaMemcpyHostToDevice)); break;
    case ECMG_FIELD_PREF_VELOCITY: CK(cudaMemcpy(c->pref_vel.p, src, sizeof(V2) * N, cudaMemcpyHostToDevice)); break;
    case ECMG_FIELD_ATTRACTION: CK(cudaMemcpy(c->attr.p, src, sizeof(V2) * N, cudaMemcpyHostToDevice)); break;
    case ECMG_FIELD_CLEARANCE:
        std::memcpy(c->clear.data(), src, sizeof(float) * N);
        CK(cudaMemcpy(c->d_clear.p, src, sizeof(float) * N, cudaMemcpyHostToDevice));
        for (size_t i = 0; i < N; i++) if (c->active[i]) note_range(c, c->clear[i], c->speed[i]);
        break;
    case ECMG_FIELD_SPEED:
        std::memcpy(c->speed.data(), src, sizeof(float) * N);
        CK(cudaMemcpy(c->d_speed.p, src, sizeof(float) * N, cudaMemcpyHostToDevice));
        for (size_t i = 0; i < N; i++) if (c->active[i]) note_range(c, c->clear[i], c->speed[i]);
        break;
    default: return fail(c, ECMG_ERR_INVALID_ARG, "field %d cannot be set", field);
    }
    return ECMG_OK;
}

ecmg_status ecmg_get_counts(const ecmg_ctx* c, int* num_agents, int* last_index, int* max_agents)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (num_agents) *num_agents = c->num_agents;
    if (last_index) *last_index = c->last_idx;
    if (max_agents) *max_agents = c->max_agents;
    return ECMG_OK;
}

ecmg_status ecmg_set_record(ecmg_ctx* c, int on)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    c->record = on != 0;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_get_record(ecmg_ctx* c, int* nbr_ids, int* nbr_count, float* v_orca, int* lp_fail, int* n_cons,
                            int* n_obst)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (!c->record || !c->rec_cnt.p) return fail(c, ECMG_ERR_STATE, "recording is off");
    size_t N = (size_t)c->max_agents;
    CK(cudaStreamSynchronize(c->stream));
    if (nbr_ids) CK(cudaMemcpy(nbr_ids, c->rec_nbr.p, sizeof(int) * N * c->prm.max_neighbors, cudaMemcpyDeviceToHost));
    if (nbr_count) CK(cudaMemcpy(nbr_count, c->rec_cnt.p, sizeof(int) * N, cudaMemcpyDeviceToHost));
    if (v_orca) CK(cudaMemcpy(v_orca, c->rec_vorca.p, sizeof(V2) * N, cudaMemcpyDeviceToHost));
    if (lp_fail) CK(cudaMemcpy(lp_fail, c->rec_fail.p, sizeof(int) * N, cudaMemcpyDeviceToHost));
    if (n_cons) CK(cudaMemcpy(n_cons, c->rec_ncons.p, sizeof(int) * N, cudaMemcpyDeviceToHost));
    if (n_obst) CK(cudaMemcpy(n_obst, c->rec_nobst.p, sizeof(int) * N, cudaMemcpyDeviceToHost));
    return ECMG_OK;
}

/* ---------------------------------------------------------------------- */
static AgentGrid knn_grid_of(float x0, float y0, float x1, float y1, float cell)
{
    AgentGrid g;
    g.cell = cell;
    g.inv = 1.0f / cell;
    g.x0 = x0 - cell;
    g.y0 = y0 - cell;
    g.gw = (int)std::ceil(std::max(0.0f, x1 - x0) / cell) + 3;
    g.gh = (int)std::ceil(std::max(0.0f, y1 - y0) / cell) + 3;
    g.ncells = g.gw * g.gh;
    return g;
}

static size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

size_t ecmg_knn_scratch_bytes(int n, float min_x, float min_y, float max_x, float max_y, float cell)
{
    if (n < 0 || !(cell > 0.0f) || !(max_x >= min_x) || !(max_y >= min_y)) return 0;
    AgentGrid g = knn_grid_of(min_x, min_y, max_x, max_y, cell);
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
    AgentGrid g = knn_grid_of(min_x, min_y, max_x, max_y, cell);
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
