/*
 * ctx.cu -- the simulation context of include/ecmg.h: device buffers, agent
 * pool, one or many independent scenes, the tick loop (optionally captured as
 * a CUDA graph), host re-planning and the launch-configuration autotuner.
 *
 * A context holds n_scenes independent scenes (the reference runs one
 * Simulator per Environment).  Scene s owns the slot range
 * [slot_base_s, slot_base_s + cap_s), its own LIFO free-slot stack
 * (Simulator.h:66-69, 167), obstacles, ECM, planner and agent grid.  All
 * scenes advance in one launch sequence per tick; the per-agent kernel is
 * persistent and load-balances work across scenes of uneven size.
 */
#include "../../include/ecmg.h"
#include "ecmg_internal.h"
#include "host_pool.h"
#include "host_scene.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <map>
#include <tuple>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

using namespace ecmg;

namespace ecmg {
/* mlp.cu */
cudaError_t mlp_infer(ecmg_mlp* mlp, const void* X, const int* n_dev, int n_max, unsigned char* cls, cudaStream_t s,
                      int sms, int* err, int errbit);
cudaError_t mlp_pack(ecmg_mlp* mlp);
}  // namespace ecmg

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

/* SpawnArea / GoalArea (Area.h:30-101) */
struct SpawnAreaH {
    int id = 0;
    float x = 0, y = 0, hw = 0, hh = 0;
    ecmg_spawn_config cfg{5.0f, 10.0f, 5.0f, 10.0f};
    std::vector<int> goals;   /* connectedGoalAreas */
    std::vector<float> rate;  /* spawnRate */
    std::vector<float> since; /* timeSinceLastSpawn */
};
struct GoalAreaH {
    int id = 0;
    float x = 0, y = 0, hw = 0, hh = 0;
};

struct SceneState {
    HostScene hs;
    /* spawn and goal areas in ID order (std::map, as Simulator.h:173-174) */
    std::map<int, SpawnAreaH> spawn_areas;
    std::map<int, GoalAreaH> goal_areas;
    int next_spawn_id = 0, next_goal_id = 0;
    bool has_obst = false;
    GridCSR ob_grid;  /* device candidate grid */
    GridCSR vis_grid; /* planner visibility grid */
    float ob_reach_needed = 0.0f;
    bool ob_dirty = true;
    AgentGrid grid{};
    bool grid_ready = false;
    int grid_agents = 0;
    int bucket_base = 0;
    DBuf<V2> d_ob_p, d_v_pos, d_he_left, d_he_right;
    DBuf<int> d_ob_next, d_ob_prev, d_v_idx, d_he_target, d_ob_gstart, d_ob_gitems, d_ecm_gstart, d_ecm_gitems;
    DBuf<unsigned char> d_ob_convex;
    DBuf<float> d_special_y;
    DBuf<int> d_sp_start, d_sp_items;
    DBuf<unsigned> d_sp_bloom;
    int slot_base = 0, slot_cap = 0;
    std::vector<int> free_stack; /* back() = top */
    int num_agents = 0;
    int last_idx = -1; /* Simulator::m_LastEntityIdx as a global slot index */

    void free_all()
    {
        d_ob_p.free_(); d_v_pos.free_(); d_he_left.free_(); d_he_right.free_();
        d_ob_next.free_(); d_ob_prev.free_(); d_v_idx.free_(); d_he_target.free_();
        d_ob_gstart.free_(); d_ob_gitems.free_(); d_ecm_gstart.free_(); d_ecm_gitems.free_();
        d_ob_convex.free_(); d_special_y.free_(); d_sp_start.free_(); d_sp_items.free_(); d_sp_bloom.free_();
    }
};

}  // namespace

struct ecmg_ctx {
    ecmg_params prm;
    int max_agents = 0;
    std::string err;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_t0 = nullptr, ev_t1 = nullptr;
    cudaEvent_t ev_k[5] = {}; /* around the attraction, neighbour, proposal and per-agent kernels */
    cudaEvent_t ev_mid = nullptr; /* after k_attract: destroyed / re-plan lists are final */
    cudaStream_t stream2 = nullptr; /* the attraction kernel, beside the neighbour search */
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    int sms = 1;
    /* launch configuration (autotuned) */
    int block = 128;
    int tile = 32;
    float cell_scale = 0.4f;
    int lp_mode = 0; /* ECMG_LP_THREAD, ECMG_LP_WARP or ECMG_LP_THREAD_FUSED */
    int occ_div = 1; /* per-thread layout: resident blocks per SM divided by this */
    int knn_wide = 0; /* neighbour kernel register budget (TickArgs::knn_wide) */
    int wgrab = 4;   /* agents per work grab in warp mode */

    /* host mirrors (Simulator bookkeeping, Simulator.h:164-171) */
    std::vector<unsigned char> active;
    std::vector<float> clear, speed;
    std::vector<std::vector<V2>> paths;
    std::vector<int> slot_scene;
    std::vector<std::unique_ptr<SceneState>> scenes;
    int num_agents = 0;

    /* device agent state */
    DBuf<V2> pos, vel, attr, pref_vel, replan_pos;
    DBuf<float> d_clear, d_speed;
    DBuf<unsigned char> d_active;
    DBuf<int> path_off, path_len, key, rank, destroyed_list, replan_list, d_slot_scene, nbr, ncnt;
    DBuf<V2> path_xy;
    size_t path_used = 0;
    /* snapshot */
    DBuf<int> s_slot;
    DBuf<V2> s_pos, s_vel;
    DBuf<float> s_clear;
    /* buckets of all scenes */
    int total_buckets = 0;
    bool table_dirty = true;
    DBuf<SceneDev> d_scenes;
    DBuf<int> cell_count, cell_start, scan_tmp, counters;
    /* planner */
    ecmg_plan_fn plan_fn = nullptr;
    void* plan_user = nullptr;
    PlanScratch scratch;
    HostPool<PlanScratch> pool; /* planner threads (built-in planner only: it is re-entrant) */
    int planner_mode = ECMG_PLANNER_REFERENCE; /* the reference's paths unless FAST is chosen */
    bool replan_enabled = true;
    bool spawn_enabled = true; /* off while the autotuner runs its trial ticks */
    /* per slot: the start edge from which the built-in planner's search
       failed for the slot's current goal and clearance (-1: none) */
    std::vector<int> fail_edge;
    DBuf<int> d_fail_edge;
    /* re-plans whose searches run on a helper thread (built-in planner)
       while the next tick's graph runs: that tick marks their agents pending
       and steps them in k_fixup once the paths are in (ecmg_set_replan_overlap) */
    struct PlanBatch {
        std::vector<int> slot; /* ascending */
        std::vector<V2> start, goal;
        std::vector<float> clr;
        std::vector<std::vector<V2>> res;
        std::vector<char> ok;
        std::vector<int> fe;
        /* a persistent helper thread: one search runs on it, several on the
           planner pool (with the helper's own scratch for its share) */
        std::thread th;
        std::mutex mu;
        std::condition_variable cv, cv_done;
        std::atomic<bool> work{false}, stop{false};
        std::atomic<bool> done{true};
        bool active = false; /* started and not yet applied (calling thread only) */
        long long seq = 0;   /* start order */
        PlanScratch scr;
    } batch[2]; /* the last tick's searches and this tick's, in flight together */
    long long batch_seq = 0;
    std::mutex pool_mu; /* one user of the planner pool at a time */
    int replan_overlap = 1; /* 0 off, 1 when a search outlasts its tick, 2 always */
    long long batch_failed = 0; /* failed searches applied outside a tick, counted with the next one */
    DBuf<int> d_pend;
    /* recording */
    bool record = false;
    DBuf<int> rec_nbr, rec_cnt, rec_fail, rec_ncons, rec_nobst;
    DBuf<V2> rec_vorca;
    /* learned proposal / trace */
    ecmg_mlp* model = nullptr;
    /* gating: a tick whose acceptance rate is below gate_min, or whose
       device time per agent exceeds that of the plain tick by 2 %, pauses
       the model for gate_pause ticks (plain ticks), then it is tried again.
       The per-agent times are running averages of the ticks with and
       without the model; without a plain time yet, 3 model ticks are
       followed by 3 plain ones to measure it. */
    float gate_min = 0.1f;
    int gate_pause = 64;
    int gate_left = 0;
    float gate_t_model = -1.0f, gate_t_plain = -1.0f; /* ms per agent, running averages */
    int gate_model_ticks = 0;
    const unsigned char* cls_override = nullptr;
    bool trace = false;
    int trace_rows = 0;
    DBuf<unsigned char> feat, cls, label;
    /* pinned staging */
    int* h_counters = nullptr; /* [3 * kCounters]: in, out, after k_attract */
    void* hview[4] = {nullptr, nullptr, nullptr, nullptr}; /* ecmg_host_view of the float2 fields */
    /* ecmg_set_host_mirror: every tick ends with a copy of the slots it may
       have moved into hview[position] and hview[velocity] (device addresses
       below); stale after any other write of positions or velocities */
    bool mirror = false, mirror_stale = true;
    V2* mirror_dev[2] = {nullptr, nullptr};
    /* the first kListStage entries of the destroyed / re-plan lists, copied
       back by every tick (no extra copy when a tick's lists fit) */
    static constexpr int kListStage = 1024;
    int* h_lists = nullptr; /* destroyed[kListStage], replan[kListStage], replan_pos[2 * kListStage] (float) */
    /* page-locked staging of the small uploads between two ticks (paths of
       re-planned agents); the copies are queued on the stream ahead of the
       next tick */
    unsigned char* h_up = nullptr;
    size_t h_up_cap = 0, h_up_used = 0;
    /* spawn stage: queued random values (rq[rq_head..] not yet consumed),
       their source, page-locked candidate / area / hit tables and the
       agents the last stage placed */
    ecmg_rand_fn rng_fn = nullptr;
    void* rng_user = nullptr;
    int rand_max = RAND_MAX;
    std::vector<int> rq;
    size_t rq_head = 0;
    V2* h_cand = nullptr;
    SpawnAreaDev* h_sarea = nullptr;
    int* h_hit = nullptr;
    DBuf<V2> d_cand;
    DBuf<SpawnAreaDev> d_sarea;
    DBuf<int> d_hit;
    DBuf<SpawnRec> d_spawn_rec;
    std::vector<int> spawned_slot;
    std::vector<V2> spawned_start, spawned_goal;
    /* neighbour mode: 0 exact kNN, 1 the reference's kd-tree (kdtree.cu) */
    int nbr_mode = 0;
    struct KdBufs {
        DBuf<unsigned char> mark, side;
        DBuf<int> n_dev, iscan, ids0, vtmp, X0, X[2], Y[2], seg_lo, seg_hi, seg_node, scan_tmp32, hist, tree, map,
            kfound, agg, prev_in, cache;
        DBuf<unsigned> keys, ktmp;
        DBuf<unsigned long long> flags, scan_tmp64;
        DBuf<V2> tree_pos;
        int levels = 0, tree_cap = 0;
        void free_all()
        {
            mark.free_(); side.free_();
            DBuf<int>* is[] = {&n_dev, &iscan, &ids0, &vtmp, &X0, &X[0], &X[1], &Y[0], &Y[1], &seg_lo, &seg_hi,
                               &seg_node, &scan_tmp32, &hist, &tree, &map, &kfound, &agg, &prev_in, &cache};
            for (auto* b : is) b->free_();
            keys.free_(); ktmp.free_(); flags.free_(); scan_tmp64.free_(); tree_pos.free_();
        }
    } kd;
    /* graph */
    cudaGraphExec_t graph[2] = {nullptr, nullptr}; /* plain tick, tick with the proposal model */
    bool graph_dirty = true;
    int graph_last = -2; /* last slot the captured launch sizes cover */

    int global_last() const
    {
        int m = -1;
        for (auto& s : scenes) m = std::max(m, s->last_idx);
        return m;
    }
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

/* applies the re-plans still in flight (defined with the tick's re-plan
   helpers); entry points that read or change paths, agents, the scene or the
   planner call it first */
static ecmg_status drain(ecmg_ctx* c);
static void batch_stop(ecmg_ctx* c);
#define DRAIN(c)                                            \
    do {                                                    \
        ecmg_status drain_status_ = drain(c);               \
        if (drain_status_ != ECMG_OK) return drain_status_; \
    } while (0)


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
    if (p->block_size != 0 && p->block_size != 64 && p->block_size != 128 && p->block_size != 256)
        return fail(c, ECMG_ERR_INVALID_ARG, "block_size must be 0, 64, 128 or 256");
    return ECMG_OK;
}

ecmg_status ecmg_create_batch(const ecmg_params* p, int n_scenes, const int* max_agents_per_scene, ecmg_ctx** out)
{
    if (!out) return ECMG_ERR_INVALID_ARG;
    *out = nullptr;
    if (n_scenes < 1 || !max_agents_per_scene) return ECMG_ERR_INVALID_ARG;
    long long total = 0;
    for (int s = 0; s < n_scenes; s++) {
        if (max_agents_per_scene[s] < 1) return ECMG_ERR_INVALID_ARG;
        total += max_agents_per_scene[s];
    }
    if (total > (1ll << 30)) return ECMG_ERR_INVALID_ARG;
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
    if (prm.block_size) c->block = prm.block_size;
    c->max_agents = (int)total;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev);
#define CKC(x) do { if ((x) != cudaSuccess) { ecmg_destroy(c); return ECMG_ERR_CUDA; } } while (0)
    CKC(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    CKC(cudaEventCreate(&c->ev_t0));
    CKC(cudaEventCreate(&c->ev_t1));
    for (auto& e : c->ev_k) CKC(cudaEventCreate(&e));
    CKC(cudaEventCreateWithFlags(&c->ev_mid, cudaEventDisableTiming));
    CKC(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    CKC(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    CKC(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking));
    size_t N = (size_t)total;
    CKC(c->pos.alloc(N)); CKC(c->vel.alloc(N)); CKC(c->attr.alloc(N)); CKC(c->pref_vel.alloc(N));
    CKC(c->d_clear.alloc(N)); CKC(c->d_speed.alloc(N)); CKC(c->d_active.alloc(N));
    CKC(c->path_off.alloc(N)); CKC(c->path_len.alloc(N)); CKC(c->key.alloc(N)); CKC(c->rank.alloc(N));
    CKC(c->destroyed_list.alloc(N)); CKC(c->replan_list.alloc(N)); CKC(c->replan_pos.alloc(N));
    CKC(c->d_pend.alloc(N));
    CKC(c->s_slot.alloc(N)); CKC(c->s_pos.alloc(N)); CKC(c->s_vel.alloc(N)); CKC(c->s_clear.alloc(N));
    CKC(c->d_slot_scene.alloc(N));
    CKC(c->nbr.alloc(N * (size_t)prm.max_neighbors));
    CKC(c->ncnt.alloc(N));
    CKC(c->d_fail_edge.alloc(N));
    CKC(cudaMemset(c->d_fail_edge.p, 0xff, sizeof(int) * N)); /* -1 */
    CKC(c->counters.alloc(kCounters));
    CKC(c->path_xy.alloc(std::max<size_t>(1024, 4 * N)));
    CKC(cudaMemset(c->pos.p, 0, sizeof(V2) * N)); CKC(cudaMemset(c->vel.p, 0, sizeof(V2) * N));
    CKC(cudaMemset(c->attr.p, 0, sizeof(V2) * N)); CKC(cudaMemset(c->pref_vel.p, 0, sizeof(V2) * N));
    CKC(cudaMemset(c->d_active.p, 0, N)); CKC(cudaMemset(c->path_len.p, 0, sizeof(int) * N));
    CKC(cudaMemset(c->path_off.p, 0, sizeof(int) * N));
    CKC(cudaMemset(c->d_clear.p, 0, sizeof(float) * N)); CKC(cudaMemset(c->d_speed.p, 0, sizeof(float) * N));
    CKC(cudaHostAlloc((void**)&c->h_counters, sizeof(int) * 3 * kCounters, cudaHostAllocDefault));
    CKC(cudaHostAlloc((void**)&c->h_lists, sizeof(int) * 4 * ecmg_ctx::kListStage, cudaHostAllocDefault));
    c->active.assign(N, 0);
    c->clear.assign(N, 0.0f);
    c->speed.assign(N, 0.0f);
    c->paths.assign(N, {});
    c->fail_edge.assign(N, -1);
    c->slot_scene.assign(N, 0);
    int base = 0;
    for (int s = 0; s < n_scenes; s++) {
        auto sc = std::make_unique<SceneState>();
        sc->slot_base = base;
        sc->slot_cap = max_agents_per_scene[s];
        sc->last_idx = base - 1;
        sc->free_stack.reserve(sc->slot_cap);
        for (int i = base + sc->slot_cap - 1; i >= base; i--) sc->free_stack.push_back(i); /* Simulator.h:66-69 */
        for (int i = base; i < base + sc->slot_cap; i++) c->slot_scene[i] = s;
        base += sc->slot_cap;
        c->scenes.push_back(std::move(sc));
    }
    CKC(cudaMemcpy(c->d_slot_scene.p, c->slot_scene.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
#undef CKC
    *out = c;
    return ECMG_OK;
}

ecmg_status ecmg_create(const ecmg_params* p, int max_agents, ecmg_ctx** out)
{
    if (!out) return ECMG_ERR_INVALID_ARG;
    *out = nullptr;
    if (max_agents < 1) return ECMG_ERR_INVALID_ARG;
    return ecmg_create_batch(p, 1, &max_agents, out);
}

ecmg_status ecmg_destroy(ecmg_ctx* c)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    batch_stop(c); /* searches in flight are waited for; their results are not needed */
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& g : c->graph)
        if (g) cudaGraphExecDestroy(g);
    DBuf<V2>* v2s[] = {&c->pos, &c->vel, &c->attr, &c->pref_vel, &c->replan_pos, &c->path_xy, &c->s_pos, &c->s_vel,
                       &c->rec_vorca};
    for (auto* b : v2s) b->free_();
    DBuf<int>* is[] = {&c->d_pend, &c->path_off, &c->path_len, &c->key, &c->rank, &c->destroyed_list, &c->replan_list,
                       &c->d_slot_scene, &c->nbr, &c->ncnt, &c->d_fail_edge, &c->s_slot, &c->cell_count, &c->cell_start, &c->scan_tmp, &c->counters,
                       &c->rec_nbr, &c->rec_cnt, &c->rec_fail, &c->rec_ncons, &c->rec_nobst};
    for (auto* b : is) b->free_();
    c->d_clear.free_();
    c->d_speed.free_();
    c->s_clear.free_();
    c->d_active.free_();
    c->feat.free_();
    c->cls.free_();
    c->label.free_();
    c->d_scenes.free_();
    for (auto& s : c->scenes) s->free_all();
    if (c->h_counters) cudaFreeHost(c->h_counters);
    if (c->h_lists) cudaFreeHost(c->h_lists);
    if (c->h_up) cudaFreeHost(c->h_up);
    if (c->h_cand) cudaFreeHost(c->h_cand);
    if (c->h_sarea) cudaFreeHost(c->h_sarea);
    if (c->h_hit) cudaFreeHost(c->h_hit);
    c->d_cand.free_();
    c->d_sarea.free_();
    c->d_hit.free_();
    c->d_spawn_rec.free_();
    c->kd.free_all();
    for (void* h : c->hview)
        if (h) cudaFreeHost(h);
    if (c->ev_t0) cudaEventDestroy(c->ev_t0);
    if (c->ev_t1) cudaEventDestroy(c->ev_t1);
    for (auto& e : c->ev_k)
        if (e) cudaEventDestroy(e);
    if (c->ev_mid) cudaEventDestroy(c->ev_mid);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->stream2) cudaStreamDestroy(c->stream2);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return ECMG_OK;
}

static void scene_bbox(SceneState& sc)
{
    HostScene& s = sc.hs;
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

static SceneState* scene_at(ecmg_ctx* c, int scene)
{
    if (!c || scene < 0 || scene >= (int)c->scenes.size()) return nullptr;
    return c->scenes[scene].get();
}

ecmg_status ecmg_scene_set_obstacles(ecmg_ctx* c, int scene, const ecmg_obstacles* o)
{
    DRAIN(c);
    SceneState* sc = scene_at(c, scene);
    if (!sc || !o) return fail(c, ECMG_ERR_INVALID_ARG, "null argument or bad scene");
    if (o->n_obstacles < 0 || (o->n_obstacles > 0 && (!o->ring_offsets || !o->xy)))
        return fail(c, ECMG_ERR_INVALID_ARG, "bad obstacle arrays");
    for (int r = 0; r < o->n_obstacles; r++)
        if (o->ring_offsets[r + 1] - o->ring_offsets[r] < 2)
            return fail(c, ECMG_ERR_INVALID_ARG, "obstacle %d has fewer than 2 vertices (Environment.cpp:288)", r);
    int nv = o->n_obstacles > 0 ? o->ring_offsets[o->n_obstacles] : 0;
    for (int i = 0; i < nv; i++)
        if (!finite2(o->xy[2 * i], o->xy[2 * i + 1])) return fail(c, ECMG_ERR_INVALID_ARG, "non-finite obstacle vertex");
    set_obstacles(sc->hs, o->n_obstacles, o->ring_offsets, o->xy);
    scene_bbox(*sc);
    HostScene& s = sc->hs;
    size_t n = std::max<size_t>(1, s.ob_p.size());
    CK(sc->d_ob_p.alloc(n)); CK(sc->d_ob_next.alloc(n)); CK(sc->d_ob_prev.alloc(n)); CK(sc->d_ob_convex.alloc(n));
    if (nv > 0) {
        CK(cudaMemcpy(sc->d_ob_p.p, s.ob_p.data(), sizeof(V2) * nv, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(sc->d_ob_next.p, s.ob_next.data(), sizeof(int) * nv, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(sc->d_ob_prev.p, s.ob_prev.data(), sizeof(int) * nv, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(sc->d_ob_convex.p, s.ob_convex.data(), nv, cudaMemcpyHostToDevice));
    }
    build_obst_grid(s, 0.0f, 4.0f, sc->vis_grid);
    sc->has_obst = true;
    sc->ob_dirty = true;
    sc->grid_ready = false;
    c->table_dirty = true;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_scene_set_ecm(ecmg_ctx* c, int scene, const ecmg_ecm* e)
{
    DRAIN(c);
    SceneState* sc = scene_at(c, scene);
    if (!sc || !e) return fail(c, ECMG_ERR_INVALID_ARG, "null argument or bad scene");
    if (e->n_vertices < 0 || e->n_edges < 0) return fail(c, ECMG_ERR_INVALID_ARG, "negative sizes");
    int V = e->n_vertices, E = e->n_edges;
    HostScene& s = sc->hs;
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
        if (!finite2(e->he_left[2 * h], e->he_left[2 * h + 1]) || !finite2(e->he_right[2 * h], e->he_right[2 * h + 1]))
            return fail(c, ECMG_ERR_INVALID_ARG, "non-finite closest point");
        s.he_left[h] = mk(e->he_left[2 * h], e->he_left[2 * h + 1]);
        s.he_right[h] = mk(e->he_right[2 * h], e->he_right[2 * h + 1]);
    }
    s.has_ecm = true;
    scene_bbox(*sc);
    build_ecm_grid(s);
    if (sc->has_obst) build_obst_grid(s, 0.0f, 4.0f, sc->vis_grid);
    size_t nV = std::max<size_t>(1, V), nH = std::max<size_t>(1, 2 * (size_t)E);
    CK(sc->d_v_pos.alloc(nV)); CK(sc->d_v_idx.alloc(nV)); CK(sc->d_he_target.alloc(nH));
    CK(sc->d_he_left.alloc(nH)); CK(sc->d_he_right.alloc(nH));
    CK(sc->d_ecm_gstart.alloc(s.ecm_grid.start.size()));
    CK(sc->d_ecm_gitems.alloc(std::max<size_t>(1, s.ecm_grid.items.size())));
    CK(sc->d_special_y.alloc(std::max<size_t>(1, s.special_y.size())));
    CK(sc->d_sp_start.alloc(std::max<size_t>(1, s.sp_start.size())));
    CK(sc->d_sp_items.alloc(std::max<size_t>(1, s.sp_items.size())));
    if (!s.sp_start.empty())
        CK(cudaMemcpy(sc->d_sp_start.p, s.sp_start.data(), sizeof(int) * s.sp_start.size(), cudaMemcpyHostToDevice));
    if (!s.sp_items.empty())
        CK(cudaMemcpy(sc->d_sp_items.p, s.sp_items.data(), sizeof(int) * s.sp_items.size(), cudaMemcpyHostToDevice));
    CK(sc->d_sp_bloom.alloc(std::max<size_t>(1, s.sp_bloom.size())));
    if (!s.sp_bloom.empty())
        CK(cudaMemcpy(sc->d_sp_bloom.p, s.sp_bloom.data(), sizeof(unsigned) * s.sp_bloom.size(), cudaMemcpyHostToDevice));
    if (V) {
        CK(cudaMemcpy(sc->d_v_pos.p, s.v_pos.data(), sizeof(V2) * V, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(sc->d_v_idx.p, s.v_idx.data(), sizeof(int) * V, cudaMemcpyHostToDevice));
    }
    if (E) {
        CK(cudaMemcpy(sc->d_he_target.p, s.he_target.data(), sizeof(int) * 2 * E, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(sc->d_he_left.p, s.he_left.data(), sizeof(V2) * 2 * E, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(sc->d_he_right.p, s.he_right.data(), sizeof(V2) * 2 * E, cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(sc->d_ecm_gstart.p, s.ecm_grid.start.data(), sizeof(int) * s.ecm_grid.start.size(), cudaMemcpyHostToDevice));
    if (!s.ecm_grid.items.empty())
        CK(cudaMemcpy(sc->d_ecm_gitems.p, s.ecm_grid.items.data(), sizeof(int) * s.ecm_grid.items.size(), cudaMemcpyHostToDevice));
    if (!s.special_y.empty())
        CK(cudaMemcpy(sc->d_special_y.p, s.special_y.data(), sizeof(float) * s.special_y.size(), cudaMemcpyHostToDevice));
    sc->grid_ready = false;
    c->table_dirty = true;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_set_obstacles(ecmg_ctx* c, const ecmg_obstacles* o) { return ecmg_scene_set_obstacles(c, 0, o); }
ecmg_status ecmg_set_ecm(ecmg_ctx* c, const ecmg_ecm* e) { return ecmg_scene_set_ecm(c, 0, e); }

ecmg_status ecmg_set_planner_mode(ecmg_ctx* c, int mode)
{
    if (!c || (mode != ECMG_PLANNER_FAST && mode != ECMG_PLANNER_REFERENCE)) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    if (mode != c->planner_mode) {
        c->planner_mode = mode;
        /* the failed-search memo belongs to the planner that made it */
        std::fill(c->fail_edge.begin(), c->fail_edge.end(), -1);
        CK(cudaMemset(c->d_fail_edge.p, 0xff, sizeof(int) * (size_t)c->max_agents));
    }
    return ECMG_OK;
}

ecmg_status ecmg_set_replan_overlap(ecmg_ctx* c, int on)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    if (on < 0 || on > 2) return fail(c, ECMG_ERR_INVALID_ARG, "overlap mode %d", on);
    c->replan_overlap = on;
    return ECMG_OK;
}

ecmg_status ecmg_set_planner(ecmg_ctx* c, ecmg_plan_fn fn, void* user)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    if ((fn == nullptr) != (c->plan_fn == nullptr)) c->graph_dirty = true; /* TickArgs::replan_dev_fail */
    c->plan_fn = fn;
    c->plan_user = user;
    return ECMG_OK;
}

/* queues a copy of host memory to the device on the context's stream,
   through the page-locked staging area (no wait for the copy) */
static ecmg_status stage_copy(ecmg_ctx* c, void* dev_dst, const void* src, size_t bytes)
{
    if (bytes == 0) return ECMG_OK;
    if (c->h_up_used + bytes > c->h_up_cap) {
        CK(cudaStreamSynchronize(c->stream)); /* staged copies done: the area is free */
        c->h_up_used = 0;
        if (bytes > c->h_up_cap) {
            if (c->h_up) cudaFreeHost(c->h_up);
            c->h_up = nullptr;
            c->h_up_cap = 0;
            size_t cap = std::max<size_t>(bytes, 1u << 20);
            CK(cudaHostAlloc((void**)&c->h_up, cap, cudaHostAllocDefault));
            c->h_up_cap = cap;
        }
    }
    unsigned char* p = c->h_up + c->h_up_used;
    std::memcpy(p, src, bytes);
    c->h_up_used += (bytes + 15) & ~(size_t)15;
    CK(cudaMemcpyAsync(dev_dst, p, bytes, cudaMemcpyHostToDevice, c->stream));
    return ECMG_OK;
}

/* forgets a slot's failed-search edge (its path, goal or clearance changed) */
static ecmg_status clear_fail_edge(ecmg_ctx* c, int slot)
{
    if (c->fail_edge[slot] < 0) return ECMG_OK;
    c->fail_edge[slot] = -1;
    const int none = -1;
    return stage_copy(c, c->d_fail_edge.p + slot, &none, sizeof(int));
}

/* makes room for `need` more path points at path_used: grows (x2) and
   compacts the path store (after the queued uploads) when it is full */
static ecmg_status ensure_path_room(ecmg_ctx* c, size_t need)
{
    if (c->path_used + need > c->path_xy.n) {
        CK(cudaStreamSynchronize(c->stream));
        size_t live = 0;
        for (int i = 0; i < c->max_agents; i++) live += c->paths[i].size();
        size_t cap = std::max(c->path_xy.n * 2, (live + need) * 2 + 1024);
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
    }
    return ECMG_OK;
}

static ecmg_status upload_path(ecmg_ctx* c, int slot)
{
    {
        ecmg_status fs = clear_fail_edge(c, slot);
        if (fs != ECMG_OK) return fs;
    }
    const std::vector<V2>& p = c->paths[slot];
    size_t n = p.size();
    if (c->path_used + n > c->path_xy.n) {
        /* the compaction uploads every slot's path, this one included */
        return ensure_path_room(c, n);
    }
    int off = (int)c->path_used, len = (int)n;
    ecmg_status s = stage_copy(c, c->path_xy.p + off, p.data(), sizeof(V2) * n);
    if (s == ECMG_OK) s = stage_copy(c, c->path_off.p + slot, &off, sizeof(int));
    if (s == ECMG_OK) s = stage_copy(c, c->path_len.p + slot, &len, sizeof(int));
    if (s != ECMG_OK) return s;
    c->path_used += n;
    return ECMG_OK;
}

static void note_range(ecmg_ctx* c, SceneState* sc, float clearance, float speed)
{
    float ms = c->prm.max_speed > 0.0f ? c->prm.max_speed : speed;
    float r = c->prm.tau_obst * ms + clearance;
    if (r > sc->ob_reach_needed) {
        sc->ob_reach_needed = r;
        if (r > sc->ob_grid.reach) sc->ob_dirty = true;
    }
}

ecmg_status ecmg_scene_add_agents(ecmg_ctx* c, int scene, int n, const float* pos, const float* clearance,
                                  const float* pref_speed, const int* path_off, const int* path_len,
                                  const float* path_xy, int* out_slots)
{
    DRAIN(c);
    SceneState* sc = scene_at(c, scene);
    if (!sc) return fail(c, ECMG_ERR_INVALID_ARG, "bad scene");
    if (n < 0 || (n > 0 && (!pos || !clearance || !pref_speed || !path_off || !path_len || !path_xy)))
        return fail(c, ECMG_ERR_INVALID_ARG, "null or negative argument");
    if ((size_t)n > sc->free_stack.size())
        return fail(c, ECMG_ERR_NO_SLOT, "%d agents requested, %zu slots free", n, sc->free_stack.size());
    CK(cudaStreamSynchronize(c->stream)); /* queued uploads land before the copies below */
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
        int idx = sc->free_stack.back();
        sc->free_stack.pop_back();
        slots[i] = idx;
        sc->num_agents++;
        c->num_agents++;
        sc->last_idx = std::max(sc->last_idx, idx);
        c->active[idx] = 1;
        c->clear[idx] = clearance[i];
        c->speed[idx] = pref_speed[i];
        c->paths[idx].assign((const V2*)(path_xy + 2 * (size_t)path_off[i]),
                             (const V2*)(path_xy + 2 * (size_t)(path_off[i] + path_len[i])));
        note_range(c, sc, clearance[i], pref_speed[i]);
        ecmg_status fs = clear_fail_edge(c, idx);
        if (fs != ECMG_OK) return fs;
    }
    /* contiguous runs of slots are uploaded in one copy each */
    for (int i = 0; i < n;) {
        int j = i;
        while (j + 1 < n && slots[j + 1] == slots[j] + 1) j++;
        int s0 = slots[i], cnt = j - i + 1;
        std::vector<V2> z((size_t)cnt, mk(0.0f, 0.0f));
        std::vector<unsigned char> one((size_t)cnt, 1);
        CK(cudaMemcpy(c->pos.p + s0, pos + 2 * (size_t)i, sizeof(V2) * cnt, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(c->vel.p + s0, z.data(), sizeof(V2) * cnt, cudaMemcpyHostToDevice));
        c->mirror_stale = true;
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
    if (sc->grid_agents == 0 || sc->num_agents > 2 * sc->grid_agents) {
        sc->grid_ready = false;
        c->table_dirty = true;
    }
    return ECMG_OK;
}

ecmg_status ecmg_add_agents(ecmg_ctx* c, int n, const float* pos, const float* clearance, const float* pref_speed,
                            const int* path_off, const int* path_len, const float* path_xy, int* out_slots)
{
    return ecmg_scene_add_agents(c, 0, n, pos, clearance, pref_speed, path_off, path_len, path_xy, out_slots);
}

/* fn(i, scratch) for i in [0, m): on the pool's threads with the built-in
   planner, on the calling thread with a caller-supplied one */
static void plan_jobs(ecmg_ctx* c, int m, const std::function<void(int, PlanScratch&)>& fn)
{
    if (c->plan_fn || m < 2) {
        for (int i = 0; i < m; i++) fn(i, c->scratch);
        return;
    }
    c->pool.start(std::min(15, (int)std::max(1u, std::thread::hardware_concurrency()) - 1));
    if (c->pool.size() == 0) {
        for (int i = 0; i < m; i++) fn(i, c->scratch);
        return;
    }
    std::lock_guard<std::mutex> l(c->pool_mu);
    c->pool.run(m, [&](int i, int w) { fn(i, c->pool.scratch[w]); });
}

static ecmg_status plan(ecmg_ctx* c, SceneState* sc, V2 s, V2 g, float clr, std::vector<V2>& out, PlanScratch& scr,
                        int* astar_fail_edge = nullptr)
{
    out.clear();
    if (astar_fail_edge) *astar_fail_edge = -1;
    if (c->plan_fn) {
        std::vector<float> buf(2 * 4096);
        int n = c->plan_fn(c->plan_user, s.x, s.y, g.x, g.y, clr, buf.data(), 4096);
        if (n < 0) return ECMG_ERR_NO_PATH;
        n = std::min(n, 4096);
        for (int i = 0; i < n; i++) out.push_back(mk(buf[2 * i], buf[2 * i + 1]));
        return n > 0 ? ECMG_OK : ECMG_ERR_NO_PATH;
    }
    if (!sc->hs.has_ecm) return ECMG_ERR_STATE;
    const bool ok = c->planner_mode == ECMG_PLANNER_REFERENCE
                        ? plan_path_reference(sc->hs, s, g, clr, out, scr.ref, astar_fail_edge)
                        : plan_path(sc->hs, sc->vis_grid, s, g, clr, out, scr, astar_fail_edge);
    return ok ? ECMG_OK : ECMG_ERR_NO_PATH;
}

ecmg_status ecmg_find_path(ecmg_ctx* c, float sx, float sy, float gx, float gy, float clearance, float* out_xy,
                           int cap, int* out_n)
{
    if (!c || !out_n || (cap > 0 && !out_xy)) return ECMG_ERR_INVALID_ARG;
    std::vector<V2> p;
    ecmg_status st = plan(c, c->scenes[0].get(), mk(sx, sy), mk(gx, gy), clearance, p, c->scratch);
    *out_n = st == ECMG_OK ? (int)p.size() : -1;
    for (int i = 0; i < (int)p.size() && i < cap; i++) { out_xy[2 * i] = p[i].x; out_xy[2 * i + 1] = p[i].y; }
    return st;
}

/* page-locked and device tables of the location checks (spawn.cu) */
/* ---- re-plans of a tick (Simulator::UpdatePath, Simulator.cpp:97-124) ----
   From the tick-start position, served in slot order.  When no path is
   found the agent keeps its previous path (the reference would keep an empty
   one and index path.x[-1]).  The built-in planner is re-entrant, so the
   searches of a tick run on several host threads. */

/* applies search results in slot order: the new path uploaded behind the
   queued device work, or the failed-search edge remembered */
static ecmg_status apply_plans(ecmg_ctx* c, const std::vector<int>& slot, std::vector<std::vector<V2>>& res,
                               const std::vector<char>& ok, const std::vector<int>& fe, long long* failed)
{
    for (size_t i = 0; i < slot.size(); i++) {
        const int sl = slot[i];
        if (ok[i]) {
            c->paths[sl] = std::move(res[i]);
            ecmg_status ps = upload_path(c, sl);
            if (ps != ECMG_OK) return ps;
        } else {
            (*failed)++;
            if (fe[i] >= 0 && c->fail_edge[sl] != fe[i]) {
                c->fail_edge[sl] = fe[i];
                ecmg_status fs = stage_copy(c, c->d_fail_edge.p + sl, &fe[i], sizeof(int));
                if (fs != ECMG_OK) return fs;
            }
        }
    }
    return ECMG_OK;
}

/* the re-plans of `slot` (ascending) from `start`, now: on the planner
   threads, or on the calling thread while a batch holds them */
static ecmg_status plan_now(ecmg_ctx* c, const std::vector<int>& slot, const std::vector<V2>& start,
                            long long* failed)
{
    const int m = (int)slot.size();
    std::vector<std::vector<V2>> res(m);
    std::vector<char> ok(m, 0);
    std::vector<int> fe(m, -1);
    auto one = [&](int i, PlanScratch& scr) {
        const int sl = slot[i];
        SceneState* sc = c->scenes[c->slot_scene[sl]].get();
        ok[i] = plan(c, sc, start[i], c->paths[sl].back(), c->clear[sl], res[i], scr, &fe[i]) == ECMG_OK &&
                !res[i].empty();
    };
    if (c->batch[0].active || c->batch[1].active) {
        for (int i = 0; i < m; i++) one(i, c->scratch);
    } else {
        plan_jobs(c, m, one);
    }
    return apply_plans(c, slot, res, ok, fe, failed);
}

/* polls flag (yielding the core between polls) until it is set or `limit`
   has passed */
constexpr std::chrono::microseconds kSpinWait{1000};
static void spin_until(const std::atomic<bool>& flag, std::chrono::microseconds limit)
{
    const auto t0 = std::chrono::steady_clock::now();
    for (int it = 0; !flag.load(); it++) {
        if ((it & 63) == 63 && std::chrono::steady_clock::now() - t0 > limit) return;
        std::this_thread::yield();
    }
}

/* the searches of batch b (on its helper thread) */
static void batch_run(ecmg_ctx* c, ecmg_ctx::PlanBatch& b)
{
    const int m = (int)b.slot.size();
    auto one = [&](int i, PlanScratch& scr) {
        SceneState* sc = c->scenes[c->slot_scene[b.slot[i]]].get();
        b.ok[i] = plan(c, sc, b.start[i], b.goal[i], b.clr[i], b.res[i], scr, &b.fe[i]) == ECMG_OK &&
                  !b.res[i].empty();
    };
    if (m < 2 || c->pool.size() == 0) {
        for (int i = 0; i < m; i++) one(i, b.scr);
    } else {
        std::lock_guard<std::mutex> l(c->pool_mu);
        c->pool.run(m, [&](int i, int w) { one(i, w == 0 ? b.scr : c->pool.scratch[w]); });
    }
}

/* the re-plans of `slot` (ascending) on batch b's helper thread; goals and
   clearances are taken now */
static void batch_start(ecmg_ctx* c, ecmg_ctx::PlanBatch& b, const std::vector<int>& slot,
                        const std::vector<V2>& start)
{
    const int m = (int)slot.size();
    b.slot = slot;
    b.start = start;
    b.goal.resize(m);
    b.clr.resize(m);
    for (int i = 0; i < m; i++) {
        b.goal[i] = c->paths[slot[i]].back();
        b.clr[i] = c->clear[slot[i]];
    }
    b.res.assign(m, {});
    b.ok.assign(m, 0);
    b.fe.assign(m, -1);
    c->pool.start(std::min(15, (int)std::max(1u, std::thread::hardware_concurrency()) - 1));
    if (!b.th.joinable())
        b.th = std::thread([c, &b] {
            for (;;) {
                /* the next batch usually comes within a tick: poll for it a
                   while before sleeping (a sleeping thread takes tens of
                   microseconds to wake) */
                spin_until(b.work, kSpinWait);
                {
                    std::unique_lock<std::mutex> l(b.mu);
                    b.cv.wait(l, [&] { return b.work.load() || b.stop.load(); });
                    if (b.stop) return;
                    b.work = false;
                }
                batch_run(c, b);
                {
                    std::lock_guard<std::mutex> l(b.mu);
                    b.done.store(true);
                }
                b.cv_done.notify_all();
            }
        });
    b.active = true;
    b.seq = ++c->batch_seq;
    {
        std::lock_guard<std::mutex> l(b.mu);
        b.done.store(false);
        b.work = true;
    }
    b.cv.notify_one();
}

/* waits for batch b's searches and applies them */
static ecmg_status batch_apply(ecmg_ctx* c, ecmg_ctx::PlanBatch& b, long long* failed)
{
    if (!b.active) return ECMG_OK;
    spin_until(b.done, kSpinWait); /* the caller has nothing else to do */
    {
        std::unique_lock<std::mutex> l(b.mu);
        b.cv_done.wait(l, [&] { return b.done.load(); });
    }
    b.active = false;
    return apply_plans(c, b.slot, b.res, b.ok, b.fe, failed);
}

/* the batch started first among those in flight (null: none) */
static ecmg_ctx::PlanBatch* oldest_batch(ecmg_ctx* c)
{
    ecmg_ctx::PlanBatch *a = &c->batch[0], *b = &c->batch[1];
    if (a->active && b->active) return a->seq < b->seq ? a : b;
    return a->active ? a : b->active ? b : nullptr;
}

/* every batch in flight applied, in the order they were started */
static ecmg_status batch_apply_all(ecmg_ctx* c, long long* failed)
{
    for (ecmg_ctx::PlanBatch* b; (b = oldest_batch(c)) != nullptr;) {
        ecmg_status s = batch_apply(c, *b, failed);
        if (s != ECMG_OK) return s;
    }
    return ECMG_OK;
}

/* stops the helper threads (the context is going away) */
static void batch_stop(ecmg_ctx* c)
{
    for (auto& b : c->batch) {
        if (!b.th.joinable()) continue;
        {
            std::lock_guard<std::mutex> l(b.mu);
            b.stop = true;
        }
        b.cv.notify_all();
        b.th.join();
        b.active = false;
    }
}

/* every re-plan in flight applied: before anything that reads or changes
   paths, agents, the scene or the planner between ticks */
static ecmg_status drain(ecmg_ctx* c)
{
    return c ? batch_apply_all(c, &c->batch_failed) : ECMG_OK;
}

static cudaError_t ensure_check_buffers(ecmg_ctx* c)
{
    if (c->h_cand) return cudaSuccess;
    cudaError_t e = cudaHostAlloc((void**)&c->h_cand, sizeof(V2) * kSpawnMaxCand, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&c->h_sarea, sizeof(SpawnAreaDev) * kSpawnMaxAreas, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&c->h_hit, sizeof(int) * kSpawnMaxCand, cudaHostAllocDefault);
    if (e == cudaSuccess) e = c->d_cand.alloc(kSpawnMaxCand);
    if (e == cudaSuccess) e = c->d_sarea.alloc(kSpawnMaxAreas);
    if (e == cudaSuccess) e = c->d_hit.alloc(kSpawnMaxCand);
    return e;
}

/* the candidate table in h_cand / h_sarea (na areas, nc candidates) against
   the active agents of the scene's slots: one launch, hits back in h_hit */
static ecmg_status check_candidates(ecmg_ctx* c, SceneState* sc, int na, size_t nc)
{
    CK(cudaMemcpyAsync(c->d_cand.p, c->h_cand, sizeof(V2) * nc, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_sarea.p, c->h_sarea, sizeof(SpawnAreaDev) * na, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(c->d_hit.p, 0, sizeof(int) * nc, c->stream));
    CK(launch_spawn_check(c->pos.p, c->d_active.p, sc->slot_base, sc->last_idx + 1, c->d_cand.p, c->d_sarea.p, na,
                          c->d_hit.p, c->sms, c->stream));
    CK(cudaMemcpyAsync(c->h_hit, c->d_hit.p, sizeof(int) * nc, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return ECMG_OK;
}

static void candidate_box(SpawnAreaDev& D, float x0, float y0, float x1, float y1, float cl, int first, int count);

/* Simulator::ValidSpawnLocation (Simulator.cpp:295-311): one candidate
   tested on the device (no copy of the agent state) */
static ecmg_status valid_spawn(ecmg_ctx* c, SceneState* sc, V2 loc, float clearance, bool* ok)
{
    *ok = true;
    if (sc->last_idx < sc->slot_base) return ECMG_OK;
    CK(ensure_check_buffers(c));
    c->h_cand[0] = loc;
    candidate_box(c->h_sarea[0], loc.x, loc.y, loc.x, loc.y, clearance, 0, 1);
    ecmg_status cs = check_candidates(c, sc, 1, 1);
    if (cs != ECMG_OK) return cs;
    *ok = c->h_hit[0] == 0;
    return ECMG_OK;
}

ecmg_status ecmg_spawn_agent(ecmg_ctx* c, float sx, float sy, float gx, float gy, float clearance, float pref_speed,
                             int* out_slot)
{
    if (!c || !out_slot) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    *out_slot = -1;
    SceneState* sc = c->scenes[0].get();
    if (!finite2(sx, sy) || !finite2(gx, gy) || !std::isfinite(clearance) || !std::isfinite(pref_speed))
        return fail(c, ECMG_ERR_INVALID_ARG, "non-finite spawn argument");
    if (sc->free_stack.empty()) return fail(c, ECMG_ERR_NO_SLOT, "no free slot");
    bool ok;
    ecmg_status st = valid_spawn(c, sc, mk(sx, sy), clearance, &ok);
    if (st != ECMG_OK) return st;
    if (!ok) return fail(c, ECMG_ERR_INVALID_SPAWN, "spawn location occupied");
    std::vector<V2> p;
    st = plan(c, sc, mk(sx, sy), mk(gx, gy), clearance, p, c->scratch);
    if (st != ECMG_OK || p.empty()) return fail(c, ECMG_ERR_NO_PATH, "no path from (%g,%g) to (%g,%g)", sx, sy, gx, gy);
    std::vector<float> xy(2 * p.size());
    for (size_t i = 0; i < p.size(); i++) { xy[2 * i] = p[i].x; xy[2 * i + 1] = p[i].y; }
    int off = 0, len = (int)p.size();
    float pos[2] = {sx, sy};
    return ecmg_scene_add_agents(c, 0, 1, pos, &clearance, &pref_speed, &off, &len, xy.data(), out_slot);
}

/* ---------------------------------------------------------------------- */
/* Spawn stage: Simulator::UpdateSpawnAreas (Simulator.cpp:494-536).

   The reference walks spawn areas in ID order and, per connected goal area,
   spawns n = (int)(timeSinceLastSpawn * rate) agents, each with up to 10
   random locations (3 random values per location, Area.h:39-53) tested by
   the O(N) ValidSpawnLocation; a valid location is followed by the goal's 3
   values.  Which values a location uses depends on how many earlier
   locations were rejected, but every location uses a whole triple of the
   stream, and a triple is either a candidate location in one of the stage's
   spawn areas or a goal.  So the stage tests triples t0..t0+w-1 as
   locations in each spawn area still due (w = 11 x the agents left, at most
   kSpawnMaxCand candidates) against the device-resident agents in one
   launch, then replays the reference's loop on the host, where the agents
   placed earlier in the same stage are checked directly.  A window that
   runs out is followed by another one (another launch). */

static int rq_at(ecmg_ctx* c, size_t i)
{
    while (c->rq.size() - c->rq_head <= i) c->rq.push_back(c->rng_fn ? c->rng_fn(c->rng_user) : std::rand());
    return c->rq[c->rq_head + i];
}

static void rq_consume(ecmg_ctx* c, size_t n)
{
    c->rq_head += n;
    if (c->rq_head > 4096 && 2 * c->rq_head > c->rq.size()) {
        c->rq.erase(c->rq.begin(), c->rq.begin() + (std::ptrdiff_t)c->rq_head);
        c->rq_head = 0;
    }
}

/* Area::GetRandomPositionInArea (Area.h:39-53) from the second and third
   value of a triple (the first feeds an unused variable), in the reference's
   float operations: x = xMin + v1 / ((float)RAND_MAX / (xMax - xMin)) */
static V2 area_point(float px, float py, float hw, float hh, int v1, int v2, int rand_max)
{
    const float xMin = px - hw, xMax = px + hw, yMin = py - hh, yMax = py + hh;
    const float rm = (float)rand_max;
    return mk(xMin + (float)v1 / (rm / (xMax - xMin)), yMin + (float)v2 / (rm / (yMax - yMin)));
}

/* int agentsToSpawn = time * rate (Simulator.cpp:505) as x86-64 converts:
   truncation toward zero, INT_MIN for NaN and out-of-range values */
static int spawn_count(float x)
{
    if (!(x > -2147483904.0f && x < 2147483648.0f)) return INT_MIN;
    return (int)x;
}

struct SpawnWindow {
    size_t t0 = 0, w = 0;                 /* triples [t0, t0 + w) */
    std::vector<const SpawnAreaH*> areas; /* candidate block a: locations in areas[a] */
    int find(const SpawnAreaH* a, size_t t) const
    {
        if (t < t0 || t >= t0 + w) return -1;
        for (size_t i = 0; i < areas.size(); i++)
            if (areas[i] == a) return (int)i;
        return -1;
    }
};

/* the window's candidates against the active agents of the scene's slots
   (one launch, one copy back) */
/* the box of an area's candidates, grown so that no agent the exact test
   would find lies outside: such an agent is within clearance * (1 + 2^-21)
   of a candidate on each axis; the margin covers that and the rounding of
   the box bounds */
static void candidate_box(SpawnAreaDev& D, float x0, float y0, float x1, float y1, float cl, int first, int count)
{
    const float big = std::fmax(std::fmax(std::fabs(x0), std::fabs(x1)), std::fmax(std::fabs(y0), std::fabs(y1)));
    const float m = std::fabs(cl) * 1.001f + 1e-3f + 1e-6f * (std::isfinite(big) ? big : 0.0f);
    D.x0 = x0 - m; D.y0 = y0 - m; D.x1 = x1 + m; D.y1 = y1 + m;
    D.c2 = cl * cl;
    D.first = first;
    D.count = count;
    D.pad = 0;
}

static ecmg_status spawn_check(ecmg_ctx* c, SceneState* sc, const SpawnWindow& win, ecmg_tick_stats& st)
{
    const auto h0 = std::chrono::steady_clock::now();
    CK(ensure_check_buffers(c));
    const int na = (int)win.areas.size(), w = (int)win.w;
    for (int a = 0; a < na; a++) {
        const SpawnAreaH& A = *win.areas[a];
        float x0 = INFINITY, y0 = INFINITY, x1 = -INFINITY, y1 = -INFINITY;
        for (int q = 0; q < w; q++) {
            const size_t t = win.t0 + (size_t)q;
            const V2 p = area_point(A.x, A.y, A.hw, A.hh, rq_at(c, 3 * t + 1), rq_at(c, 3 * t + 2), c->rand_max);
            c->h_cand[a * w + q] = p;
            x0 = std::fmin(x0, p.x); y0 = std::fmin(y0, p.y);
            x1 = std::fmax(x1, p.x); y1 = std::fmax(y1, p.y);
        }
        candidate_box(c->h_sarea[a], x0, y0, x1, y1, A.cfg.clearance_min, a * w, w);
    }
    const size_t nc = (size_t)na * (size_t)w;
    {
        ecmg_status cs = check_candidates(c, sc, na, nc);
        if (cs != ECMG_OK) return cs;
    }
    st.spawn_candidates += (long long)nc;
    st.spawn_kernels++;
    st.spawn_check_ms += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - h0).count();
    return ECMG_OK;
}

struct SpawnPair {
    SpawnAreaH* a;
    int ga, n;
};
struct SpawnPick {
    V2 start, goal;
    float clr, speed;
};

/* SpawnAgent (Simulator.cpp:168-200) for the agents a stage placed, in
   order: LIFO slots, components, zero velocities and the planned paths.  The
   device side is one copy of the new path points, one copy of per-agent
   records and one scatter kernel, queued ahead of the tick. */
static ecmg_status place_agents(ecmg_ctx* c, SceneState* sc, const std::vector<SpawnPick>& picks,
                                std::vector<std::vector<V2>>& paths)
{
    const int n = (int)picks.size();
    if (n == 0) return ECMG_OK;
    size_t total = 0;
    for (auto& p : paths) total += p.size();
    {
        ecmg_status rs = ensure_path_room(c, total);
        if (rs != ECMG_OK) return rs;
    }
    std::vector<SpawnRec> rec((size_t)n);
    std::vector<V2> pts;
    pts.reserve(total);
    for (int i = 0; i < n; i++) {
        const SpawnPick& p = picks[i];
        const int idx = sc->free_stack.back();
        sc->free_stack.pop_back();
        sc->num_agents++;
        c->num_agents++;
        sc->last_idx = std::max(sc->last_idx, idx);
        c->active[idx] = 1;
        c->clear[idx] = p.clr;
        c->speed[idx] = p.speed;
        c->fail_edge[idx] = -1;
        note_range(c, sc, p.clr, p.speed);
        rec[i] = SpawnRec{idx, p.start.x, p.start.y, p.clr, p.speed, (int)(c->path_used + pts.size()),
                          (int)paths[i].size(), 0};
        pts.insert(pts.end(), paths[i].begin(), paths[i].end());
        c->paths[idx].swap(paths[i]);
        c->spawned_slot.push_back(idx);
        c->spawned_start.push_back(p.start);
        c->spawned_goal.push_back(p.goal);
    }
    ecmg_status s = stage_copy(c, c->path_xy.p + c->path_used, pts.data(), sizeof(V2) * pts.size());
    if (s != ECMG_OK) return s;
    c->path_used += pts.size();
    CK(c->d_spawn_rec.alloc((size_t)n));
    s = stage_copy(c, c->d_spawn_rec.p, rec.data(), sizeof(SpawnRec) * rec.size());
    if (s != ECMG_OK) return s;
    SpawnTargets tg{c->pos.p, c->vel.p, c->pref_vel.p, c->d_clear.p, c->d_speed.p, c->d_active.p,
                    c->path_off.p, c->path_len.p, c->d_fail_edge.p};
    CK(launch_spawn_place(c->d_spawn_rec.p, n, tg, c->stream));
    if (sc->grid_agents == 0 || sc->num_agents > 2 * sc->grid_agents) {
        sc->grid_ready = false;
        c->table_dirty = true;
    }
    return ECMG_OK;
}

/* One replay of the reference's loop over the stage's agents.  Agents with a
   valid location and a free slot are placed unless the planner is known to
   fail for their (start, goal, clearance); their paths are planned after the
   walk (on several host threads), and a walk in which an unplanned agent then
   turns out to have no path is replayed with that knowledge -- an agent that
   is not placed frees its location for the ones after it. */
struct PlanKey {
    float sx, sy, gx, gy, c;
    bool operator<(const PlanKey& o) const
    {
        return std::tie(sx, sy, gx, gy, c) < std::tie(o.sx, o.sy, o.gx, o.gy, o.c);
    }
};

static ecmg_status spawn_walk(ecmg_ctx* c, SceneState* sc, const std::vector<SpawnPair>& pairs, long long total,
                              const std::map<PlanKey, std::vector<V2>>& planned, std::vector<SpawnPick>& picks,
                              size_t* triples, long long* failed, long long* refused, ecmg_tick_stats& st)
{
    picks.clear();
    *failed = *refused = 0;
    SpawnWindow win;
    std::vector<V2> placed; /* this stage's agents: tested on the host */
    long long left = total;
    size_t free_left = sc->free_stack.size();
    size_t t = 0; /* triples used so far */
    for (size_t pi = 0; pi < pairs.size(); pi++) {
        const SpawnPair& P = pairs[pi];
        const SpawnAreaH& A = *P.a;
        const float clr = A.cfg.clearance_min, speed = A.cfg.preferred_speed_min;
        const float c2 = clr * clr;
        for (int i = 0; i < P.n; i++, left--) {
            bool found = false;
            V2 start = mk(0.0f, 0.0f);
            for (int att = 0; att < 10 && !found; att++, t++) {
                int ai = win.find(&A, t);
                if (ai < 0) {
                    win.t0 = t;
                    win.areas.assign(1, &A);
                    for (size_t q = pi + 1; q < pairs.size() && (int)win.areas.size() < kSpawnMaxAreas; q++)
                        if (pairs[q].n > 0 &&
                            std::find(win.areas.begin(), win.areas.end(), pairs[q].a) == win.areas.end())
                            win.areas.push_back(pairs[q].a);
                    const long long cap = kSpawnMaxCand / (long long)win.areas.size();
                    win.w = (size_t)std::max(1LL, std::min(11 * left, cap));
                    ecmg_status cs = spawn_check(c, sc, win, st);
                    if (cs != ECMG_OK) return cs;
                    ai = 0;
                }
                const size_t j = (size_t)ai * win.w + (t - win.t0);
                start = c->h_cand[j];
                bool occupied = c->h_hit[j] != 0;
                for (size_t q = 0; q < placed.size() && !occupied; q++) {
                    const float dx = start.x - placed[q].x, dy = start.y - placed[q].y;
                    occupied = dx * dx + dy * dy < c2;
                }
                found = !occupied;
            }
            if (!found) { /* "Could not find a valid spawn position" */
                (*failed)++;
                continue;
            }
            /* the goal's triple; a goal area that no longer exists gives (0, 0)
               (the reference would default-construct one) */
            const int v1 = rq_at(c, 3 * t + 1), v2 = rq_at(c, 3 * t + 2);
            t++;
            auto git = sc->goal_areas.find(A.goals[P.ga]);
            const V2 goal = git != sc->goal_areas.end()
                                ? area_point(git->second.x, git->second.y, git->second.hw, git->second.hh, v1, v2,
                                             c->rand_max)
                                : mk(0.0f, 0.0f);
            if (free_left == 0) { /* SpawnAgent returns -1 (Simulator.cpp:170) */
                (*refused)++;
                continue;
            }
            auto it = planned.find(PlanKey{start.x, start.y, goal.x, goal.y, clr});
            if (it != planned.end() && it->second.empty()) { /* no path */
                (*refused)++;
                continue;
            }
            free_left--;
            placed.push_back(start);
            picks.push_back({start, goal, clr, speed});
        }
    }
    *triples = t;
    return ECMG_OK;
}

static ecmg_status spawn_stage(ecmg_ctx* c, ecmg_tick_stats& st)
{
    c->spawned_slot.clear();
    c->spawned_start.clear();
    c->spawned_goal.clear();
    for (auto& scp : c->scenes) {
        SceneState* sc = scp.get();
        if (sc->spawn_areas.empty()) continue;
        std::vector<SpawnPair> pairs;
        long long total = 0;
        for (auto& kv : sc->spawn_areas) {
            SpawnAreaH& A = kv.second;
            for (int ga = 0; ga < (int)A.goals.size(); ga++) {
                A.since[ga] += c->prm.dt;
                const int n = spawn_count(A.since[ga] * A.rate[ga]);
                pairs.push_back({&A, ga, n});
                if (n > 0) total += n;
            }
        }
        std::map<PlanKey, std::vector<V2>> planned; /* empty path: the planner failed */
        std::vector<SpawnPick> picks;
        size_t triples = 0;
        long long failed = 0, refused = 0;
        for (;;) {
            ecmg_status ws = spawn_walk(c, sc, pairs, total, planned, picks, &triples, &failed, &refused, st);
            if (ws != ECMG_OK) return ws;
            std::vector<int> todo;
            for (int i = 0; i < (int)picks.size(); i++)
                if (!planned.count(PlanKey{picks[i].start.x, picks[i].start.y, picks[i].goal.x, picks[i].goal.y,
                                           picks[i].clr}))
                    todo.push_back(i);
            if (todo.empty()) break;
            /* SpawnAgent's UpdatePath (Simulator.cpp:190); the built-in planner
               is re-entrant, a caller-supplied one runs on this thread */
            const int m = (int)todo.size();
            std::vector<std::vector<V2>> res(m);
            plan_jobs(c, m, [&](int q, PlanScratch& scr) {
                const SpawnPick& p = picks[todo[q]];
                if (plan(c, sc, p.start, p.goal, p.clr, res[q], scr) != ECMG_OK) res[q].clear();
            });
            bool replay = false;
            for (int q = 0; q < m; q++) {
                const SpawnPick& p = picks[todo[q]];
                if (res[q].empty()) replay = true;
                planned[PlanKey{p.start.x, p.start.y, p.goal.x, p.goal.y, p.clr}] = std::move(res[q]);
            }
            if (!replay) break;
        }
        std::vector<std::vector<V2>> paths(picks.size());
        for (size_t i = 0; i < picks.size(); i++) {
            const SpawnPick& p = picks[i];
            paths[i] = planned[PlanKey{p.start.x, p.start.y, p.goal.x, p.goal.y, p.clr}];
        }
        ecmg_status ps = place_agents(c, sc, picks, paths);
        if (ps != ECMG_OK) return ps;
        if (!picks.empty()) st.spawn_kernels++;
        st.spawned += (long long)picks.size();
        st.spawn_failed += failed;
        st.spawn_refused += refused;
        for (const SpawnPair& P : pairs) P.a->since[P.ga] -= (float)P.n / P.a->rate[P.ga];
        rq_consume(c, 3 * triples);
    }
    return ECMG_OK;
}

/* an area whose corners and extent are finite floats (its random locations
   are then finite too) */
static bool area_ok(float x, float y, float hw, float hh)
{
    const float x0 = x - hw, x1 = x + hw, y0 = y - hh, y1 = y + hh;
    return finite2(x, y) && finite2(hw, hh) && finite2(x0, x1) && finite2(y0, y1) && std::isfinite(x1 - x0) &&
           std::isfinite(y1 - y0);
}

ecmg_status ecmg_add_spawn_area(ecmg_ctx* c, float x, float y, float half_w, float half_h,
                                const ecmg_spawn_config* config, int id, int* out_id)
{
    if (!c || !out_id) return ECMG_ERR_INVALID_ARG;
    if (!area_ok(x, y, half_w, half_h)) return fail(c, ECMG_ERR_INVALID_ARG, "non-finite area");
    if (config && !(finite2(config->preferred_speed_min, config->preferred_speed_max) &&
                    finite2(config->clearance_min, config->clearance_max)))
        return fail(c, ECMG_ERR_INVALID_ARG, "non-finite spawn configuration");
    SceneState* sc = c->scenes[0].get();
    SpawnAreaH a;
    a.id = id == -1 ? sc->next_spawn_id++ : id;
    a.x = x; a.y = y; a.hw = half_w; a.hh = half_h;
    if (config) a.cfg = *config;
    sc->spawn_areas.emplace(a.id, a);
    *out_id = a.id;
    return ECMG_OK;
}

ecmg_status ecmg_add_goal_area(ecmg_ctx* c, float x, float y, float half_w, float half_h, int id, int* out_id)
{
    if (!c || !out_id) return ECMG_ERR_INVALID_ARG;
    if (!area_ok(x, y, half_w, half_h)) return fail(c, ECMG_ERR_INVALID_ARG, "non-finite area");
    SceneState* sc = c->scenes[0].get();
    GoalAreaH g;
    g.id = id == -1 ? sc->next_goal_id++ : id;
    g.x = x; g.y = y; g.hw = half_w; g.hh = half_h;
    sc->goal_areas.emplace(g.id, g);
    *out_id = g.id;
    return ECMG_OK;
}

ecmg_status ecmg_remove_area(ecmg_ctx* c, int type, int id)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    SceneState* sc = c->scenes[0].get();
    if (type == ECMG_AREA_SPAWN) sc->spawn_areas.erase(id);
    if (type == ECMG_AREA_GOAL) sc->goal_areas.erase(id);
    return ECMG_OK;
}

ecmg_status ecmg_connect_areas(ecmg_ctx* c, int spawn_id, int goal_id, float spawn_rate)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (!std::isfinite(spawn_rate)) return fail(c, ECMG_ERR_INVALID_ARG, "non-finite spawn rate");
    SceneState* sc = c->scenes[0].get();
    auto it = sc->spawn_areas.find(spawn_id);
    if (it == sc->spawn_areas.end()) return fail(c, ECMG_ERR_INVALID_ARG, "no spawn area %d", spawn_id);
    SpawnAreaH& a = it->second;
    for (int g : a.goals)
        if (g == goal_id) return ECMG_OK;
    a.goals.push_back(goal_id);
    a.since.push_back(0.0f);
    a.rate.push_back(spawn_rate);
    return ECMG_OK;
}

ecmg_status ecmg_disconnect_areas(ecmg_ctx* c, int spawn_id, int goal_id)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    SceneState* sc = c->scenes[0].get();
    if (spawn_id < 0 || spawn_id >= (int)sc->spawn_areas.size()) return ECMG_OK;
    auto it = sc->spawn_areas.find(spawn_id);
    if (it == sc->spawn_areas.end()) return ECMG_OK;
    std::vector<int>& g = it->second.goals;
    auto q = std::find(g.begin(), g.end(), goal_id);
    if (q != g.end()) g.erase(q); /* rates and timers keep their entries */
    return ECMG_OK;
}

ecmg_status ecmg_set_area(ecmg_ctx* c, int type, int id, float x, float y, float half_w, float half_h)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (!area_ok(x, y, half_w, half_h)) return fail(c, ECMG_ERR_INVALID_ARG, "non-finite area");
    SceneState* sc = c->scenes[0].get();
    if (type == ECMG_AREA_SPAWN) {
        auto it = sc->spawn_areas.find(id);
        if (it == sc->spawn_areas.end()) return fail(c, ECMG_ERR_INVALID_ARG, "no spawn area %d", id);
        it->second.x = x; it->second.y = y; it->second.hw = half_w; it->second.hh = half_h;
        return ECMG_OK;
    }
    if (type == ECMG_AREA_GOAL) {
        auto it = sc->goal_areas.find(id);
        if (it == sc->goal_areas.end()) return fail(c, ECMG_ERR_INVALID_ARG, "no goal area %d", id);
        it->second.x = x; it->second.y = y; it->second.hw = half_w; it->second.hh = half_h;
        return ECMG_OK;
    }
    return fail(c, ECMG_ERR_INVALID_ARG, "area type %d", type);
}

ecmg_status ecmg_get_area(ecmg_ctx* c, int type, int id, ecmg_area_info* out, int* goal_ids, float* rates,
                          float* since_last_spawn, int cap)
{
    if (!c || !out) return ECMG_ERR_INVALID_ARG;
    SceneState* sc = c->scenes[0].get();
    std::memset(out, 0, sizeof(*out));
    if (type == ECMG_AREA_SPAWN) {
        auto it = sc->spawn_areas.find(id);
        if (it == sc->spawn_areas.end()) return fail(c, ECMG_ERR_INVALID_ARG, "no spawn area %d", id);
        const SpawnAreaH& a = it->second;
        out->id = a.id; out->x = a.x; out->y = a.y; out->half_w = a.hw; out->half_h = a.hh;
        out->config = a.cfg;
        out->n_connected = (int)a.goals.size();
        out->n_timers = (int)a.rate.size();
        for (int i = 0; i < cap && i < (int)a.goals.size(); i++)
            if (goal_ids) goal_ids[i] = a.goals[i];
        for (int i = 0; i < cap && i < (int)a.rate.size(); i++) {
            if (rates) rates[i] = a.rate[i];
            if (since_last_spawn) since_last_spawn[i] = a.since[i];
        }
        return ECMG_OK;
    }
    if (type == ECMG_AREA_GOAL) {
        auto it = sc->goal_areas.find(id);
        if (it == sc->goal_areas.end()) return fail(c, ECMG_ERR_INVALID_ARG, "no goal area %d", id);
        const GoalAreaH& g = it->second;
        out->id = g.id; out->x = g.x; out->y = g.y; out->half_w = g.hw; out->half_h = g.hh;
        return ECMG_OK;
    }
    return fail(c, ECMG_ERR_INVALID_ARG, "area type %d", type);
}

ecmg_status ecmg_area_ids(ecmg_ctx* c, int type, int* ids, int cap, int* n)
{
    if (!c || !n || (cap > 0 && !ids)) return ECMG_ERR_INVALID_ARG;
    SceneState* sc = c->scenes[0].get();
    int k = 0;
    if (type == ECMG_AREA_SPAWN)
        for (auto& kv : sc->spawn_areas) { if (k < cap) ids[k] = kv.first; k++; }
    else if (type == ECMG_AREA_GOAL)
        for (auto& kv : sc->goal_areas) { if (k < cap) ids[k] = kv.first; k++; }
    else
        return fail(c, ECMG_ERR_INVALID_ARG, "area type %d", type);
    *n = k;
    return ECMG_OK;
}

ecmg_status ecmg_set_spawn_rng(ecmg_ctx* c, ecmg_rand_fn fn, void* user, int rand_max)
{
    if (!c || (fn && rand_max < 1)) return ECMG_ERR_INVALID_ARG;
    c->rng_fn = fn;
    c->rng_user = user;
    c->rand_max = fn ? rand_max : RAND_MAX;
    return ECMG_OK;
}

ecmg_status ecmg_push_spawn_random(ecmg_ctx* c, const int* values, int n)
{
    if (!c || n < 0 || (n > 0 && !values)) return ECMG_ERR_INVALID_ARG;
    c->rq.insert(c->rq.end(), values, values + n);
    return ECMG_OK;
}

ecmg_status ecmg_spawn_random_pending(const ecmg_ctx* c, long long* n)
{
    if (!c || !n) return ECMG_ERR_INVALID_ARG;
    *n = (long long)(c->rq.size() - c->rq_head);
    return ECMG_OK;
}

ecmg_status ecmg_update_spawn_areas(ecmg_ctx* c, ecmg_tick_stats* stats)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    ecmg_tick_stats st{};
    auto h0 = std::chrono::steady_clock::now();
    CK(cudaStreamSynchronize(c->stream));
    ecmg_status s = spawn_stage(c, st);
    st.spawn_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - h0).count();
    st.active_agents = c->num_agents;
    st.last_index = c->global_last();
    if (stats) *stats = st;
    return s;
}

ecmg_status ecmg_get_spawned(const ecmg_ctx* c, int* slots, float* start_xy, float* goal_xy, int cap, int* n)
{
    if (!c || !n || cap < 0) return ECMG_ERR_INVALID_ARG;
    const int m = (int)c->spawned_slot.size();
    for (int i = 0; i < m && i < cap; i++) {
        if (slots) slots[i] = c->spawned_slot[i];
        if (start_xy) { start_xy[2 * i] = c->spawned_start[i].x; start_xy[2 * i + 1] = c->spawned_start[i].y; }
        if (goal_xy) { goal_xy[2 * i] = c->spawned_goal[i].x; goal_xy[2 * i + 1] = c->spawned_goal[i].y; }
    }
    *n = m;
    return ECMG_OK;
}

ecmg_status ecmg_destroy_agent(ecmg_ctx* c, int slot)
{
    if (!c || slot < 0 || slot >= c->max_agents) return fail(c, ECMG_ERR_INVALID_ARG, "bad slot");
    DRAIN(c);
    if (!c->active[slot]) return fail(c, ECMG_ERR_INVALID_ARG, "slot %d is not active", slot);
    SceneState* sc = c->scenes[c->slot_scene[slot]].get();
    sc->num_agents--;
    c->num_agents--;
    c->active[slot] = 0;
    sc->free_stack.push_back(slot);
    unsigned char z = 0;
    CK(cudaMemcpy(c->d_active.p + slot, &z, 1, cudaMemcpyHostToDevice));
    return ECMG_OK;
}

ecmg_status ecmg_reset(ecmg_ctx* c)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    for (auto& scp : c->scenes) { /* Simulator.cpp:327-332 */
        SceneState* sc = scp.get();
        for (int i = sc->slot_base; i <= sc->last_idx; i++)
            if (c->active[i]) {
                sc->num_agents--;
                c->num_agents--;
                c->active[i] = 0;
                sc->free_stack.push_back(i);
            }
    }
    int last = c->global_last();
    if (last >= 0) CK(cudaMemset(c->d_active.p, 0, (size_t)last + 1));
    return ECMG_OK;
}

ecmg_status ecmg_set_path(ecmg_ctx* c, int slot, const float* xy, int n)
{
    if (!c || slot < 0 || slot >= c->max_agents || n < 1 || !xy) return fail(c, ECMG_ERR_INVALID_ARG, "bad path argument");
    DRAIN(c);
    for (int i = 0; i < n; i++)
        if (!finite2(xy[2 * i], xy[2 * i + 1])) return fail(c, ECMG_ERR_INVALID_ARG, "non-finite path point");
    c->paths[slot].assign((const V2*)xy, (const V2*)(xy + 2 * (size_t)n));
    return upload_path(c, slot);
}

ecmg_status ecmg_get_path(ecmg_ctx* c, int slot, float* out_xy, int cap, int* out_n)
{
    if (!c || slot < 0 || slot >= c->max_agents || !out_n) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    const auto& p = c->paths[slot];
    *out_n = (int)p.size();
    for (int i = 0; i < (int)p.size() && i < cap; i++) { out_xy[2 * i] = p[i].x; out_xy[2 * i + 1] = p[i].y; }
    return ECMG_OK;
}

/* ---------------------------------------------------------------------- */
static ecmg_status ensure_grids(ecmg_ctx* c)
{
    for (auto& scp : c->scenes) {
        SceneState* sc = scp.get();
        HostScene& s = sc->hs;
        if (sc->ob_dirty) {
            float reach = std::max(sc->ob_reach_needed, 1.0f) * 1.05f + 0.1f;
            build_obst_grid(s, reach, std::max(2.0f, std::min(reach, 8.0f)), sc->ob_grid);
            CK(sc->d_ob_gstart.alloc(sc->ob_grid.start.size()));
            CK(sc->d_ob_gitems.alloc(std::max<size_t>(1, sc->ob_grid.items.size())));
            CK(cudaMemcpy(sc->d_ob_gstart.p, sc->ob_grid.start.data(), sizeof(int) * sc->ob_grid.start.size(),
                          cudaMemcpyHostToDevice));
            if (!sc->ob_grid.items.empty())
                CK(cudaMemcpy(sc->d_ob_gitems.p, sc->ob_grid.items.data(), sizeof(int) * sc->ob_grid.items.size(),
                              cudaMemcpyHostToDevice));
            sc->ob_dirty = false;
            c->table_dirty = true;
        }
        if (!sc->grid_ready) {
            float w = std::max(1.0f, s.bx1 - s.bx0), h = std::max(1.0f, s.by1 - s.by0);
            float cell = c->prm.grid_cell;
            if (!(cell > 0.0f)) {
                float dens = (float)std::max(1, sc->num_agents) / (w * h);
                cell = std::sqrt((float)c->prm.max_neighbors / dens) * c->cell_scale;
                cell = std::min(std::max(cell, 0.3f), std::max(0.3f, c->prm.neighbor_dist));
            }
            while ((double)(w / cell + 3) * (double)(h / cell + 3) > 32.0e6) cell *= 1.5f; /* <= 32M cells */
            AgentGrid g;
            g.cell = cell;
            g.inv = 1.0f / cell;
            g.x0 = s.bx0 - cell;
            g.y0 = s.by0 - cell;
            g.gw = (int)std::ceil(w / cell) + 3;
            g.gh = (int)std::ceil(h / cell) + 3;
            g.ncells = g.gw * g.gh;
            sc->grid = g;
            sc->grid_ready = true;
            sc->grid_agents = std::max(1, sc->num_agents);
            c->table_dirty = true;
        }
    }
    if (c->table_dirty) {
        int base = 0;
        std::vector<SceneDev> tab(c->scenes.size());
        for (size_t i = 0; i < c->scenes.size(); i++) {
            SceneState* sc = c->scenes[i].get();
            HostScene& s = sc->hs;
            sc->bucket_base = base;
            base += sc->grid.ncells + 1;
            SceneDev& d = tab[i];
            d = SceneDev{};
            d.grid = sc->grid;
            d.bucket_base = sc->bucket_base;
            ObstView& o = d.ob;
            o.p = sc->d_ob_p.p;
            o.next = sc->d_ob_next.p;
            o.prev = sc->d_ob_prev.p;
            o.convex = sc->d_ob_convex.p;
            o.n_verts = sc->has_obst ? (int)s.ob_p.size() : 0;
            if (sc->ob_grid.gw > 0) {
                o.gx0 = sc->ob_grid.x0; o.gy0 = sc->ob_grid.y0; o.ginv = sc->ob_grid.inv;
                o.gw = sc->ob_grid.gw; o.gh = sc->ob_grid.gh; o.reach = sc->ob_grid.reach;
                o.g_start = sc->d_ob_gstart.p;
                o.g_items = sc->d_ob_gitems.p;
            }
            EcmView& e = d.ecm;
            e.v_pos = sc->d_v_pos.p;
            e.v_idx = sc->d_v_idx.p;
            e.he_target = sc->d_he_target.p;
            e.he_left = sc->d_he_left.p;
            e.he_right = sc->d_he_right.p;
            e.n_edges = (int)(s.he_target.size() / 2);
            e.gx0 = s.ecm_grid.x0; e.gy0 = s.ecm_grid.y0; e.ginv = s.ecm_grid.inv;
            e.gw = s.ecm_grid.gw; e.gh = s.ecm_grid.gh;
            e.g_start = sc->d_ecm_gstart.p;
            e.g_items = sc->d_ecm_gitems.p;
            e.special_y = sc->d_special_y.p;
            e.n_special = (int)s.special_y.size();
            e.sp_start = sc->d_sp_start.p;
            e.sp_items = sc->d_sp_items.p;
            e.sp_bloom = s.sp_bloom.empty() ? nullptr : sc->d_sp_bloom.p;
        }
        c->total_buckets = base;
        CK(c->d_scenes.alloc(tab.size()));
        CK(cudaMemcpy(c->d_scenes.p, tab.data(), sizeof(SceneDev) * tab.size(), cudaMemcpyHostToDevice));
        CK(c->cell_count.alloc((size_t)base + 2));
        CK(c->cell_start.alloc((size_t)base + 2));
        CK(c->scan_tmp.alloc((size_t)scan_tmp_ints(base)));
        c->table_dirty = false;
        c->graph_dirty = true;
    }
    if (c->model || c->trace) {
        size_t N = (size_t)c->max_agents;
        CK(c->feat.alloc(N * kMlpIn * 2));
        if (c->model) CK(c->cls.alloc(N));
        if (c->trace) CK(c->label.alloc(N));
    }
    if (c->record) {
        size_t N = (size_t)c->max_agents;
        int k = c->prm.max_neighbors;
        CK(c->rec_nbr.alloc(N * k)); CK(c->rec_cnt.alloc(N)); CK(c->rec_fail.alloc(N));
        CK(c->rec_ncons.alloc(N)); CK(c->rec_nobst.alloc(N)); CK(c->rec_vorca.alloc(N));
    }
    return ECMG_OK;
}

static void fill_args(ecmg_ctx* c, BinArgs& b, TickArgs& t, bool use_model)
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
    b.scenes = c->d_scenes.p;
    b.slot_scene = c->scenes.size() > 1 ? c->d_slot_scene.p : nullptr;
    b.total_buckets = c->total_buckets;

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
    t.nbr = c->nbr.p;
    t.ncnt = c->ncnt.p;
    t.slot_bucket = c->key.p;
    t.slot_rank = c->rank.p;
    t.scenes = c->d_scenes.p;
    t.slot_scene = b.slot_scene;
    t.tile = c->lp_mode == ECMG_LP_WARP ? c->wgrab : c->tile;
    t.lp_mode = c->lp_mode;
    t.occ_div = c->occ_div;
    t.knn_wide = c->knn_wide;
    const ecmg_params& p = c->prm;
    t.dt = p.dt;
    t.tau_a = p.tau_agent;
    {
        /* a power of two (normal, so that 1/tau is exact too) */
        int ex = 0;
        const float fr = std::frexp(p.tau_agent, &ex);
        t.inv_tau_a = (fr == 0.5f && ex > -125 && ex < 126) ? 1.0f / p.tau_agent : 0.0f;
    }
    t.tau_o = p.tau_obst;
    t.rnb = p.neighbor_dist;
    t.rnb2 = p.neighbor_dist * p.neighbor_dist;
    t.max_speed = p.max_speed;
    t.mass_recip = 1.0f / p.mass; /* Simulator.cpp:623 */
    t.arr_sq = p.arrival_radius * p.arrival_radius;
    t.del_sq = p.delete_radius * p.delete_radius;
    t.k = p.max_neighbors;
    t.lp3d_fp64 = p.lp3d_fp64;
    t.replan_dev_fail = c->plan_fn == nullptr ? 1 : 0;
    t.fail_edge = c->d_fail_edge.p;
    t.counters = c->counters.p;
    t.destroyed_list = c->destroyed_list.p;
    t.replan_list = c->replan_list.p;
    t.replan_pos = c->replan_pos.p;
    t.list_cap = c->max_agents;
    if (use_model || c->trace) t.feat = c->feat.p;
    if (use_model) t.cls = c->cls.p;
    t.cls_slot = c->cls_override;
    if (c->trace) t.label = c->label.p;
    if (c->record) {
        t.rec_nbr = c->rec_nbr.p;
        t.rec_cnt = c->rec_cnt.p;
        t.rec_vorca = c->rec_vorca.p;
        t.rec_fail = c->rec_fail.p;
        t.rec_ncons = c->rec_ncons.p;
        t.rec_nobst = c->rec_nobst.p;
    }
}

struct ProposeCall {
    ecmg_mlp* model;
    const void* feat;
    const int* n_dev;
    int n_max;
    unsigned char* cls;
    int sms;
    int* err;
};

static cudaError_t propose_cb(void* user, cudaStream_t s)
{
    const ProposeCall* pc = (const ProposeCall*)user;
    return mlp_infer(pc->model, pc->feat, pc->n_dev, pc->n_max, pc->cls, s, pc->sms, pc->err, ECMG_DEV_ERR_MLP);
}

/* after k_attract: the destroyed / re-plan lists are final; copy them and
   the counters back and mark the point, so that the host can start the
   re-plans while the neighbour and ORCA kernels run */
static cudaError_t after_attract_cb(void* user, cudaStream_t s, unsigned evflags)
{
    ecmg_ctx* c = (ecmg_ctx*)user;
    cudaError_t e = cudaMemcpyAsync(c->h_counters + 2 * kCounters, c->counters.p, sizeof(int) * kCounters,
                                    cudaMemcpyDeviceToHost, s);
    const size_t ls = (size_t)std::min(ecmg_ctx::kListStage, c->max_agents);
    int* hl = c->h_lists;
    if (e == cudaSuccess) e = cudaMemcpyAsync(hl, c->destroyed_list.p, sizeof(int) * ls, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hl + ecmg_ctx::kListStage, c->replan_list.p, sizeof(int) * ls, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(hl + 2 * ecmg_ctx::kListStage, c->replan_pos.p, sizeof(V2) * ls, cudaMemcpyDeviceToHost,
                            s);
    if (e == cudaSuccess) e = cudaEventRecordWithFlags(c->ev_mid, s, evflags);
    return e;
}

/* the device work of one tick: counters in, kernels, counters out */
static cudaError_t enqueue_tick(ecmg_ctx* c, int launch_slots, bool use_model)
{
    BinArgs b;
    TickArgs t;
    fill_args(c, b, t, use_model);
    cudaGetLastError(); /* launch errors below must not be confused with older ones */
    cudaError_t e = cudaMemcpyAsync(c->counters.p, c->h_counters, sizeof(int) * kCounters, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return e;
    if (c->trace) {
        e = cudaMemsetAsync(c->label.p, kClsOther, (size_t)launch_slots, c->stream);
        if (e != cudaSuccess) return e;
    }
    ProposeCall pc{c->model, c->feat.p, c->counters.p + C_NSORTED, launch_slots, c->cls.p, c->sms,
                   c->counters.p + C_ERROR};
    KdArgs kd{};
    if (c->nbr_mode == 1) {
        auto& K = c->kd;
        kd.max_slots = c->max_agents;
        kd.cap = c->max_agents;
        kd.k = c->prm.max_neighbors;
        kd.levels = K.levels;
        kd.tree_cap = K.tree_cap;
        kd.pos = c->pos.p;
        kd.s_slot = c->s_slot.p;
        kd.counters = c->counters.p;
        kd.active = c->d_active.p;
        kd.cell_start = c->cell_start.p;
        kd.slot_bucket = c->key.p;
        kd.slot_rank = c->rank.p;
        kd.mark = K.mark.p;
        kd.n_dev = K.n_dev.p;
        kd.iscan = K.iscan.p;
        kd.ids0 = K.ids0.p;
        kd.keys = K.keys.p;
        kd.ktmp = K.ktmp.p;
        kd.vtmp = K.vtmp.p;
        kd.X0 = K.X0.p;
        kd.X[0] = K.X[0].p; kd.X[1] = K.X[1].p;
        kd.Y[0] = K.Y[0].p; kd.Y[1] = K.Y[1].p;
        kd.seg_lo = K.seg_lo.p; kd.seg_hi = K.seg_hi.p; kd.seg_node = K.seg_node.p;
        kd.side = K.side.p;
        kd.flags = K.flags.p;
        kd.scan_tmp32 = K.scan_tmp32.p;
        kd.scan_tmp64 = K.scan_tmp64.p;
        kd.hist = K.hist.p;
        kd.tree = K.tree.p;
        kd.tree_pos = K.tree_pos.p;
        kd.map = K.map.p;
        kd.kfound = K.kfound.p;
        kd.agg = K.agg.p;
        kd.prev_in = K.prev_in.p;
        kd.cache = K.cache.p;
        kd.nbr = c->nbr.p;
        kd.ncnt = c->ncnt.p;
    }
    e = launch_tick(b, t, launch_slots, c->scan_tmp.p, c->block, c->sms, c->stream, c->stream2, c->ev_fork,
                    c->ev_join, c->ev_k,
                    use_model ? propose_cb : nullptr, &pc, after_attract_cb, c, c->nbr_mode == 1 ? &kd : nullptr);
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(c->h_counters + kCounters, c->counters.p, sizeof(int) * kCounters, cudaMemcpyDeviceToHost,
                           c->stream);
}

void* ecmg_stream(const ecmg_ctx* c) { return c ? (void*)c->stream : nullptr; }

int ecmg_kernels_per_tick(const ecmg_ctx* c)
{
    /* k_bin, k_scan_local, k_scan_top, k_scan_add, k_scatter, k_attract,
       k_neighbors, k_agents; k_features with a proposal model or a trace;
       k_mlp_infer with a proposal model */
    if (!c) return 8;
    int n = 8 + ((c->model || c->trace) ? 1 : 0) + (c->model ? 1 : 0);
    /* kd-tree mode, instead of k_neighbors: members and slot-order list (6),
       four radix sorts of four passes (84), segment init (1), level 0 (11),
       levels 1.. (side + partition), the query (2) and the composition (4) */
    if (c->nbr_mode == ECMG_NEIGHBORS_KDTREE) {
        const int L = c->kd.levels;
        n += -1 + 6 + 84 + 1 + 11 + (L - 1) + 5 * std::max(0, L - 2) + 2 + 4;
    } else if (c->lp_mode == ECMG_LP_THREAD_FUSED && !c->model && !c->trace) {
        n -= 1; /* the search runs inside the per-agent kernel */
    }
    return n;
}

static ecmg_status run_ticks(ecmg_ctx* c, int n_ticks, ecmg_tick_stats* stats)
{
    for (auto& scp : c->scenes)
        if (!scp->hs.has_ecm) return fail(c, ECMG_ERR_STATE, "every scene needs an ECM before ecmg_tick");
    ecmg_tick_stats st{};
    ecmg_status result = ECMG_OK;
    if (c->model) CK(mlp_pack(c->model)); /* BF16 fragments of the current weights */
    for (int tk = 0; tk < n_ticks; tk++) {
        auto hs = std::chrono::steady_clock::now();
        /* UpdateMaxAgentIndex (Simulator.cpp:481-492), per scene */
        for (auto& scp : c->scenes) {
            SceneState* sc = scp.get();
            while (sc->last_idx >= sc->slot_base && !c->active[sc->last_idx]) sc->last_idx--;
        }
        st.ticks++;
        bool spawning = false;
        for (auto& scp : c->scenes) spawning |= c->spawn_enabled && !scp->spawn_areas.empty();
        /* re-plans of the last tick still in flight: their agents are marked
           pending for this tick and stepped by k_fixup after it (the spawn
           stage needs the planner threads and the paths: apply them first) */
        if (oldest_batch(c) && (spawning || c->global_last() < 0)) {
            ecmg_status ds = batch_apply_all(c, &st.replans_failed);
            if (ds != ECMG_OK) return ds;
        }
        st.replans_failed += c->batch_failed;
        c->batch_failed = 0;
        if (c->spawn_enabled) { /* UpdateSpawnAreas (Simulator.cpp:317) */
            auto s0 = std::chrono::steady_clock::now();
            ecmg_status ss = spawn_stage(c, st);
            if (ss != ECMG_OK) return ss;
            st.spawn_ms += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - s0).count();
        }
        int last = c->global_last();
        if (last < 0) continue;
        ecmg_status gs = ensure_grids(c);
        if (gs != ECMG_OK) return gs;
        std::memset(c->h_counters, 0, sizeof(int) * kCounters);
        c->h_counters[C_LAST] = last;
        const bool use_model = c->model && c->gate_left == 0;
        if (c->model && !use_model) {
            c->gate_left--;
            st.gated++;
        }
        /* at most one batch is in flight here: the last tick's */
        ecmg_ctx::PlanBatch* carried = oldest_batch(c);
        const int npend = carried ? (int)carried->slot.size() : 0;
        if (npend > 0) {
            ecmg_status ps = stage_copy(c, c->d_pend.p, carried->slot.data(), sizeof(int) * (size_t)npend);
            if (ps != ECMG_OK) return ps;
            BinArgs bm;
            TickArgs tm;
            fill_args(c, bm, tm, use_model);
            CK(launch_mark_pending(tm, c->d_pend.p, npend, c->stream));
        }
        st.host_ms += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - hs).count();
        if (c->prm.use_graph) {
            /* a graph bakes in launch sizes covering slots [0, max_agents) */
            if (c->graph_dirty) {
                for (auto& g : c->graph)
                    if (g) cudaGraphExecDestroy(g);
                c->graph[0] = c->graph[1] = nullptr;
                c->graph_dirty = false;
            }
            cudaGraphExec_t& ge = c->graph[use_model ? 1 : 0];
            if (!ge) {
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                cudaError_t e = enqueue_tick(c, c->max_agents, use_model);
                cudaError_t e2 = cudaStreamEndCapture(c->stream, &g);
                if (e != cudaSuccess) return fail(c, ECMG_ERR_CUDA, "capture: %s", cudaGetErrorString(e));
                if (e2 != cudaSuccess) return fail(c, ECMG_ERR_CUDA, "end capture: %s", cudaGetErrorString(e2));
                CK(cudaGraphInstantiate(&ge, g, 0));
                cudaGraphDestroy(g);
                st.graph_builds++;
            }
            /* device time from here: a (re)capture is host time */
            CK(cudaEventRecord(c->ev_t0, c->stream));
            CK(cudaGraphLaunch(ge, c->stream));
        } else {
            CK(cudaEventRecord(c->ev_t0, c->stream));
            CK(enqueue_tick(c, last + 1, use_model));
        }
        CK(cudaEventRecord(c->ev_t1, c->stream));
        /* the lists of the attraction kernel are final after it: bookkeeping
           and re-plans run on the host while the rest of the tick runs on the
           device; path uploads are queued behind the tick */
        CK(cudaEventSynchronize(c->ev_mid));
        auto h0 = std::chrono::steady_clock::now();
        const int* mid = c->h_counters + 2 * kCounters;
        const int nd_mid = mid[C_DESTROYED], nr = mid[C_REPLAN];
        st.replans_host += nr;
        /* the destroys of a tick with a fix-up are known only after it */
        auto destroy = [&](int nd) -> ecmg_status {
            if (nd <= 0) return ECMG_OK;
            std::vector<int> d(std::min(nd, c->max_agents));
            if ((int)d.size() <= ecmg_ctx::kListStage && npend == 0)
                std::memcpy(d.data(), c->h_lists, sizeof(int) * d.size());
            else
                CK(cudaMemcpy(d.data(), c->destroyed_list.p, sizeof(int) * d.size(), cudaMemcpyDeviceToHost));
            std::sort(d.begin(), d.end()); /* DestroyAgent order: slot order of the loop */
            for (int s : d) {
                SceneState* sc = c->scenes[c->slot_scene[s]].get();
                sc->num_agents--;
                c->num_agents--;
                c->active[s] = 0;
                sc->free_stack.push_back(s);
            }
            return ECMG_OK;
        };
        if (npend == 0) {
            ecmg_status ds = destroy(nd_mid);
            if (ds != ECMG_OK) return ds;
        }
        /* the re-plan list [from, to) (ascending slots with their positions) */
        auto replans = [&](int from, int to, std::vector<int>& r, std::vector<V2>& rp) -> ecmg_status {
            to = std::min(to, c->max_agents);
            const int m = to - from;
            if (m <= 0) return ECMG_OK;
            std::vector<int> r0(m);
            std::vector<V2> p0(m);
            if (to <= ecmg_ctx::kListStage && from == 0) {
                std::memcpy(r0.data(), c->h_lists + ecmg_ctx::kListStage, sizeof(int) * m);
                std::memcpy(p0.data(), c->h_lists + 2 * ecmg_ctx::kListStage, sizeof(V2) * m);
            } else {
                CK(cudaMemcpy(r0.data(), c->replan_list.p + from, sizeof(int) * m, cudaMemcpyDeviceToHost));
                CK(cudaMemcpy(p0.data(), c->replan_pos.p + from, sizeof(V2) * m, cudaMemcpyDeviceToHost));
            }
            std::vector<int> order(m);
            for (int i = 0; i < m; i++) order[i] = i;
            std::sort(order.begin(), order.end(), [&](int x, int y) { return r0[x] < r0[y]; });
            r.resize(m);
            rp.resize(m);
            for (int i = 0; i < m; i++) {
                r[i] = r0[order[i]];
                rp[i] = p0[order[i]];
            }
            return ECMG_OK;
        };
        /* searches overlap the next tick when the built-in planner serves them
           and no spawn stage needs the planner threads first */
        const bool overlap = c->replan_overlap != 0 && !c->plan_fn && !spawning;
        if (nr > 0 && c->replan_enabled) {
            std::vector<int> r;
            std::vector<V2> rp;
            ecmg_status rs = replans(0, nr, r, rp);
            if (rs != ECMG_OK) return rs;
            if (overlap) {
                /* on the idle helper, beside the last tick's searches */
                batch_start(c, c->batch[0].active ? c->batch[1] : c->batch[0], r, rp);
            } else {
                rs = plan_now(c, r, rp, &st.replans_failed);
                if (rs != ECMG_OK) return rs;
            }
        }
        if (npend > 0) {
            /* the last tick's searches, their paths queued behind this tick's
               kernels, then the pending agents' step of this tick */
            ecmg_status bs = batch_apply(c, *carried, &st.replans_failed);
            if (bs != ECMG_OK) return bs;
            BinArgs bf;
            TickArgs tf;
            fill_args(c, bf, tf, use_model);
            CK(launch_fixup(tf, c->d_pend.p, npend, c->stream));
            CK(cudaMemcpyAsync(c->h_counters + kCounters, c->counters.p, sizeof(int) * kCounters,
                               cudaMemcpyDeviceToHost, c->stream));
        }
        /* the getters' host arrays: slots [0, last] are all this tick can
           have moved (spawns included); the copy runs while the host does
           the tick's bookkeeping */
        if (c->mirror && !c->mirror_stale)
            CK(launch_mirror(c->pos.p, c->vel.p, c->mirror_dev[0], c->mirror_dev[1], last + 1, c->sms, c->stream));
        st.host_ms += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - h0).count();
        CK(cudaStreamSynchronize(c->stream));
        c->h_up_used = 0; /* every queued upload has been applied */
        const int* fin = c->h_counters + kCounters;
        if (npend > 0) {
            /* the fix-up's destroys join the tick's; its re-plans (an agent whose
               new path already fails) are served now */
            ecmg_status ds = destroy(fin[C_DESTROYED]);
            if (ds != ECMG_OK) return ds;
            if (fin[C_REPLAN] > nr && c->replan_enabled) {
                std::vector<int> r;
                std::vector<V2> rp;
                ecmg_status rs = replans(nr, fin[C_REPLAN], r, rp);
                if (rs == ECMG_OK) rs = plan_now(c, r, rp, &st.replans_failed);
                if (rs != ECMG_OK) return rs;
                st.replans_host += fin[C_REPLAN] - nr;
                CK(cudaStreamSynchronize(c->stream));
                c->h_up_used = 0;
            }
        }
        st.destroyed += fin[C_DESTROYED];
        st.replans += fin[C_REPLAN] + fin[C_REPLAN_DEV];
        st.replans_failed += fin[C_REPLAN_DEV];
        /* searches that ended while the tick's kernels ran are applied now, as
           re-plans served inside the tick; the others overlap the next tick */
        if (ecmg_ctx::PlanBatch* nb = oldest_batch(c))
            if (nb->done.load() && c->replan_overlap != 2) {
                ecmg_status bs = batch_apply(c, *nb, &st.replans_failed);
                if (bs != ECMG_OK) return bs;
            }
        auto h1 = std::chrono::steady_clock::now();
        /* attraction and neighbour kernels run side by side: both are timed
           from their common start */
        float ms = 0, tot = 0, att = 0, nbr = 0, prop = 0, orca = 0;
        if (cudaEventElapsedTime(&ms, c->ev_t0, c->ev_t1) != cudaSuccess) ms = 0;
        if (cudaEventElapsedTime(&tot, c->ev_k[0], c->ev_k[4]) != cudaSuccess) tot = 0;
        if (cudaEventElapsedTime(&att, c->ev_k[0], c->ev_k[1]) != cudaSuccess) att = 0;
        if (cudaEventElapsedTime(&nbr, c->ev_k[0], c->ev_k[2]) != cudaSuccess) nbr = 0;
        if (cudaEventElapsedTime(&prop, c->ev_k[2], c->ev_k[3]) != cudaSuccess) prop = 0;
        if (cudaEventElapsedTime(&orca, c->ev_k[3], c->ev_k[4]) != cudaSuccess) orca = 0;
        cudaGetLastError();
        st.device_ms += ms;
        st.agent_kernel_ms += tot;
        st.attract_ms += att;
        st.neighbors_ms += nbr;
        st.proposal_ms += prop;
        st.orca_ms += orca;
        const int* out = c->h_counters + kCounters;
        st.agent_steps += out[C_NSORTED];
        st.lp3d += out[C_LP3D];
        st.proposed += out[C_PROPOSED];
        st.accepted += out[C_ACCEPTED];
        if (c->model && c->gate_min > 0.0f && out[C_NSORTED] > 0 && tot > 0.0f) {
            const float per = tot / (float)out[C_NSORTED];
            float& avg = use_model ? c->gate_t_model : c->gate_t_plain;
            avg = avg < 0.0f ? per : 0.5f * avg + 0.5f * per;
        }
        if (use_model && c->gate_min > 0.0f) {
            c->gate_model_ticks++;
            if ((float)out[C_ACCEPTED] < c->gate_min * (float)out[C_NSORTED])
                c->gate_left = c->gate_pause;
            else if (c->gate_t_plain < 0.0f && c->gate_model_ticks >= 3)
                c->gate_left = 3; /* measure the plain tick */
            else if (c->gate_t_plain > 0.0f && c->gate_model_ticks >= 2 && c->gate_t_model > 1.02f * c->gate_t_plain)
                c->gate_left = c->gate_pause;
            if (c->gate_left > 0) c->gate_model_ticks = 0;
        }
        c->trace_rows = out[C_NSORTED];
        if (out[C_ERROR]) {
            result = fail(c, ECMG_ERR_BOUND, "device bound exceeded (flags 0x%x): %s", out[C_ERROR],
                          (out[C_ERROR] & ECMG_DEV_ERR_CONSTRAINTS) ? "more than 24 obstacle half-planes for one agent"
                          : (out[C_ERROR] & ECMG_DEV_ERR_MLP)       ? "proposal network: a tensor-core wait timed out"
                                                                    : "event list overflow");
        }
        st.host_ms += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - h1).count();
    }
    st.active_agents = c->num_agents;
    st.last_index = c->global_last();
    if (stats) *stats = st;
    return result;
}

ecmg_status ecmg_tick(ecmg_ctx* c, int n_ticks, ecmg_tick_stats* stats)
{
    if (!c || n_ticks < 0) return ECMG_ERR_INVALID_ARG;
    return run_ticks(c, n_ticks, stats);
}

/* ---------------------------------------------------------------------- */
/* Autotuner: times whole ticks for each launch configuration on copies of
   the current state (the state is restored after every trial; trial ticks
   serve no re-plans) and keeps the fastest. */
ecmg_status ecmg_autotune(ecmg_ctx* c, int ticks_per_trial, ecmg_tune_result* out)
{
    if (!c || ticks_per_trial < 1) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    if (c->num_agents == 0) return fail(c, ECMG_ERR_STATE, "autotune needs agents");
    size_t N = (size_t)c->max_agents;
    DBuf<V2> sp, sv, sa, spv;
    DBuf<unsigned char> sact;
    CK(sp.alloc(N)); CK(sv.alloc(N)); CK(sa.alloc(N)); CK(spv.alloc(N)); CK(sact.alloc(N));
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(sp.p, c->pos.p, sizeof(V2) * N, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(sv.p, c->vel.p, sizeof(V2) * N, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(sa.p, c->attr.p, sizeof(V2) * N, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(spv.p, c->pref_vel.p, sizeof(V2) * N, cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(sact.p, c->d_active.p, N, cudaMemcpyDeviceToDevice));
    /* kd-tree mode: the neighbour cache the next tick starts from */
    std::vector<int> kd_cache;
    if (c->nbr_mode == ECMG_NEIGHBORS_KDTREE) {
        kd_cache.resize((size_t)c->prm.max_neighbors);
        CK(cudaMemcpy(kd_cache.data(), c->kd.cache.p, sizeof(int) * kd_cache.size(), cudaMemcpyDeviceToHost));
    }
    std::vector<unsigned char> act = c->active;
    std::vector<std::vector<int>> stacks;
    std::vector<int> nums, lasts;
    for (auto& s : c->scenes) { stacks.push_back(s->free_stack); nums.push_back(s->num_agents); lasts.push_back(s->last_idx); }
    int num = c->num_agents;
    auto restore = [&]() -> ecmg_status {
        CK(cudaMemcpy(c->pos.p, sp.p, sizeof(V2) * N, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(c->vel.p, sv.p, sizeof(V2) * N, cudaMemcpyDeviceToDevice));
        c->mirror_stale = true;
        CK(cudaMemcpy(c->attr.p, sa.p, sizeof(V2) * N, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(c->pref_vel.p, spv.p, sizeof(V2) * N, cudaMemcpyDeviceToDevice));
        CK(cudaMemcpy(c->d_active.p, sact.p, N, cudaMemcpyDeviceToDevice));
        if (!kd_cache.empty())
            CK(cudaMemcpy(c->kd.cache.p, kd_cache.data(), sizeof(int) * kd_cache.size(), cudaMemcpyHostToDevice));
        c->active = act;
        for (size_t i = 0; i < c->scenes.size(); i++) {
            c->scenes[i]->free_stack = stacks[i];
            c->scenes[i]->num_agents = nums[i];
            c->scenes[i]->last_idx = lasts[i];
        }
        c->num_agents = num;
        return ECMG_OK;
    };
    struct Launch {
        float scale;
        int mode, block, tile, occ_div, wgrab, knn_wide;
    };
    Launch bestL{c->cell_scale, c->lp_mode, c->block, c->tile, c->occ_div, c->wgrab, c->knn_wide};
    float best = 1e30f;
    int trials = 0;
    c->replan_enabled = false;
    c->spawn_enabled = false;
    auto trial = [&](const Launch& L, bool* better) -> ecmg_status {
        if (L.scale != c->cell_scale) {
            c->cell_scale = L.scale;
            for (auto& s : c->scenes) s->grid_ready = false;
        }
        c->lp_mode = L.mode;
        c->block = L.block;
        c->tile = L.tile;
        c->occ_div = L.occ_div;
        c->wgrab = L.wgrab;
        c->knn_wide = L.knn_wide;
        c->graph_dirty = true;
        ecmg_tick_stats ts{};
        ecmg_status st = run_ticks(c, 1, &ts); /* warm-up and graph capture */
        if (st == ECMG_OK) st = run_ticks(c, ticks_per_trial, &ts);
        ecmg_status rs = restore();
        if (st != ECMG_OK) return st;
        if (rs != ECMG_OK) return rs;
        trials++;
        const float ms = ts.device_ms / (float)ticks_per_trial;
        *better = ms < best;
        if (*better) {
            best = ms;
            bestL = L;
        }
        return ECMG_OK;
    };
    /* stage 1: the agent-grid cell (mostly the neighbour search), default
       launch; stage 2: the per-agent kernel's launch at the best cell */
    const float scales[] = {0.2f, 0.25f, 0.3f, 0.4f, 0.5f, 0.6f, 0.8f};
    const int blocks[] = {64, 128, 256};
    const int tiles[] = {32, 64, 128};
    const int divs[] = {1, 2, 3};
    const int wgrabs[] = {1, 2, 4, 8};
    const bool fixed_cell = c->prm.grid_cell > 0.0f;
    const int def_block = c->prm.block_size ? c->prm.block_size : 128;
    bool better = false;
    ecmg_status st = ECMG_OK;
    for (float sc : scales) {
        if (fixed_cell && sc != scales[0]) break;
        for (int kw = 0; kw < 2 && st == ECMG_OK; kw++)
            st = trial(Launch{sc, 0, def_block, 32, 1, c->wgrab, kw}, &better);
        if (st != ECMG_OK) break;
    }
    const float cell = bestL.scale;
    const int kw = bestL.knn_wide;
    for (int b : blocks) {
        if (st != ECMG_OK) break;
        if (c->prm.block_size && b != c->prm.block_size) continue;
        for (int tl : tiles)
            for (int dv : divs) {
                if (st != ECMG_OK) break;
                st = trial(Launch{cell, 0, b, tl, dv, c->wgrab, kw}, &better);
            }
    }
    /* the per-thread layout fused with the neighbour search, at the best
       per-thread launch (the kd-tree mode builds its lists separately) */
    const Launch thr = bestL;
    for (int dv : divs) {
        if (st != ECMG_OK || c->nbr_mode == ECMG_NEIGHBORS_KDTREE) break;
        st = trial(Launch{cell, ECMG_LP_THREAD_FUSED, thr.block, thr.tile, dv, c->wgrab, kw}, &better);
    }
    for (int w : wgrabs) {
        if (st != ECMG_OK || c->nbr_mode == ECMG_NEIGHBORS_KDTREE) break; /* one thread per agent there */
        st = trial(Launch{cell, 1, thr.block, thr.tile, 1, w, kw}, &better);
    }
    if (st != ECMG_OK) {
        c->replan_enabled = true;
        c->spawn_enabled = true;
        return st;
    }
    int bb = bestL.block, bt = bestL.tile, bmode = bestL.mode, bw = bestL.wgrab;
    float bs = bestL.scale;
    c->occ_div = bestL.occ_div;
    c->replan_enabled = true;
    c->spawn_enabled = true;
    c->block = bb;
    c->tile = bt;
    c->lp_mode = bmode;
    c->wgrab = bw;
    c->cell_scale = bs;
    c->knn_wide = bestL.knn_wide;
    for (auto& s : c->scenes) s->grid_ready = false;
    c->graph_dirty = true;
    sp.free_(); sv.free_(); sa.free_(); spv.free_(); sact.free_();
    if (out) {
        out->block_size = bb;
        out->agents_per_warp_grab = bmode == ECMG_LP_WARP ? bw : bt;
        out->lp_mode = bmode;
        out->grid_cell_scale = bs;
        out->best_tick_ms = best;
        out->trials = trials;
        out->occupancy_divisor = bestL.occ_div;
        out->neighbor_blocks_per_sm = bestL.knn_wide ? 6 : 8;
    }
    return ECMG_OK;
}

ecmg_status ecmg_set_neighbor_mode(ecmg_ctx* c, int mode)
{
    if (!c || (mode != ECMG_NEIGHBORS_EXACT && mode != ECMG_NEIGHBORS_KDTREE)) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    if (mode == c->nbr_mode) return ECMG_OK;
    if (mode == ECMG_NEIGHBORS_KDTREE) {
        if (c->model || c->trace || c->cls_override)
            return fail(c, ECMG_ERR_STATE, "the kd-tree neighbour mode runs without the learned proposal and trace");
        if (c->scenes.size() != 1)
            return fail(c, ECMG_ERR_STATE, "the kd-tree neighbour mode needs a single-scene context (one tree, one cache)");
        if (c->max_agents > (1 << 24)) return fail(c, ECMG_ERR_BOUND, "the kd-tree neighbour mode supports 2^24 slots");
        const size_t N = (size_t)c->max_agents;
        const int k = c->prm.max_neighbors;
        auto& K = c->kd;
        K.levels = 32 - __builtin_clz((unsigned)c->max_agents); /* depth 0 .. bit length - 1 */
        K.tree_cap = (int)((1u << K.levels) - 1u);
        const int hist = kd_hist_ints(c->max_agents);
        CK(K.mark.alloc(N)); CK(K.side.alloc(N));
        CK(K.n_dev.alloc(2)); CK(K.iscan.alloc(N)); CK(K.ids0.alloc(N)); CK(K.vtmp.alloc(N)); CK(K.X0.alloc(N));
        CK(K.X[0].alloc(N)); CK(K.X[1].alloc(N)); CK(K.Y[0].alloc(N)); CK(K.Y[1].alloc(N));
        CK(K.seg_lo.alloc(N)); CK(K.seg_hi.alloc(N)); CK(K.seg_node.alloc(N));
        CK(K.scan_tmp32.alloc((size_t)kd_scan_tmp(std::max<int>(c->max_agents, hist))));
        CK(K.scan_tmp64.alloc((size_t)kd_scan_tmp(c->max_agents)));
        CK(K.hist.alloc((size_t)hist)); CK(K.tree.alloc((size_t)K.tree_cap));
        CK(K.tree_pos.alloc((size_t)K.tree_cap));
        CK(K.map.alloc(N * (size_t)k)); CK(K.kfound.alloc(N));
        CK(K.agg.alloc((size_t)kd_compose_blocks(c->max_agents) * k));
        CK(K.prev_in.alloc((size_t)kd_compose_blocks(c->max_agents) * k));
        CK(K.cache.alloc((size_t)k));
        CK(K.keys.alloc(N)); CK(K.ktmp.alloc(N)); CK(K.flags.alloc(N));
        /* ORCA::m_NeighborCache starts as std::vector<Entity>(k): zeros */
        CK(cudaMemset(K.cache.p, 0, sizeof(int) * (size_t)k));
        c->lp_mode = ECMG_LP_THREAD;
    } else {
        c->kd.free_all();
    }
    c->nbr_mode = mode;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_set_lp_mode(ecmg_ctx* c, int mode, int agents_per_warp_grab)
{
    if (!c || (mode != ECMG_LP_THREAD && mode != ECMG_LP_WARP && mode != ECMG_LP_THREAD_FUSED))
        return ECMG_ERR_INVALID_ARG;
    if (mode == ECMG_LP_WARP && c->nbr_mode == ECMG_NEIGHBORS_KDTREE)
        return fail(c, ECMG_ERR_STATE, "the kd-tree neighbour mode runs one thread per agent");
    if (mode == ECMG_LP_WARP && (agents_per_warp_grab < 1 || agents_per_warp_grab > 64)) return ECMG_ERR_INVALID_ARG;
    c->lp_mode = mode;
    if (mode == ECMG_LP_WARP) c->wgrab = agents_per_warp_grab;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_set_occupancy(ecmg_ctx* c, int divisor)
{
    if (!c || divisor < 1 || divisor > 8) return ECMG_ERR_INVALID_ARG;
    c->occ_div = divisor;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_set_neighbor_blocks(ecmg_ctx* c, int blocks_per_sm)
{
    if (!c || (blocks_per_sm != 8 && blocks_per_sm != 6)) return ECMG_ERR_INVALID_ARG;
    const int w = blocks_per_sm == 6 ? 1 : 0;
    if (w != c->knn_wide) {
        c->knn_wide = w;
        c->graph_dirty = true;
    }
    return ECMG_OK;
}

ecmg_status ecmg_set_launch(ecmg_ctx* c, int block_size, int agents_per_warp_grab, float grid_cell_scale)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (block_size != 64 && block_size != 128 && block_size != 256) return fail(c, ECMG_ERR_INVALID_ARG, "block size");
    if (agents_per_warp_grab < 32 || agents_per_warp_grab % 32 || agents_per_warp_grab > 1024)
        return fail(c, ECMG_ERR_INVALID_ARG, "agents per warp grab must be a multiple of 32 in [32, 1024]");
    if (!(grid_cell_scale > 0.0f) || !std::isfinite(grid_cell_scale)) return fail(c, ECMG_ERR_INVALID_ARG, "grid scale");
    c->block = block_size;
    c->tile = agents_per_warp_grab;
    if (grid_cell_scale != c->cell_scale) {
        c->cell_scale = grid_cell_scale;
        for (auto& s : c->scenes) s->grid_ready = false;
    }
    c->graph_dirty = true;
    return ECMG_OK;
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

ecmg_status ecmg_host_view(ecmg_ctx* c, int field, const void** out)
{
    if (!c || !out) return ECMG_ERR_INVALID_ARG;
    size_t N = (size_t)c->max_agents;
    switch (field) {
    case ECMG_FIELD_CLEARANCE: *out = c->clear.data(); return ECMG_OK;
    case ECMG_FIELD_SPEED: *out = c->speed.data(); return ECMG_OK;
    case ECMG_FIELD_ACTIVE: *out = c->active.data(); return ECMG_OK;
    case ECMG_FIELD_POSITION:
    case ECMG_FIELD_VELOCITY:
    case ECMG_FIELD_PREF_VELOCITY:
    case ECMG_FIELD_ATTRACTION: {
        if (c->mirror && field <= ECMG_FIELD_VELOCITY) {
            /* kept by the ticks; refreshed here after any other write */
            if (c->mirror_stale) {
                CK(cudaMemcpyAsync(c->hview[0], c->pos.p, sizeof(V2) * N, cudaMemcpyDeviceToHost, c->stream));
                CK(cudaMemcpyAsync(c->hview[1], c->vel.p, sizeof(V2) * N, cudaMemcpyDeviceToHost, c->stream));
                CK(cudaStreamSynchronize(c->stream));
                c->mirror_stale = false;
            }
            *out = c->hview[field];
            return ECMG_OK;
        }
        void*& h = c->hview[field];
        if (!h) CK(cudaHostAlloc(&h, sizeof(V2) * N, cudaHostAllocMapped));
        const V2* src = field == ECMG_FIELD_POSITION ? c->pos.p
                        : field == ECMG_FIELD_VELOCITY ? c->vel.p
                        : field == ECMG_FIELD_PREF_VELOCITY ? c->pref_vel.p : c->attr.p;
        CK(cudaMemcpyAsync(h, src, sizeof(V2) * N, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        *out = h;
        return ECMG_OK;
    }
    default: return fail(c, ECMG_ERR_INVALID_ARG, "unknown field %d", field);
    }
}

ecmg_status ecmg_set_host_mirror(ecmg_ctx* c, int on)
{
    if (!c || (on != 0 && on != 1)) return ECMG_ERR_INVALID_ARG;
    if ((on != 0) == c->mirror) return ECMG_OK;
    CK(cudaStreamSynchronize(c->stream));
    if (on) {
        const size_t N = (size_t)c->max_agents;
        for (int f = 0; f < 2; f++) {
            if (!c->hview[f]) CK(cudaHostAlloc(&c->hview[f], sizeof(V2) * N, cudaHostAllocMapped));
            void* d = nullptr;
            CK(cudaHostGetDevicePointer(&d, c->hview[f], 0));
            c->mirror_dev[f] = (V2*)d;
        }
    }
    c->mirror = on != 0;
    c->mirror_stale = true; /* the copy after the tick, outside the graph: no recapture */
    return ECMG_OK;
}

ecmg_status ecmg_set_state(ecmg_ctx* c, int field, const void* src)
{
    if (!c || !src) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    size_t N = (size_t)c->max_agents;
    CK(cudaStreamSynchronize(c->stream));
    switch (field) {
    case ECMG_FIELD_POSITION:
        CK(cudaMemcpy(c->pos.p, src, sizeof(V2) * N, cudaMemcpyHostToDevice));
        c->mirror_stale = true;
        break;
    case ECMG_FIELD_VELOCITY:
        CK(cudaMemcpy(c->vel.p, src, sizeof(V2) * N, cudaMemcpyHostToDevice));
        c->mirror_stale = true;
        break;
    case ECMG_FIELD_PREF_VELOCITY: CK(cudaMemcpy(c->pref_vel.p, src, sizeof(V2) * N, cudaMemcpyHostToDevice)); break;
    case ECMG_FIELD_ATTRACTION: CK(cudaMemcpy(c->attr.p, src, sizeof(V2) * N, cudaMemcpyHostToDevice)); break;
    case ECMG_FIELD_CLEARANCE:
        std::memcpy(c->clear.data(), src, sizeof(float) * N);
        CK(cudaMemcpy(c->d_clear.p, src, sizeof(float) * N, cudaMemcpyHostToDevice));
        /* remembered failed searches were for the old clearances */
        std::fill(c->fail_edge.begin(), c->fail_edge.end(), -1);
        CK(cudaMemset(c->d_fail_edge.p, 0xff, sizeof(int) * N));
        for (size_t i = 0; i < N; i++)
            if (c->active[i]) note_range(c, c->scenes[c->slot_scene[i]].get(), c->clear[i], c->speed[i]);
        break;
    case ECMG_FIELD_SPEED:
        std::memcpy(c->speed.data(), src, sizeof(float) * N);
        CK(cudaMemcpy(c->d_speed.p, src, sizeof(float) * N, cudaMemcpyHostToDevice));
        for (size_t i = 0; i < N; i++)
            if (c->active[i]) note_range(c, c->scenes[c->slot_scene[i]].get(), c->clear[i], c->speed[i]);
        break;
    default: return fail(c, ECMG_ERR_INVALID_ARG, "field %d cannot be set", field);
    }
    return ECMG_OK;
}

/* ---------------------------------------------------------------------- */
/* Checkpoint / resume: a binary snapshot of everything a tick depends on.
   Layout: "ECMGSNAP", version, sizes, then the sections in a fixed order
   (device state as slot arrays, host mirrors, paths, per-scene bookkeeping
   and areas, queued random values, neighbour cache, failed-search memo). */
}  /* extern "C" */
namespace {
struct SnapWriter {
    FILE* f;
    bool ok = true;
    template <class T>
    void put(const T& v) { ok = ok && fwrite(&v, sizeof(T), 1, f) == 1; }
    template <class T>
    void arr(const T* p, size_t n)
    {
        put<unsigned long long>(n);
        if (n) ok = ok && fwrite(p, sizeof(T), n, f) == n;
    }
};
struct SnapReader {
    FILE* f;
    bool ok = true;
    template <class T>
    void get(T& v) { ok = ok && fread(&v, sizeof(T), 1, f) == 1; }
    template <class T>
    void arr(std::vector<T>& v, size_t expect = (size_t)-1)
    {
        unsigned long long n = 0;
        get(n);
        if (!ok || (expect != (size_t)-1 && n != expect) || n > (1ull << 34)) { ok = false; return; }
        v.resize((size_t)n);
        if (n) ok = ok && fread(v.data(), sizeof(T), (size_t)n, f) == n;
    }
};
constexpr unsigned kSnapVersion = 1;
}  // namespace
extern "C" {

ecmg_status ecmg_save_state(ecmg_ctx* c, const char* path)
{
    if (!c || !path) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    CK(cudaStreamSynchronize(c->stream));
    const size_t N = (size_t)c->max_agents;
    std::vector<V2> pos(N), vel(N), attr(N), pv(N);
    CK(cudaMemcpy(pos.data(), c->pos.p, sizeof(V2) * N, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(vel.data(), c->vel.p, sizeof(V2) * N, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(attr.data(), c->attr.p, sizeof(V2) * N, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(pv.data(), c->pref_vel.p, sizeof(V2) * N, cudaMemcpyDeviceToHost));
    std::vector<int> kd_cache;
    if (c->nbr_mode == ECMG_NEIGHBORS_KDTREE) {
        kd_cache.resize((size_t)c->prm.max_neighbors);
        CK(cudaMemcpy(kd_cache.data(), c->kd.cache.p, sizeof(int) * kd_cache.size(), cudaMemcpyDeviceToHost));
    }
    FILE* f = fopen(path, "wb");
    if (!f) return fail(c, ECMG_ERR_INVALID_ARG, "cannot write %s", path);
    SnapWriter w{f};
    fwrite("ECMGSNAP", 1, 8, f);
    w.put(kSnapVersion);
    w.put(c->max_agents);
    w.put((int)c->scenes.size());
    w.put(c->prm.max_neighbors);
    w.put(c->nbr_mode);
    w.put(c->num_agents);
    w.arr(pos.data(), N);
    w.arr(vel.data(), N);
    w.arr(attr.data(), N);
    w.arr(pv.data(), N);
    w.arr(c->clear.data(), N);
    w.arr(c->speed.data(), N);
    w.arr(c->active.data(), N);
    w.arr(c->fail_edge.data(), N);
    std::vector<int> plen(N);
    size_t total = 0;
    for (size_t i = 0; i < N; i++) {
        plen[i] = (int)c->paths[i].size();
        total += c->paths[i].size();
    }
    std::vector<V2> pts;
    pts.reserve(total);
    for (size_t i = 0; i < N; i++) pts.insert(pts.end(), c->paths[i].begin(), c->paths[i].end());
    w.arr(plen.data(), N);
    w.arr(pts.data(), pts.size());
    for (auto& scp : c->scenes) {
        const SceneState* sc = scp.get();
        w.put(sc->num_agents);
        w.put(sc->last_idx);
        w.arr(sc->free_stack.data(), sc->free_stack.size());
        w.put(sc->next_spawn_id);
        w.put(sc->next_goal_id);
        w.put((int)sc->spawn_areas.size());
        for (auto& kv : sc->spawn_areas) {
            const SpawnAreaH& a = kv.second;
            w.put(a.id); w.put(a.x); w.put(a.y); w.put(a.hw); w.put(a.hh); w.put(a.cfg);
            w.arr(a.goals.data(), a.goals.size());
            w.arr(a.rate.data(), a.rate.size());
            w.arr(a.since.data(), a.since.size());
        }
        w.put((int)sc->goal_areas.size());
        for (auto& kv : sc->goal_areas) {
            const GoalAreaH& g = kv.second;
            w.put(g.id); w.put(g.x); w.put(g.y); w.put(g.hw); w.put(g.hh);
        }
    }
    w.arr(c->rq.data() + c->rq_head, c->rq.size() - c->rq_head);
    w.put(c->rand_max);
    w.arr(kd_cache.data(), kd_cache.size());
    const bool ok = w.ok && fclose(f) == 0;
    if (!ok) return fail(c, ECMG_ERR_INVALID_ARG, "writing %s failed", path);
    return ECMG_OK;
}

ecmg_status ecmg_load_state(ecmg_ctx* c, const char* path)
{
    if (!c || !path) return ECMG_ERR_INVALID_ARG;
    DRAIN(c);
    FILE* f = fopen(path, "rb");
    if (!f) return fail(c, ECMG_ERR_INVALID_ARG, "cannot read %s", path);
    SnapReader r{f};
    char magic[8] = {};
    r.ok = fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "ECMGSNAP", 8) == 0;
    unsigned ver = 0;
    int n_slots = 0, n_scenes = 0, k = 0, mode = 0, num = 0;
    r.get(ver); r.get(n_slots); r.get(n_scenes); r.get(k); r.get(mode); r.get(num);
    if (!r.ok || ver != kSnapVersion || n_slots != c->max_agents || n_scenes != (int)c->scenes.size() ||
        k != c->prm.max_neighbors) {
        fclose(f);
        return fail(c, ECMG_ERR_INVALID_ARG, "%s is not a snapshot of a context like this one", path);
    }
    const size_t N = (size_t)c->max_agents;
    std::vector<V2> pos, vel, attr, pv, pts;
    std::vector<float> clear, speed;
    std::vector<unsigned char> active;
    std::vector<int> fe, plen;
    r.arr(pos, N); r.arr(vel, N); r.arr(attr, N); r.arr(pv, N);
    r.arr(clear, N); r.arr(speed, N); r.arr(active, N); r.arr(fe, N);
    r.arr(plen, N); r.arr(pts);
    struct SceneSnap {
        int num, last, next_spawn, next_goal;
        std::vector<int> free_stack;
        std::map<int, SpawnAreaH> spawn;
        std::map<int, GoalAreaH> goal;
    };
    std::vector<SceneSnap> ss((size_t)n_scenes);
    for (auto& q : ss) {
        r.get(q.num); r.get(q.last);
        r.arr(q.free_stack);
        r.get(q.next_spawn); r.get(q.next_goal);
        int ns = 0;
        r.get(ns);
        for (int i = 0; r.ok && i < ns; i++) {
            SpawnAreaH a;
            r.get(a.id); r.get(a.x); r.get(a.y); r.get(a.hw); r.get(a.hh); r.get(a.cfg);
            r.arr(a.goals); r.arr(a.rate); r.arr(a.since);
            if (a.rate.size() != a.since.size() || a.goals.size() > a.rate.size()) r.ok = false;
            q.spawn.emplace(a.id, a);
        }
        int ng = 0;
        r.get(ng);
        for (int i = 0; r.ok && i < ng; i++) {
            GoalAreaH g;
            r.get(g.id); r.get(g.x); r.get(g.y); r.get(g.hw); r.get(g.hh);
            q.goal.emplace(g.id, g);
        }
    }
    std::vector<int> rq, kd_cache;
    int rand_max = RAND_MAX;
    r.arr(rq);
    r.get(rand_max);
    r.arr(kd_cache);
    fclose(f);
    size_t total = 0;
    for (size_t i = 0; r.ok && i < N; i++) {
        if (plen[i] < 0) r.ok = false;
        total += (size_t)std::max(0, plen[i]);
    }
    if (!r.ok || total != pts.size() || (mode == ECMG_NEIGHBORS_KDTREE && (int)kd_cache.size() != k))
        return fail(c, ECMG_ERR_INVALID_ARG, "%s is damaged", path);
    /* the neighbour mode of the snapshot */
    {
        ecmg_status ms = ecmg_set_neighbor_mode(c, mode);
        if (ms != ECMG_OK) return ms;
    }
    CK(cudaStreamSynchronize(c->stream));
    CK(cudaMemcpy(c->pos.p, pos.data(), sizeof(V2) * N, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->vel.p, vel.data(), sizeof(V2) * N, cudaMemcpyHostToDevice));
    c->mirror_stale = true;
    CK(cudaMemcpy(c->attr.p, attr.data(), sizeof(V2) * N, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->pref_vel.p, pv.data(), sizeof(V2) * N, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_clear.p, clear.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_speed.p, speed.data(), sizeof(float) * N, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_active.p, active.data(), N, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_fail_edge.p, fe.data(), sizeof(int) * N, cudaMemcpyHostToDevice));
    c->clear = clear;
    c->speed = speed;
    c->active = active;
    c->fail_edge = fe;
    c->num_agents = num;
    size_t o = 0;
    for (size_t i = 0; i < N; i++) {
        c->paths[i].assign(pts.begin() + (std::ptrdiff_t)o, pts.begin() + (std::ptrdiff_t)(o + (size_t)plen[i]));
        o += (size_t)plen[i];
    }
    /* every path again, packed (the compaction path of the path store) */
    c->path_used = c->path_xy.n; /* forces the repack */
    {
        ecmg_status ps = ensure_path_room(c, 1);
        if (ps != ECMG_OK) return ps;
    }
    for (size_t s = 0; s < ss.size(); s++) {
        SceneState* sc = c->scenes[s].get();
        sc->num_agents = ss[s].num;
        sc->last_idx = ss[s].last;
        sc->free_stack = ss[s].free_stack;
        sc->next_spawn_id = ss[s].next_spawn;
        sc->next_goal_id = ss[s].next_goal;
        sc->spawn_areas = ss[s].spawn;
        sc->goal_areas = ss[s].goal;
        sc->grid_ready = false;
        for (int i = sc->slot_base; i <= sc->last_idx; i++)
            if (c->active[i]) note_range(c, sc, c->clear[i], c->speed[i]);
    }
    c->rq = rq;
    c->rq_head = 0;
    c->rand_max = rand_max;
    if (mode == ECMG_NEIGHBORS_KDTREE)
        CK(cudaMemcpy(c->kd.cache.p, kd_cache.data(), sizeof(int) * kd_cache.size(), cudaMemcpyHostToDevice));
    c->table_dirty = true;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_get_counts(const ecmg_ctx* c, int* num_agents, int* last_index, int* max_agents)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (num_agents) *num_agents = c->num_agents;
    if (last_index) *last_index = c->global_last();
    if (max_agents) *max_agents = c->max_agents;
    return ECMG_OK;
}

ecmg_status ecmg_scene_counts(const ecmg_ctx* c, int scene, int* num_agents, int* last_index, int* slot_base,
                              int* slot_count)
{
    if (!c || scene < 0 || scene >= (int)c->scenes.size()) return ECMG_ERR_INVALID_ARG;
    const SceneState* sc = c->scenes[scene].get();
    if (num_agents) *num_agents = sc->num_agents;
    if (last_index) *last_index = sc->last_idx;
    if (slot_base) *slot_base = sc->slot_base;
    if (slot_count) *slot_count = sc->slot_cap;
    return ECMG_OK;
}

int ecmg_scene_count(const ecmg_ctx* c) { return c ? (int)c->scenes.size() : 0; }

ecmg_status ecmg_set_record(ecmg_ctx* c, int on)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    c->record = on != 0;
    c->graph_dirty = true;
    return ECMG_OK;
}

ecmg_status ecmg_set_proposal(ecmg_ctx* c, ecmg_mlp* model)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (model && c->nbr_mode == ECMG_NEIGHBORS_KDTREE)
        return fail(c, ECMG_ERR_STATE, "the learned proposal and the trace need the exact neighbour mode");
    if (model != c->model) {
        c->model = model;
        c->gate_left = 0;
        c->gate_t_model = c->gate_t_plain = -1.0f;
        c->gate_model_ticks = 0;
        c->graph_dirty = true;
    }
    return ECMG_OK;
}

ecmg_status ecmg_set_proposal_gate(ecmg_ctx* c, float min_accept_rate, int pause_ticks)
{
    if (!c || !(min_accept_rate >= 0.0f && min_accept_rate <= 1.0f) || pause_ticks < 0) return ECMG_ERR_INVALID_ARG;
    c->gate_min = min_accept_rate;
    c->gate_pause = pause_ticks;
    c->gate_left = 0;
    c->gate_t_model = c->gate_t_plain = -1.0f;
    c->gate_model_ticks = 0;
    return ECMG_OK;
}

ecmg_status ecmg_set_trace(ecmg_ctx* c, int on)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (on && c->nbr_mode == ECMG_NEIGHBORS_KDTREE)
        return fail(c, ECMG_ERR_STATE, "the learned proposal and the trace need the exact neighbour mode");
    if ((on != 0) != c->trace) {
        c->trace = on != 0;
        c->trace_rows = 0;
        c->graph_dirty = true;
    }
    return ECMG_OK;
}

ecmg_status ecmg_set_proposal_classes(ecmg_ctx* c, const unsigned char* dev_cls_by_slot)
{
    if (!c) return ECMG_ERR_INVALID_ARG;
    if (dev_cls_by_slot && c->nbr_mode == ECMG_NEIGHBORS_KDTREE)
        return fail(c, ECMG_ERR_STATE, "the learned proposal and the trace need the exact neighbour mode");
    if (dev_cls_by_slot != c->cls_override) {
        c->cls_override = dev_cls_by_slot;
        c->graph_dirty = true;
    }
    return ECMG_OK;
}

ecmg_status ecmg_get_trace(ecmg_ctx* c, void* feat_dst, unsigned char* label_dst, int* slot_dst, int cap,
                           int* n_rows)
{
    if (!c || cap < 0) return ECMG_ERR_INVALID_ARG;
    if (!c->trace || !c->label.p) return fail(c, ECMG_ERR_STATE, "tracing is off");
    CK(cudaStreamSynchronize(c->stream));
    int n = std::min(cap, c->trace_rows);
    if (n > 0 && feat_dst) CK(cudaMemcpy(feat_dst, c->feat.p, (size_t)n * kMlpIn * 2, cudaMemcpyDefault));
    if (n > 0 && label_dst) CK(cudaMemcpy(label_dst, c->label.p, (size_t)n, cudaMemcpyDefault));
    if (n > 0 && slot_dst) CK(cudaMemcpy(slot_dst, c->s_slot.p, sizeof(int) * n, cudaMemcpyDefault));
    if (n_rows) *n_rows = n;
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

}  // extern "C"
