/*
 * ecmg_internal.h -- device-side layout shared by the kernels and the host
 * context (not part of the C ABI).
 */
#ifndef ECMG_INTERNAL_H
#define ECMG_INTERNAL_H

#include <cuda_runtime.h>
#include "ecmg_geom.cuh"

namespace ecmg {

/* Constraint capacity per agent: the k neighbour half-planes plus
   kMaxObstCons obstacle half-planes.  An agent that would need more obstacle
   half-planes sets ECMG_DEV_ERR_CONSTRAINTS and is computed with the first
   kMaxObstCons only; the tick then returns ECMG_ERR_BOUND. */
constexpr int kMaxObstCons = 24;
constexpr int kMaxK = 32;

/* device active flag: bit 0 active; kActivePending marks an active agent
   whose re-plan from the previous tick is still being computed on the host
   when the tick starts (its attraction and ORCA step come from k_fixup) */
constexpr unsigned char kActivePending = 2;

/* Learned active-set proposal (mlp.cu).  Features: 16 neighbours x 5 + 2,
   zero-padded to kMlpIn.  Classes of an agent's 2D LP result, in terms of
   its neighbour half-planes q (constraint index nObst + q):
     kClsPref          no half-plane moved the initial velocity
     kClsSingle + q    projection of the preferred velocity onto q
     kClsPair + p      q_hi's line, bounded by q_lo's (q_lo < q_hi),
                       p = q_hi * (q_hi - 1) / 2 + q_lo
     kClsCircle + q    q's line, bounded by the speed circle
     kClsOther         anything else (obstacle half-plane, neighbour >= 16,
                       infeasible 2D LP) */
constexpr int kMlpIn = 96, kMlpHid = 128, kMlpOut = 160, kMlpNbrs = 16;
constexpr int kClsPref = 0, kClsSingle = 1, kClsPair = 17, kClsCircle = 137, kClsOther = 153;

/* device counters (int[kCounters]) */
enum {
    C_DESTROYED = 0,
    C_REPLAN = 1,
    C_LP3D = 2,
    C_ERROR = 3,       /* bitmask of ECMG_DEV_ERR_* */
    C_PROCESSED = 4,   /* agents processed by the per-agent kernel */
    C_WORK = 5,        /* work counter of the persistent agent kernel */
    C_LAST = 6,        /* last slot index to scan (host-written before the tick) */
    C_NSORTED = 7,     /* agents in the neighbour grid */
    C_PROPOSED = 8,    /* LPs that received a learned proposal */
    C_ACCEPTED = 9,    /* proposals that passed the exact check */
    C_REPLAN_DEV = 10, /* re-plans that fail at the start retraction (not listed) */
    C_NBR_WORK = 11,   /* work counter of the persistent neighbour kernel */
    kCounters = 16
};

enum {
    ECMG_DEV_ERR_CONSTRAINTS = 1,
    ECMG_DEV_ERR_LIST = 2,
    ECMG_DEV_ERR_MLP = 4, /* a bounded wait of the tensor-core inference gave up */
};

/* Uniform agent grid: cells [0, gw*gh) cover the scene rectangle; agents
   outside it go to the overflow bucket gw*gh, which every query scans. */
struct AgentGrid {
    float x0, y0, cell, inv;
    int gw, gh;
    int ncells; /* gw*gh, overflow bucket index */
};

/* One independent scene of a batch: its agent grid, the first of its
   buckets in the global bucket array, and its static obstacle / ECM views
   (indices inside a view are local to the scene). */
struct SceneDev {
    AgentGrid grid;
    int bucket_base;
    ObstView ob;
    EcmView ecm;
};

struct TickArgs {
    /* slot-indexed state */
    V2* pos;
    V2* vel;
    V2* attr;
    V2* pref_vel;
    const float* clear;
    const float* speed;
    unsigned char* active;
    const int* path_off;
    const int* path_len;
    const V2* path_xy;
    /* tick-start snapshot in grid order */
    const int* s_slot;
    const V2* s_pos;
    const V2* s_vel;
    const float* s_clear;
    const int* cell_start; /* total buckets + 1 */
    int* nbr;              /* [n * k] neighbours of grid-order agent t, as grid-order indices */
    int* ncnt;             /* [n] neighbour count */
    const int* slot_bucket; /* slot -> bucket of this tick's binning */
    const int* slot_rank;   /* slot -> rank inside its bucket */
    void* feat;            /* [n, kMlpIn] bf16 proposal features (learned mode / tracing) */
    const unsigned char* cls; /* [n] proposed class (null: plain LP) */
    const unsigned char* cls_slot; /* [slots] proposed class by slot (overrides cls) */
    unsigned char* label;  /* [n] class of the LP result (null: not traced) */
    const SceneDev* scenes;
    const int* slot_scene; /* slot -> scene (null: one scene) */
    int tile;              /* agents a warp takes per work grab (per-thread mode: multiple of 32) */
    int lp_mode;           /* 0: one thread per agent, 1: one warp per agent */
    int occ_div;           /* per-thread layout: resident blocks per SM divided by this */
    int knn_wide;          /* neighbour kernel: 0 = 8 blocks of 128 threads per SM (64 registers), 1 = 6 (80) */
    /* parameters */
    float dt, tau_a, tau_o, rnb, rnb2, max_speed, mass_recip, arr_sq, del_sq;
    float inv_tau_a;       /* 1 / tau_a when tau_a is a power of two (exact), else 0 */
    int k;
    int lp3d_fp64;
    int replan_dev_fail;   /* built-in planner: settle known-failing re-plans on the device */
    const int* fail_edge;  /* slot -> ECM edge from which its re-plan search failed (-1: none) */
    /* outputs */
    int* counters;
    int* destroyed_list;
    int* replan_list;
    V2* replan_pos;
    int list_cap;
    /* recording (may be null) */
    int* rec_nbr;
    int* rec_cnt;
    V2* rec_vorca;
    int* rec_fail;
    int* rec_ncons;
    int* rec_nobst;
};

struct BinArgs {
    const V2* pos;
    const float* clear;
    const V2* vel;
    const unsigned char* active;
    int* key;        /* slot -> bucket */
    int* rank;       /* slot -> rank inside the bucket */
    int* cell_count; /* ncells + 1 buckets (+1 sentinel) */
    int* s_slot;
    V2* s_pos;
    V2* s_vel;
    float* s_clear;
    const int* cell_start;
    int* counters;
    AgentGrid grid;           /* used when scenes is null */
    const SceneDev* scenes;   /* batch: per-scene grid and bucket base */
    const int* slot_scene;
    int total_buckets;        /* sum over scenes of (cells + overflow) */
    int n_fixed;              /* > 0: bin slots [0, n_fixed) (stand-alone kNN); 0: [0, counters[C_LAST]] */
};

/* kernels.cu; propose (may be null) runs between the feature kernel and the
   per-agent kernel and fills TickArgs::cls */
typedef cudaError_t (*ProposeFn)(void* user, cudaStream_t s);
/* after_attract (may be null) runs right after the attraction kernel, when
   the destroyed and re-plan lists are final; evflags are the flags for an
   event record at that point (external when the stream is being captured) */
typedef cudaError_t (*HookFn)(void* user, cudaStream_t s, unsigned evflags);
/* The attraction kernel runs on s2 beside the neighbour kernel on s (fork and
   join through ev_fork / ev_join).  ev (may be null): five events -- before
   both, after the attraction kernel (on s2), after the neighbour kernel, after
   the proposal (features + inference) and after the per-agent kernel. */
struct KdArgs;
/* kd (may be null): the kd-tree neighbour mode replaces the neighbour kernel */
cudaError_t launch_tick(const BinArgs& b, const TickArgs& t, int max_slots, int* scan_tmp, int block, int sms,
                        cudaStream_t s, cudaStream_t s2, cudaEvent_t ev_fork, cudaEvent_t ev_join,
                        const cudaEvent_t* ev, ProposeFn propose, void* propose_user,
                        HookFn after_attract, void* after_attract_user, const KdArgs* kd);
/* api_host.cu: the checked grid of the stand-alone kNN (ecmg_knn,
   ecmg_knn_noalloc); false for a non-finite box or cell, or more than
   kKnnMaxCells cells */
constexpr double kKnnMaxCells = 32.0e6;
bool knn_grid_of(float x0, float y0, float x1, float y1, float cell, AgentGrid* out);
cudaError_t launch_knn(const V2* pos, const unsigned char* active, int n, int k, float r, AgentGrid g,
                       int* key, int* rank, int* cell_count, int* cell_start, int* s_slot, V2* s_pos,
                       int* scan_tmp, int scan_blocks, int* out_ids, int* out_cnt, cudaStream_t s);
int scan_tmp_ints(int n);
/* kernels.cu: mark the agents of `list` pending (before the tick's graph);
   after the graph and the upload of their paths, their attraction and ORCA
   step of the tick (k_fixup) */
cudaError_t launch_mark_pending(const TickArgs& t, const int* list, int n, cudaStream_t s);
/* pos / vel of slots [0, n) into page-locked host memory (device addresses
   of it): 16-byte loads and stores, coalesced on both sides */
cudaError_t launch_mirror(const V2* pos, const V2* vel, V2* h_pos, V2* h_vel, int n, int sms, cudaStream_t s);
cudaError_t launch_fixup(const TickArgs& t, const int* list, int n, cudaStream_t s);

/* spawn.cu: Simulator::ValidSpawnLocation (Simulator.cpp:295-311) for a batch
   of candidate locations.  Candidates of one spawn area share a clearance;
   an agent is tested against an area's candidates only when it lies in the
   area's box (the candidates' bounding box grown by more than the
   clearance, so no agent the exact test would find is skipped). */
constexpr int kSpawnMaxAreas = 64;
constexpr int kSpawnMaxCand = 4096;
struct SpawnAreaDev {
    float x0, y0, x1, y1; /* box of the candidates, grown */
    float c2;             /* clearance * clearance */
    int first, count, pad;
};
/* hit[j] = 1 when an active agent in slots [b, e) is closer than the area's
   clearance to candidate j (hit must be zeroed by the caller) */
cudaError_t launch_spawn_check(const V2* pos, const unsigned char* active, int b, int e, const V2* cand,
                               const SpawnAreaDev* areas, int n_areas, int* hit, int sms, cudaStream_t s);
/* one spawned agent: its slot, start, clearance, preferred speed and path */
struct SpawnRec {
    int slot;
    float x, y, clr, speed;
    int path_off, path_len, pad;
};
struct SpawnTargets {
    V2 *pos, *vel, *pref_vel;
    float *clear, *speed;
    unsigned char* active;
    int *path_off, *path_len, *fail_edge;
};
/* writes the records into the agent arrays (velocities zeroed, active set,
   failed-search edge cleared) */
cudaError_t launch_spawn_place(const SpawnRec* rec, int n, const SpawnTargets& t, cudaStream_t s);

/* kdtree.cu: the reference's kd-tree neighbour query (neighbour mode
   ECMG_NEIGHBORS_KDTREE).  Members = agents in this tick's grid (active at
   the start of the tick); lists hold slots. */
constexpr int kKdMaxDepth = 30;
struct KdArgs {
    int max_slots, cap, k, levels, tree_cap;
    const V2* pos;              /* slot-indexed positions at the start of the tick */
    const int* s_slot;          /* grid order -> slot */
    const int* counters;        /* C_NSORTED (members), C_LAST */
    const unsigned char* active; /* after the attraction kernel (kd_finish) */
    const int* cell_start;
    const int* slot_bucket;
    const int* slot_rank;
    unsigned char* mark;        /* [max_slots] member flags */
    int* n_dev;                 /* [2] members, max depth */
    int* iscan;                 /* [max_slots] */
    int* ids0;                  /* [cap] members in slot order */
    unsigned* keys;
    unsigned* ktmp;
    int* vtmp;                  /* [cap] radix buffers */
    int* X0;                    /* [cap] (x, index) */
    int* X[2];                  /* [cap] (x, y, index), partitioned per level */
    int* Y[2];                  /* [cap] (y, x, index), partitioned per level */
    int* seg_lo;
    int* seg_hi;
    int* seg_node;              /* [cap] segment of each position */
    unsigned char* side;        /* [max_slots] 0 left, 1 node, 2 right */
    unsigned long long* flags;  /* [cap] left | right << 32 */
    int* scan_tmp32;
    unsigned long long* scan_tmp64;
    int* hist;                  /* [kd_hist_ints(cap)] */
    int* tree;                  /* [tree_cap] KDTree::m_Tree */
    V2* tree_pos;               /* [tree_cap] position of each node's agent */
    int* map;                   /* [max_slots * k] per-member cache maps, then local prefixes */
    int* kfound;                /* [max_slots] */
    int* agg;
    int* prev_in;               /* [kd_compose_blocks * k] */
    int* cache;                 /* [k] ORCA::m_NeighborCache, kept across ticks */
    int* nbr;                   /* [cap * k] per-agent kernel input, grid order */
    int* ncnt;                  /* [cap] */
};
int kd_compose_blocks(int max_slots);
int kd_hist_ints(int cap);
int kd_scan_tmp(int n);
cudaError_t kd_build_and_query(const KdArgs& a, cudaStream_t s, int sms);
cudaError_t kd_finish(const KdArgs& a, cudaStream_t s, int sms);

}  // namespace ecmg
#endif
