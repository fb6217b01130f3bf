/*
 * ecmg.h -- C ABI of the GB300 crowd-tick library (libecmg.so).
 *
 * The library replaces the per-tick update of the ECMGenerator crowd simulator,
 * ECM::Simulation::Simulator (ECMAgentSimulator/Simulator.h:59-188): neighbour
 * query, ORCA velocity selection, IRM path following and integration, executed
 * as sm_103a kernels on one GPU with the agent state resident in device memory.
 * Scene construction (obstacles, the Explicit Corridor Map) and path planning
 * stay on the host.
 *
 * Conventions: every entry point returns an ecmg_status (0 = ECMG_OK).  Arrays
 * are host arrays unless the name says "dev".  Slot indices are the reference's
 * Entity ids: slots are handed out by a LIFO free-slot stack exactly like
 * Simulator::m_freeEntitySpaces (Simulator.h:66-69, 167).  One context must not
 * be used from two threads at once (the reference is single-threaded).
 * ecmg_last_error() describes the most recent failure of a context.
 */
#ifndef ECMG_H
#define ECMG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    ECMG_OK = 0,
    ECMG_ERR_INVALID_ARG = 1,   /* bad pointer, size or value (NaN/inf input, empty path, ...) */
    ECMG_ERR_CUDA = 2,          /* a CUDA runtime call failed                                   */
    ECMG_ERR_BOUND = 3,         /* a device capacity or loop bound was exceeded (see last_error) */
    ECMG_ERR_NO_SLOT = 4,       /* no free agent slot (SpawnAgent returns -1, Simulator.cpp:170) */
    ECMG_ERR_STATE = 5,         /* call made in the wrong state (e.g. tick before set_ecm)     */
    ECMG_ERR_INVALID_SPAWN = 6, /* spawn location occupied (ValidSpawnLocation, Simulator.cpp:295) */
    ECMG_ERR_NO_PATH = 7,       /* the planner found no path                                    */
    ECMG_ERR_NO_DEVICE = 8      /* no CUDA device                                               */
} ecmg_status;

typedef struct ecmg_ctx ecmg_ctx;

/* Tick parameters.  ecmg_default_params() gives the reference's values:
   ORCA(5) (Simulator.cpp:55), time horizons 10 s (ORCA.h:102-103), mass 0.8
   (Simulator.cpp:622), arrival / delete radii 20 m / 2 m (Simulator.cpp:542-543).
   max_speed <= 0 reproduces the reference, whose LP radius is each agent's
   preferred speed (Simulator.cpp:671). */
typedef struct {
    float dt;              /* Simulator::m_SimStepTime (ctor argument)            */
    float tau_agent;       /* ORCA::m_lookAheadAgent                              */
    float tau_obst;        /* ORCA::m_lookAheadObstacle                           */
    float neighbor_dist;   /* neighbour cut-off of the grid kNN (metres)          */
    float max_speed;       /* <= 0: preferred speed per agent                     */
    float mass;
    float arrival_radius;
    float delete_radius;
    int max_neighbors;     /* ORCA(numNeighbors); 1..32                           */
    int lp3d_fp64;         /* 1: build the 3D-LP projection lines in FP64         */
    int use_graph;         /* 1: capture the tick as a CUDA graph                 */
    int block_size;        /* 0: autotuned                                        */
    float grid_cell;       /* agent grid cell (metres); 0: derived from density  */
} ecmg_params;

/* Per-tick counters (summed over the ticks of one ecmg_tick call). */
typedef struct {
    int ticks;
    int active_agents;     /* after the last tick (Simulator::GetNumAgents)       */
    int last_index;        /* Simulator::GetLastIndex after the last tick          */
    long long agent_steps; /* sum over ticks of agents processed                  */
    long long destroyed;   /* agents that reached their goal (DestroyAgent)       */
    long long replans;     /* IRM failures handed to the host planner             */
    long long replans_failed;
    long long lp3d;        /* agents whose 2D LP was infeasible                   */
    float device_ms;       /* device time of the ticks (CUDA events)              */
    float agent_kernel_ms; /* device time of the attraction, neighbour, proposal and per-agent kernels */
    float host_ms;         /* host time between ticks (bookkeeping, re-planning)  */
    long long proposed;    /* learned mode: LPs that received an active-set proposal */
    long long accepted;    /* learned mode: proposals that passed the exact check     */
    long long gated;       /* learned mode: ticks run without the model (gate closed) */
    long long replans_host; /* re-plans served by the host planner (the rest were settled on the device) */
    float attract_ms;      /* attraction / steering kernel (from the common start)  */
    float neighbors_ms;    /* neighbour (kNN) kernel, which runs beside it          */
    float proposal_ms;     /* learned mode: feature and inference kernels          */
    float orca_ms;         /* device time of the per-agent ORCA kernel             */
    long long spawned;       /* agents placed by the spawn areas                   */
    long long spawn_failed;  /* no valid location in 10 attempts (Simulator.cpp:526-530) */
    long long spawn_refused; /* valid location, but no free slot or no path        */
    float spawn_ms;          /* host time of the spawn stage, device check included */
    float spawn_check_ms;    /* of which the location tests on the device (copies and wait included) */
    long long spawn_candidates; /* candidate locations tested on the device      */
    int graph_builds;        /* tick graphs captured and instantiated (host time; after launch-configuration, mode or path-store changes) */
    int spawn_kernels;       /* kernel launches of the spawn stage (location checks, placement) */
} ecmg_tick_stats;

/* Static obstacles: n_obstacles rings, ring r = xy[2*ring_offsets[r] ..
   2*ring_offsets[r+1]), counter-clockwise as Environment::AddObstacle expects
   (Environment.cpp:199-229).  Convexity and prev/next links are derived as
   Obstacle::Initialize does (ECMDataTypes.cpp:23-61). */
typedef struct {
    int n_obstacles;
    const int* ring_offsets;  /* n_obstacles + 1 */
    const float* xy;
} ecmg_obstacles;

/* Explicit Corridor Map in ECMGraph's layout (ECMGenerator/ECM.h:20-116):
   vertex i = (v_pos[2i], v_pos[2i+1]); half-edge h of edge e has index 2e+h. */
typedef struct {
    int n_vertices;
    const float* v_pos;       /* 2*V  ECMVertex::position        */
    const float* v_clear;     /* V    ECMVertex::clearance       */
    const int* v_idx;         /* V    ECMVertex::idx             */
    const int* v_halfedge;    /* V    ECMVertex::half_edge_idx   */
    int n_edges;
    const int* he_target;     /* 2E   ECMHalfEdge::v_target_idx  */
    const int* he_next;       /* 2E   ECMHalfEdge::next_idx      */
    const float* he_left;     /* 4E   ECMHalfEdge::closest_left  */
    const float* he_right;    /* 4E   ECMHalfEdge::closest_right */
} ecmg_ecm;

/* Host planner used for spawning and for re-planning after an IRM failure
   (Simulator::UpdatePath, Simulator.cpp:97-124).  Write at most cap points
   to out_xy and return their count, or a negative value for "no path". */
typedef int (*ecmg_plan_fn)(void* user, float sx, float sy, float gx, float gy,
                            float clearance, float* out_xy, int cap);

enum {
    ECMG_FIELD_POSITION = 0,       /* float[2*n]  GetPositionData           */
    ECMG_FIELD_VELOCITY = 1,       /* float[2*n]  GetVelocityData           */
    ECMG_FIELD_PREF_VELOCITY = 2,  /* float[2*n]  GetPreferredVelocityData  */
    ECMG_FIELD_ATTRACTION = 3,     /* float[2*n]  GetAttractionPointData    */
    ECMG_FIELD_CLEARANCE = 4,      /* float[n]    GetClearanceData          */
    ECMG_FIELD_SPEED = 5,          /* float[n]    preferred speed           */
    ECMG_FIELD_ACTIVE = 6          /* uint8[n]    GetActiveFlags            */
};

/* defaults as listed above; dt = 0.1 (ECMApplication/main.cpp:53) */
void ecmg_default_params(ecmg_params* p);

/* Simulator(ecm, planner, env, maxAgents, simStepTime) + Initialize()
   (Simulator.h:63-74, Simulator.cpp:21-60); device 0 of the process. */
ecmg_status ecmg_create(const ecmg_params* p, int max_agents, ecmg_ctx** out);
/* ~Simulator / ClearSimulator (Simulator.cpp:62-95) */
ecmg_status ecmg_destroy(ecmg_ctx* ctx);
const char* ecmg_last_error(const ecmg_ctx* ctx);
ecmg_status ecmg_get_params(const ecmg_ctx* ctx, ecmg_params* out);

/* Environment::GetObstacles (Environment.h:55), read by FindNearestObstacles */
ecmg_status ecmg_set_obstacles(ecmg_ctx* ctx, const ecmg_obstacles* o);
/* the ECM the Simulator and its planner hold (Simulator.h:154-155) */
ecmg_status ecmg_set_ecm(ecmg_ctx* ctx, const ecmg_ecm* e);
/* replaces the built-in A* planner (NULL restores it) */
ecmg_status ecmg_set_planner(ecmg_ctx* ctx, ecmg_plan_fn fn, void* user);
/* Built-in planner.  ECMG_PLANNER_REFERENCE (default):
   ECMPathPlanner::FindPath restated (ECMPathPlanner.cpp:22-411,
   AStar.cpp:44-210): the reference's A* -- its open list included --,
   corridor, portals and funnel, giving the reference planner's paths.
   ECMG_PLANNER_FAST (opt-in, not the reference's paths): A* over the ECM
   vertices with the clearance filter (landmark lower bounds), then the
   polyline is shortened greedily where a straight piece keeps the
   clearance. */
#define ECMG_PLANNER_FAST 0
#define ECMG_PLANNER_REFERENCE 1
ecmg_status ecmg_set_planner_mode(ecmg_ctx* ctx, int mode);
/* Re-plans overlapping the next tick (the built-in planner only, and not
   while spawn areas need the planner at the start of a tick).  The searches
   of a tick's re-plans start on host threads while the tick's neighbour and
   ORCA kernels run.  Mode 1 (default): searches that end with the tick are
   applied then, as re-plans served inside the tick; longer ones keep running
   after ecmg_tick returns, and the next tick skips those agents in its
   attraction and ORCA kernels and steps them, with their new paths, in a
   small launch after its own kernels -- the same inputs and functions, so the
   same results, the searches overlapping a whole tick of device work (the
   next tick's own searches start beside them).
   Mode 2: every search is carried into the next tick that way.  Mode 0: the
   tick waits for its searches.  Every entry point that reads or changes
   paths, agents, the scene or the planner waits for the searches first. */
ecmg_status ecmg_set_replan_overlap(ecmg_ctx* ctx, int mode);

/* Simulator::SpawnAgent (Simulator.cpp:168-200): ValidSpawnLocation, then a
   planned path.  *out_slot = slot, or -1 with ECMG_ERR_NO_SLOT /
   ECMG_ERR_INVALID_SPAWN / ECMG_ERR_NO_PATH. */
ecmg_status ecmg_spawn_agent(ecmg_ctx* ctx, float sx, float sy, float gx, float gy,
                             float clearance, float pref_speed, int* out_slot);
/* Bulk spawn with caller-supplied paths (agent i's path is
   path_xy[2*path_off[i] .. 2*(path_off[i]+path_len[i]))); no spawn-location
   check.  out_slots may be NULL. */
ecmg_status ecmg_add_agents(ecmg_ctx* ctx, int n, const float* pos, const float* clearance,
                            const float* pref_speed, const int* path_off, const int* path_len,
                            const float* path_xy, int* out_slots);
/* Simulator::DestroyAgent (Simulator.cpp:202-208) */
ecmg_status ecmg_destroy_agent(ecmg_ctx* ctx, int slot);
/* Simulator::Reset (Simulator.cpp:325-333) */
ecmg_status ecmg_reset(ecmg_ctx* ctx);
/* replace one agent's path (Simulator::UpdatePath with a given polyline) */
ecmg_status ecmg_set_path(ecmg_ctx* ctx, int slot, const float* xy, int n);
/* plan with the context's planner (ECMPathPlanner::FindPath) */
ecmg_status ecmg_find_path(ecmg_ctx* ctx, float sx, float sy, float gx, float gy, float clearance,
                           float* out_xy, int cap, int* out_n);
/* Host-only planner over a scene (needs no GPU): the same planner the context
   uses, for scene set-up and batch planning on `threads` host threads.
   out_xy holds cap_per_path points per request; out_n[i] is the point count,
   -1 when no path exists, -2 when the path has more than cap_per_path points. */
typedef struct ecmg_planner ecmg_planner;
ecmg_status ecmg_planner_create(const ecmg_obstacles* o, const ecmg_ecm* e, ecmg_planner** out);
ecmg_status ecmg_planner_destroy(ecmg_planner* p);
ecmg_status ecmg_planner_find_paths(ecmg_planner* p, int n, const float* starts, const float* goals,
                                    const float* clearances, int threads, int cap_per_path,
                                    float* out_xy, int* out_n);
/* ECMG_PLANNER_REFERENCE (default) or ECMG_PLANNER_FAST, as ecmg_set_planner_mode */
ecmg_status ecmg_planner_set_mode(ecmg_planner* p, int mode);
/* ECMGraph::FindCell for n points: cell index (2*edge + side) or -1 */
ecmg_status ecmg_planner_locate(ecmg_planner* p, int n, const float* xy, int* out_cell);

/* ---- spawn and goal areas (Simulator.h:92-104, Area.h) ---------------------
   Every tick starts with the reference's UpdateSpawnAreas
   (Simulator.cpp:494-536): per spawn area in ID order and per connected goal
   area, timeSinceLastSpawn += dt, n = (int)(time * rate) agents are spawned
   with up to 10 random locations each, then time -= n / rate.  A location is
   valid when no active agent is closer than the area's clearanceMin
   (ValidSpawnLocation, Simulator.cpp:295-311); the library tests the
   candidate locations of a tick against the device-resident agents in one
   batched kernel and the agents placed earlier in the same stage on the
   host.  Spawned agents get clearanceMin / preferredSpeedMin as in the
   reference and a path from the context's planner; a spawn with no free slot
   or no path is refused (the reference would keep an agent with an empty
   path) -- its random numbers are consumed all the same.
   Random numbers: Area::GetRandomPositionInArea (Area.h:39-53) draws three
   values per location, x = xMin + v1 / ((float)RAND_MAX / (xMax - xMin)),
   likewise y with v2 (v0 is unused).  Values come first from the queue
   filled by ecmg_push_spawn_random, then from the source set by
   ecmg_set_spawn_rng (default: the C library's rand() with RAND_MAX).  The
   library draws up to 33 values per agent due in a tick ahead of use; values
   a tick does not use stay queued for the next one, so the values consumed
   are those the reference's sequence of rand() calls would see. */
#define ECMG_AREA_SPAWN 2 /* SimAreaType::SPAWN (Area.h:11-18) */
#define ECMG_AREA_GOAL 3  /* SimAreaType::GOAL                 */
/* SpawnConfiguration (Area.h:82-88); the reference's defaults are 5/10/5/10 */
typedef struct {
    float preferred_speed_min, preferred_speed_max;
    float clearance_min, clearance_max;
} ecmg_spawn_config;
typedef struct {
    int id;
    float x, y;              /* Area::Position                              */
    float half_w, half_h;    /* Area::HalfWidth, Area::HalfHeight           */
    ecmg_spawn_config config; /* spawn areas                                */
    int n_connected;         /* spawn areas: connectedGoalAreas.size()      */
    int n_timers;            /* spawn areas: spawnRate.size() (see disconnect) */
} ecmg_area_info;
typedef int (*ecmg_rand_fn)(void* user);
/* AddSpawnArea / AddGoalArea (Simulator.cpp:336-381): id -1 takes the
   counter's next value; *out_id = the area's ID.  An ID already present
   keeps its area (std::map::emplace does not replace). */
ecmg_status ecmg_add_spawn_area(ecmg_ctx* ctx, float x, float y, float half_w, float half_h,
                                const ecmg_spawn_config* config, int id, int* out_id);
ecmg_status ecmg_add_goal_area(ecmg_ctx* ctx, float x, float y, float half_w, float half_h, int id, int* out_id);
/* RemoveArea (Simulator.cpp:414-424); connections to a removed goal area stay */
ecmg_status ecmg_remove_area(ecmg_ctx* ctx, int type, int id);
/* ConnectSpawnGoalAreas (Simulator.cpp:426-438): no-op if already connected */
ecmg_status ecmg_connect_areas(ecmg_ctx* ctx, int spawn_id, int goal_id, float spawn_rate);
/* DeconnectSpawnGoalAreas (Simulator.cpp:440-457), as the reference: the goal
   leaves connectedGoalAreas while spawnRate / timeSinceLastSpawn keep their
   entries, so later goals are paired with the rates of earlier positions;
   ignored when spawn_id is not below the number of spawn areas */
ecmg_status ecmg_disconnect_areas(ecmg_ctx* ctx, int spawn_id, int goal_id);
/* Area::Translate / Area::Scale as absolute values */
ecmg_status ecmg_set_area(ecmg_ctx* ctx, int type, int id, float x, float y, float half_w, float half_h);
/* GetSpawnArea / GetGoalArea (Simulator.cpp:459-479); for spawn areas the
   connected goal IDs, rates and timers (up to cap entries each, any NULL) */
ecmg_status ecmg_get_area(ecmg_ctx* ctx, int type, int id, ecmg_area_info* out, int* goal_ids, float* rates,
                          float* since_last_spawn, int cap);
/* IDs of the spawn or goal areas in ascending order (GetSpawnAreas / GetGoalAreas) */
ecmg_status ecmg_area_ids(ecmg_ctx* ctx, int type, int* ids, int cap, int* n);
/* source of random values in [0, rand_max]; fn NULL: rand() / RAND_MAX */
ecmg_status ecmg_set_spawn_rng(ecmg_ctx* ctx, ecmg_rand_fn fn, void* user, int rand_max);
/* appends recorded values to the queue consumed before the source */
ecmg_status ecmg_push_spawn_random(ecmg_ctx* ctx, const int* values, int n);
/* values queued and not yet consumed */
ecmg_status ecmg_spawn_random_pending(const ecmg_ctx* ctx, long long* n);
/* UpdateSpawnAreas alone (the stage every ecmg_tick starts with) */
ecmg_status ecmg_update_spawn_areas(ecmg_ctx* ctx, ecmg_tick_stats* stats);
/* agents placed by the last spawn stage: slot, start and goal (float[2] each) */
ecmg_status ecmg_get_spawned(const ecmg_ctx* ctx, int* slots, float* start_xy, float* goal_xy, int cap, int* n);

/* n_ticks x Simulator::Update (Simulator.cpp:314-323).  Re-planning requests
   raised by a tick are served on the host before the next tick starts. */
ecmg_status ecmg_tick(ecmg_ctx* ctx, int n_ticks, ecmg_tick_stats* stats);

/* Getters of Simulator.h:114-126, copied to caller memory (n_slots entries) */
ecmg_status ecmg_get_state(ecmg_ctx* ctx, int field, void* host_dst);
/* The getters as the reference has them: a pointer to library-owned host
   memory (page-locked for the device fields, refreshed from the device by
   this call).  The pointer stays valid until ecmg_destroy; its contents are
   those of this call until the next ecmg_host_view of the same field. */
ecmg_status ecmg_host_view(ecmg_ctx* ctx, int field, const void** out);
/* Host mirror of the positions and velocities (no reference counterpart:
   the reference's getters point into arrays that Update itself writes).
   on = 1: every tick ends by writing the positions and velocities of the
   slots it may have moved into the page-locked host views of
   ECMG_FIELD_POSITION and ECMG_FIELD_VELOCITY (a device-side copy that runs
   while the host finishes the tick), so that ecmg_host_view of those fields
   returns without a copy (it copies once after anything other than a tick
   changed them: adding, spawning through ecmg_spawn_agent, ecmg_set_state,
   ecmg_load_state, ecmg_autotune).  The two views are then rewritten by every
   tick, as the reference's arrays are by Update.  on = 0 (default):
   ecmg_host_view copies on every call. */
ecmg_status ecmg_set_host_mirror(ecmg_ctx* ctx, int on);
/* Overwrite slot-indexed state from the host (float[2*n] for the 2-vectors);
   used to start a tick from a given state. */
ecmg_status ecmg_set_state(ecmg_ctx* ctx, int field, const void* host_src);
ecmg_status ecmg_get_counts(const ecmg_ctx* ctx, int* num_agents, int* last_index, int* max_agents);
/* Checkpoint / resume (no reference counterpart): everything the following
   ticks depend on -- agent state, paths, free-slot stacks, spawn and goal
   areas with their timers, queued random values, the kd-tree mode's
   neighbour cache, the failed-search memo -- to a binary file, and back
   into a context created with the same slot capacity, scene count,
   max_neighbors and scene.  Ticks after a load reproduce the ticks after the
   save bit for bit.  The random source set by ecmg_set_spawn_rng, the
   planner and the launch configuration are not part of a snapshot. */
ecmg_status ecmg_save_state(ecmg_ctx* ctx, const char* path);
ecmg_status ecmg_load_state(ecmg_ctx* ctx, const char* path);
ecmg_status ecmg_get_path(ecmg_ctx* ctx, int slot, float* out_xy, int cap, int* out_n);

/* Record per-agent results of the following ticks for inspection:
   neighbour list (slot ids, -1 padded, max_neighbors per slot), LP result,
   failed index of the 2D LP (== n_constraints when feasible), constraint
   counts.  Recording costs bandwidth; it is off by default. */
ecmg_status ecmg_set_record(ecmg_ctx* ctx, int on);
ecmg_status ecmg_get_record(ecmg_ctx* ctx, int* nbr_ids, int* nbr_count, float* v_orca,
                            int* lp_fail, int* n_constraints, int* n_obst_constraints);

/* ---- batches of independent scenes (one launch sequence per tick) ----------
   Scene s owns the slot range [slot_base_s, slot_base_s + max_agents_s) with
   its own free-slot stack, obstacles, ECM and planner; a scene is what one
   reference Simulator + Environment hold.  ecmg_create(p, n, &ctx) is
   ecmg_create_batch(p, 1, &n, &ctx); the single-scene calls act on scene 0. */
ecmg_status ecmg_create_batch(const ecmg_params* p, int n_scenes, const int* max_agents_per_scene, ecmg_ctx** out);
int ecmg_scene_count(const ecmg_ctx* ctx);
ecmg_status ecmg_scene_set_obstacles(ecmg_ctx* ctx, int scene, const ecmg_obstacles* o);
ecmg_status ecmg_scene_set_ecm(ecmg_ctx* ctx, int scene, const ecmg_ecm* e);
ecmg_status ecmg_scene_add_agents(ecmg_ctx* ctx, int scene, int n, const float* pos, const float* clearance,
                                  const float* pref_speed, const int* path_off, const int* path_len,
                                  const float* path_xy, int* out_slots);
ecmg_status ecmg_scene_counts(const ecmg_ctx* ctx, int scene, int* num_agents, int* last_index, int* slot_base,
                              int* slot_count);

/* ---- launch configuration ------------------------------------------------
   The per-agent kernel is persistent: each warp takes agents_per_warp_grab
   grid-order agents per atomic work grab.  The agent grid cell is
   grid_cell_scale * sqrt(max_neighbors / agent density), unless
   ecmg_params.grid_cell fixes it. */
typedef struct {
    int block_size;
    int agents_per_warp_grab;
    float grid_cell_scale;
    float best_tick_ms;
    int trials;
    int lp_mode;             /* ECMG_LP_THREAD, ECMG_LP_WARP or ECMG_LP_THREAD_FUSED */
    int occupancy_divisor;   /* per-thread layout: resident blocks per SM divided by this */
    int neighbor_blocks_per_sm; /* exact-kNN kernel (k <= 16): 8 resident blocks at 64 registers or 6 at 80 */
} ecmg_tune_result;
ecmg_status ecmg_set_launch(ecmg_ctx* ctx, int block_size, int agents_per_warp_grab, float grid_cell_scale);
/* Per-agent kernel layout.  ECMG_LP_THREAD: one thread per agent (work
   grabs of agents_per_warp_grab from ecmg_set_launch).  ECMG_LP_WARP: one
   warp per agent -- the lanes build the constraints in parallel and share
   the inner loops of the LPs -- taking agents_per_warp_grab agents per work
   grab (1..64).  ECMG_LP_THREAD_FUSED: the per-thread layout with the
   neighbour search in the same kernel (each thread finds its agent's k
   nearest, then steps it; the separate search kernel is skipped; with a
   learned proposal or the kd-tree neighbour mode the per-thread layout runs
   instead).  All give identical results. */
/* per-thread layout: run the persistent per-agent kernel with the resident
   blocks per SM divided by `divisor` (1..8; fewer resident warps leave more
   L1 to each thread's local constraint arrays) */
ecmg_status ecmg_set_occupancy(ecmg_ctx* ctx, int divisor);
/* exact-kNN kernel for k <= 16: 8 resident blocks of 128 threads per SM
   (64 registers) or 6 (80 registers, no spills); the autotuner picks one */
ecmg_status ecmg_set_neighbor_blocks(ecmg_ctx* ctx, int blocks_per_sm);
#define ECMG_LP_THREAD 0
#define ECMG_LP_WARP 1
#define ECMG_LP_THREAD_FUSED 2
ecmg_status ecmg_set_lp_mode(ecmg_ctx* ctx, int mode, int agents_per_warp_grab);
/* Neighbour query of the tick.  ECMG_NEIGHBORS_EXACT (default): the exact k
   nearest within neighbor_dist, ordered by (d^2, index).
   ECMG_NEIGHBORS_KDTREE: the reference's own query -- KDTree::Construct and
   KNearestAgents_R (KDTree.cpp:22-202), quirks included, with ORCA's
   neighbour cache carried from agent to agent and from tick to tick
   (ORCA.h:87,100) -- i.e. the neighbour lists of the unmodified
   Simulator::Update; agents whose x (or y) coordinates are equal keep the
   order of the level above (std::sort agrees on subtrees of up to 16 agents).
   neighbor_dist is not used.  Runs the per-agent kernel one thread per agent,
   without the learned proposal or the trace; single-scene contexts, up to
   2^24 slots. */
#define ECMG_NEIGHBORS_EXACT 0
#define ECMG_NEIGHBORS_KDTREE 1
ecmg_status ecmg_set_neighbor_mode(ecmg_ctx* ctx, int mode);
/* times ticks_per_trial ticks per configuration -- first the grid cell with
   the default launch, then, at the best cell, the per-agent kernel's layout,
   block size, work grab and occupancy -- on a copy of the current state, restores the state after each
   trial (no re-plans are served during trials) and keeps the fastest */
ecmg_status ecmg_autotune(ecmg_ctx* ctx, int ticks_per_trial, ecmg_tune_result* out);

/* the cudaStream_t the context launches on (for callers that record CUDA
   events or order their own work around the tick) */
void* ecmg_stream(const ecmg_ctx* ctx);

/* Kernel launch list of the last tick (names in launch order); returns the
   number of kernels per tick. */
int ecmg_kernels_per_tick(const ecmg_ctx* ctx);

/* Stand-alone exact kNN on device arrays: for each of n agents at dev_pos
   (float2) with dev_active != 0, the k nearest other active agents with
   1e-4 < d^2 < radius^2, ordered by (d^2, index) -- the neighbour definition
   of the tick.  dev_scratch must hold ecmg_knn_scratch_bytes(n, ...) bytes;
   stream is a cudaStream_t (NULL = legacy default stream). */
size_t ecmg_knn_scratch_bytes(int n, float min_x, float min_y, float max_x, float max_y, float cell);
ecmg_status ecmg_knn(const float* dev_pos, const unsigned char* dev_active, int n, int k, float radius,
                     float min_x, float min_y, float max_x, float max_y, float cell,
                     int* dev_out_ids, int* dev_out_count, void* dev_scratch, size_t scratch_bytes,
                     void* stream);

/* ecmg_knn without caller scratch.  No counterpart in the reference: it is
   for callers that may not allocate device memory at query time (a real-time
   frame loop, where cudaMalloc would synchronise the device, or a plug-in
   whose host application owns the allocator).  Scratch is a fixed device
   array of ECMG_KNN_STATIC_SCRATCH_BYTES held by every GPU that loads the
   library until the process exits; a query needing more
   (ecmg_knn_scratch_bytes > the limit) returns ECMG_ERR_BOUND.  The first call
   on a device resolves the array's device address -- make it before any
   stream capture; later calls may be captured into a CUDA graph (a query
   enqueues only memsets and kernels, no host copies).  The address is kept per device for its primary context:
   other contexts made current through the driver API, and calls after a
   cudaDeviceReset, are not supported.  Calls share the array: overlapping
   calls on one device race.  Allocates nothing. */
#define ECMG_KNN_STATIC_SCRATCH_BYTES (16u * 1024u * 1024u)
ecmg_status ecmg_knn_noalloc(const float* dev_pos, const unsigned char* dev_active, int n, int k, float radius,
                             float min_x, float min_y, float max_x, float max_y, float cell,
                             int* dev_out_ids, int* dev_out_count, void* stream);

/* ---- learned active-set proposal (no reference counterpart) --------------
   A small MLP (96 inputs: 16 sorted neighbours x (relative position /
   neighbor_dist, relative velocity / 2, radius sum) + preferred velocity /
   LP radius, zero-padded; two hidden layers of 128 with GELU; 160 classes)
   proposes which constraints bound the optimum of an agent's 2D LP
   (ORCA.cpp:428-587): none, the projection onto neighbour q's half-plane,
   q's line bounded by neighbour p's, or q's line bounded by the speed
   circle.  The tick checks every proposal exactly (the proposed last update
   of the incremental LP, containment by every later half-plane, KKT
   multipliers and slack of the rest) and runs the full LP when the check
   fails.  Inference runs in BF16 on the tensor cores with FP32 accumulation;
   training (FP32 master weights, Adam) runs on the GPU in this library. */
typedef struct ecmg_mlp ecmg_mlp;
#define ECMG_MLP_IN 96
#define ECMG_MLP_CLASSES 160
ecmg_status ecmg_mlp_create(unsigned long long seed, ecmg_mlp** out);
ecmg_status ecmg_mlp_destroy(ecmg_mlp* model);
int ecmg_mlp_param_count(void);
/* parameters as one float array: W1 [96x128] row-major, b1 [128],
   W2 [128x128], b2 [128], W3 [128x160], b3 [160] */
ecmg_status ecmg_mlp_get_params(ecmg_mlp* model, float* host_out);
ecmg_status ecmg_mlp_set_params(ecmg_mlp* model, const float* host_in);
/* mean softmax cross-entropy and its gradient (host float[param_count]) over
   all n rows; dev_x: bf16 [n x 96], dev_y: class per row (device memory) */
ecmg_status ecmg_mlp_loss_grad(ecmg_mlp* model, const void* dev_x, const unsigned char* dev_y, int n,
                               float* loss, float* host_grad);
/* `steps` Adam steps on minibatches of `batch` rows drawn with replacement
   from the n rows (seeded); per-step loss / accuracy to host arrays if given */
ecmg_status ecmg_mlp_train(ecmg_mlp* model, const void* dev_x, const unsigned char* dev_y, int n, int steps,
                           int batch, float lr, unsigned long long seed, float* host_loss, float* host_acc);
/* class of every row (argmax of the BF16 tensor-core forward); returns
   ECMG_ERR_BOUND when a bounded wait of the inference kernel gave up (the
   kernel drains its copies and MMAs, frees its tensor memory and returns) */
ecmg_status ecmg_mlp_predict(ecmg_mlp* model, const void* dev_x, int n, unsigned char* dev_cls);
/* how many times the inference kernel polls an mbarrier (a feature-tile copy
   or an MMA chain) before it gives up with ECMG_ERR_BOUND; 0 restores the
   default (2^22).  A diagnostic of the device-side timeout path: a tiny
   limit makes the first wait run out. */
ecmg_status ecmg_mlp_set_wait_limit(ecmg_mlp* model, int polls);

/* Learned mode for a context: model != NULL turns it on (the context does
   not own the model; keep it alive while it is set), NULL turns it off.
   Results are those of the plain LP whether or not a proposal is accepted. */
ecmg_status ecmg_set_proposal(ecmg_ctx* ctx, ecmg_mlp* model);
/* Gate of the learned mode: a tick whose accepted proposals are fewer than
   min_accept_rate x its agents, or whose device time per agent exceeds the
   plain tick's by more than 2 % (running averages of both kinds of tick; the
   plain time is measured by 3 plain ticks after the first 3 model ticks),
   runs the next pause_ticks ticks without the model (no features, no
   inference), then tries it again.  Default 0.1 / 64; min_accept_rate 0
   keeps the model on every tick. */
ecmg_status ecmg_set_proposal_gate(ecmg_ctx* ctx, float min_accept_rate, int pause_ticks);
/* Trace mode: every tick also writes, for each agent in grid order, its
   proposal features and the class of its plain LP result (training data). */
ecmg_status ecmg_set_trace(ecmg_ctx* ctx, int on);
/* the last tick's trace: rows of bf16 [96] features, class labels and the
   agent slot of each row, copied to dst pointers in host or device memory
   (any may be NULL; at most cap rows; *n_rows set) */
ecmg_status ecmg_get_trace(ecmg_ctx* ctx, void* feat_dst, unsigned char* label_dst, int* slot_dst, int cap,
                           int* n_rows);
/* Proposals given per agent slot (device array of max_agents classes)
   instead of by a model, e.g. the labels of a trace; NULL turns it off.
   Exercises the exact check with known answers. */
ecmg_status ecmg_set_proposal_classes(ecmg_ctx* ctx, const unsigned char* dev_cls_by_slot);

#ifdef __cplusplus
}
#endif
#endif /* ECMG_H */
