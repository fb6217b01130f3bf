/*
 * ecmg_oracle.h -- CPU oracle for the per-tick crowd update.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * simulator's tick (ECMAgentSimulator/Simulator.cpp:314-323 and everything it
 * calls on the hot path), used by tests/, by __graft_entry__.smoke() and by the
 * cpu_baseline leg of bench.py as the checker.  The product library never links
 * or calls it.
 *
 * Parity is pinned: tests/test_oracle_vs_reference.py runs this file next to
 * the reference's own sources (compiled by oracle/Makefile into oracle/_ref)
 * and requires bit-identical results when both use the host libm, and
 * tests/golden/ holds fixtures produced by the reference itself.
 *
 * Floating point: every expression keeps the reference's operand order; the
 * file is compiled with -ffp-contract=off so nothing is fused.  og_params.libm
 * selects the transcendental source: 1 = the host libm (atanf/sinf/cosf/powf,
 * as the reference), 0 = the deterministic ecmg_tmath.h routines that the CUDA
 * kernels also use (and x*x for powf(x, 2)).
 */
#ifndef ECMG_ORACLE_H
#define ECMG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* The arithmetic type.  float: the restatement (bit for bit the reference).
   Built with -DOG_REAL_DOUBLE (liboracle64.so) the same code computes in
   double with the host libm: the FP64 run that FP32 results are measured
   against. */
#ifdef OG_REAL_DOUBLE
typedef double og_real;
#else
typedef float og_real;
#endif

typedef struct { og_real x, y; } og_v2;

/* Static obstacles, flattened in the reference's global order
   (Environment::GetObstacles() obstacle by obstacle, vertex by vertex). */
typedef struct {
    int n_verts;
    const og_v2* p;              /* ObstacleVertex::p                         */
    const int* next;             /* ObstacleVertex::nextObstacle (index)      */
    const int* prev;             /* ObstacleVertex::prevObstacle (index)      */
    const unsigned char* convex; /* ObstacleVertex::isConvex                  */
} og_obstacles;

/* ECM graph (ECMGenerator/ECM.h:20-50); half-edge h of edge e is 2e+h. */
typedef struct {
    int n_vertices;
    const og_v2* v_pos;     /* ECMVertex::position       */
    const og_real* v_clear;   /* ECMVertex::clearance      */
    const int* v_idx;       /* ECMVertex::idx            */
    const int* v_halfedge;  /* ECMVertex::half_edge_idx  */
    int n_edges;
    const int* he_target;   /* [2E] ECMHalfEdge::v_target_idx */
    const int* he_next;     /* [2E] ECMHalfEdge::next_idx     */
    const og_v2* he_left;   /* [2E] ECMHalfEdge::closest_left */
    const og_v2* he_right;  /* [2E] ECMHalfEdge::closest_right */
} og_ecm;

typedef struct {
    og_real dt;               /* Simulator::m_SimStepTime                      */
    og_real tau_agent;        /* ORCA::m_lookAheadAgent                        */
    og_real tau_obst;         /* ORCA::m_lookAheadObstacle                     */
    og_real neighbor_dist;    /* kNN cut-off radius (exact-kNN mode only)      */
    og_real max_speed;        /* <= 0: LP radius = preferred speed (Simulator.cpp:671) */
    og_real mass;             /* Simulator.cpp:622                             */
    og_real arrival_radius;   /* Simulator.cpp:543                             */
    og_real delete_radius;    /* Simulator.cpp:542                             */
    int k;                  /* ORCA(numNeighbors)                            */
    int knn_mode;           /* 0 = exact kNN (d2,id) within neighbor_dist; 1 = kd-tree as the reference */
    int libm;               /* 1 = host libm transcendentals; 0 = ecmg_tmath.h */
    int threads;            /* >1: split the per-agent stages over threads (exact-kNN mode only) */
    int lp3d_fp64;          /* 1: 3D-LP bisector intersections in double (the GPU's lp3d_fp64 mode) */
} og_params;

/* Slot-indexed agent state (Simulator component arrays). */
typedef struct {
    int n_slots;
    int last_idx;           /* Simulator::m_LastEntityIdx */
    int num_agents;         /* Simulator::m_NumEntities   */
    og_v2* pos;
    og_v2* vel;
    og_v2* attr;            /* attraction points          */
    og_v2* pref_vel;
    og_real* clear;
    og_real* pref_speed;
    unsigned char* active;
    int* path_off;          /* path CSR: agent i owns path_xy[path_off[i] .. +path_len[i]) */
    int* path_len;
    const og_v2* path_xy;
} og_state;

/* Optional per-tick outputs; any pointer may be NULL. */
typedef struct {
    int* destroyed;         /* slots destroyed this tick, in slot order      */
    int n_destroyed;
    int* replan;            /* slots whose IRM query failed, in slot order    */
    og_v2* replan_pos;      /* position used for the replan                   */
    int n_replan;
    int* nbr_ids;           /* [n_slots * k] neighbour list per slot (-1 pad)  */
    int* nbr_count;         /* [n_slots]                                      */
    og_v2* v_orca;          /* [n_slots] LP result                            */
    int* n_constraints;     /* [n_slots]                                      */
    int* n_obst_constraints;/* [n_slots]                                      */
    int* lp_fail;           /* [n_slots] failed index of the 2D LP (== n if none) */
    int n_lp3d;             /* agents that needed the 3D LP                   */
} og_tick_out;

/* kd-tree state of the reference (KDTree.h:57-80) plus ORCA's neighbour cache
   (ORCA.h:100), which the reference carries across agents and ticks. */
typedef struct og_kdtree og_kdtree;

og_kdtree* og_kdtree_create(int k);
void og_kdtree_destroy(og_kdtree* t);
void og_kdtree_build(og_kdtree* t, const og_state* s);
int og_kdtree_query(og_kdtree* t, const og_state* s, int agent, int* out_ids);

/* exact k nearest (d2, id) with EPSILON < d2 < r2; returns the count */
int og_knn_exact(const og_state* s, int agent, int k, og_real r2, int* out_ids, og_real* out_d2);

int og_find_obstacles(const og_obstacles* o, og_v2 pos, og_real range_sq, int* out, int cap, int libm);

/* ORCA constraints + LP + LP3D for one agent with the given neighbour list.
   Returns the number of constraints. */
int og_orca_velocity(const og_obstacles* o, const og_state* s, const og_params* p,
                     int agent, const int* nbrs, int n_nbrs, og_v2 pref_vel,
                     og_v2* out_vel, int* out_n_obst, int* out_fail);

/* half-plane LP of ORCA.cpp:428-587; constraints as (point, normal) quadruples */
int og_lp(const og_real* cons, int n, og_v2 opt, og_real max_speed, int use_dir_opt, og_v2* out);
void og_lp3d(const og_real* cons, int n, int n_obst, og_real max_speed, int failed, og_v2* out);
int og_generate_constraints(const og_obstacles* o, const og_state* s, const og_params* p, int agent,
                            const int* nbrs, int n_nbrs, const int* obst, int n_obst_cand,
                            og_real* cons_out, int cap, int* out_n_obst);

int og_point_location(const og_ecm* e, og_v2 p);
int og_retract(const og_ecm* e, og_v2 p, og_v2* out, int* out_edge);
int og_irm(const og_ecm* e, og_v2 pos, const og_v2* path, int n, og_v2* out);

/* One Simulator::Update.  kd may be NULL unless p->knn_mode == 1. */
int og_tick(const og_obstacles* o, const og_ecm* e, og_state* s, const og_params* p,
            og_kdtree* kd, og_tick_out* out);

/* CPU-baseline timing on a bounded sample: builds the reference kd-tree over
   every active agent (timed as *t_build) and runs the per-agent stages of the
   tick -- IRM attraction point with the linear point location, steering,
   kd-tree kNN, obstacle scan, constraints, LP and LP3D -- for the n_sample
   listed agents on `threads` host threads (timed as *t_agents, seconds).
   State is not modified. */
int og_time_sample(const og_obstacles* o, const og_ecm* e, const og_state* s, const og_params* p,
                   const int* sample, int n_sample, int threads, double* t_build, double* t_agents);

/* One Simulator::Update (exact-kNN mode) for the n_sample listed agents only,
   from the state at the start of the tick, on `threads` host threads; the
   state is not modified.  For sample q: status[q] = 0 (updated), 1 (destroyed
   by the attraction stage), 2 (updated, re-plan flagged) or 3 (not active);
   attr[q] the attraction point after the attraction stage; nbr_ids[q * k ..]
   (-1 padded) and nbr_count[q] its neighbours among the agents active at the
   start of the tick; v_orca[q], vel[q], pos[q] the LP result and the new
   velocity and position.  For parity checks at sizes where a whole-tick
   oracle run would take minutes. */
typedef struct {
    unsigned char* status;
    og_v2* attr;
    int* nbr_ids;
    int* nbr_count;
    og_v2* v_orca;
    og_v2* vel;
    og_v2* pos;
} og_sample_out;

int og_tick_sample(const og_obstacles* o, const og_ecm* e, const og_state* s, const og_params* p,
                   const int* sample, int n_sample, int threads, og_sample_out* out);

/* ECMPathPlanner::FindPath (ECMGenerator/ECMPathPlanner.cpp:22-136) with
   AStar::FindPath (AStar.cpp:44-210), as Simulator::UpdatePath calls it
   (preferred additional clearance 0).  An og_planner holds one thread's A*
   node arrays.  og_find_path writes at most cap points and returns their
   count, -1 when the reference finds no path, -2 when the path has more than
   cap points.  og_find_paths plans n requests on `threads` host threads (out
   holds cap points per request). */
typedef struct og_planner og_planner;
og_planner* og_planner_create(const og_ecm* e);
void og_planner_destroy(og_planner* pl);
int og_find_path(og_planner* pl, og_v2 start, og_v2 goal, og_real clearance, og_v2* out, int cap);
int og_find_paths(const og_ecm* e, int n, const og_v2* starts, const og_v2* goals, const og_real* clr, int threads,
                  int cap, og_v2* out, int* out_n);

/* One Simulator::Update in the reference's kd-tree neighbour mode
   (p->knn_mode is ignored) with the per-agent stages split over `threads`
   host threads: the timed CPU arm of the benchmark.  The kd-tree is built on
   one thread as the reference does; each thread carries its own neighbour
   cache (ORCA.h:100), so stale cache entries are those of its own agents
   rather than of the previous agent in slot order; everything else is
   og_tick's arithmetic.  Destroyed agents and re-plan requests are listed in
   out in slot order; re-plans are left to the caller. */
int og_tick_mt(const og_obstacles* o, const og_ecm* e, og_state* s, const og_params* p, og_kdtree* kd, int threads,
               og_tick_out* out);

#ifdef __cplusplus
}
#endif
#endif
