/*
 * host_scene.h -- host copies of the static scene (obstacles, ECM), the
 * acceleration grids built from them, and the host path planner.
 */
#ifndef ECMG_HOST_SCENE_H
#define ECMG_HOST_SCENE_H

#include <vector>
#include "ecmg_geom.cuh"

namespace ecmg {

struct GridCSR {
    float x0 = 0, y0 = 0, cell = 1, inv = 1;
    int gw = 0, gh = 0;
    float reach = 0;
    std::vector<int> start; /* gw*gh + 1 */
    std::vector<int> items;
};

struct HostScene {
    /* obstacles, global (obstacle, vertex) order */
    std::vector<V2> ob_p;
    std::vector<int> ob_next, ob_prev;
    std::vector<unsigned char> ob_convex;
    std::vector<int> ob_ring_off;
    /* ECM */
    std::vector<V2> v_pos;
    std::vector<float> v_clear;
    std::vector<int> v_idx, v_halfedge, he_target, he_next;
    std::vector<V2> he_left, he_right;
    GridCSR ecm_grid;
    std::vector<float> special_y;
    std::vector<int> sp_start, sp_items; /* quads with a corner at special_y[s] */
    std::vector<unsigned> sp_bloom;      /* 2048 words: filter of the special heights */
    /* scene rectangle (ECM and obstacle bounding box) */
    float bx0 = 0, by0 = 0, bx1 = 0, by1 = 0;
    bool has_ecm = false;
    /* planner landmarks: graph distance from each of n_land vertices to
       every vertex, vertex-major [V * n_land] (infinity: not connected) */
    int n_land = 0;
    std::vector<float> land_d;

    EcmView ecm_view() const;
    ObstView obst_view(const GridCSR* g) const;
};

/* Obstacle::Initialize (ECMDataTypes.cpp:23-61): links and convexity */
void set_obstacles(HostScene& s, int n_obst, const int* off, const float* xy);
/* point-location grid + special y list over the ECM cell quads, and the
   planner's landmark distances */
void build_ecm_grid(HostScene& s);
/* candidate lists: every obstacle edge within `reach` of each cell */
void build_obst_grid(const HostScene& s, float reach, float cell, GridCSR& g);

/* working arrays of the reference planner's A* (ref_planner.cpp) */
struct RefPlanScratch {
    std::vector<float> g, f;
    std::vector<int> parent;
    std::vector<unsigned char> visited;
    std::vector<int> heap;
    std::vector<int> touched; /* nodes whose g was set by the current search */
};

struct PlanScratch {
    std::vector<float> g;
    std::vector<int> parent;
    std::vector<int> stamp;
    std::vector<unsigned char> closed;
    std::vector<std::pair<float, int>> open; /* binary min-heap, kept between searches */
    int gen = 0;
    std::vector<unsigned> ob_stamp; /* obstacle edges tested by the current straight-piece check */
    unsigned ob_gen = 0;
    RefPlanScratch ref;
};

/* ECMPathPlanner::FindPath (ECMGenerator/ECMPathPlanner.cpp:22-136) as an
   indicative route: locate and retract start and goal; same edge -> straight
   line; otherwise A* over ECM vertices with the clearance filter of
   AStar::FindPath (AStar.cpp:44-160), then the polyline start, vertices, goal
   is shortened greedily wherever a straight piece keeps `clearance` from every
   obstacle edge.  Returns false when no path exists. */
/* *astar_fail_edge (optional) is set to the start's ECM edge when the search
   itself fails (a property of that edge, the goal and the clearance only),
   else to -1 */
bool plan_path(const HostScene& s, const GridCSR& vis, V2 start, V2 goal, float clearance,
               std::vector<V2>& out, PlanScratch& scr, int* astar_fail_edge = nullptr);

/* ECMPathPlanner::FindPath (ECMPathPlanner.cpp:22-136) restated: the
   reference's A*, corridor, portals and funnel (ref_planner.cpp); the same
   paths as the reference planner */
bool plan_path_reference(const HostScene& s, V2 start, V2 goal, float clearance, std::vector<V2>& out,
                         RefPlanScratch& r, int* astar_fail_edge = nullptr);

}  // namespace ecmg
#endif
