/*
 * ref_harness.cpp -- drives the reference simulator's own C++ classes.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
 * the unmodified reference sources (ECMAgentSimulator/*.cpp and
 * ECMGenerator/*.cpp minus ECMGenerator.cpp) into oracle/_ref/libecmref.so.
 * Tests use it to pin the C oracle (ecmg_oracle.c) and to produce the golden
 * fixtures in tests/golden/.
 *
 * Boost.Polygon is absent, so ECMGenerator::GenerateECM (ECMGenerator.cpp:235-256)
 * is replaced here: the ECM graph arrives already built (the same arrays the
 * oracle and the GPU library receive) and is written into ECMGraph's members,
 * after which the reference's own ECMGraph::ConstructECMCells runs.
 *
 * Overrides applied through the reference's members (no source edits):
 * ORCA(k), m_lookAheadAgent/m_lookAheadObstacle, m_SimStepTime, and direct
 * component writes for mass spawning (Simulator.cpp:168-200 minus the O(N)
 * ValidSpawnLocation and the planner call; the path is supplied).
 */
#include "Simulator.h"
#include "KDTree.h"
#include "ORCA.h"
#include "IRMPathFollower.h"
#include "Environment.h"
#include "ECMGenerator.h"
#include "ECM.h"
#include "ECMCellCollection.h"
#include "ECMPathPlanner.h"
#include "UtilityFunctions.h"

#include <cstring>

using namespace ECM;
using namespace ECM::Simulation;

namespace ECM {
/* Environment::ComputeECM/UpdateECM link against this; the harness never
   calls them, the ECM is installed by ref_create. */
ECM* ECMGenerator::GenerateECM(const Environment&, ECM* ecm) { return ecm; }
}

struct RefSim {
    Environment env;
    ECM::ECM* ecm = nullptr;
    PathPlanning::ECMPathPlanner* planner = nullptr;
    Simulator* sim = nullptr;
    int k = 5;
};

extern "C" {

/* obstacles: n_obst rings, ring r = xy[2*off[r] .. 2*off[r+1]) in the
   reference's CCW order; walkable: 4 segments x0,y0,x1,y1.
   ECM: vertex arrays, edge arrays (2 half-edges per edge). */
void* ref_create(int max_agents, float dt, int k, float tau_agent, float tau_obst,
                 int n_obst, const int* off, const float* xy, const float* walk,
                 int n_vert, const float* v_xy, const float* v_clear, const int* v_he,
                 int n_edge, const int* he_target, const int* he_next,
                 const float* he_left, const float* he_right)
{
    RefSim* r = new RefSim();
    std::vector<Segment> wa;
    for (int i = 0; i < 4; i++)
        wa.push_back(Segment(walk[4 * i], walk[4 * i + 1], walk[4 * i + 2], walk[4 * i + 3]));
    r->env.AddWalkableArea(wa);
    for (int o = 0; o < n_obst; o++) {
        std::vector<Point> verts;
        for (int i = off[o]; i < off[o + 1]; i++) verts.push_back(Point(xy[2 * i], xy[2 * i + 1]));
        r->env.AddObstacle(verts);
    }
    r->ecm = new ECM::ECM();
    ECMGraph& g = r->ecm->GetECMGraph();
    for (int i = 0; i < n_vert; i++) {
        ECMVertex* v = g.AddVertex(Point(v_xy[2 * i], v_xy[2 * i + 1]));
        v->clearance = v_clear[i];
        v->half_edge_idx = v_he[i];
    }
    for (int e = 0; e < n_edge; e++) {
        ECMEdge* ed = g.AddEdge();
        for (int h = 0; h < 2; h++) {
            int q = 2 * e + h;
            g.AddHalfEdge(ed->idx, he_target[q], Point(he_left[2 * q], he_left[2 * q + 1]),
                          Point(he_right[2 * q], he_right[2 * q + 1]), (short)h);
            g.m_Edges[e].half_edges[h].next_idx = he_next[q];
        }
    }
    g.ConstructECMCells();
    r->env.m_Ecms.push_back(r->ecm);
    r->planner = new PathPlanning::ECMPathPlanner(&g);
    r->sim = new Simulator(r->ecm, r->planner, &r->env, max_agents, dt);
    r->sim->Initialize();
    delete r->sim->m_ORCA;
    r->sim->m_ORCA = new ORCA(k);
    r->sim->m_ORCA->m_lookAheadAgent = tau_agent;
    r->sim->m_ORCA->m_lookAheadObstacle = tau_obst;
    r->k = k;
    return r;
}

void ref_destroy(void* h)
{
    RefSim* r = (RefSim*)h;
    delete r->sim;
    delete r->planner;
    /* the Environment destructor deletes its ECMs */
    delete r;
}

/* Simulator::SpawnAgent without ValidSpawnLocation and with a given path */
int ref_spawn_direct(void* h, float x, float y, float clearance, float speed, const float* path_xy, int n)
{
    Simulator* s = ((RefSim*)h)->sim;
    if (s->m_freeEntitySpaces.empty() || n <= 0) return -1;
    s->m_NumEntities++;
    int idx = s->m_freeEntitySpaces.top();
    s->m_freeEntitySpaces.pop();
    s->m_LastEntityIdx = s->m_LastEntityIdx < idx ? idx : s->m_LastEntityIdx;
    s->m_Positions[idx].x = x;
    s->m_Positions[idx].y = y;
    s->m_Clearances[idx].clearance = clearance;
    s->m_PreferredSpeed[idx].speed = speed;
    s->m_ActiveAgents[idx] = true;
    PathComponent& pc = s->m_Paths[idx];
    if (pc.numPoints > 0) { delete[] pc.x; delete[] pc.y; }
    pc.x = new float[n];
    pc.y = new float[n];
    pc.numPoints = n;
    pc.currentIndex = 0;
    for (int j = 0; j < n; j++) { pc.x[j] = path_xy[2 * j]; pc.y[j] = path_xy[2 * j + 1]; }
    s->m_PreferredVelocities[idx].dx = 0.0f;
    s->m_PreferredVelocities[idx].dy = 0.0f;
    s->m_Velocities[idx].dx = 0.0f;
    s->m_Velocities[idx].dy = 0.0f;
    s->m_Forces[idx].dx = 0.0f;
    s->m_Forces[idx].dy = 0.0f;
    return idx;
}

/* the reference's own SpawnAgent (ValidSpawnLocation + planner) */
int ref_spawn(void* h, float sx, float sy, float gx, float gy, float clearance, float speed)
{
    return ((RefSim*)h)->sim->SpawnAgent(Point(sx, sy), Point(gx, gy), clearance, speed);
}

void ref_set_path(void* h, int idx, const float* path_xy, int n)
{
    Simulator* s = ((RefSim*)h)->sim;
    PathComponent& pc = s->m_Paths[idx];
    if (pc.numPoints > 0) { delete[] pc.x; delete[] pc.y; }
    pc.x = new float[n];
    pc.y = new float[n];
    pc.numPoints = n;
    pc.currentIndex = 0;
    for (int j = 0; j < n; j++) { pc.x[j] = path_xy[2 * j]; pc.y[j] = path_xy[2 * j + 1]; }
}

int ref_get_path(void* h, int idx, float* out_xy, int cap)
{
    Simulator* s = ((RefSim*)h)->sim;
    PathComponent& pc = s->m_Paths[idx];
    for (int j = 0; j < pc.numPoints && j < cap; j++) { out_xy[2 * j] = pc.x[j]; out_xy[2 * j + 1] = pc.y[j]; }
    return pc.numPoints;
}

/* Simulator::DestroyAgent */
void ref_destroy_agent(void* h, int idx) { ((RefSim*)h)->sim->DestroyAgent(idx); }

/* the unmodified Simulator::Update */
void ref_update(void* h) { Simulator* s = ((RefSim*)h)->sim; s->Update(s->m_SimStepTime); }

/* exact (d2, id) kNN over active agents, d2 as KDTree.cpp:107-108 */
static int exact_knn(Simulator* s, const std::vector<char>& act, int agent, int k, float r2, std::vector<Entity>& out)
{
    std::vector<std::pair<float, int>> c;
    float tx = s->m_Positions[agent].x, ty = s->m_Positions[agent].y;
    for (int j = 0; j <= s->m_LastEntityIdx; j++) {
        if (!act[j]) continue;
        float dx = s->m_Positions[j].x - tx, dy = s->m_Positions[j].y - ty;
        float d2 = dx * dx + dy * dy;
        if (d2 > Utility::EPSILON && d2 < r2) c.push_back(std::make_pair(d2, j));
    }
    std::sort(c.begin(), c.end());
    int n = (int)c.size() < k ? (int)c.size() : k;
    for (int i = 0; i < n; i++) out[i] = c[i].second;
    return n;
}

/* Simulator::Update with the kd-tree kNN replaced by the exact (d2, id) kNN
   within neighbor_dist; every other stage is the reference's own member
   function, called in Update's order (Simulator.cpp:314-323, 611-686). */
void ref_tick_exact(void* h, float neighbor_dist, int* nbr_out, float* vorca_out, int* lp_fail_out, int* n_cons_out)
{
    RefSim* r = (RefSim*)h;
    Simulator* s = r->sim;
    s->UpdateMaxAgentIndex();
    s->UpdateSpawnAreas();
    std::vector<char> act(s->m_MaxNumEntities);
    for (int i = 0; i < s->m_MaxNumEntities; i++) act[i] = s->m_ActiveAgents[i];
    s->UpdateAttractionPointSystem();
    s->ApplySteeringForce();
    ORCA* orca = s->m_ORCA;
    int k = r->k;
    float r2 = neighbor_dist * neighbor_dist;
    std::vector<Entity> nb(k);
    for (int i = 0; i <= s->m_LastEntityIdx; i++) {
        if (!s->m_ActiveAgents[i]) continue;
        const Entity e = s->m_Entities[i];
        float maxSpeed = s->m_PreferredSpeed[i].speed;
        int nn = exact_knn(s, act, e, k, r2, nb);
        std::vector<const ObstacleVertex*> obst;
        float range = orca->m_lookAheadObstacle * maxSpeed + s->GetClearanceData()[e].clearance;
        s->FindNearestObstacles(e, range * range, obst);
        std::vector<Constraint> cons;
        int nObst;
        orca->GenerateConstraints(s, e, nn, nb, obst, s->m_SimStepTime, nObst, cons);
        const VelocityComponent& pv = s->GetPreferredVelocityData()[e];
        Vec2 prefVel(pv.dx, pv.dy);
        Vec2 outVel;
        int failed = orca->RandomizedLP(cons, prefVel, maxSpeed, false, outVel);
        if (failed < (int)cons.size()) orca->RandomizedLP3D(nObst, cons, maxSpeed, failed, outVel);
        s->m_Forces[e].dx = (outVel.x - s->m_Velocities[e].dx);
        s->m_Forces[e].dy = (outVel.y - s->m_Velocities[e].dy);
        if (nbr_out) for (int q = 0; q < k; q++) nbr_out[(size_t)e * k + q] = q < nn ? nb[q] : -1;
        if (vorca_out) { vorca_out[2 * e] = outVel.x; vorca_out[2 * e + 1] = outVel.y; }
        if (lp_fail_out) lp_fail_out[e] = failed;
        if (n_cons_out) n_cons_out[e] = (int)cons.size();
    }
    s->UpdateVelocitySystem();
    s->UpdatePositionSystem();
}

/* component arrays out/in (slot-indexed, n_slots entries) */
void ref_get_state(void* h, float* pos, float* vel, float* attr, float* pref_vel, unsigned char* active,
                   float* clear, float* speed, int* last_idx, int* num_agents)
{
    Simulator* s = ((RefSim*)h)->sim;
    int n = s->m_MaxNumEntities;
    for (int i = 0; i < n; i++) {
        if (pos) { pos[2 * i] = s->m_Positions[i].x; pos[2 * i + 1] = s->m_Positions[i].y; }
        if (vel) { vel[2 * i] = s->m_Velocities[i].dx; vel[2 * i + 1] = s->m_Velocities[i].dy; }
        if (attr) { attr[2 * i] = s->m_AttractionPoints[i].x; attr[2 * i + 1] = s->m_AttractionPoints[i].y; }
        if (pref_vel) { pref_vel[2 * i] = s->m_PreferredVelocities[i].dx; pref_vel[2 * i + 1] = s->m_PreferredVelocities[i].dy; }
        if (active) active[i] = s->m_ActiveAgents[i] ? 1 : 0;
        if (clear) clear[i] = s->m_Clearances[i].clearance;
        if (speed) speed[i] = s->m_PreferredSpeed[i].speed;
    }
    if (last_idx) *last_idx = s->m_LastEntityIdx;
    if (num_agents) *num_agents = s->m_NumEntities;
}

void ref_set_state(void* h, const float* pos, const float* vel, const float* attr)
{
    Simulator* s = ((RefSim*)h)->sim;
    int n = s->m_MaxNumEntities;
    for (int i = 0; i < n; i++) {
        if (pos) { s->m_Positions[i].x = pos[2 * i]; s->m_Positions[i].y = pos[2 * i + 1]; }
        if (vel) { s->m_Velocities[i].dx = vel[2 * i]; s->m_Velocities[i].dy = vel[2 * i + 1]; }
        if (attr) { s->m_AttractionPoints[i].x = attr[2 * i]; s->m_AttractionPoints[i].y = attr[2 * i + 1]; }
    }
}

/* KDTree::Construct + Simulator::FindNNearestNeighbors for every active agent
   in slot order through ORCA's persistent neighbour cache, exactly as
   ORCA::GetVelocity consumes it (ORCA.cpp:18-21). out: [n_slots*k], counts. */
void ref_knn_kdtree(void* h, int* out, int* counts)
{
    RefSim* r = (RefSim*)h;
    Simulator* s = r->sim;
    s->m_KDTree->Construct(s);
    ORCA* orca = s->m_ORCA;
    int k = r->k;
    for (int i = 0; i <= s->m_LastEntityIdx; i++) {
        if (!s->m_ActiveAgents[i]) continue;
        int n = 0;
        s->FindNNearestNeighbors(i, k, orca->m_NeighborCache, n);
        for (int q = 0; q < k; q++) out[(size_t)i * k + q] = orca->m_NeighborCache[q];
        counts[i] = n;
    }
}

int ref_find_obstacles(void* h, int agent, float range_sq, int* out, int cap)
{
    RefSim* r = (RefSim*)h;
    std::vector<const ObstacleVertex*> obst;
    r->sim->FindNearestObstacles(agent, range_sq, obst);
    /* map vertex pointers back to the global (obstacle, vertex) index */
    const std::vector<Obstacle>& os = r->env.GetObstacles();
    int n = 0;
    for (const ObstacleVertex* v : obst) {
        int g = 0, found = -1;
        for (const Obstacle& o : os) {
            for (size_t i = 0; i < o.verts.size(); i++, g++)
                if (o.verts[i] == v) found = g;
        }
        if (n < cap) out[n] = found;
        n++;
    }
    return n;
}

/* ORCA constraints + LP + LP3D for one agent and a given neighbour list.
   cons_out: 4 floats per constraint (point, normal). */
int ref_orca(void* h, int agent, const int* nbrs, int n_nbrs, float max_speed,
             float* out_vel, float* cons_out, int cap, int* n_obst_out, int* fail_out)
{
    RefSim* r = (RefSim*)h;
    Simulator* s = r->sim;
    ORCA* orca = s->m_ORCA;
    std::vector<Entity> nb(nbrs, nbrs + n_nbrs);
    std::vector<const ObstacleVertex*> obst;
    float range = orca->m_lookAheadObstacle * max_speed + s->GetClearanceData()[agent].clearance;
    s->FindNearestObstacles(agent, range * range, obst);
    std::vector<Constraint> cons;
    int nObst;
    orca->GenerateConstraints(s, agent, n_nbrs, nb, obst, s->m_SimStepTime, nObst, cons);
    const VelocityComponent& pv = s->GetPreferredVelocityData()[agent];
    Vec2 prefVel(pv.dx, pv.dy), outVel;
    int failed = orca->RandomizedLP(cons, prefVel, max_speed, false, outVel);
    if (failed < (int)cons.size()) orca->RandomizedLP3D(nObst, cons, max_speed, failed, outVel);
    out_vel[0] = outVel.x;
    out_vel[1] = outVel.y;
    for (int i = 0; i < (int)cons.size() && i < cap; i++) {
        cons_out[4 * i] = cons[i].PointOnLine().x;
        cons_out[4 * i + 1] = cons[i].PointOnLine().y;
        cons_out[4 * i + 2] = cons[i].Normal().x;
        cons_out[4 * i + 3] = cons[i].Normal().y;
    }
    if (n_obst_out) *n_obst_out = nObst;
    if (fail_out) *fail_out = failed;
    return (int)cons.size();
}

/* ORCA::RandomizedLP / RandomizedLP3D on caller-given half-planes */
int ref_lp(void* h, const float* cons, int n, float ox, float oy, float max_speed, int use_dir_opt, float* out)
{
    ORCA* orca = ((RefSim*)h)->sim->m_ORCA;
    std::vector<Constraint> c(n);
    for (int i = 0; i < n; i++) c[i].Init(Point(cons[4 * i], cons[4 * i + 1]), Vec2(cons[4 * i + 2], cons[4 * i + 3]));
    Vec2 o;
    int f = orca->RandomizedLP(c, Vec2(ox, oy), max_speed, use_dir_opt != 0, o);
    out[0] = o.x;
    out[1] = o.y;
    return f;
}

void ref_lp3d(void* h, const float* cons, int n, int n_obst, float max_speed, int failed, float* inout)
{
    ORCA* orca = ((RefSim*)h)->sim->m_ORCA;
    std::vector<Constraint> c(n);
    for (int i = 0; i < n; i++) c[i].Init(Point(cons[4 * i], cons[4 * i + 1]), Vec2(cons[4 * i + 2], cons[4 * i + 3]));
    Vec2 o(inout[0], inout[1]);
    orca->RandomizedLP3D(n_obst, c, max_speed, failed, o);
    inout[0] = o.x;
    inout[1] = o.y;
}

/* ECMGraph::FindCell -> index into the cell list (2e = left, 2e+1 = right) */
int ref_point_location(void* h, float x, float y)
{
    RefSim* r = (RefSim*)h;
    const ECMCell* c = r->ecm->GetECMCell(x, y);
    if (!c) return -1;
    const ECMCell* base = &r->ecm->GetECMGraph().m_Cells->m_ECMCells[0];
    return (int)(c - base);
}

int ref_retract(void* h, float x, float y, float* out, int* edge)
{
    RefSim* r = (RefSim*)h;
    Point o;
    ECMEdge e;
    bool ok = r->ecm->RetractPoint(Point(x, y), o, e);
    out[0] = o.x;
    out[1] = o.y;
    if (edge) *edge = ok ? e.idx : -1;
    return ok ? 1 : 0;
}

int ref_irm(void* h, float x, float y, const float* path_xy, int n, float* out)
{
    RefSim* r = (RefSim*)h;
    PathComponent pc;
    std::vector<float> px(n), py(n);
    for (int i = 0; i < n; i++) { px[i] = path_xy[2 * i]; py[i] = path_xy[2 * i + 1]; }
    pc.x = px.data();
    pc.y = py.data();
    pc.numPoints = n;
    pc.currentIndex = 0;
    Point o;
    IRMPathFollower f;
    bool ok = f.FindAttractionPoint(*r->ecm, r->ecm->GetECMGraph(), Point(x, y), pc, o);
    out[0] = o.x;
    out[1] = o.y;
    return ok ? 1 : 0;
}

/* ECMPathPlanner::FindPath; returns the point count or -1 on failure */
int ref_find_path(void* h, float sx, float sy, float gx, float gy, float clearance, float* out_xy, int cap)
{
    RefSim* r = (RefSim*)h;
    PathPlanning::Corridor cor;
    std::vector<Segment> portals;
    PathPlanning::Path path;
    bool ok = r->planner->FindPath(r->env, Point(sx, sy), Point(gx, gy), clearance, 0.0f, cor, portals, path);
    if (!ok) return -1;
    for (int i = 0; i < (int)path.size() && i < cap; i++) { out_xy[2 * i] = path[i].x; out_xy[2 * i + 1] = path[i].y; }
    return (int)path.size();
}

/* obstacle vertex convexity as computed by Obstacle::Initialize */
void ref_obstacle_convexity(void* h, unsigned char* out)
{
    RefSim* r = (RefSim*)h;
    int g = 0;
    for (const Obstacle& o : r->env.GetObstacles())
        for (size_t i = 0; i < o.verts.size(); i++) out[g++] = o.verts[i]->isConvex ? 1 : 0;
}

/* ---- spawn and goal areas (Simulator.cpp:336-457, 494-536) ------------ */
int ref_add_spawn_area(void* h, float x, float y, float hw, float hh, float speed_min, float speed_max,
                       float clear_min, float clear_max, int id)
{
    SpawnConfiguration cfg;
    cfg.preferredSpeedMin = speed_min;
    cfg.preferredSpeedMax = speed_max;
    cfg.clearanceMin = clear_min;
    cfg.clearanceMax = clear_max;
    return ((RefSim*)h)->sim->AddSpawnArea(Point(x, y), Vec2(hw, hh), cfg, id);
}

int ref_add_goal_area(void* h, float x, float y, float hw, float hh, int id)
{
    return ((RefSim*)h)->sim->AddGoalArea(Point(x, y), Vec2(hw, hh), id);
}

void ref_remove_area(void* h, int type, int id) { ((RefSim*)h)->sim->RemoveArea((SimAreaType)type, id); }
void ref_connect_areas(void* h, int s, int g, float rate) { ((RefSim*)h)->sim->ConnectSpawnGoalAreas(s, g, rate); }
void ref_disconnect_areas(void* h, int s, int g) { ((RefSim*)h)->sim->DeconnectSpawnGoalAreas(s, g); }
/* the reference's UpdateSpawnAreas alone (private, opened by pre.h) */
void ref_update_spawn_areas(void* h) { ((RefSim*)h)->sim->UpdateSpawnAreas(); }
/* the C library's generator the reference draws from */
void ref_srand(unsigned seed) { srand(seed); }
int ref_rand(void) { return rand(); }
int ref_rand_max(void) { return RAND_MAX; }

/* connected goals, rates and timers of a spawn area; returns the size of
   the rate vector, or -1 when the area does not exist */
int ref_spawn_area_state(void* h, int id, int* goals, int* n_goals, float* rates, float* since, int cap)
{
    SpawnArea* a = ((RefSim*)h)->sim->GetSpawnArea(id);
    if (!a) return -1;
    *n_goals = (int)a->connectedGoalAreas.size();
    for (int i = 0; i < *n_goals && i < cap; i++) goals[i] = a->connectedGoalAreas[i];
    for (int i = 0; i < (int)a->spawnRate.size() && i < cap; i++) {
        rates[i] = a->spawnRate[i];
        since[i] = a->timeSinceLastSpawn[i];
    }
    return (int)a->spawnRate.size();
}

/* the top of the free-slot stack (-1 when empty) and its size */
int ref_free_top(void* h, int* size)
{
    Simulator* s = ((RefSim*)h)->sim;
    *size = (int)s->m_freeEntitySpaces.size();
    return s->m_freeEntitySpaces.empty() ? -1 : s->m_freeEntitySpaces.top();
}

} /* extern "C" */
