/*
 * ecmg_simulator.hpp -- header-only C++17 facade with the public surface of
 * ECM::Simulation::Simulator (ECMAgentSimulator/Simulator.h:59-188), forwarding
 * to the C ABI of libecmg.so.  A caller of the reference class swaps the
 * include and the type name; component getters keep returning raw host
 * pointers (Simulator.h:114-126), which are host mirrors refreshed lazily after
 * each Update(), so renderer-style readers work unchanged.
 *
 * Scene input: the reference hands the Simulator an ECM, a planner and an
 * Environment (Simulator.h:63).  Here the constructor takes the flattened
 * obstacle rings and ECM graph (ecmg_obstacles / ecmg_ecm); path planning uses
 * the library's restatement of the reference planner (ECMG_PLANNER_REFERENCE,
 * the reference's paths) unless SetPlanner() installs another one.
 */
#ifndef ECMG_SIMULATOR_HPP
#define ECMG_SIMULATOR_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "ecmg.h"

namespace ecmg {

struct Point {
    float x = 0, y = 0;
};
struct Vec2 {
    float x = 0, y = 0;
};
/* Area.h:11-18, 82-88 */
enum SimAreaType { NONE, WALKABLE, SPAWN, GOAL, OBSTACLE };
struct SpawnConfiguration {
    float preferredSpeedMin = 5.0f;
    float preferredSpeedMax = 10.0f;
    float clearanceMin = 5.0f;
    float clearanceMax = 10.0f;
};
/* component layouts of Simulator.h:29-49 */
struct PositionComponent {
    float x, y;
};
struct VelocityComponent {
    float dx, dy;
};
struct ClearanceComponent {
    float clearance;
};
struct SpeedComponent {
    float speed;
};

class Simulator {
public:
    /* Simulator(ecm, planner, environment, maxAgents, simStepTime) */
    Simulator(const ecmg_obstacles& obstacles, const ecmg_ecm& ecm, int maxAgents, float simStepTime,
              const ecmg_params* params = nullptr)
        : m_Max(maxAgents)
    {
        ecmg_params p;
        if (params) p = *params;
        else ecmg_default_params(&p);
        p.dt = simStepTime;
        check(ecmg_create(&p, maxAgents, &m_Ctx), "ecmg_create");
        check(ecmg_set_obstacles(m_Ctx, &obstacles), "ecmg_set_obstacles");
        check(ecmg_set_ecm(m_Ctx, &ecm), "ecmg_set_ecm");
        /* spawns and re-plans get the reference planner's paths */
        check(ecmg_set_planner_mode(m_Ctx, ECMG_PLANNER_REFERENCE), "ecmg_set_planner_mode");
    }
    ~Simulator()
    {
        if (m_Ctx) ecmg_destroy(m_Ctx);
    }
    Simulator(const Simulator&) = delete;
    Simulator& operator=(const Simulator&) = delete;

    void Initialize() {} /* storage is created by the constructor */

    /* returns the slot, or -1 (no slot / occupied / no path) as the reference */
    int SpawnAgent(const Point& start, const Point& goal, float clearance, float preferredSpeed)
    {
        int slot = -1;
        ecmg_status s = ecmg_spawn_agent(m_Ctx, start.x, start.y, goal.x, goal.y, clearance, preferredSpeed, &slot);
        if (s == ECMG_ERR_NO_SLOT || s == ECMG_ERR_INVALID_SPAWN || s == ECMG_ERR_NO_PATH) return -1;
        check(s, "ecmg_spawn_agent");
        m_Dirty = 0x7fu;
        return slot;
    }
    void DestroyAgent(int idx)
    {
        check(ecmg_destroy_agent(m_Ctx, idx), "ecmg_destroy_agent");
        m_Dirty = 0x7fu;
    }
    /* like the reference, the argument is ignored in favour of the step time */
    void Update(float /*dt*/)
    {
        check(ecmg_tick(m_Ctx, 1, &m_Stats), "ecmg_tick");
        m_Dirty = 0x7fu;
    }
    void Reset()
    {
        check(ecmg_reset(m_Ctx), "ecmg_reset");
        m_Dirty = 0x7fu;
    }
    void SetPlanner(ecmg_plan_fn fn, void* user) { check(ecmg_set_planner(m_Ctx, fn, user), "ecmg_set_planner"); }
    /* re-plan searches overlapping the next Update (ecmg_set_replan_overlap:
       1 default, when a search outlasts its tick; 2 always; 0 never) */
    void SetReplanOverlap(int mode) { check(ecmg_set_replan_overlap(m_Ctx, mode), "ecmg_set_replan_overlap"); }
    /* positions and velocities written to the getters' host arrays by every
       Update (ecmg_set_host_mirror) */
    void SetHostMirror(bool on) { check(ecmg_set_host_mirror(m_Ctx, on ? 1 : 0), "ecmg_set_host_mirror"); }

    /* spawn / goal areas (Simulator.h:92-104); Update() runs their spawn stage */
    int AddSpawnArea(const Point& position, const Vec2& halfSize, const SpawnConfiguration& config, int ID = -1)
    {
        ecmg_spawn_config c{config.preferredSpeedMin, config.preferredSpeedMax, config.clearanceMin,
                            config.clearanceMax};
        int id = -1;
        check(ecmg_add_spawn_area(m_Ctx, position.x, position.y, halfSize.x, halfSize.y, &c, ID, &id),
              "ecmg_add_spawn_area");
        return id;
    }
    int AddGoalArea(const Point& position, const Vec2& halfSize, int ID = -1)
    {
        int id = -1;
        check(ecmg_add_goal_area(m_Ctx, position.x, position.y, halfSize.x, halfSize.y, ID, &id), "ecmg_add_goal_area");
        return id;
    }
    void RemoveArea(SimAreaType areaType, int ID) { check(ecmg_remove_area(m_Ctx, (int)areaType, ID), "ecmg_remove_area"); }
    void ConnectSpawnGoalAreas(int spawnID, int goalID, float spawnRate = 0.0f)
    {
        check(ecmg_connect_areas(m_Ctx, spawnID, goalID, spawnRate), "ecmg_connect_areas");
    }
    void DeconnectSpawnGoalAreas(int spawnID, int goalID)
    {
        check(ecmg_disconnect_areas(m_Ctx, spawnID, goalID), "ecmg_disconnect_areas");
    }
    /* SPAWN: the goal areas a spawn area feeds; GOAL: the spawn areas that
       feed a goal area (Simulator.cpp:126-166 intends this; its GOAL branch
       compares goal IDs by list position) */
    std::vector<int> GetConnectedAreas(int sourceID, SimAreaType type) const
    {
        std::vector<int> out;
        ecmg_area_info info;
        if (type == SPAWN) {
            if (ecmg_get_area(m_Ctx, ECMG_AREA_SPAWN, sourceID, &info, nullptr, nullptr, nullptr, 0) != ECMG_OK)
                return out;
            out.resize(info.n_connected);
            ecmg_get_area(m_Ctx, ECMG_AREA_SPAWN, sourceID, &info, out.data(), nullptr, nullptr, info.n_connected);
            return out;
        }
        if (type == GOAL) {
            if (ecmg_get_area(m_Ctx, ECMG_AREA_GOAL, sourceID, &info, nullptr, nullptr, nullptr, 0) != ECMG_OK)
                return out;
            int n = 0;
            ecmg_area_ids(m_Ctx, ECMG_AREA_SPAWN, nullptr, 0, &n);
            std::vector<int> ids(n);
            ecmg_area_ids(m_Ctx, ECMG_AREA_SPAWN, ids.data(), n, &n);
            for (int id : ids)
                for (int g : GetConnectedAreas(id, SPAWN))
                    if (g == sourceID) {
                        out.push_back(id);
                        break;
                    }
        }
        return out;
    }

    int GetNumAgents() const
    {
        int n = 0;
        ecmg_get_counts(m_Ctx, &n, nullptr, nullptr);
        return n;
    }
    int GetLastIndex() const
    {
        int n = -1;
        ecmg_get_counts(m_Ctx, nullptr, &n, nullptr);
        return n;
    }
    /* raw host pointers as the reference returns them: library-owned host
       copies, refreshed on the first call after the state changed */
    PositionComponent* GetPositionData() { return static_cast<PositionComponent*>(view(ECMG_FIELD_POSITION)); }
    VelocityComponent* GetVelocityData() { return static_cast<VelocityComponent*>(view(ECMG_FIELD_VELOCITY)); }
    VelocityComponent* GetPreferredVelocityData()
    {
        return static_cast<VelocityComponent*>(view(ECMG_FIELD_PREF_VELOCITY));
    }
    PositionComponent* GetAttractionPointData() { return static_cast<PositionComponent*>(view(ECMG_FIELD_ATTRACTION)); }
    ClearanceComponent* GetClearanceData() { return static_cast<ClearanceComponent*>(view(ECMG_FIELD_CLEARANCE)); }
    SpeedComponent* GetSpeedData() { return static_cast<SpeedComponent*>(view(ECMG_FIELD_SPEED)); }
    bool* GetActiveFlags() { return static_cast<bool*>(view(ECMG_FIELD_ACTIVE)); }
    float GetSimulationStepTime() const
    {
        ecmg_params p;
        ecmg_get_params(m_Ctx, &p);
        return p.dt;
    }
    const ecmg_tick_stats& LastTickStats() const { return m_Stats; }
    ecmg_ctx* Handle() const { return m_Ctx; }

private:
    void check(ecmg_status s, const char* what) const
    {
        if (s != ECMG_OK)
            throw std::runtime_error(std::string(what) + ": " + (m_Ctx ? ecmg_last_error(m_Ctx) : "no context"));
    }
    void* view(int field)
    {
        if (m_Dirty & (1u << field)) {
            const void* p = nullptr;
            check(ecmg_host_view(m_Ctx, field, &p), "ecmg_host_view");
            m_View[field] = const_cast<void*>(p);
            m_Dirty &= ~(1u << field);
        }
        return m_View[field];
    }

    ecmg_ctx* m_Ctx = nullptr;
    int m_Max;
    unsigned m_Dirty = 0x7fu; /* one bit per ECMG_FIELD_* */
    void* m_View[7] = {};
    ecmg_tick_stats m_Stats{};
};

}  // namespace ecmg
#endif
