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
 * the library's host planner unless SetPlanner() installs another one (e.g. a
 * wrapper around the reference's ECMPathPlanner::FindPath).
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
        m_Pos.resize(maxAgents);
        m_Vel.resize(maxAgents);
        m_PrefVel.resize(maxAgents);
        m_Attr.resize(maxAgents);
        m_Clear.resize(maxAgents);
        m_Speed.resize(maxAgents);
        m_Active.resize(maxAgents);
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
        m_Dirty = true;
        return slot;
    }
    void DestroyAgent(int idx)
    {
        check(ecmg_destroy_agent(m_Ctx, idx), "ecmg_destroy_agent");
        m_Dirty = true;
    }
    /* like the reference, the argument is ignored in favour of the step time */
    void Update(float /*dt*/)
    {
        check(ecmg_tick(m_Ctx, 1, &m_Stats), "ecmg_tick");
        m_Dirty = true;
    }
    void Reset()
    {
        check(ecmg_reset(m_Ctx), "ecmg_reset");
        m_Dirty = true;
    }
    void SetPlanner(ecmg_plan_fn fn, void* user) { check(ecmg_set_planner(m_Ctx, fn, user), "ecmg_set_planner"); }

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
    PositionComponent* GetPositionData() { sync(); return m_Pos.data(); }
    VelocityComponent* GetVelocityData() { sync(); return m_Vel.data(); }
    VelocityComponent* GetPreferredVelocityData() { sync(); return m_PrefVel.data(); }
    PositionComponent* GetAttractionPointData() { sync(); return m_Attr.data(); }
    ClearanceComponent* GetClearanceData() { sync(); return m_Clear.data(); }
    SpeedComponent* GetSpeedData() { sync(); return m_Speed.data(); }
    bool* GetActiveFlags() { sync(); return reinterpret_cast<bool*>(m_Active.data()); }
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
    void sync()
    {
        if (!m_Dirty) return;
        check(ecmg_get_state(m_Ctx, ECMG_FIELD_POSITION, m_Pos.data()), "get position");
        check(ecmg_get_state(m_Ctx, ECMG_FIELD_VELOCITY, m_Vel.data()), "get velocity");
        check(ecmg_get_state(m_Ctx, ECMG_FIELD_PREF_VELOCITY, m_PrefVel.data()), "get preferred velocity");
        check(ecmg_get_state(m_Ctx, ECMG_FIELD_ATTRACTION, m_Attr.data()), "get attraction");
        check(ecmg_get_state(m_Ctx, ECMG_FIELD_CLEARANCE, m_Clear.data()), "get clearance");
        check(ecmg_get_state(m_Ctx, ECMG_FIELD_SPEED, m_Speed.data()), "get speed");
        check(ecmg_get_state(m_Ctx, ECMG_FIELD_ACTIVE, m_Active.data()), "get active");
        m_Dirty = false;
    }

    ecmg_ctx* m_Ctx = nullptr;
    int m_Max;
    bool m_Dirty = true;
    ecmg_tick_stats m_Stats{};
    std::vector<PositionComponent> m_Pos, m_Attr;
    std::vector<VelocityComponent> m_Vel, m_PrefVel;
    std::vector<ClearanceComponent> m_Clear;
    std::vector<SpeedComponent> m_Speed;
    std::vector<std::uint8_t> m_Active;
};

}  // namespace ecmg
#endif
