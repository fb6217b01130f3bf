// Drives the C++ facade (include/ecmg_simulator.hpp) the way the reference's
// application drives ECM::Simulation::Simulator: construct, spawn, Update,
// read the raw component pointers.  Scene: one 4x4 m box in a 40x40 m room,
// with a hand-written ECM (four corridors around the box).
// Exit codes: 0 ok, 2 no CUDA device, 1 failure.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "ecmg_simulator.hpp"

int main(int argc, char** argv)
{
    const int ring_off[2] = {0, 4};
    const float ring[8] = {22, 22, 18, 22, 18, 18, 22, 18}; /* AddObstacleArea order */
    ecmg_obstacles ob{1, ring_off, ring};
    /* medial axis around the box: a square loop of 4 vertices at (9,9)..(31,31)
       joined by 4 edges; closest points: the box on the inside, walls outside */
    const float vpos[8] = {9, 9, 31, 9, 31, 31, 9, 31};
    const float vclr[4] = {9, 9, 9, 9};
    const int vidx[4] = {0, 1, 2, 3};
    const int vhe[4] = {0, 2, 4, 6};
    const int tgt[8] = {1, 0, 2, 1, 3, 2, 0, 3};
    const int nxt[8] = {7, 2, 1, 4, 3, 6, 5, 0};
    /* edge e goes v_e -> v_{e+1} counter-clockwise with the box on its left;
       half-edge 0 stores the closest points at v_e, half-edge 1 (reversed
       direction) those at v_{e+1} (ECMGenerator.cpp:194-195) */
    const float left[16] = {18, 18, 31, 0, 22, 18, 40, 31, 22, 22, 9, 40, 18, 22, 0, 9};
    const float right[16] = {9, 0, 22, 18, 40, 9, 22, 22, 31, 40, 18, 22, 0, 31, 18, 18};
    ecmg_ecm ecm{4, vpos, vclr, vidx, vhe, 4, tgt, nxt, left, right};
    try {
        ecmg_params p;
        ecmg_default_params(&p);
        p.max_neighbors = 4;
        ecmg::Simulator sim(ob, ecm, 16, 1.0f / 60.0f, &p);
        sim.Initialize();
        int a = sim.SpawnAgent({12, 4}, {35, 28}, 0.3f, 1.3f);
        int b = sim.SpawnAgent({28, 36}, {4, 12}, 0.3f, 1.3f);
        if (a != 0 || b != 1) { std::printf("spawn slots %d %d\n", a, b); return 1; }
        if (sim.SpawnAgent({12.1f, 4.0f}, {35, 28}, 0.3f, 1.3f) != -1) { std::printf("overlap accepted\n"); return 1; }
        for (int t = 0; t < 120; t++) sim.Update(1.0f / 60.0f);
        ecmg::PositionComponent* pos = sim.GetPositionData();
        bool* act = sim.GetActiveFlags();
        std::printf("agents %d last %d pos0 %.3f %.3f pos1 %.3f %.3f active %d %d\n", sim.GetNumAgents(),
                    sim.GetLastIndex(), pos[0].x, pos[0].y, pos[1].x, pos[1].y, (int)act[0], (int)act[1]);
        if (!(pos[0].x > 12.5f && pos[0].y > 4.5f && pos[1].x < 27.5f)) return 1;
        sim.DestroyAgent(a);
        if (sim.GetNumAgents() != 1) return 1;
        sim.Reset();
        if (sim.GetNumAgents() != 0) return 1;
        /* spawn areas, as the editor's commands set them up (Command.cpp:31-160) */
        ecmg::SpawnConfiguration cfg;
        cfg.clearanceMin = 0.3f;
        cfg.preferredSpeedMin = 1.2f;
        int sa = sim.AddSpawnArea({12, 4}, {2, 1}, cfg);
        int ga = sim.AddGoalArea({35, 28}, {1, 1});
        sim.ConnectSpawnGoalAreas(sa, ga, 30.0f);
        if (sim.GetConnectedAreas(sa, ecmg::SPAWN).size() != 1 || sim.GetConnectedAreas(ga, ecmg::GOAL).size() != 1)
            return 1;
        long long refused = 0, failed = 0;
        for (int t = 0; t < 60; t++) {
            sim.Update(1.0f / 60.0f);
            refused += sim.LastTickStats().spawn_refused;
            failed += sim.LastTickStats().spawn_failed;
        }
        std::printf("spawned agents %d (no location %lld, refused %lld)\n", sim.GetNumAgents(), failed, refused);
        if (sim.GetNumAgents() < 10) return 1;
        sim.DeconnectSpawnGoalAreas(sa, ga);
        if (!sim.GetConnectedAreas(sa, ecmg::SPAWN).empty()) return 1;
        sim.RemoveArea(ecmg::SPAWN, sa);
    } catch (const std::runtime_error& e) {
        std::string m = e.what();
        std::printf("%s\n", m.c_str());
        return m.find("ecmg_create") != std::string::npos ? 2 : 1;
    }
    return 0;
}
