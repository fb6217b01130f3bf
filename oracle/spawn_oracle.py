"""Python restatement of the reference's spawn areas (test infrastructure only).

It checks the library's spawn stage (ecmg_update_spawn_areas, run at the start
of every ecmg_tick) and never runs on the product path.  It restates, in float32
arithmetic with the reference's operation order:

  * ``Area::GetRandomPositionInArea`` (ECMAgentSimulator/Area.h:39-53): three
    random values per location, the first unused,
    x = xMin + v1 / ((float)RAND_MAX / (xMax - xMin)), y likewise with v2;
  * ``Simulator::ValidSpawnLocation`` (Simulator.cpp:295-311): no active agent
    with diff.LengthSquared() < clearance * clearance;
  * ``Simulator::UpdateSpawnAreas`` (Simulator.cpp:494-536): spawn areas in ID
    order, per connected goal area timeSinceLastSpawn += dt,
    n = (int)(time * rate), per agent up to 10 locations, then the goal's
    location, ``SpawnAgent`` (Simulator.cpp:168-200: LIFO slot, clearanceMin,
    preferredSpeedMin), and time -= (float)n / rate;
  * the area bookkeeping of Simulator.cpp:336-457 (AddSpawnArea, AddGoalArea,
    RemoveArea, ConnectSpawnGoalAreas, DeconnectSpawnGoalAreas), including
    DeconnectSpawnGoalAreas leaving spawnRate / timeSinceLastSpawn untouched.

Deviations, where the reference's behaviour is undefined: a connection to a
goal area that no longer exists gives the goal (0, 0) (the reference
default-constructs an area with indeterminate size); ``plan_ok`` decides
whether a spawn with a valid location gets its agent (the reference keeps an
agent with an empty path when its planner fails; the library refuses it).
The float -> int conversion of the agent count follows x86-64 (INT_MIN for
NaN or out-of-range values).  The restatement is pinned against the reference
compiled in oracle/_ref by tests/test_spawn_oracle.py.
"""
from __future__ import annotations

import numpy as np

F32 = np.float32
INT_MIN = -2147483648


def area_point(px, py, hw, hh, v1, v2, rand_max):
    """Area::GetRandomPositionInArea (Area.h:39-53) with values v1, v2"""
    px, py, hw, hh = F32(px), F32(py), F32(hw), F32(hh)
    x_min, x_max, y_min, y_max = px - hw, px + hw, py - hh, py + hh
    rm = F32(rand_max)
    with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
        x = x_min + F32(v1) / (rm / (x_max - x_min))
        y = y_min + F32(v2) / (rm / (y_max - y_min))
    return F32(x), F32(y)


def spawn_count(x):
    """int agentsToSpawn = time * rate (Simulator.cpp:505), x86-64 conversion"""
    x = F32(x)
    if not (x > F32(-2147483904.0) and x < F32(2147483648.0)):
        return INT_MIN
    return int(x)


def valid_location(loc, clearance, pos, active):
    """Simulator::ValidSpawnLocation (Simulator.cpp:295-311) over arrays"""
    c2 = F32(clearance) * F32(clearance)
    m = np.asarray(active, bool)
    if not m.any():
        return True
    p = np.asarray(pos, F32)[m]
    with np.errstate(over="ignore", invalid="ignore"):
        dx = F32(loc[0]) - p[:, 0]
        dy = F32(loc[1]) - p[:, 1]
        d2 = dx * dx + dy * dy
    return not bool(np.any(d2 < c2))


class Areas:
    """The spawn / goal area members of Simulator (Simulator.h:173-177)."""

    def __init__(self):
        self.spawn = {}  # id -> dict(x, y, hw, hh, cfg, goals, rate, since)
        self.goal = {}   # id -> dict(x, y, hw, hh)
        self.next_spawn = 0
        self.next_goal = 0

    def add_spawn_area(self, x, y, hw, hh, cfg=None, ID=-1):
        """Simulator::AddSpawnArea (Simulator.cpp:336-360); emplace keeps an existing ID"""
        if ID == -1:
            ID = self.next_spawn
            self.next_spawn += 1
        c = dict(preferred_speed_min=5.0, preferred_speed_max=10.0, clearance_min=5.0, clearance_max=10.0)
        c.update(cfg or {})
        if ID not in self.spawn:
            self.spawn[ID] = dict(x=F32(x), y=F32(y), hw=F32(hw), hh=F32(hh),
                                  cfg={k: F32(v) for k, v in c.items()}, goals=[], rate=[], since=[])
        return ID

    def add_goal_area(self, x, y, hw, hh, ID=-1):
        """Simulator::AddGoalArea (Simulator.cpp:362-381)"""
        if ID == -1:
            ID = self.next_goal
            self.next_goal += 1
        if ID not in self.goal:
            self.goal[ID] = dict(x=F32(x), y=F32(y), hw=F32(hw), hh=F32(hh))
        return ID

    def remove_area(self, area_type, ID):
        """Simulator::RemoveArea (Simulator.cpp:414-424): 2 = SPAWN, 3 = GOAL"""
        if area_type == 2:
            self.spawn.pop(ID, None)
        if area_type == 3:
            self.goal.pop(ID, None)

    def connect(self, spawn_id, goal_id, rate=0.0):
        """Simulator::ConnectSpawnGoalAreas (Simulator.cpp:426-438)"""
        a = self.spawn[spawn_id]
        if goal_id in a["goals"]:
            return
        a["goals"].append(goal_id)
        a["since"].append(F32(0.0))
        a["rate"].append(F32(rate))

    def disconnect(self, spawn_id, goal_id):
        """Simulator::DeconnectSpawnGoalAreas (Simulator.cpp:440-457): only
        the goal list loses the entry"""
        if spawn_id < 0 or spawn_id >= len(self.spawn) or spawn_id not in self.spawn:
            return
        g = self.spawn[spawn_id]["goals"]
        if goal_id in g:
            g.remove(goal_id)


def spawn_stage(areas: Areas, pos, active, free_stack, stream, head, dt, rand_max, plan_ok=None):
    """Simulator::UpdateSpawnAreas (Simulator.cpp:494-536).

    pos [n, 2] float32 and active [n] are the agent state at the start of the
    stage (copied, not modified); free_stack is the LIFO slot stack (last
    element = top; popped in place); stream[head:] are the random values still
    to be consumed.  Returns (spawns, head, counts): spawns = list of
    (slot, start, goal, clearance, speed), counts = dict(spawned, failed,
    refused)."""
    pos = np.array(pos, F32, copy=True)
    active = np.array(active, bool, copy=True)
    dt = F32(dt)
    spawns = []
    counts = dict(spawned=0, failed=0, refused=0)

    def triple():
        nonlocal head
        v = stream[head:head + 3]
        if len(v) < 3:
            raise IndexError("random stream exhausted")
        head += 3
        return int(v[1]), int(v[2])

    for sid in sorted(areas.spawn):
        a = areas.spawn[sid]
        for ga in range(len(a["goals"])):
            a["since"][ga] = F32(a["since"][ga] + dt)
            n = spawn_count(a["since"][ga] * a["rate"][ga])
            for _ in range(max(n, 0)):
                clr = a["cfg"]["clearance_min"]
                speed = a["cfg"]["preferred_speed_min"]
                found = False
                start = None
                for _att in range(10):
                    v1, v2 = triple()
                    start = area_point(a["x"], a["y"], a["hw"], a["hh"], v1, v2, rand_max)
                    if valid_location(start, clr, pos, active):
                        found = True
                        break
                if not found:
                    counts["failed"] += 1
                    continue
                v1, v2 = triple()
                g = areas.goal.get(a["goals"][ga])
                goal = area_point(g["x"], g["y"], g["hw"], g["hh"], v1, v2, rand_max) if g else (F32(0), F32(0))
                if not free_stack:
                    counts["refused"] += 1
                    continue
                if plan_ok is not None and not plan_ok(start, goal, clr):
                    counts["refused"] += 1
                    continue
                slot = free_stack.pop()
                pos[slot] = start
                active[slot] = True
                spawns.append((slot, start, goal, clr, speed))
                counts["spawned"] += 1
            with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
                a["since"][ga] = F32(a["since"][ga] - F32(F32(n) / a["rate"][ga]))
    return spawns, head, counts
