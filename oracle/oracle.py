"""ctypes bindings for the CPU oracle (test infrastructure only).

``Port``  wraps oracle/_build/liboracle.so, the C restatement (ecmg_oracle.c).
``Ref``   wraps oracle/_ref/libecmref.so, the reference's own C++ sources
          compiled with ref_harness.cpp; it exists only where the reference
          tree was available at build time.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "liboracle.so")
PORT64_SO = os.path.join(HERE, "_build", "liboracle64.so")
REF_SO = os.path.join(HERE, "_ref", "libecmref.so")

F32, I32, U8 = np.float32, np.int32, np.uint8


def build(ref: bool = False, ref_tree: str | None = None) -> None:
    """Compile the C restatement (and the reference, when its sources exist;
    ref_tree overrides the Makefile's default location of the source tree)."""
    targets = ["oracle"]
    if ref:
        targets.append("ref")
    extra = [f"REF={ref_tree}"] if ref and ref_tree else []
    subprocess.run(["make", "-s", "-C", HERE] + targets + extra, check=True)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


class V2(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


class Obst(C.Structure):
    _fields_ = [("n_verts", C.c_int), ("p", C.c_void_p), ("next", C.c_void_p),
                ("prev", C.c_void_p), ("convex", C.c_void_p)]


class EcmS(C.Structure):
    _fields_ = [("n_vertices", C.c_int), ("v_pos", C.c_void_p), ("v_clear", C.c_void_p),
                ("v_idx", C.c_void_p), ("v_halfedge", C.c_void_p), ("n_edges", C.c_int),
                ("he_target", C.c_void_p), ("he_next", C.c_void_p), ("he_left", C.c_void_p),
                ("he_right", C.c_void_p)]


class Params64(C.Structure):
    _fields_ = [("dt", C.c_double), ("tau_agent", C.c_double), ("tau_obst", C.c_double),
                ("neighbor_dist", C.c_double), ("max_speed", C.c_double), ("mass", C.c_double),
                ("arrival_radius", C.c_double), ("delete_radius", C.c_double), ("k", C.c_int),
                ("knn_mode", C.c_int), ("libm", C.c_int), ("threads", C.c_int), ("lp3d_fp64", C.c_int)]


class Params(C.Structure):
    _fields_ = [("dt", C.c_float), ("tau_agent", C.c_float), ("tau_obst", C.c_float),
                ("neighbor_dist", C.c_float), ("max_speed", C.c_float), ("mass", C.c_float),
                ("arrival_radius", C.c_float), ("delete_radius", C.c_float), ("k", C.c_int),
                ("knn_mode", C.c_int), ("libm", C.c_int), ("threads", C.c_int), ("lp3d_fp64", C.c_int)]


class State(C.Structure):
    _fields_ = [("n_slots", C.c_int), ("last_idx", C.c_int), ("num_agents", C.c_int),
                ("pos", C.c_void_p), ("vel", C.c_void_p), ("attr", C.c_void_p), ("pref_vel", C.c_void_p),
                ("clear", C.c_void_p), ("pref_speed", C.c_void_p), ("active", C.c_void_p),
                ("path_off", C.c_void_p), ("path_len", C.c_void_p), ("path_xy", C.c_void_p)]


class TickOut(C.Structure):
    _fields_ = [("destroyed", C.c_void_p), ("n_destroyed", C.c_int), ("replan", C.c_void_p),
                ("replan_pos", C.c_void_p), ("n_replan", C.c_int), ("nbr_ids", C.c_void_p),
                ("nbr_count", C.c_void_p), ("v_orca", C.c_void_p), ("n_constraints", C.c_void_p),
                ("n_obst_constraints", C.c_void_p), ("lp_fail", C.c_void_p), ("n_lp3d", C.c_int)]


class SampleOut(C.Structure):
    _fields_ = [("status", C.c_void_p), ("attr", C.c_void_p), ("nbr_ids", C.c_void_p), ("nbr_count", C.c_void_p),
                ("v_orca", C.c_void_p), ("vel", C.c_void_p), ("pos", C.c_void_p)]


def _addr(a):
    return a.ctypes.data if a is not None else None


class Port:
    """The C restatement.  Holds numpy-owned state mirrored to C structs."""

    REAL = F32

    def __init__(self, so=PORT_SO):
        if not os.path.exists(so):
            build()
        self.lib = C.CDLL(so)
        L = self.lib
        L.og_tick.restype = C.c_int
        L.og_point_location.restype = C.c_int
        L.og_point_location.argtypes = [C.POINTER(EcmS), V2]
        L.og_retract.argtypes = [C.POINTER(EcmS), V2, C.POINTER(V2), C.POINTER(C.c_int)]
        L.og_irm.argtypes = [C.POINTER(EcmS), V2, C.c_void_p, C.c_int, C.POINTER(V2)]
        L.og_find_obstacles.argtypes = [C.POINTER(Obst), V2, C.c_float, C.c_void_p, C.c_int, C.c_int]
        L.og_knn_exact.argtypes = [C.POINTER(State), C.c_int, C.c_int, C.c_float, C.c_void_p, C.c_void_p]
        L.og_lp.argtypes = [C.c_void_p, C.c_int, V2, C.c_float, C.c_int, C.POINTER(V2)]
        L.og_lp3d.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_int, C.POINTER(V2)]
        L.og_orca_velocity.argtypes = [C.POINTER(Obst), C.POINTER(State), C.POINTER(Params), C.c_int,
                                       C.c_void_p, C.c_int, V2, C.POINTER(V2), C.POINTER(C.c_int),
                                       C.POINTER(C.c_int)]
        L.og_kdtree_create.restype = C.c_void_p
        L.og_kdtree_create.argtypes = [C.c_int]
        L.og_kdtree_destroy.argtypes = [C.c_void_p]
        L.og_kdtree_build.argtypes = [C.c_void_p, C.POINTER(State)]
        L.og_kdtree_query.argtypes = [C.c_void_p, C.POINTER(State), C.c_int, C.c_void_p]
        L.og_tick.argtypes = [C.POINTER(Obst), C.POINTER(EcmS), C.POINTER(State), C.POINTER(Params),
                              C.c_void_p, C.POINTER(TickOut)]

    # -- structs ---------------------------------------------------------
    def obstacles(self, scene):
        keep = [np.ascontiguousarray(scene.obst_xy, self.REAL), np.ascontiguousarray(scene.obst_next, I32),
                np.ascontiguousarray(scene.obst_prev, I32), np.ascontiguousarray(scene.obst_convex, U8)]
        o = Obst(int(keep[0].shape[0]), *[_addr(a) for a in keep])
        o._keep = keep
        return o

    def ecm(self, e):
        R = self.REAL
        keep = [np.ascontiguousarray(e.v_pos, R), np.ascontiguousarray(e.v_clear, R),
                np.ascontiguousarray(e.v_idx, I32), np.ascontiguousarray(e.v_halfedge, I32),
                np.ascontiguousarray(e.he_target, I32), np.ascontiguousarray(e.he_next, I32),
                np.ascontiguousarray(e.he_left, R), np.ascontiguousarray(e.he_right, R)]
        s = EcmS(e.n_vertices, _addr(keep[0]), _addr(keep[1]), _addr(keep[2]), _addr(keep[3]),
                 e.n_edges, _addr(keep[4]), _addr(keep[5]), _addr(keep[6]), _addr(keep[7]))
        s._keep = keep
        return s

    @staticmethod
    def params(**kw):
        d = dict(dt=1.0 / 60.0, tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0, max_speed=0.0, mass=0.8,
                 arrival_radius=20.0, delete_radius=2.0, k=10, knn_mode=0, libm=0, threads=1, lp3d_fp64=0)
        d.update(kw)
        return Params(**d)

    def state(self, st):
        """st: AgentState (numpy arrays, see ecmgenerator_gb300.agents)."""
        s = State(st.n_slots, st.last_idx, st.num_agents, _addr(st.pos), _addr(st.vel), _addr(st.attr),
                  _addr(st.pref_vel), _addr(st.clear), _addr(st.pref_speed), _addr(st.active),
                  _addr(st.path_off), _addr(st.path_len), _addr(st.path_xy))
        return s

    # -- queries ---------------------------------------------------------
    def point_location(self, ecm_s, x, y):
        return self.lib.og_point_location(C.byref(ecm_s), V2(x, y))

    def retract(self, ecm_s, x, y):
        o = V2()
        ed = C.c_int(-1)
        ok = self.lib.og_retract(C.byref(ecm_s), V2(x, y), C.byref(o), C.byref(ed))
        return bool(ok), (o.x, o.y), ed.value

    def irm(self, ecm_s, x, y, path):
        path = np.ascontiguousarray(path, F32)
        o = V2(0.0, 0.0)
        ok = self.lib.og_irm(C.byref(ecm_s), V2(x, y), _addr(path), int(path.shape[0]), C.byref(o))
        return bool(ok), (o.x, o.y)

    def find_obstacles(self, obst_s, x, y, range_sq, libm=0, cap=256):
        out = np.zeros(cap, I32)
        n = self.lib.og_find_obstacles(C.byref(obst_s), V2(x, y), C.c_float(range_sq), _addr(out), cap, libm)
        return out[:min(n, cap)].copy()

    def lp(self, cons, opt, max_speed, use_dir_opt=0):
        cons = np.ascontiguousarray(cons, F32).reshape(-1, 4)
        o = V2()
        f = self.lib.og_lp(_addr(cons), int(cons.shape[0]), V2(*opt), C.c_float(max_speed), use_dir_opt, C.byref(o))
        return f, (o.x, o.y)

    def lp3d(self, cons, n_obst, max_speed, failed, start):
        cons = np.ascontiguousarray(cons, F32).reshape(-1, 4)
        o = V2(*start)
        self.lib.og_lp3d(_addr(cons), int(cons.shape[0]), n_obst, C.c_float(max_speed), failed, C.byref(o))
        return (o.x, o.y)

    def tick(self, obst_s, ecm_s, st, params, kd=None, record=True, k=None):
        """One Simulator::Update on ``st`` (modified in place).  Returns a dict
        of the per-tick outputs."""
        s = self.state(st)
        n = st.n_slots
        k = params.k if k is None else k
        R = self.REAL
        for f in ("pos", "vel", "attr", "pref_vel", "clear", "pref_speed", "path_xy"):
            assert getattr(st, f).dtype == R, f"state array {f} must be {np.dtype(R).name}"
        res = dict(destroyed=np.zeros(n, I32), replan=np.zeros(n, I32), replan_pos=np.zeros((n, 2), R))
        if record:
            res.update(nbr_ids=np.full((n, max(k, 1)), -1, I32), nbr_count=np.zeros(n, I32),
                       v_orca=np.zeros((n, 2), R), n_constraints=np.zeros(n, I32),
                       n_obst_constraints=np.zeros(n, I32), lp_fail=np.zeros(n, I32))
        out = TickOut(_addr(res["destroyed"]), 0, _addr(res["replan"]), _addr(res["replan_pos"]), 0,
                      _addr(res.get("nbr_ids")), _addr(res.get("nbr_count")), _addr(res.get("v_orca")),
                      _addr(res.get("n_constraints")), _addr(res.get("n_obst_constraints")),
                      _addr(res.get("lp_fail")), 0)
        self.lib.og_tick(C.byref(obst_s), C.byref(ecm_s), C.byref(s), C.byref(params), kd, C.byref(out))
        st.last_idx = s.last_idx
        st.num_agents = s.num_agents
        res["destroyed"] = res["destroyed"][:out.n_destroyed].copy()
        res["replan"] = res["replan"][:out.n_replan].copy()
        res["replan_pos"] = res["replan_pos"][:out.n_replan].copy()
        res["n_lp3d"] = out.n_lp3d
        return res

    def kdtree(self, k):
        return self.lib.og_kdtree_create(k)

    def find_paths(self, ecm_s, starts, goals, clearances, threads=1, cap=256):
        """ECMPathPlanner::FindPath restated (og_find_paths) for n requests on
        `threads` host threads: a list of (m, 2) arrays, None where the
        reference finds no path (or the path has more than cap points)."""
        L = self.lib
        L.og_find_paths.argtypes = [C.POINTER(EcmS), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                    C.c_int, C.c_void_p, C.c_void_p]
        R = self.REAL
        starts = np.ascontiguousarray(np.asarray(starts).reshape(-1, 2), R)
        goals = np.ascontiguousarray(np.asarray(goals).reshape(-1, 2), R)
        clr = np.ascontiguousarray(clearances, R)
        n = starts.shape[0]
        out = np.zeros((n, cap, 2), R)
        cnt = np.zeros(n, I32)
        L.og_find_paths(C.byref(ecm_s), n, _addr(starts), _addr(goals), _addr(clr), int(threads), int(cap),
                        _addr(out), _addr(cnt))
        return [out[i, :cnt[i]].copy() if cnt[i] > 0 else None for i in range(n)]

    def tick_mt(self, obst_s, ecm_s, st, params, kd, threads):
        """One Simulator::Update in the kd-tree mode on `threads` host threads
        (og_tick_mt; ``st`` modified in place): destroyed slots and re-plan
        requests (slots, positions)."""
        L = self.lib
        L.og_tick_mt.argtypes = [C.POINTER(Obst), C.POINTER(EcmS), C.POINTER(State), C.POINTER(Params),
                                 C.c_void_p, C.c_int, C.POINTER(TickOut)]
        s = self.state(st)
        n = st.n_slots
        res = dict(destroyed=np.zeros(n, I32), replan=np.zeros(n, I32), replan_pos=np.zeros((n, 2), self.REAL))
        out = TickOut(_addr(res["destroyed"]), 0, _addr(res["replan"]), _addr(res["replan_pos"]), 0,
                      None, None, None, None, None, None, 0)
        L.og_tick_mt(C.byref(obst_s), C.byref(ecm_s), C.byref(s), C.byref(params), kd, int(threads), C.byref(out))
        st.last_idx = s.last_idx
        st.num_agents = s.num_agents
        return (res["destroyed"][:out.n_destroyed].copy(), res["replan"][:out.n_replan].copy(),
                res["replan_pos"][:out.n_replan].copy(), out.n_lp3d)

    def tick_sample(self, obst_s, ecm_s, st, params, sample, threads=1):
        """One exact-kNN tick for the listed slots only, from ``st`` (not
        modified); see og_tick_sample.  Returns a dict of per-sample arrays."""
        L = self.lib
        L.og_tick_sample.argtypes = [C.POINTER(Obst), C.POINTER(EcmS), C.POINTER(State), C.POINTER(Params),
                                     C.c_void_p, C.c_int, C.c_int, C.POINTER(SampleOut)]
        sample = np.ascontiguousarray(sample, I32)
        m, k = int(sample.shape[0]), max(int(params.k), 1)
        res = dict(status=np.zeros(m, U8), attr=np.zeros((m, 2), F32), nbr_ids=np.full((m, k), -1, I32),
                   nbr_count=np.zeros(m, I32), v_orca=np.zeros((m, 2), F32), vel=np.zeros((m, 2), F32),
                   pos=np.zeros((m, 2), F32))
        out = SampleOut(*[_addr(res[f]) for f in ("status", "attr", "nbr_ids", "nbr_count", "v_orca", "vel", "pos")])
        s = self.state(st)
        L.og_tick_sample(C.byref(obst_s), C.byref(ecm_s), C.byref(s), C.byref(params), _addr(sample), m,
                         int(threads), C.byref(out))
        return res

    def time_sample(self, obst_s, ecm_s, st, params, sample, threads=1):
        """Seconds spent building the kd-tree and running the per-agent tick
        stages for ``sample`` (see og_time_sample)."""
        L = self.lib
        L.og_time_sample.argtypes = [C.POINTER(Obst), C.POINTER(EcmS), C.POINTER(State), C.POINTER(Params),
                                     C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        sample = np.ascontiguousarray(sample, I32)
        s = self.state(st)
        tb, ta = C.c_double(), C.c_double()
        L.og_time_sample(C.byref(obst_s), C.byref(ecm_s), C.byref(s), C.byref(params), _addr(sample),
                         int(sample.shape[0]), int(threads), C.byref(tb), C.byref(ta))
        return tb.value, ta.value


class Port64(Port):
    """The same restatement computing in double with the host libm
    (liboracle64.so, built with -DOG_REAL_DOUBLE): the FP64 run that the FP32
    tick is measured against.  Its states hold float64 arrays (as_f64)."""

    REAL = np.float64

    def __init__(self):
        super().__init__(PORT64_SO)
        self.lib.og_tick.argtypes = [C.POINTER(Obst), C.POINTER(EcmS), C.POINTER(State), C.POINTER(Params64),
                                     C.c_void_p, C.POINTER(TickOut)]

    @staticmethod
    def params(**kw):
        d = dict(dt=1.0 / 60.0, tau_agent=2.0, tau_obst=2.0, neighbor_dist=5.0, max_speed=0.0, mass=0.8,
                 arrival_radius=20.0, delete_radius=2.0, k=10, knn_mode=0, libm=1, threads=1)
        d.update(kw)
        assert d["libm"] == 1, "the FP64 run uses the host libm"
        return Params64(**d)

    @staticmethod
    def as_f64(st):
        c = st.copy()
        for f in ("pos", "vel", "attr", "pref_vel", "clear", "pref_speed", "path_xy"):
            setattr(c, f, np.ascontiguousarray(getattr(c, f), np.float64))
        return c


class Ref:
    """The reference's own simulator, driven through ref_harness.cpp."""

    def __init__(self, scene, max_agents, dt, k, tau_agent, tau_obst):
        if not ref_available():
            raise RuntimeError("oracle/_ref/libecmref.so is not built (reference sources absent)")
        self.lib = L = C.CDLL(REF_SO)
        L.ref_create.restype = C.c_void_p
        vp = C.c_void_p
        L.ref_create.argtypes = [C.c_int, C.c_float, C.c_int, C.c_float, C.c_float, C.c_int, vp, vp, vp,
                                 C.c_int, vp, vp, vp, C.c_int, vp, vp, vp, vp]
        for name in ("ref_destroy", "ref_update"):
            getattr(L, name).argtypes = [vp]
        L.ref_spawn_direct.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_float, vp, C.c_int]
        L.ref_spawn.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]
        L.ref_set_path.argtypes = [vp, C.c_int, vp, C.c_int]
        L.ref_get_path.argtypes = [vp, C.c_int, vp, C.c_int]
        L.ref_destroy_agent.argtypes = [vp, C.c_int]
        L.ref_tick_exact.argtypes = [vp, C.c_float, vp, vp, vp, vp]
        L.ref_get_state.argtypes = [vp] * 8 + [vp, vp]
        L.ref_set_state.argtypes = [vp, vp, vp, vp]
        L.ref_knn_kdtree.argtypes = [vp, vp, vp]
        L.ref_find_obstacles.argtypes = [vp, C.c_int, C.c_float, vp, C.c_int]
        L.ref_orca.argtypes = [vp, C.c_int, vp, C.c_int, C.c_float, vp, vp, C.c_int, vp, vp]
        L.ref_lp.argtypes = [vp, vp, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, vp]
        L.ref_lp3d.argtypes = [vp, vp, C.c_int, C.c_int, C.c_float, C.c_int, vp]
        L.ref_point_location.argtypes = [vp, C.c_float, C.c_float]
        L.ref_retract.argtypes = [vp, C.c_float, C.c_float, vp, vp]
        L.ref_irm.argtypes = [vp, C.c_float, C.c_float, vp, C.c_int, vp]
        L.ref_find_path.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, vp, C.c_int]
        L.ref_obstacle_convexity.argtypes = [vp, vp]
        e = scene.ecm
        self._keep = [np.ascontiguousarray(scene.obst_off, I32), np.ascontiguousarray(scene.obst_xy, F32),
                      np.ascontiguousarray(scene.walk, F32), np.ascontiguousarray(e.v_pos, F32),
                      np.ascontiguousarray(e.v_clear, F32), np.ascontiguousarray(e.v_halfedge, I32),
                      np.ascontiguousarray(e.he_target, I32), np.ascontiguousarray(e.he_next, I32),
                      np.ascontiguousarray(e.he_left, F32), np.ascontiguousarray(e.he_right, F32)]
        k_ = self._keep
        self.h = L.ref_create(max_agents, dt, k, tau_agent, tau_obst, scene.n_obstacles, _addr(k_[0]),
                              _addr(k_[1]), _addr(k_[2]), e.n_vertices, _addr(k_[3]), _addr(k_[4]),
                              _addr(k_[5]), e.n_edges, _addr(k_[6]), _addr(k_[7]), _addr(k_[8]),
                              _addr(k_[9]))
        self.n = max_agents
        self.k = k

    def close(self):
        if self.h:
            self.lib.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def spawn_direct(self, x, y, clearance, speed, path):
        path = np.ascontiguousarray(path, F32)
        return self.lib.ref_spawn_direct(self.h, x, y, clearance, speed, _addr(path), int(path.shape[0]))

    def set_path(self, idx, path):
        path = np.ascontiguousarray(path, F32)
        self.lib.ref_set_path(self.h, idx, _addr(path), int(path.shape[0]))

    def update(self):
        self.lib.ref_update(self.h)

    def tick_exact(self, neighbor_dist):
        n, k = self.n, self.k
        nb = np.full((n, k), -1, I32)
        vo = np.zeros((n, 2), F32)
        lf = np.zeros(n, I32)
        nc = np.zeros(n, I32)
        self.lib.ref_tick_exact(self.h, C.c_float(neighbor_dist), _addr(nb), _addr(vo), _addr(lf), _addr(nc))
        return dict(nbr_ids=nb, v_orca=vo, lp_fail=lf, n_constraints=nc)

    def get_state(self):
        n = self.n
        d = dict(pos=np.zeros((n, 2), F32), vel=np.zeros((n, 2), F32), attr=np.zeros((n, 2), F32),
                 pref_vel=np.zeros((n, 2), F32), active=np.zeros(n, U8), clear=np.zeros(n, F32),
                 pref_speed=np.zeros(n, F32))
        last = C.c_int()
        num = C.c_int()
        self.lib.ref_get_state(self.h, _addr(d["pos"]), _addr(d["vel"]), _addr(d["attr"]), _addr(d["pref_vel"]),
                               _addr(d["active"]), _addr(d["clear"]), _addr(d["pref_speed"]), C.byref(last),
                               C.byref(num))
        d["last_idx"] = last.value
        d["num_agents"] = num.value
        return d

    def set_state(self, pos=None, vel=None, attr=None):
        f = lambda a: None if a is None else np.ascontiguousarray(a, F32)
        pos, vel, attr = f(pos), f(vel), f(attr)
        self.lib.ref_set_state(self.h, _addr(pos), _addr(vel), _addr(attr))

    def knn_kdtree(self):
        out = np.zeros((self.n, self.k), I32)
        cnt = np.zeros(self.n, I32)
        self.lib.ref_knn_kdtree(self.h, _addr(out), _addr(cnt))
        return out, cnt

    def find_obstacles(self, agent, range_sq, cap=256):
        out = np.zeros(cap, I32)
        n = self.lib.ref_find_obstacles(self.h, agent, C.c_float(range_sq), _addr(out), cap)
        return out[:min(n, cap)].copy()

    def orca(self, agent, nbrs, max_speed, cap=256):
        nbrs = np.ascontiguousarray(nbrs, I32)
        v = np.zeros(2, F32)
        cons = np.zeros((cap, 4), F32)
        no = C.c_int()
        fl = C.c_int()
        m = self.lib.ref_orca(self.h, agent, _addr(nbrs), int(nbrs.shape[0]), C.c_float(max_speed), _addr(v),
                              _addr(cons), cap, C.byref(no), C.byref(fl))
        return (float(v[0]), float(v[1])), cons[:m].copy(), no.value, fl.value

    def lp(self, cons, opt, max_speed, use_dir_opt=0):
        cons = np.ascontiguousarray(cons, F32).reshape(-1, 4)
        o = np.zeros(2, F32)
        f = self.lib.ref_lp(self.h, _addr(cons), int(cons.shape[0]), C.c_float(opt[0]), C.c_float(opt[1]),
                            C.c_float(max_speed), use_dir_opt, _addr(o))
        return f, (float(o[0]), float(o[1]))

    def lp3d(self, cons, n_obst, max_speed, failed, start):
        cons = np.ascontiguousarray(cons, F32).reshape(-1, 4)
        o = np.array(start, F32)
        self.lib.ref_lp3d(self.h, _addr(cons), int(cons.shape[0]), n_obst, C.c_float(max_speed), failed, _addr(o))
        return (float(o[0]), float(o[1]))

    def point_location(self, x, y):
        return self.lib.ref_point_location(self.h, C.c_float(x), C.c_float(y))

    def retract(self, x, y):
        o = np.zeros(2, F32)
        ed = C.c_int(-1)
        ok = self.lib.ref_retract(self.h, C.c_float(x), C.c_float(y), _addr(o), C.byref(ed))
        return bool(ok), (float(o[0]), float(o[1])), ed.value

    def irm(self, x, y, path):
        path = np.ascontiguousarray(path, F32)
        o = np.zeros(2, F32)
        ok = self.lib.ref_irm(self.h, C.c_float(x), C.c_float(y), _addr(path), int(path.shape[0]), _addr(o))
        return bool(ok), (float(o[0]), float(o[1]))

    def find_path(self, start, goal, clearance, cap=4096):
        out = np.zeros((cap, 2), F32)
        n = self.lib.ref_find_path(self.h, C.c_float(start[0]), C.c_float(start[1]), C.c_float(goal[0]),
                                   C.c_float(goal[1]), C.c_float(clearance), _addr(out), cap)
        return None if n < 0 else out[:n].copy()

    def convexity(self, nv):
        out = np.zeros(nv, U8)
        self.lib.ref_obstacle_convexity(self.h, _addr(out))
        return out

    # ---- spawn and goal areas --------------------------------------------
    def _spawn_sigs(self):
        L, vp = self.lib, C.c_void_p
        if getattr(self, "_spawn_ready", False):
            return L
        L.ref_add_spawn_area.argtypes = [vp] + [C.c_float] * 8 + [C.c_int]
        L.ref_add_goal_area.argtypes = [vp] + [C.c_float] * 4 + [C.c_int]
        L.ref_remove_area.argtypes = [vp, C.c_int, C.c_int]
        L.ref_connect_areas.argtypes = [vp, C.c_int, C.c_int, C.c_float]
        L.ref_disconnect_areas.argtypes = [vp, C.c_int, C.c_int]
        L.ref_update_spawn_areas.argtypes = [vp]
        L.ref_srand.argtypes = [C.c_uint]
        L.ref_spawn_area_state.argtypes = [vp, C.c_int, vp, vp, vp, vp, C.c_int]
        L.ref_free_top.argtypes = [vp, vp]
        self._spawn_ready = True
        return L

    def add_spawn_area(self, x, y, hw, hh, cfg=None, ID=-1):
        c = dict(preferred_speed_min=5.0, preferred_speed_max=10.0, clearance_min=5.0, clearance_max=10.0)
        c.update(cfg or {})
        return self._spawn_sigs().ref_add_spawn_area(self.h, x, y, hw, hh, c["preferred_speed_min"],
                                                     c["preferred_speed_max"], c["clearance_min"],
                                                     c["clearance_max"], ID)

    def add_goal_area(self, x, y, hw, hh, ID=-1):
        return self._spawn_sigs().ref_add_goal_area(self.h, x, y, hw, hh, ID)

    def remove_area(self, area_type, ID):
        self._spawn_sigs().ref_remove_area(self.h, area_type, ID)

    def connect(self, spawn_id, goal_id, rate=0.0):
        self._spawn_sigs().ref_connect_areas(self.h, spawn_id, goal_id, rate)

    def disconnect(self, spawn_id, goal_id):
        self._spawn_sigs().ref_disconnect_areas(self.h, spawn_id, goal_id)

    def update_spawn_areas(self):
        self._spawn_sigs().ref_update_spawn_areas(self.h)

    def srand(self, seed):
        self._spawn_sigs().ref_srand(seed)

    def rand(self):
        return self._spawn_sigs().ref_rand()

    def rand_max(self):
        return self._spawn_sigs().ref_rand_max()

    def spawn_area_state(self, ID, cap=64):
        g, r, t = np.zeros(cap, I32), np.zeros(cap, F32), np.zeros(cap, F32)
        ng = C.c_int()
        n = self._spawn_sigs().ref_spawn_area_state(self.h, ID, _addr(g), C.byref(ng), _addr(r), _addr(t), cap)
        if n < 0:
            return None
        return dict(goals=g[:ng.value].tolist(), rate=r[:n].copy(), since=t[:n].copy())

    def free_top(self):
        size = C.c_int()
        top = self._spawn_sigs().ref_free_top(self.h, C.byref(size))
        return top, size.value

    def get_path(self, idx, cap=4096):
        out = np.zeros((cap, 2), F32)
        n = self.lib.ref_get_path(self.h, idx, _addr(out), cap)
        return out[:min(n, cap)].copy()
