"""ctypes binding of libecmg.so (include/ecmg.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared library has not been built, and every call that
needs the GPU raises EcmgError with the library's own message when it fails.
"""
from __future__ import annotations

import ctypes as C
import os
import re

from . import build as _build

LIB_PATH = _build.LIB
HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "ecmg.h")

STATUS = {0: "ECMG_OK", 1: "ECMG_ERR_INVALID_ARG", 2: "ECMG_ERR_CUDA", 3: "ECMG_ERR_BOUND", 4: "ECMG_ERR_NO_SLOT",
          5: "ECMG_ERR_STATE", 6: "ECMG_ERR_INVALID_SPAWN", 7: "ECMG_ERR_NO_PATH", 8: "ECMG_ERR_NO_DEVICE"}
FIELD = dict(position=0, velocity=1, pref_velocity=2, attraction=3, clearance=4, speed=5, active=6)


class EcmgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Params(C.Structure):
    _fields_ = [("dt", C.c_float), ("tau_agent", C.c_float), ("tau_obst", C.c_float),
                ("neighbor_dist", C.c_float), ("max_speed", C.c_float), ("mass", C.c_float),
                ("arrival_radius", C.c_float), ("delete_radius", C.c_float), ("max_neighbors", C.c_int),
                ("lp3d_fp64", C.c_int), ("use_graph", C.c_int), ("block_size", C.c_int), ("grid_cell", C.c_float)]


class TickStats(C.Structure):
    _fields_ = [("ticks", C.c_int), ("active_agents", C.c_int), ("last_index", C.c_int),
                ("agent_steps", C.c_longlong), ("destroyed", C.c_longlong), ("replans", C.c_longlong),
                ("replans_failed", C.c_longlong), ("lp3d", C.c_longlong), ("device_ms", C.c_float),
                ("agent_kernel_ms", C.c_float), ("host_ms", C.c_float), ("proposed", C.c_longlong),
                ("accepted", C.c_longlong), ("gated", C.c_longlong), ("replans_host", C.c_longlong),
                ("attract_ms", C.c_float), ("neighbors_ms", C.c_float), ("proposal_ms", C.c_float),
                ("orca_ms", C.c_float), ("spawned", C.c_longlong), ("spawn_failed", C.c_longlong),
                ("spawn_refused", C.c_longlong), ("spawn_ms", C.c_float), ("spawn_check_ms", C.c_float),
                ("spawn_candidates", C.c_longlong), ("graph_builds", C.c_int), ("spawn_kernels", C.c_int)]


class SpawnConfig(C.Structure):
    _fields_ = [("preferred_speed_min", C.c_float), ("preferred_speed_max", C.c_float),
                ("clearance_min", C.c_float), ("clearance_max", C.c_float)]


class AreaInfo(C.Structure):
    _fields_ = [("id", C.c_int), ("x", C.c_float), ("y", C.c_float), ("half_w", C.c_float), ("half_h", C.c_float),
                ("config", SpawnConfig), ("n_connected", C.c_int), ("n_timers", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("block_size", C.c_int), ("agents_per_warp_grab", C.c_int), ("grid_cell_scale", C.c_float),
                ("best_tick_ms", C.c_float), ("trials", C.c_int), ("lp_mode", C.c_int),
                ("occupancy_divisor", C.c_int), ("neighbor_blocks_per_sm", C.c_int)]


class Obstacles(C.Structure):
    _fields_ = [("n_obstacles", C.c_int), ("ring_offsets", C.c_void_p), ("xy", C.c_void_p)]


class Ecm(C.Structure):
    _fields_ = [("n_vertices", C.c_int), ("v_pos", C.c_void_p), ("v_clear", C.c_void_p), ("v_idx", C.c_void_p),
                ("v_halfedge", C.c_void_p), ("n_edges", C.c_int), ("he_target", C.c_void_p),
                ("he_next", C.c_void_p), ("he_left", C.c_void_p), ("he_right", C.c_void_p)]


RAND_FN = C.CFUNCTYPE(C.c_int, C.c_void_p)
AREA_SPAWN, AREA_GOAL = 2, 3

PLAN_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                      C.POINTER(C.c_float), C.c_int)

_lib = None


def declared_symbols() -> list[str]:
    """Every function the public header declares."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    names = set()
    for line in src.splitlines():
        line = line.strip()
        if not line or line.startswith(("#", "typedef")):
            continue
        m = re.match(r"^[A-Za-z_][\w\s\*]*?\b(ecmg_[a-z0-9_]+)\s*\(", line)
        if m:
            names.add(m.group(1))
    return sorted(names)


def load(build_if_missing: bool = False):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError(f"{LIB_PATH} is not built; run `python -m ecmgenerator_gb300.build`")
    L = C.CDLL(LIB_PATH)
    vp, ip, fp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_float)
    sig = {
        "ecmg_default_params": (None, [C.POINTER(Params)]),
        "ecmg_create": (C.c_int, [C.POINTER(Params), C.c_int, C.POINTER(vp)]),
        "ecmg_destroy": (C.c_int, [vp]),
        "ecmg_last_error": (C.c_char_p, [vp]),
        "ecmg_get_params": (C.c_int, [vp, C.POINTER(Params)]),
        "ecmg_set_obstacles": (C.c_int, [vp, C.POINTER(Obstacles)]),
        "ecmg_set_ecm": (C.c_int, [vp, C.POINTER(Ecm)]),
        "ecmg_set_planner": (C.c_int, [vp, PLAN_FN, vp]),
        "ecmg_spawn_agent": (C.c_int, [vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, ip]),
        "ecmg_add_agents": (C.c_int, [vp, C.c_int, vp, vp, vp, vp, vp, vp, vp]),
        "ecmg_destroy_agent": (C.c_int, [vp, C.c_int]),
        "ecmg_reset": (C.c_int, [vp]),
        "ecmg_set_path": (C.c_int, [vp, C.c_int, vp, C.c_int]),
        "ecmg_find_path": (C.c_int, [vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, vp, C.c_int, ip]),
        "ecmg_planner_create": (C.c_int, [C.POINTER(Obstacles), C.POINTER(Ecm), C.POINTER(vp)]),
        "ecmg_planner_destroy": (C.c_int, [vp]),
        "ecmg_planner_find_paths": (C.c_int, [vp, C.c_int, vp, vp, vp, C.c_int, C.c_int, vp, vp]),
        "ecmg_planner_locate": (C.c_int, [vp, C.c_int, vp, vp]),
        "ecmg_planner_set_mode": (C.c_int, [vp, C.c_int]),
        "ecmg_set_planner_mode": (C.c_int, [vp, C.c_int]),
        "ecmg_set_replan_overlap": (C.c_int, [vp, C.c_int]),
        "ecmg_save_state": (C.c_int, [vp, C.c_char_p]),
        "ecmg_load_state": (C.c_int, [vp, C.c_char_p]),
        "ecmg_tick": (C.c_int, [vp, C.c_int, C.POINTER(TickStats)]),
        "ecmg_get_state": (C.c_int, [vp, C.c_int, vp]),
        "ecmg_host_view": (C.c_int, [vp, C.c_int, C.POINTER(vp)]),
        "ecmg_set_host_mirror": (C.c_int, [vp, C.c_int]),
        "ecmg_set_state": (C.c_int, [vp, C.c_int, vp]),
        "ecmg_get_counts": (C.c_int, [vp, ip, ip, ip]),
        "ecmg_get_path": (C.c_int, [vp, C.c_int, vp, C.c_int, ip]),
        "ecmg_set_record": (C.c_int, [vp, C.c_int]),
        "ecmg_get_record": (C.c_int, [vp, vp, vp, vp, vp, vp, vp]),
        "ecmg_kernels_per_tick": (C.c_int, [vp]),
        "ecmg_stream": (vp, [vp]),
        "ecmg_create_batch": (C.c_int, [C.POINTER(Params), C.c_int, vp, C.POINTER(vp)]),
        "ecmg_scene_count": (C.c_int, [vp]),
        "ecmg_scene_set_obstacles": (C.c_int, [vp, C.c_int, C.POINTER(Obstacles)]),
        "ecmg_scene_set_ecm": (C.c_int, [vp, C.c_int, C.POINTER(Ecm)]),
        "ecmg_scene_add_agents": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, vp]),
        "ecmg_scene_counts": (C.c_int, [vp, C.c_int, ip, ip, ip, ip]),
        "ecmg_set_launch": (C.c_int, [vp, C.c_int, C.c_int, C.c_float]),
        "ecmg_set_lp_mode": (C.c_int, [vp, C.c_int, C.c_int]),
        "ecmg_set_occupancy": (C.c_int, [vp, C.c_int]),
        "ecmg_set_neighbor_mode": (C.c_int, [vp, C.c_int]),
        "ecmg_autotune": (C.c_int, [vp, C.c_int, C.POINTER(TuneResult)]),
        "ecmg_knn_noalloc": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                       C.c_float, C.c_float, vp, vp, vp]),
        "ecmg_knn_scratch_bytes": (C.c_size_t, [C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float]),
        "ecmg_knn": (C.c_int, [vp, vp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                               C.c_float, vp, vp, vp, C.c_size_t, vp]),
        "ecmg_mlp_create": (C.c_int, [C.c_ulonglong, C.POINTER(vp)]),
        "ecmg_mlp_destroy": (C.c_int, [vp]),
        "ecmg_mlp_param_count": (C.c_int, []),
        "ecmg_mlp_get_params": (C.c_int, [vp, vp]),
        "ecmg_mlp_set_params": (C.c_int, [vp, vp]),
        "ecmg_mlp_loss_grad": (C.c_int, [vp, vp, vp, C.c_int, fp, vp]),
        "ecmg_mlp_train": (C.c_int, [vp, vp, vp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_ulonglong, vp, vp]),
        "ecmg_mlp_predict": (C.c_int, [vp, vp, C.c_int, vp]),
        "ecmg_mlp_set_wait_limit": (C.c_int, [vp, C.c_int]),
        "ecmg_set_neighbor_blocks": (C.c_int, [vp, C.c_int]),
        "ecmg_set_proposal": (C.c_int, [vp, vp]),
        "ecmg_set_trace": (C.c_int, [vp, C.c_int]),
        "ecmg_set_proposal_gate": (C.c_int, [vp, C.c_float, C.c_int]),
        "ecmg_get_trace": (C.c_int, [vp, vp, vp, vp, C.c_int, ip]),
        "ecmg_set_proposal_classes": (C.c_int, [vp, vp]),
        "ecmg_add_spawn_area": (C.c_int, [vp, C.c_float, C.c_float, C.c_float, C.c_float, C.POINTER(SpawnConfig),
                                          C.c_int, ip]),
        "ecmg_add_goal_area": (C.c_int, [vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, ip]),
        "ecmg_remove_area": (C.c_int, [vp, C.c_int, C.c_int]),
        "ecmg_connect_areas": (C.c_int, [vp, C.c_int, C.c_int, C.c_float]),
        "ecmg_disconnect_areas": (C.c_int, [vp, C.c_int, C.c_int]),
        "ecmg_set_area": (C.c_int, [vp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float]),
        "ecmg_get_area": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(AreaInfo), vp, vp, vp, C.c_int]),
        "ecmg_area_ids": (C.c_int, [vp, C.c_int, vp, C.c_int, ip]),
        "ecmg_set_spawn_rng": (C.c_int, [vp, RAND_FN, vp, C.c_int]),
        "ecmg_push_spawn_random": (C.c_int, [vp, vp, C.c_int]),
        "ecmg_spawn_random_pending": (C.c_int, [vp, C.POINTER(C.c_longlong)]),
        "ecmg_update_spawn_areas": (C.c_int, [vp, C.POINTER(TickStats)]),
        "ecmg_get_spawned": (C.c_int, [vp, vp, vp, vp, C.c_int, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def default_params(**over) -> Params:
    L = load()
    p = Params()
    L.ecmg_default_params(C.byref(p))
    for k, v in over.items():
        setattr(p, k, v)
    return p
