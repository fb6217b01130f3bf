"""Loading of the committed golden fixtures (tests/golden/*.npz)."""
import os

import numpy as np

from ecmgenerator_gb300 import agents as ag
from ecmgenerator_gb300 import scene as sc

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def scene_of(d):
    s = sc.make_scene(float(d["w"]), float(d["h"]), d["boxes"])
    assert np.array_equal(s.obst_xy, d["obst_xy"])
    s.ecm = sc.Ecm(v_pos=d["v_pos"], v_clear=d["v_clear"], v_idx=d["v_idx"], v_halfedge=d["v_halfedge"],
                   he_target=d["he_target"], he_next=d["he_next"], he_left=d["he_left"], he_right=d["he_right"])
    return s


def state_of(d):
    n = d["clear"].shape[0]
    st = ag.AgentState.empty(n)
    st.pos[:] = d["pos"][0]
    st.vel[:] = d["vel"][0]
    st.attr[:] = d["attr"][0]
    st.active[:] = d["active"][0]
    st.clear[:] = d["clear"]
    st.pref_speed[:] = d["speed"]
    off = np.concatenate([[0], np.cumsum(d["path_len"])[:-1]]).astype(np.int32)
    paths = [d["path_xy"][off[i]:off[i] + d["path_len"][i]] for i in range(n)]
    st.set_paths(paths)
    st.last_idx, st.num_agents = n - 1, int(st.active.sum())
    return st, paths


def path_events(d, tick):
    """(slot, path) pairs the reference re-planned during `tick`."""
    off = np.concatenate([[0], np.cumsum(d["ev_len"])]).astype(np.int64)
    out = []
    for e in np.nonzero(d["ev_tick"] == tick)[0]:
        out.append((int(d["ev_slot"][e]), d["ev_xy"][off[e]:off[e + 1]]))
    return out
