import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "ref: needs the reference build in oracle/_ref (this container only)")


def pytest_collection_modifyitems(config, items):
    import oracle as orc

    have_ref = orc.ref_available()
    for it in items:
        if "ref" in it.keywords and not have_ref:
            it.add_marker(pytest.mark.skip(reason="oracle/_ref not built (reference sources absent)"))


@pytest.fixture(scope="session")
def port():
    import oracle as orc

    orc.build()
    return orc.Port()


@pytest.fixture(scope="session")
def lib():
    from ecmgenerator_gb300 import _lib, build

    build.build()
    return _lib.load()


@pytest.fixture(scope="session")
def c1_small():
    """300-agent instance of the 100x100 m, 40-box scene (seed 5), with
    paths from the host planner."""
    import numpy as np

    from ecmgenerator_gb300 import agents as ag
    from ecmgenerator_gb300 import build
    from ecmgenerator_gb300.simulator import Planner

    build.build()
    cfg = ag.scaled("c1", agents=300)
    scene = ag.build_scene(cfg, seed=5)
    st = ag.spawn_agents(cfg, scene, seed=5)
    paths = Planner(scene).find_paths(st.pos, st.goal, st.clear)
    paths = [p if p is not None else np.stack([st.pos[i], st.goal[i]]) for i, p in enumerate(paths)]
    st.set_paths(paths)
    return scene, st, paths
