import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "rigid-ipc_gb300"), os.path.join(ROOT, "oracle"), ROOT,
          os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built librigc.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def rigc_mod():
    import rigc

    return rigc


@pytest.fixture(scope="session")
def cube_scene():
    from rigc import scene as S

    return S.scene_from_json(S.spec_cubes(0))


def contact_poses(scene, seed=0, gap=5e-4):
    """Poses with each lattice column stacked on the floor: every cube rests
    gap * U[0.2, 1.2] above the one below (or the floor), so stacked cubes
    and the floor are within the barrier distance."""
    x = scene.poses().reshape(-1, 6).copy()
    V = scene.world_vertices(scene.poses())
    rng = np.random.default_rng(seed)
    cols = {}
    for b in range(scene.num_bodies):
        if scene.bodies[b].type != 2:
            continue
        key = (round(x[b, 0], 3), round(x[b, 2], 3))
        cols.setdefault(key, []).append(b)
    for bs in cols.values():
        bs.sort(key=lambda b: x[b, 1])
        top = 0.0
        for b in bs:
            a, c = scene.body_vertex_start[b], scene.body_vertex_start[b + 1]
            lo, hi = V[a:c, 1].min(), V[a:c, 1].max()
            shift = top + gap * rng.uniform(0.2, 1.2) - lo
            x[b, 1] += shift
            top = hi + shift
    return x.reshape(-1)


@pytest.fixture(scope="session")
def cube_contact(cube_scene):
    return contact_poses(cube_scene)
