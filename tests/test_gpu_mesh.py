"""Mass properties of many meshes on the device (d2g_mass_properties): the
same bits as the host scene set-up gives for the same meshes (volume =
mass at density 1, centre of mass, inverse inertia), and the oracle's
restatement of the reference's formulas within rounding, for closed meshes
(volume model) and thin shells (surface model)."""
import time

import numpy as np
import pytest

import delta2_gb300 as D
from oracle import oracle as O
from tests.test_tree_build import cube_mesh, grid_mesh, icosphere

pytestmark = pytest.mark.gpu


def test_device_mass_properties_match_host_and_oracle(gpu_required):
    from delta2_gb300 import build as B
    B.build()
    rng = np.random.default_rng(3)
    meshes, surface = [cube_mesh(0.5)], [0]
    for k in range(24):
        V, F = icosphere(2 + k % 2, radius=0.3 + 0.05 * k, noise=0.2, seed=k)
        meshes.append((V + rng.normal(0, 0.3, 3), F))  # off-centre: the centre of mass is found, not assumed
        surface.append(0)
    for k in range(3):  # 80 faces: a chunk of 32 faces and a ragged last chunk
        V, F = icosphere(1, radius=0.4, noise=0.3, seed=100 + k)
        meshes.append((V + rng.normal(0, 0.3, 3), F))
        surface.append(0)
    meshes.append(grid_mesh(4))  # a thin shell (the surface model, as static planes use): 32 faces
    surface.append(1)
    meshes.append(grid_mesh(7))  # 98 faces
    surface.append(1)
    ctx = D.Context(0)
    try:
        dev = ctx.mass_properties(meshes, surface=surface, thickness=0.01)
    finally:
        ctx.close()
    b = D.SceneBuilder(dt=1 / 240, gravity_z=-9.8)
    coms = []
    for (V, F), s in zip(meshes, surface):
        mid, com = b.add_mesh(V, F, surface=bool(s))
        coms.append(com)
        b.add_body(mid, static=bool(s), density=1.0)
    sc = b.finish()
    for i in range(len(meshes)):
        assert dev[i, 0].view(np.uint64) == np.float64(sc.mass[i]).view(np.uint64), i
        assert np.array_equal(dev[i, 1:4].view(np.uint64), np.asarray(coms[i]).view(np.uint64)), i
        assert np.array_equal(dev[i, 13:22].view(np.uint64), sc.inv_inertia[i].view(np.uint64)), i
        vol, com, I = O.mass_properties(*meshes[i], surface=bool(surface[i]), thickness=0.01)
        assert abs(dev[i, 0] - vol) <= 1e-12 * abs(vol)
        assert np.abs(dev[i, 1:4] - com).max() <= 1e-12 * (1 + np.abs(com).max())
        assert np.abs(dev[i, 4:13].reshape(3, 3) - I).max() <= 1e-10 * np.abs(I).max()
        assert np.abs(dev[i, 4:13].reshape(3, 3) @ dev[i, 13:22].reshape(3, 3) - np.eye(3)).max() < 1e-9


def test_device_mass_properties_of_a_large_mesh_set(gpu_required):
    """4,096 distinct noisy subdivision-3 icospheres (1,280 triangles each)
    in one call; each equals the oracle's within rounding."""
    from delta2_gb300 import build as B
    B.build()
    base_V, F = icosphere(3, radius=0.5)
    rng = np.random.default_rng(11)
    meshes = [(base_V * (1.0 + 0.2 * rng.uniform(-1, 1, (len(base_V), 1))), F) for _ in range(4096)]
    ctx = D.Context(0)
    try:
        ctx.mass_properties(meshes[:64])
        t0 = time.perf_counter()
        dev = ctx.mass_properties(meshes)
        dt = time.perf_counter() - t0
    finally:
        ctx.close()
    for i in range(0, 4096, 97):
        vol, com, I = O.mass_properties(*meshes[i])
        assert abs(dev[i, 0] - vol) <= 1e-12 * vol
        assert np.abs(dev[i, 4:13].reshape(3, 3) - I).max() <= 1e-10 * np.abs(I).max()
    print(f"4096 meshes x 1280 triangles: {dt * 1e3:.1f} ms including the copies")
