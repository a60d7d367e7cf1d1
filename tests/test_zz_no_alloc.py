"""The allocation-free narrow phase (d2g_compare_trees_full_noalloc).

Callers that may not allocate device memory during a call — work captured
into a CUDA graph, real-time loops with a fixed memory budget, runtimes that
own every allocation — use this entry point: the caller passes the scene,
pairs and outputs in device memory and the library works in a fixed static
scratch array.  This checks, through the C ABI, that two calls in a row give
exactly the contacts and offsets of the allocating entry point
d2g_compare_trees_full (bit for bit, the tolerance the parity tests use), and
that requests beyond the documented limits are refused.  The file name makes
pytest collect it last.
"""
import ctypes as C

import numpy as np
import pytest

import delta2_gb300 as D

pytestmark = pytest.mark.gpu


def _project_futures(scene):
    from oracle import oracle as O
    for i in range(scene.n_bodies):
        scene.fut[i] = O.state_extrapolate(scene.cur[i], scene.last_dt[i], scene.inv_inertia[i])
    return scene


def test_noalloc_matches_allocating_entry_point(gpu_required):
    import torch

    from delta2_gb300 import build as B
    B.build()
    scene = _project_futures(D.make_scene(1, nx=2, ny=2, nz=1, spacing=1.12, speed_sigma=3.0, seed=5))
    pairs = D.broad_phase(scene)
    assert 0 < len(pairs) <= D.NOALLOC_MAX_PAIRS

    ctx = D.Context(0)
    try:
        ctx.set_scene(scene.copy())
        ref, ref_off, _ = ctx.compare_trees_full(pairs)
    finally:
        ctx.close()
    assert len(ref) > 0

    dev = torch.device("cuda", 0)
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(scene, k))).to(dev) for k in
         ["mesh_node_off", "nodes", "ntris", "tris", "eps", "inner_eps", "mesh", "fut", "geo_eps"]}
    ds = D.DeviceScene(len(scene.mesh_node_off) - 1, int(scene.nodes.shape[0]), t["mesh_node_off"].data_ptr(),
                       t["nodes"].data_ptr(), t["ntris"].data_ptr(), t["tris"].data_ptr(), t["eps"].data_ptr(),
                       t["inner_eps"].data_ptr(), scene.n_bodies, t["mesh"].data_ptr(), t["fut"].data_ptr(),
                       t["geo_eps"].data_ptr())
    d_pairs = torch.from_numpy(np.ascontiguousarray(pairs, dtype=np.int32)).to(dev)
    cap = len(ref) + 8
    d_out = torch.full((cap, D.CONTACT_LEN), float("nan"), dtype=torch.float64, device=dev)
    d_off = torch.zeros(len(pairs) + 1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    for call in range(2):  # the scratch keeps the last call's contents; both calls must agree
        d_out.fill_(float("nan"))
        d_off.zero_()
        torch.cuda.synchronize()
        n = D.compare_trees_full_noalloc(ds, d_pairs.data_ptr(), len(pairs), d_out.data_ptr(), cap,
                                         d_off.data_ptr())
        assert n == len(ref), (call, n, len(ref))
        got = d_out[:n].cpu().numpy()
        assert np.array_equal(d_off.cpu().numpy(), ref_off), call
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), call

    # requests beyond the limits are refused with a clear error, not run
    big = torch.zeros((D.NOALLOC_MAX_PAIRS + 1, 2), dtype=torch.int32, device=dev)
    with pytest.raises(D.D2GError, match="exceed the limit"):
        D.compare_trees_full_noalloc(ds, big.data_ptr(), D.NOALLOC_MAX_PAIRS + 1, d_out.data_ptr(), cap,
                                     d_off.data_ptr())
    # a too-small output buffer reports the count without writing contacts
    with pytest.raises(D.CapacityError):
        D.compare_trees_full_noalloc(ds, d_pairs.data_ptr(), len(pairs), d_out.data_ptr(), 1, d_off.data_ptr())
