"""The allocation-free narrow phase (d2g_compare_trees_full_noalloc).

Some hosts cannot allocate device memory while a call runs: real-time loops
that fix their memory budget up front (an allocation can stall or fail
mid-frame) and runtimes that own every allocation themselves.  They use this
entry point: the caller passes the scene, pairs and outputs in device memory
and the library works in a fixed static scratch array.  This checks, through
the C ABI, that two calls in a row give exactly the contacts and offsets of
the allocating entry point d2g_compare_trees_full (bit for bit, the tolerance
the parity tests use), that requests beyond the documented limits are refused
(before the traversal, and at the tree level that would pass the per-level
limit), and that a call after a refused one is still exact.  The file name
makes pytest collect it last.
"""
import itertools

import numpy as np
import pytest

import delta2_gb300 as D

pytestmark = pytest.mark.gpu


def _project_futures(scene):
    from oracle import oracle as O
    for i in range(scene.n_bodies):
        scene.fut[i] = O.state_extrapolate(scene.cur[i], scene.last_dt[i], scene.inv_inertia[i])
    return scene


def _device_scene(scene, dev):
    import torch

    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(scene, k))).to(dev) for k in
         ["mesh_node_off", "nodes", "ntris", "tris", "eps", "inner_eps", "mesh", "fut", "geo_eps"]}
    ds = D.DeviceScene(len(scene.mesh_node_off) - 1, int(scene.nodes.shape[0]), t["mesh_node_off"].data_ptr(),
                       t["nodes"].data_ptr(), t["ntris"].data_ptr(), t["tris"].data_ptr(), t["eps"].data_ptr(),
                       t["inner_eps"].data_ptr(), scene.n_bodies, t["mesh"].data_ptr(), t["fut"].data_ptr(),
                       t["geo_eps"].data_ptr())
    return ds, t  # the tensors keep the device buffers alive


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
    ds, keep = _device_scene(scene, dev)
    d_pairs = torch.from_numpy(np.ascontiguousarray(pairs, dtype=np.int32)).to(dev)
    cap = len(ref) + 8
    d_out = torch.full((cap, D.CONTACT_LEN), float("nan"), dtype=torch.float64, device=dev)
    d_off = torch.zeros(len(pairs) + 1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()

    def call_and_check(tag):
        d_out.fill_(float("nan"))
        d_off.zero_()
        torch.cuda.synchronize()
        n = D.compare_trees_full_noalloc(ds, d_pairs.data_ptr(), len(pairs), d_out.data_ptr(), cap,
                                         d_off.data_ptr())
        assert n == len(ref), (tag, n, len(ref))
        got = d_out[:n].cpu().numpy()
        assert np.array_equal(d_off.cpu().numpy(), ref_off), tag
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), tag

    for call in range(2):  # the scratch keeps the last call's contents; both calls must agree
        call_and_check(call)

    # more body pairs than the limit (2,048: the first level holds one root node pair per body pair)
    # are refused before any work, with a clear error
    big_n = 3000
    big = torch.from_numpy(np.tile(np.ascontiguousarray(pairs[:1], dtype=np.int32), (big_n, 1))).to(dev)
    with pytest.raises(D.D2GError, match="3000 pairs exceed the limit of 2048"):
        D.compare_trees_full_noalloc(ds, big.data_ptr(), big_n, d_out.data_ptr(), cap, d_off.data_ptr())
    # a too-small output buffer reports the count without writing contacts
    with pytest.raises(D.CapacityError):
        D.compare_trees_full_noalloc(ds, d_pairs.data_ptr(), len(pairs), d_out.data_ptr(), 1, d_off.data_ptr())
    call_and_check("after the refusals")


def test_noalloc_refuses_a_level_beyond_its_limit_then_recovers(gpu_required):
    """Twelve coincident cubes: 66 body pairs, 528 node pairs at the second
    level and 4,224 at the third (every node pair hits), more than the
    2,048-entry level buffers.  The call stops at that level with an error;
    the next call on the same scratch is exact again."""
    import torch

    from delta2_gb300 import build as B
    B.build()
    dense = D.make_scene(1, nx=12, ny=1, nz=1, spacing=1.5, speed_sigma=0.5, seed=7)
    moving = np.where(dense.is_static == 0)[0]
    for i in moving:
        dense.fut[i] = dense.cur[i]
        dense.fut[i, 8:11] = dense.cur[moving[0], 8:11]
    dpairs = np.array(list(itertools.combinations(moving, 2)), dtype=np.int32)
    assert len(dpairs) == 66

    dev = torch.device("cuda", 0)
    ds, keep = _device_scene(dense, dev)
    d_pairs = torch.from_numpy(dpairs).to(dev)
    cap = 1 << 14
    d_out = torch.zeros((cap, D.CONTACT_LEN), dtype=torch.float64, device=dev)
    d_off = torch.zeros(len(dpairs) + 1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    with pytest.raises(D.D2GError, match="4224 node pairs at level 2 exceed the limit of 2048"):
        D.compare_trees_full_noalloc(ds, d_pairs.data_ptr(), len(dpairs), d_out.data_ptr(), cap, d_off.data_ptr())

    # the first eight pairs stay within every limit: exact against the allocating path
    sub = dpairs[:8]
    ctx = D.Context(0)
    try:
        ctx.set_scene(dense.copy())
        ref, ref_off, _ = ctx.compare_trees_full(sub)
    finally:
        ctx.close()
    d_sub = torch.from_numpy(np.ascontiguousarray(sub)).to(dev)
    d_off2 = torch.zeros(len(sub) + 1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    n = D.compare_trees_full_noalloc(ds, d_sub.data_ptr(), len(sub), d_out.data_ptr(), cap, d_off2.data_ptr())
    assert n == len(ref) > 0
    assert np.array_equal(d_off2.cpu().numpy(), ref_off)
    assert np.array_equal(d_out[:n].cpu().numpy().view(np.uint64), ref.view(np.uint64))
