"""Host logic of the z-slab sharding (CPU): the slab plan, and the stitching
exchange run as two gloo ranks.  Each rank's window mesh is made from the
oracle's whole mesh (its triangles of the rank's cells plus a guard band,
vertices renumbered in a shuffled order); the stitched meshes, concatenated
in rank order, must hold exactly the whole mesh's vertices and triangles."""
import os
import socket

import numpy as np
import pytest

from broxy_gb300 import shard, synth
from oracle import oracle as O


def test_plan_partitions_the_grid():
    for res, world, rmax in [(64, 2, 4), (128, 3, 12), (512, 8, 32), (256, 1, 8)]:
        slabs = shard.plan_slabs(res, world, rmax, bilateral_iters=20)
        assert slabs[0].z0 == 0 and slabs[-1].z1 == res
        for a, b in zip(slabs, slabs[1:]):
            assert a.z1 == b.z0
        for s in slabs:
            assert s.z0 % 16 == 0 and s.z1 > s.z0
            assert s.zlo % 16 == 0 and s.zhi % 16 == 0 or s.zhi == res
            halo = rmax + shard.HALO_SPARE + s.guard
            assert s.zlo <= max(0, s.z0 - halo) and s.zhi >= min(res, s.z1 + halo)
    with pytest.raises(ValueError):
        shard.plan_slabs(40, 2, 4)


def _whole(res=32, seed=61):
    X = synth.blob_grid(res, seed, count=30)  # solid away from the grid border
    _, _, Cg = O.close(X, res, [res] * 3, O.scale_grid(res, uniform=3), 0, 0)
    V, T = O.mc(Cg, res, np.zeros(3, np.float32), 1.0 / res)
    N = O.normals(V, T, 0)
    return V, N, T.astype(np.int64)


def _rank_window(slab, V, N, T, res, seed):
    cs_f = 0.5 / res
    vz = shard._lattice_z(V, 0.0, cs_f)
    tcell = np.floor_divide(vz[T].min(axis=1), 2)
    sel = (tcell >= max(slab.z0 - slab.guard, 0)) & (tcell < min(slab.z1 + slab.guard, res))
    Tw = T[sel]
    ids = np.unique(Tw)
    perm = np.random.default_rng(seed).permutation(len(ids))
    new_of_old = np.full(len(V), -1, np.int64)
    new_of_old[ids[perm]] = np.arange(len(ids))
    Vw = np.empty((len(ids), 3), np.float32)
    Nw = np.empty((len(ids), 3), np.float32)
    Vw[new_of_old[ids]] = V[ids]
    Nw[new_of_old[ids]] = N[ids]
    return Vw, Nw, new_of_old[Tw]


def _rank_main(rank, world, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    res = 32
    V, N, T = _whole(res)
    slab = shard.plan_slabs(res, world, 3, bilateral_iters=0)[rank]
    Vw, Nw, Tw = _rank_window(slab, V, N, T, res, seed=rank + 7)
    part = shard.local_mesh(slab, Vw, Nw, Tw, 0.0, 1.0 / res)
    assert part["dropped"] == 0
    Vs, Ns, Ts = shard.stitch(slab, part, shard.TorchGroup())
    np.savez(os.path.join(outdir, "rank%d.npz" % rank), V=Vs, N=Ns, T=Ts)
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_stitch_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn")
    parts = [np.load(tmp_path / ("rank%d.npz" % r)) for r in range(world)]
    Vs = np.concatenate([p["V"] for p in parts])
    Ts = np.concatenate([p["T"] for p in parts])
    V, N, T = _whole()
    assert len(Vs) == len(np.unique(T)) and Ts.max() < len(Vs)
    key = lambda A, B: sorted(map(bytes, np.ascontiguousarray(A[B]).view(np.uint8).reshape(len(B), -1)))
    assert key(Vs, Ts) == key(V, T)
    # every vertex appears once
    vk = sorted(map(bytes, Vs.view(np.uint8).reshape(len(Vs), -1)))
    assert len(set(vk)) == len(vk)
