"""Multi-GPU layout, run as two gloo ranks.

A single frame does not shard: N GPUs render N independent replicas and the
only collectives are a barrier and a max over ranks of the timed duration.
A batch of views shards by view (gorender_gb300.shard): each rank renders the
views the partition gives it.  These tests run both protocols with two ranks
and check that the replicas agree, that the reduction is a max, and that the
union of the ranks' per-view frames is exactly the single-rank set.  Without
a GPU the ranks render with the oracle; the GPU variant renders each rank's
share with the library's CUDA-graph batch (both ranks on GPU 0, independent
processes whose kernels never wait on each other)."""
import hashlib
import os
import socket
import sys

import numpy as np
import pytest

from gorender_gb300 import scenes, shard

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _init(rank, world, port):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)


def _digest(rgba, z):
    return hashlib.sha256(np.ascontiguousarray(rgba).tobytes() + np.ascontiguousarray(z).tobytes()).hexdigest()


def _views():
    return scenes.multiview_batch(18, seed=21, min_tris=100, max_tris=20000,
                                  resolutions=((96, 64), (128, 128), (160, 90), (200, 120)))


def _replica_rank(rank, world, port, q):
    _init(rank, world, port)
    from oracle import oracle
    from tests.golden_scenes import heightfield_small
    dist.barrier()
    rgba, z, tpf, st = oracle.draw_scene(heightfield_small(), nthreads=1)
    elapsed = torch.tensor([float(rank + 1)], dtype=torch.float64)  # stand-in durations 1, 2
    dist.all_reduce(elapsed, op=dist.ReduceOp.MAX)
    q.put((rank, st, tpf, _digest(rgba, z), float(elapsed.item())))
    dist.destroy_process_group()


def _shard_rank(rank, world, port, q, use_gpu):
    _init(rank, world, port)
    vs = _views()
    ws, r, local = shard.dist_env()
    assert (ws, r, local) == (world, rank, rank)
    mine = shard.shard_of(vs, r, ws)
    out = {}
    if use_gpu:
        from gorender_gb300 import renderer as R
        ctx = R.Context(0)
        sb = shard.ShardedBatch(ctx, vs, mine, autotune=False)
        sb.run()
        sb.sync()
        for k, (i, tpf) in enumerate(zip(mine, sb.view_tpf())):
            rgba, z = sb.frame(k)
            out[i] = (_digest(rgba, z), tpf)
        sb.close()
        ctx.close()
    else:
        from oracle import oracle
        for i in mine:
            rgba, z, tpf, st = oracle.draw_scene(vs[i], nthreads=1)
            assert st == 0
            out[i] = (_digest(rgba, z), tpf)
    dist.barrier()
    q.put((rank, out))
    dist.destroy_process_group()


def _spawn(target, world, *args):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=target, args=(r, world, port, q) + args) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=600) for _ in procs), key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return res


def test_two_rank_replicas():
    res = _spawn(_replica_rank, 2)
    assert all(r[1] == 0 for r in res)
    assert res[0][2:4] == res[1][2:4]           # identical replicas
    assert res[0][4] == res[1][4] == 2.0         # max over ranks


def test_partition_covers_every_view_once_and_balances():
    vs = scenes.multiview_batch(256, seed=0)
    costs = [shard.view_cost(s) for s in vs]
    for world in (1, 2, 3, 4, 8):
        parts = shard.partition_views(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(vs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs) + 1e-6
        assert parts == shard.partition_views(costs, world)  # deterministic
    assert shard.partition_views([5.0, 1.0, 1.0], 4) == [[0], [1], [2], []]


def _check_union(res, use_gpu):
    vs = _views()
    seen = {}
    for _, out in res:
        for i, v in out.items():
            assert i not in seen, f"view {i} rendered twice"
            seen[i] = v
    assert sorted(seen) == list(range(len(vs)))
    from oracle import oracle
    for i, sc in enumerate(vs):
        rgba, z, tpf, st = oracle.draw_scene(sc, nthreads=2)
        assert st == 0 and seen[i] == (_digest(rgba, z), tpf), f"view {i}"


def test_two_rank_view_shards_oracle():
    _check_union(_spawn(_shard_rank, 2, False), False)


@pytest.mark.gpu
def test_two_rank_view_shards_library():
    _check_union(_spawn(_shard_rank, 2, True), True)


# ---- the differentiable step sharded by view: loss and gradients are sums of the ranks' shares ----

def _diff_case():
    from gorender_gb300 import scenes as S
    return S.diff_scene(views=4, size=48, level=2, tex_size=16, seed=5)


def _oracle_share(sc, idx):
    """FP64 loss and gradients of the views idx (the oracle's adjoint), with
    the target rendered from the perturbed parameters over those views."""
    import dataclasses as dc_
    from oracle import oracle
    from tests import diff_cases as dc
    views_all, world = dc.oracle_views(sc)
    sub = dc_.replace(sc, cameras=[sc.cameras[i] for i in idx])
    views = [views_all[i] for i in idx]
    ids = dc.oracle_ids(sub)
    tgt_ids = dc.oracle_ids(sub, sc.target_params["pos"])
    tp = dc.params_of(sc, world, target=True)
    tgt = oracle.diff_eval(sc.mesh, views, tp, tgt_ids, np.zeros((ids.size, 4), np.float32), grads=False, image=True)
    params = {k: (np.array(v, np.float64) if k != "world" else v) for k, v in dc.params_of(sc, world).items()}
    r = oracle.diff_eval(sc.mesh, views, params, ids, tgt["image"].astype(np.float32))
    return [np.array([r["loss"]], np.float64)] + [np.array(r[k], np.float64) for k in ("g_light", "g_pos", "g_vcol", "g_tex")]


def _diff_rank_oracle(rank, world, port, q):
    _init(rank, world, port)
    sc = _diff_case()
    mine = shard.partition_views([1.0] * len(sc.cameras), world)[rank]
    parts = _oracle_share(sc, mine)
    shard.allreduce_host(dist)(parts)
    q.put((rank, mine, parts))
    dist.destroy_process_group()


def test_two_rank_diff_shards_sum_to_the_whole_step():
    """Each rank's FP64 adjoint over its views, summed over two gloo ranks,
    equals the adjoint of all views in one process."""
    res = _spawn(_diff_rank_oracle, 2)
    assert sorted(res[0][1] + res[1][1]) == [0, 1, 2, 3]
    whole = _oracle_share(_diff_case(), [0, 1, 2, 3])
    for got in (res[0][2], res[1][2]):
        for a, b in zip(got, whole):
            assert np.allclose(a, b, rtol=1e-9, atol=1e-12 * max(1.0, float(np.abs(b).max())))


def _diff_rank_library(rank, world, port, q):
    _init(rank, world, port)
    from gorender_gb300 import renderer as R
    sc = _diff_case()
    ctx = R.Context(0)
    mesh = ctx.mesh(sc.mesh)
    world_m, views = R.diff_views(sc)
    mine = shard.partition_views([1.0] * len(views), world)[rank]
    sd = shard.ShardedDiff(ctx, mesh, world_m, views, mine, tex_size=sc.tex.shape[:2])

    def dev(a):
        a = np.ascontiguousarray(a, np.float32)
        return ctx.device_buffer(a.nbytes).upload(a)
    tp = sc.target_params
    p = [dev(sc.mesh.pos), dev(sc.vcol), dev(sc.tex)]
    q_ = [dev(tp["pos"]), dev(tp["vcol"]), dev(tp["tex"])]
    target = dev(np.zeros((sd.pixels, 4)))
    zeros = dev(np.zeros((sd.pixels, 4)))
    sd.forward(q_[0].ptr, q_[1].ptr, q_[2].ptr, tp["light"], zeros.ptr, target.ptr)  # this rank's targets
    nv = sc.mesh.nv
    g = [ctx.device_buffer(nv * 16), ctx.device_buffer(nv * 12), ctx.device_buffer(sc.tex.nbytes)]
    shapes = [((nv, 4), np.float32), ((nv, 3), np.float32), (sc.tex.shape, np.float32)]
    loss, g_light, host = sd.step(p[0].ptr, p[1].ptr, p[2].ptr, sc.light, target.ptr, [x.ptr for x in g], shapes,
                                  shard.allreduce_host(dist))
    sd.close()
    for x in p + q_ + g + [target, zeros]:
        x.free()
    ctx.close()
    q.put((rank, loss, g_light, host))
    dist.destroy_process_group()


@pytest.mark.gpu
def test_two_rank_diff_shards_library():
    """Two ranks (both on GPU 0) differentiate two views each with the
    library; their summed loss and gradients equal one process's over all
    four views (float32 atomics add in another order: 1e-5 relative)."""
    res = _spawn(_diff_rank_library, 2)
    from gorender_gb300 import renderer as R
    sc = _diff_case()
    ctx = R.Context(0)
    try:
        mesh = ctx.mesh(sc.mesh)
        world_m, views = R.diff_views(sc)
        sd = shard.ShardedDiff(ctx, mesh, world_m, views, list(range(len(views))), tex_size=sc.tex.shape[:2])

        def dev(a):
            a = np.ascontiguousarray(a, np.float32)
            return ctx.device_buffer(a.nbytes).upload(a)
        tp = sc.target_params
        p = [dev(sc.mesh.pos), dev(sc.vcol), dev(sc.tex)]
        q_ = [dev(tp["pos"]), dev(tp["vcol"]), dev(tp["tex"])]
        target = dev(np.zeros((sd.pixels, 4)))
        zeros = dev(np.zeros((sd.pixels, 4)))
        sd.forward(q_[0].ptr, q_[1].ptr, q_[2].ptr, tp["light"], zeros.ptr, target.ptr)
        nv = sc.mesh.nv
        g = [ctx.device_buffer(nv * 16), ctx.device_buffer(nv * 12), ctx.device_buffer(sc.tex.nbytes)]
        shapes = [((nv, 4), np.float32), ((nv, 3), np.float32), (sc.tex.shape, np.float32)]
        loss, g_light, host = sd.step(p[0].ptr, p[1].ptr, p[2].ptr, sc.light, target.ptr, [x.ptr for x in g], shapes,
                                      lambda arrays: None)
        sd.close()
    finally:
        ctx.close()
    for _, l2, gl2, h2 in res:
        assert abs(l2 - loss) <= 1e-6 * abs(loss)
        assert np.allclose(gl2, g_light, rtol=1e-5, atol=1e-7 * np.abs(g_light).max())
        for a, b in zip(h2, host):
            assert np.abs(a - b).max() <= 1e-5 * max(np.abs(b).max(), 1e-30)
