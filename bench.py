"""Frame-pipeline benchmark: Mtris/s on the 199,712-triangle heightfield at 1280x720.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

A step is one frame: Clear + DotGrid + the textured, flat-shaded, clipped
heightfield (317x317 vertices, heights U[-0.1,0.1], seed 0) at 1280x720.
Throughput counts submitted faces (Scene.NumTriangles, scene.go:48-54).

value       device-timed: CUDA events around each frame on the library's
            stream, mesh resident in HBM, L2 flushed (512 MiB write) between
            frames outside the timed events.
e2e         the same frames through the public C-ABI call gr_draw with host
            (page-locked) output buffers: draw items in, RGBA + Z out, copies
            inside the wall-clock timed region.
roofline    the kernel with the largest share of frame time, its algorithmic
            bytes per launch over its CUDA-event duration (profiled pass).
cpu_baseline the CPU restatement of the reference frame path (the oracle),
            timed on this host's cores on a bounded number of frames.

--impl reference runs that CPU frame path (all host threads) as the
reference arm, since the Go reference has no toolchain here.
N > 1 (under torchrun, or --gpus N alone, which starts one process per GPU
itself): the frame is rendered as independent replicas, one per GPU, and
value counts every rank's frames over the slowest rank's time; the 256-view
batch is partitioned by view across the ranks (gorender_gb300.shard).  The
ranks share only a gloo barrier and max-reductions of their timings.  The
stress frame and the differentiable pass are reported at N = 1 only.
parity      the last timed end-to-end frame (and every batch view, and the
            stress frame) compared with the oracle outside the timed regions.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "heightfield-199712tris-1280x720-textured-flat-clipped"
METRIC = "Mtris/s at 1280x720 (plain per-frame)"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self.proc = None
        self.t0 = self.t1 = None

    def start(self):
        q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.reader = threading.Thread(target=self._read, daemon=True)
        self.reader.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), [x.strip() for x in line.split(",")]))

    def mark(self, begin: bool):
        if begin:
            self.t0 = time.time()
        else:
            self.t1 = time.time()

    def stop(self):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = [s for t, s in self.samples if self.t0 and self.t1 and self.t0 - 0.15 <= t <= self.t1 + 0.15]
        if not rows:
            rows = [s for _, s in self.samples]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        mx = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if len(r) > 6 + k and r[6 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_bytes(scene):
    """Bytes a frame must move at minimum, split by the stage that moves them
    (the per-view formula of the measurement plan): per object 16 B a vertex
    position and 12 B a face's indices; flat lighting 16 B a face normal,
    Gouraud 16 B a vertex normal plus 12 B a face's normal indices; textured
    faces 24 B of corner UVs; vertex colours 12 B a vertex; then the texels
    (4 B each) and the framebuffer, RGBA8 + fp32 Z written once (8 B a pixel).
    Intermediate records (bins, triangle set-up) are not algorithmic."""
    project = 0
    lit = bool(scene.flags & 0x08)
    flat = bool(scene.flags & 0x10)
    tex_on = bool(scene.flags & 0x20)
    for o in scene.objects:
        m = o.mesh
        project += 16 * m.nv + 12 * m.nf
        if lit and (flat or m.vnrm is None):
            project += 16 * m.nf
        elif lit:
            project += 16 * m.vnrm.shape[0] + 12 * m.nf
        textured = tex_on and m.uv is not None and m.tex is not None and bool((m.tex >= 0).any())
        if textured:
            project += 24 * m.nf
        if m.vcolor is not None and not (textured and bool((m.tex >= 0).all())):
            project += 12 * m.nv
    texels = sum(4 * t.width * t.height for t in scene.textures if t.pixels is not None)
    raster = 8 * scene.width * scene.height + texels
    return {"project": project, "bin": 0, "raster": raster, "frame": project + raster}


# Stages of the profiled pass (CUDA events between them; every kernel on the
# context stream, so k_clip runs inside the project stage here, while a graph
# replay runs it beside k_setup and k_bin_big).
STAGES = {"project_stage": "k_light + k_vertex + k_cull + k_clip + k_setup",
          "bin_stage": "k_bin_big (+ k_overlay)",
          "raster_stage": "k_plan + k_raster + k_resolve (one view) or k_plan + k_raster, which also clears the empty tiles (a batch)"}
STAGE_KERNELS = {"project_stage": ["k_light", "k_vertex", "k_cull", "k_clip", "k_setup"],
                 "bin_stage": ["k_bin_big", "k_overlay"],
                 "raster_stage": ["k_plan", "k_raster", "k_resolve"],
                 "forward": ["k_diff_vertices", "k_diff_tables", "k_diff_shade"],
                 "backward": ["k_diff_grad", "k_diff_scatter"]}


def _ncu_summary(workload):
    """Per-workload figures from the committed ncu summaries
    (profiles/ncu_workloads.json): DRAM traffic per stage and the issue
    utilisation of each kernel, from one-kernel captures."""
    path = os.path.join(ROOT, "profiles", "ncu_workloads.json")
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f).get(workload, {})


def roofline_of(workload, stage_ms, stage_bytes, stages_desc, launches_per_step=1):
    """The roofline object of a workload: the stage with the largest share of
    the step's device time, its algorithmic bytes over its CUDA-event time,
    against the measured HBM copy bandwidth; traffic and SM issue
    utilisation of the stage's kernels from the ncu summaries."""
    top = max(stage_ms, key=lambda k: stage_ms[k])
    peak, peak_kind = _peaks()
    ms = stage_ms[top]
    achieved = stage_bytes[top] / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
    ncu = _ncu_summary(workload)
    issue = {k: v for k, v in ncu.get("issue_active_pct", {}).items()
             if any(k.startswith(p) for p in STAGE_KERNELS.get(top, []))}
    traffic = ncu.get("stage_dram_bytes", {}).get(top)
    stage_issue = ncu.get("stage_issue_active_pct_time_weighted", {}).get(top)
    return {"bound": "hbm", "kernel": top, "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 5), "traffic": traffic, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": int(stage_bytes[top]),
            "stage_ms": {k: round(float(v), 5) for k, v in stage_ms.items()},
            "stages": stages_desc,
            "sm_issue_active": None if stage_issue is None else {
                "stage_pct_of_peak": stage_issue, "frac": round(stage_issue / 100.0, 4), "per_kernel_pct": issue},
            "ncu_source": ncu.get("source")}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def config_of(scene, ws):
    """The workload both arms report (the GPU tuning goes under "run")."""
    return {"workload": WORKLOAD, "faces": scene.num_triangles, "width": scene.width, "height": scene.height,
            "parallelism": f"replicas x{ws}"}


def spawn_ranks(n):
    """--gpus N outside a launcher: one process per GPU (RANK, LOCAL_RANK,
    WORLD_SIZE and a rendezvous on 127.0.0.1 in each one's environment), the
    same layout torchrun gives; rank 0 prints the line.  Returns the largest
    exit status."""
    import socket
    sock = socket.socket()
    sock.bind(("127.0.0.1", 0))
    port = sock.getsockname()[1]
    sock.close()
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__)] + sys.argv[1:], env=env))
    return max(p.wait() for p in procs)


def run_ours(args):
    import gorender_gb300 as gr
    from gorender_gb300 import _native as N
    from gorender_gb300 import scenes
    import ctypes as C

    ws, rank, local = dist_env()
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    scene = scenes.scene_heightfield_1280x720()
    faces = scene.num_triangles
    ctx = gr.Context(local)
    up = gr.UploadedScene(ctx, scene)
    W, H = scene.width, scene.height
    npx = W * H
    L = N.lib()
    # device outputs owned by the context (NULL pointers)
    n = len(scene.objects)
    # tile size, raster slice and bin capacity for this frame, picked by the
    # library's autotuner (part of warm-up)
    N.check(L.gr_context_autotune(ctx.handle, up.items, n, C.byref(up.params)))
    tuning = ctx.tuning() + (ctx.raster()[0],)  # tile size, bin capacity, slice cost
    for _ in range(max(3, args.warmup)):
        gr.draw_async(ctx, up.items, n, up.params)
        ctx.flush_l2()
    ctx.sync()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if pg:
        pg.barrier()
    ctx.sync()
    sampler.mark(True)
    total_ms = 0.0
    pairs = 31
    k = 0
    while k < args.steps:
        m = min(pairs, args.steps - k)
        for j in range(m):
            ctx.event(2 * j)
            gr.draw_async(ctx, up.items, n, up.params)
            ctx.event(2 * j + 1)
            ctx.flush_l2()
        for j in range(m):
            total_ms += ctx.elapsed_ms(2 * j, 2 * j + 1)
        k += m
    ctx.sync()
    sampler.mark(False)
    launches_per_frame = ctx.last_launches()
    if pg:
        import torch
        t = torch.tensor([total_ms], dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        total_ms = float(t.item())
    sampler.stop()
    ms_per_frame = total_ms / args.steps
    value = faces * args.steps * ws / (total_ms * 1e-3) / 1e6

    # per-kernel profiled pass (same workload, same stream, events around each kernel)
    kms = np.zeros(3)
    kprof = max(20, min(200, args.steps))
    buf = (C.c_float * 3)()
    for _ in range(kprof):
        N.check(L.gr_draw_profiled(ctx.handle, up.items, n, C.byref(up.params), None, None, buf))
        kms += np.array(buf[:])
        ctx.flush_l2()
    kms /= kprof
    # the profiled pass brackets three stages: k_light + k_vertex + k_cull +
    # k_setup (k_clip starts beside k_setup) | k_bin_big and the rest of
    # k_clip | k_plan + k_raster + k_resolve (k_plan is a one-thread-per-tile
    # scan; k_resolve shades the one view's pixels)
    ab = algorithmic_bytes(scene)
    roof = roofline_of("heightfield", dict(zip(["project_stage", "bin_stage", "raster_stage"], kms)),
                       {"project_stage": ab["project"], "bin_stage": 0, "raster_stage": ab["raster"]}, STAGES)
    roof["frame_algorithmic_bytes"] = int(ab["frame"])

    # end to end through gr_draw with page-locked host outputs
    hp = C.c_void_p()
    N.check(L.gr_host_alloc(npx * 8, C.byref(hp)))
    rgba_h = hp.value
    z_h = hp.value + npx * 4
    tpf = C.c_int64()
    e2e_frames = max(10, min(args.steps, 300))
    for _ in range(3):
        N.check(L.gr_draw(ctx.handle, up.items, n, C.byref(up.params), rgba_h, z_h, C.byref(tpf)))
    if pg:
        pg.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_frames):
        N.check(L.gr_draw(ctx.handle, up.items, n, C.byref(up.params), rgba_h, z_h, C.byref(tpf)))
    e2e_s = time.perf_counter() - t0
    if pg:
        import torch
        t = torch.tensor([e2e_s], dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e2e_s = float(t.item())
    h2d = C.c_int64()
    d2h = C.c_int64()
    N.check(L.gr_context_last_transfer_bytes(ctx.handle, C.byref(h2d), C.byref(d2h)))
    # the last timed end-to-end frame, checked against the oracle outside the timed region
    host = np.frombuffer((C.c_uint8 * (npx * 8)).from_address(hp.value), np.uint8)
    last_rgba = host[:npx * 4].reshape(H, W, 4).copy()
    last_z = host[npx * 4:].view(np.float32).reshape(H, W).copy()
    N.check(L.gr_host_free(hp))
    parity = frame_parity(scene, last_rgba, last_z, int(tpf.value)) if rank == 0 else None
    e2e_value = faces * e2e_frames * ws / e2e_s / 1e6

    present = bench_present(ctx, up, scene, e2e_frames)
    batched = bench_batched(ctx, args, local, pg) if not args.skip_batched else None
    # the stress frame and the differentiable pass are single-GPU lines
    stress = bench_stress(local, args) if not args.skip_batched and ws == 1 else None
    diff = bench_diff(local) if not args.skip_batched and ws == 1 else None

    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mtris/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_frame, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+int64",
        "data": "synthetic (seeded heightfield, seeded 16x16 RGBA8 texture)",
        "config": config_of(scene, ws),
        "run": {"binned_triangles": int(tpf.value),
                "l2": "flushed between frames (512 MiB write outside the timed events)",
                "tile_size": tuning[0], "bin_capacity": tuning[1], "slice_cost": tuning[2]},
        "e2e": {"value": round(e2e_value, 3), "unit": "Mtris/s", "h2d_bytes_per_step": int(h2d.value),
                "d2h_bytes_per_step": int(d2h.value), "frames": e2e_frames,
                "ms_per_frame": round(e2e_s * 1e3 / e2e_frames, 4)},
        "roofline": roof,
        "parity": None if parity is None else parity["identical"],
        "parity_check": parity,
        "gpu_launches": int(launches_per_frame * args.steps),
        "clocks": sampler.summary(),
        "e2e_present": present,
        "batched_multiview": batched,
        "stress_1080p": stress,
        "diff_fwd_bwd": diff,
    }
    if rank == 0:
        out["cpu_baseline"] = cpu_baseline(scene, args)
        print(json.dumps(out), flush=True)
    ctx.close()
    if pg:
        pg.destroy_process_group()


def frame_parity(scene, rgba, z, tpf):
    """One rendered frame against the oracle's frame of the same scene (the
    oracle's own matrices): RGBA8 and z-buffer bit patterns and TPF."""
    from oracle import oracle
    oracle.build()
    nt = max(1, min(os.cpu_count() or 1, 64))
    ref_rgba, ref_z, ref_tpf, st = oracle.draw_scene(scene, nthreads=nt, items_override=_oracle_matrices(oracle, scene))
    drgba = int((rgba != ref_rgba).any(axis=-1).sum())
    dz = int((z.view(np.uint32) != ref_z.view(np.uint32)).sum())
    return {"identical": bool(st == 0 and drgba == 0 and dz == 0 and tpf == ref_tpf), "rgba_pixels_differing": drgba,
            "z_values_differing": dz, "tpf": tpf, "oracle_tpf": ref_tpf,
            "rgba_sha256": __import__("hashlib").sha256(rgba.tobytes()).hexdigest()[:16]}


def bench_batched(ctx, args, device, pg=None):
    """256 seeded views (heightfields and icospheres, 100..200k triangles
    log-uniform, four resolutions, mixed materials): one autotuned CUDA-graph
    batch against the same views drawn by plain per-view launches
    (gr_draw_async, one per view, back to back on the same stream).  Both are
    device-timed with events on the library stream; outputs (820 MB over all
    views) exceed L2, so no flush is needed.  Each rank renders the views the
    partition by view gives it (all of them at N = 1); the timed durations
    are the maximum over ranks.  The batch's frames are compared with the
    plain launches' bit for bit and every view with the oracle's frame of
    that view alone (outside the timed regions)."""
    import hashlib

    from gorender_gb300 import renderer as R
    from gorender_gb300 import scenes, shard

    ws, rank, _ = shard.dist_env()
    vs = scenes.multiview_batch(256, seed=0)
    mine = shard.shard_of(vs, rank, ws)
    sb = shard.ShardedBatch(ctx, vs, mine, autotune=True)
    plain_out = [(ctx.device_buffer(sc.width * sc.height * 4), ctx.device_buffer(sc.width * sc.height * 4))
                 for sc in sb.scenes]
    tuning = sb.batch.tuning()
    reps = 10
    for _ in range(3):
        sb.run()
    sb.sync()
    ctx.sync()
    if pg:
        pg.barrier()
    t_batch = []
    for _ in range(reps):
        ctx.event(0)
        sb.run()
        ctx.event(1)
        sb.sync()
        t_batch.append(ctx.elapsed_ms(0, 1))

    def plain_pass():
        for up, (r, z) in zip(sb.uploads, plain_out):
            R.draw_async(ctx, up.items, len(up.scene.objects), up.params, r.ptr, z.ptr)

    for _ in range(2):
        plain_pass()
        try:
            ctx.sync()
        except R.N.GrError as e:  # the first pass may grow the bins; it is re-issued
            if e.code != R.N.GR_ERR_BIN_OVERFLOW:
                raise
    if pg:
        pg.barrier()
    t_plain = []
    for _ in range(reps):
        ctx.event(2)
        plain_pass()
        ctx.event(3)
        ctx.sync()
        t_plain.append(ctx.elapsed_ms(2, 3))
    kms = np.zeros(3)
    for _ in range(5):
        ctx.flush_l2()
        kms += np.array(sb.batch.profile())
    kms /= 5
    per_view = [algorithmic_bytes(sc) for sc in sb.scenes]
    stage_bytes = {"project_stage": sum(b["project"] for b in per_view), "bin_stage": 0,
                   "raster_stage": sum(b["raster"] for b in per_view)}
    if pg:
        import torch
        t = torch.tensor(list(kms), dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        kms = t.numpy()
        for k in ("project_stage", "raster_stage"):
            t = torch.tensor([float(stage_bytes[k])], dtype=torch.float64)
            pg.all_reduce(t, op=pg.ReduceOp.SUM)
            stage_bytes[k] = int(t.item())
    roof = roofline_of("batch256", dict(zip(["project_stage", "bin_stage", "raster_stage"], kms)), stage_bytes,
                       STAGES)
    roof["note"] = ("stages timed outside the graph, one launch sequence per rank; bytes summed over every "
                    "rank's views, time the slowest rank's")
    sb.run()
    sb.sync()
    launches = ctx.last_launches()
    view_tpf = sb.view_tpf()
    mb, mp = statistics.median(t_batch), statistics.median(t_plain)
    same, differing = True, []
    for k, sc in enumerate(sb.scenes):
        rgba, z = sb.frame(k)
        pr = plain_out[k][0].download(rgba.shape, np.uint8)
        pz = plain_out[k][1].download(z.shape, np.float32)
        same = same and np.array_equal(rgba, pr) and np.array_equal(z.view(np.uint32), pz.view(np.uint32))
        if not frame_parity(sc, rgba, z, view_tpf[k])["identical"]:
            differing.append(mine[k])
    my_faces = sb.faces
    for r, z in plain_out:
        r.free()
        z.free()
    sb.close()
    if pg:
        import torch
        t = torch.tensor([mb, mp, 0.0 if same else 1.0, float(len(differing))], dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        mb, mp = float(t[0]), float(t[1])
        same = same and float(t[2]) == 0.0
        if float(t[3]) > 0 and not differing:
            differing = ["on another rank"]
    faces = sum(sc.num_triangles for sc in vs)
    pixels = sum(sc.width * sc.height for sc in vs)
    return {"views": len(vs), "faces": faces, "pixels": pixels, "ranks": ws, "views_this_rank": len(mine),
            "faces_this_rank": my_faces, "partition": "by view, cost = faces + pixels/4, largest first",
            "graph_ms": round(mb, 4), "plain_ms": round(mp, 4),
            "views_per_s": round(len(vs) / (mb * 1e-3), 1), "plain_views_per_s": round(len(vs) / (mp * 1e-3), 1),
            "Mtris_per_s": round(faces / (mb * 1e-3) / 1e6, 2),
            "plain_Mtris_per_s": round(faces / (mp * 1e-3) / 1e6, 2),
            "speedup_vs_plain": round(mp / mb, 3), "identical_output": bool(same), "reps": reps,
            "parity": not differing, "views_differing_from_oracle": differing,
            "tuning": tuning, "kernel_launches_per_batch": launches, "roofline": roof}


def bench_diff(device):
    """Differentiable forward + backward: 64 views at 512x512 of the 81,920-face
    icosphere (level 6, +-5% radial noise), vertex RGB, a 256x256 RGBA fp32
    texture and the light as parameters, per-pixel L2 loss against a target
    rendered from parameters perturbed by N(0, 0.05).  Each call is timed with
    events on the library stream (the calls return after their results are on
    the host: the loss, the light gradient)."""
    import gorender_gb300 as gr
    from gorender_gb300 import renderer as R
    from gorender_gb300 import scenes

    sc = scenes.diff_scene(views=64, size=512, level=6, tex_size=256, seed=0)
    ctx = gr.Context(device)

    def t(a):
        a = np.ascontiguousarray(a, np.float32)
        return ctx.device_buffer(a.nbytes).upload(a)

    mesh = ctx.mesh(sc.mesh)
    world, views = R.diff_views(sc)
    d = R.Diff(ctx, mesh, world, views, tex_size=sc.tex.shape[:2])
    npx = sum(w * h for w, h, _, _, _ in views)
    p = [t(sc.mesh.pos), t(sc.vcol), t(sc.tex)]
    tp = sc.target_params
    q = [t(tp["pos"]), t(tp["vcol"]), t(tp["tex"])]
    target = t(np.zeros((npx, 4), np.float32))
    zeros = t(np.zeros((npx, 4), np.float32))
    d.forward(q[0].ptr, q[1].ptr, q[2].ptr, tp["light"], zeros.ptr, target.ptr)
    g = [ctx.device_buffer(sc.mesh.nv * 16), ctx.device_buffer(sc.mesh.nv * 12), ctx.device_buffer(sc.tex.nbytes)]
    ctx.sync()

    def fwd():
        return d.forward(p[0].ptr, p[1].ptr, p[2].ptr, sc.light, target.ptr)

    def bwd():
        return d.backward(*(x.ptr for x in g))

    for _ in range(3):
        fwd()
        bwd()
    reps = 20
    tf, tb = [], []
    for _ in range(reps):
        ctx.event(6)
        loss = fwd()
        ctx.event(7)
        bwd()
        ctx.event(8)
        ctx.flush_l2()
        tf.append(ctx.elapsed_ms(6, 7))
        tb.append(ctx.elapsed_ms(7, 8))
    mf, mb = statistics.median(tf), statistics.median(tb)
    roof = roofline_of("diff64", {"forward": mf, "backward": mb}, diff_bytes(sc, views),
                       {"forward": "visibility pass (the frame kernels in face-id mode) + k_diff_vertices + "
                                   "k_diff_tables + k_diff_shade",
                        "backward": "k_diff_grad + k_diff_scatter"})
    d.close()
    for x in p + q + g + [target, zeros]:
        x.free()
    ctx.close()
    return {"workload": "diff-icosphere6-81920f-64views-512x512-tex256", "views": 64, "faces": sc.mesh.nf,
            "pixels": npx, "forward_ms": round(mf, 4), "backward_ms": round(mb, 4),
            "backward_over_forward": round(mb / mf, 3), "views_per_s": round(64 / ((mf + mb) * 1e-3), 1),
            "loss": loss, "reps": reps, "l2": "flushed between iterations", "roofline": roof}


def diff_bytes(sc, views):
    """Algorithmic bytes of one differentiable step.  Forward, per view: the
    parameter positions (16 B a vertex), indices (12 B a face) and vertex
    colours (12 B a vertex), then per pixel the 16-byte record the backward
    pass reads and the 16-byte target; once, the fp32 texture (16 B a texel).
    Backward: per pixel the record and the target again (32 B), the
    parameters read once and their gradients written once (positions 16 B,
    colours 12 B a vertex, texels 16 B)."""
    V, F = sc.mesh.nv, sc.mesh.nf
    texels = sc.tex.shape[0] * sc.tex.shape[1]
    px = sum(w * h for w, h, _, _, _ in views)
    fwd = len(views) * (16 * V + 12 * F + 12 * V) + 32 * px + 16 * texels
    bwd = 32 * px + 2 * (16 * V + 12 * V + 16 * texels) + 12 * F
    return {"forward": fwd, "backward": bwd}


def bench_present(ctx, up, scene, frames):
    """The present loop of the reference (Draw, SwapBuffers, show the finished
    frame while the next one renders) through gr_presenter_frame: each call
    queues a frame and returns the previous one's pixels in host memory, the
    device-to-host copy overlapping the next frame.  Wall clock, Python loop."""
    import gorender_gb300 as gr
    r = gr.Renderer(ctx, scene.width, scene.height)
    r.FlatShading = bool(scene.flags & gr.FLAT_SHADING)
    r.set_fov(up.fov)
    objs = [gr.Object(h, o.scale, o.rotation, o.translation) for h, o in zip(up.mesh_handles, scene.objects)]
    cam = gr.Camera(scene.camera.position, scene.camera.direction, scene.camera.up)
    p = gr.Presenter(r)
    for _ in range(5):
        p.frame(objs, cam)
    p.flush()
    t0 = time.perf_counter()
    for _ in range(frames):
        rgba, _ = p.frame(objs, cam, copy=False)  # the host frame, valid until the next call
    p.flush(copy=False)
    dt = time.perf_counter() - t0
    import ctypes as C
    from gorender_gb300 import _native as N
    h2d, d2h = C.c_int64(), C.c_int64()
    N.check(N.lib().gr_context_last_transfer_bytes(ctx.handle, C.byref(h2d), C.byref(d2h)))
    p.close()
    r.close()
    return {"value": round(scene.num_triangles * frames / dt / 1e6, 3), "unit": "Mtris/s", "frames": frames,
            "ms_per_frame": round(dt * 1e3 / frames, 4), "h2d_bytes_per_step": int(h2d.value),
            "d2h_bytes_per_step": scene.width * scene.height * 4,
            "note": "pixels only (the reference presents Pixels2); matrices built by the library per frame"}


def bench_stress(device, args):
    """The 64-icosphere 1920x1080 scene (5.0M faces, per-vertex colours) on a
    context of its own: device-timed frames after the autotuner, L2 flushed
    between frames."""
    import ctypes as C
    import gorender_gb300 as gr
    from gorender_gb300 import _native as N
    from gorender_gb300 import renderer as R
    from gorender_gb300 import scenes

    ctx = gr.Context(device)
    sc = scenes.scene_icospheres_1920x1080()
    up = R.UploadedScene(ctx, sc)
    n = len(sc.objects)
    N.check(N.lib().gr_context_autotune(ctx.handle, up.items, n, C.byref(up.params)))
    for _ in range(3):
        R.draw_async(ctx, up.items, n, up.params)
    ctx.sync()
    frames = 30
    t = []
    for _ in range(frames):
        ctx.event(4)
        R.draw_async(ctx, up.items, n, up.params)
        ctx.event(5)
        ctx.flush_l2()
        ctx.sync()
        t.append(ctx.elapsed_ms(4, 5))
    ms = statistics.median(t)
    kms = np.zeros(3)
    buf = (C.c_float * 3)()
    for _ in range(10):
        N.check(N.lib().gr_draw_profiled(ctx.handle, up.items, n, C.byref(up.params), None, None, buf))
        kms += np.array(buf[:])
        ctx.flush_l2()
    kms /= 10
    ab = algorithmic_bytes(sc)
    roof = roofline_of("icospheres", dict(zip(["project_stage", "bin_stage", "raster_stage"], kms)),
                       {"project_stage": ab["project"], "bin_stage": 0, "raster_stage": ab["raster"]}, STAGES)
    roof["frame_algorithmic_bytes"] = int(ab["frame"])
    rgba, z, tpf = up.render()
    chk = frame_parity(sc, rgba, z, tpf)
    out = {"workload": "icospheres-64obj-1920x1080-gouraud-vertex-rgb", "faces": sc.num_triangles,
           "parity": chk["identical"], "parity_check": chk,
           "ms_per_frame": round(ms, 4), "Mtris_per_s": round(sc.num_triangles / (ms * 1e-3) / 1e6, 2),
           "frames": frames, "tile_size": ctx.tuning()[0], "slice_cost": ctx.raster()[0], "roofline": roof}
    ctx.close()
    return out


def _oracle_matrices(oracle, scene):
    """Per-object (mvp, world) built by the oracle's own restatement of
    projectObject (renderer.go:255-262): the CPU arms load nothing from the
    library."""
    fov = oracle.fov_radians(scene.fov_deg)
    return [oracle.object_matrices(o, scene.camera, scene.width, scene.height, fov) for o in scene.objects]


def _oracle_frames(scene, nthreads: int, budget_s: float, max_frames: int):
    from oracle import oracle
    oracle.build()
    mats = _oracle_matrices(oracle, scene)
    # first frame untimed (builds the ctypes structures, warms caches)
    oracle.draw_scene(scene, nthreads=nthreads, items_override=mats)
    times = []
    t_start = time.perf_counter()
    while len(times) < max_frames and (time.perf_counter() - t_start) < budget_s:
        t0 = time.perf_counter()
        _, _, _, st = oracle.draw_scene(scene, nthreads=nthreads, items_override=mats)
        times.append(time.perf_counter() - t0)
        assert st == 0
    return times


def cpu_baseline(scene, args):
    import platform
    cores = os.cpu_count() or 1
    nt = min(cores, 64)
    times = _oracle_frames(scene, nt, budget_s=10.0, max_frames=200)
    med = statistics.median(times)
    # the same restatement on one thread (a smaller bounded sample)
    times1 = _oracle_frames(scene, 1, budget_s=6.0, max_frames=20)
    med1 = statistics.median(times1)
    return {"value": round(scene.num_triangles / med / 1e6, 4), "unit": "Mtris/s", "cores": nt,
            "kind": "port", "arch": platform.machine(),
            "sample": f"{len(times)} full frames of {WORKLOAD}, median frame time "
            f"{med * 1e3:.2f} ms (C restatement of the reference frame path, objects projected per "
            f"task, raster in {nt} disjoint row bands)",
            "single_thread": {"value": round(scene.num_triangles / med1 / 1e6, 4), "unit": "Mtris/s",
                              "frames": len(times1), "median_ms": round(med1 * 1e3, 2)}}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from gorender_gb300 import scenes
    scene = scenes.scene_heightfield_1280x720()
    cores = os.cpu_count() or 1
    nt = min(cores, 64)
    from oracle import oracle
    oracle.build()
    mats = _oracle_matrices(oracle, scene)
    for _ in range(args.warmup):
        oracle.draw_scene(scene, nthreads=nt, items_override=mats)
    # bounded sample: at most ~60 s of frames, at most K frames
    t0 = time.perf_counter()
    frames = 0
    while frames < args.steps and (time.perf_counter() - t0) < 60.0:
        _, _, _, st = oracle.draw_scene(scene, nthreads=nt, items_override=mats)
        assert st == 0
        frames += 1
    el = time.perf_counter() - t0
    value = scene.num_triangles * frames / el / 1e6
    out = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mtris/s", "n_gpus": ws,
        "steps": frames, "warmup": args.warmup, "ms_per_step": round(el * 1e3 / frames, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+int64",
        "data": "synthetic (seeded heightfield, seeded 16x16 RGBA8 texture)",
        "config": config_of(scene, ws),
        "cpu_baseline": {"value": round(value, 4), "unit": "Mtris/s", "cores": nt, "kind": "port",
                         "sample": f"{frames} of the requested {args.steps} frames (bounded at 60 s) "
                                   f"on {nt} threads: C restatement of the reference frame path"},
        "e2e": {"value": round(value, 4), "unit": "Mtris/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--skip-batched", action="store_true", help="only the plain heightfield frame")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(spawn_ranks(args.gpus))
    if args.impl == "reference":
        run_reference(args)
    else:
        from gorender_gb300 import build as b
        b.build()
        run_ours(args)


if __name__ == "__main__":
    main()
