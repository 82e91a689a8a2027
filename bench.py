"""Benchmark of the GMorpho hot path on GB300: variable-radius ball closing
plus contour marching cubes (with normals and 20 bilateral iterations) of a
1024^3 fine grid, in the reference's bit-exact two-level mode.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0.  ``value`` is whole-job Gvoxel/s with the inputs
resident in HBM (device-timed with CUDA events); ``e2e`` is the same metric
through the host-buffer C ABI call gm_update_to_host (pinned host
buffers, H2D of the grid and the radius field and D2H of the mesh inside the
timed region; gm_update_to_host overlaps them with the work).  Under
torchrun every rank closes its own replica (weak scaling, no collective on
the data path).

Two more objects ride on rank 0's line: ``batch`` (64 uneven grids, edges
log-uniform in [64, 512], own radius U{1..24}: one batched call against 64
plain calls) and ``serving`` (resident 2048^3 grid, Poisson 200/s brush
edits: edits/s and p50/p99 latency).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gvoxel/s closing+MC at 1024^3 (bit-exact)"
UNIT = "Gvoxel/s"
RES = 512                # base cells per axis -> 1024^3 fine voxels
SEED = 3000              # seed = 1000 * config + instance
BLOBS = 200
BILATERAL = 20           # symmetric closing (GMorpho.cu:7808-7811)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_inputs(ctx, res):
    """Configuration 3: the ~4M-triangle blob isosurface voxelized into the grid
    (grid attributes from the mesh's box, conservative voxelization, timed
    apart), and the radius field r = 2 + floor(30 s(x))."""
    from broxy_gb300 import synth
    return synth.config_inputs(ctx, 3, res=res, voxelize_reps=5)


# Algorithmic bytes per fine voxel of each kernel (its compulsory input and
# output streams in the layout it works on).
KERNEL_BYTES_PER_VOXEL = {
    "k_dil_pass_x": 1 / 8 + 1,            # packed grid in, u8 distance out
    "k_pass_dil_y": 1 + 2,                # u8 distances in, u16 partial sums out
    "k_pass_dil_z": 2 + 1 + 1 / 8,        # u16 in, radius in, packed dilation bits out
    "k_pass_ero_y": 2 + 2,                # u16 in, u16 out (voxel centres)
    "k_pass_ero_z": 2 + 1 / 8,            # u16 in, packed eroded bits out
    "k_pass_erob_y": 1 + 0.5,             # lattice points 2c+1: (res, N, N) u16 in, (res, res, N) out
    "k_pass_erob_z": 0.5 + 1 / 8,         # (res, res, N) u16 in, one flag per cell out
    "k_ero_pass_x": 1 / 8 + 1 + 2 + 1,    # contour bits + radius in, centre + lattice fields out
    "k_axis_pass": 2 + 2,                 # general-radius fallback passes
    "k_final_z": 2 + 1 + 1 / 8,
}


# What limits each kernel, from its ncu capture (profiles/): the min-plus
# passes are bound by the integer ALU pipe of their packed DPX taps, not by
# HBM, so their HBM fraction is low by construction.
LIMITER = {
    "k_pass_dil_z": "integer ALU pipe (packed DPX min-plus taps, up to 2 (r + 2) per output); DRAM traffic = algorithmic",
    "k_pass_dil_y": "integer ALU pipe (packed DPX min-plus taps)",
    "k_pass_ero_y": "integer ALU pipe (packed DPX min-plus taps)",
    "k_pass_ero_z": "integer ALU pipe (packed DPX min-plus taps)",
    "k_bilateral": "HBM (gathers of neighbour normals and records)",
}


# ALU pipe utilisation of the min-plus passes from their ncu capture
# (sm__pipe_alu_cycles_active, profiles/k_pass_dpx_512.md, 512^3 case).
ALU_PIPE_NCU = {"k_pass_dil_y": 0.691, "k_pass_dil_z": 0.735}


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from
# one ncu capture of each kernel, scaled to the 1024^3 workload by the
# units processed (see profiles/).
TRAFFIC = {
    "k_bilateral": 550_000_000,     # 129.0 MB at 1.70M vertices / 3.40M triangles, x4.26
    "k_pass_dil_z": 3_358_000_000,  # 419.7 MB at 512^3 fine voxels, x8
}


def run_ours(args, rank, world):
    import torch
    from broxy_gb300 import api
    torch.cuda.set_device(rank % max(1, torch.cuda.device_count()))
    dev = torch.device("cuda", torch.cuda.current_device())
    ctx = api.Context(dev.index)
    res = args.res
    V = (2 * res) ** 3
    inp = make_inputs(ctx, res)
    X, R, desc = inp["X"], inp["R"], inp["desc"]
    # the voxelizer's kernels, one more run with per-kernel events
    ctx.profile(True)
    ctx.profile_reset()
    ctx.voxelize(desc, inp["P"], inp["T"], out=X)
    torch.cuda.synchronize()
    vox_kernels = {k: round(v["ms"], 3) for k, v in ctx.profile_read().items()}
    ctx.profile(False)
    out = torch.empty_like(X)

    def step():
        ctx.close(desc, X, R, 0, api.L.GM_REF, api.L.GM_SE_SPHERE, out=out)
        Vm, Nm, Tm = ctx.mesh(desc, out, BILATERAL)
        return Vm.shape[0], Tm.shape[0]

    for _ in range(args.warmup):
        nv, nt = step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches0 = ctx.kernel_launches
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev.index) as clk:
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(args.steps):
            nv, nt = step()
        e1.record(st)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    launches = ctx.kernel_launches - launches0
    # per-kernel events (kernels, roofline) from the same number of further
    # steps, outside the timed region
    ctx.profile(True)
    ctx.profile_reset()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile(False)
    ms_max = ms
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_max = float(t.item())
    value = world * V / (ms_max * 1e-3) / 1e9

    # ---- e2e through the host-buffer C ABI (gm_update_to_host)
    e2e_extra = {}
    if args.no_e2e:
        e2e_ms, nv2, nt2 = float("nan"), nv, nt
    else:
        e2e_ms, nv2, nt2, e2e_extra = run_e2e(args, ctx, desc, X, R, nv, nt, world, dev)
    assert (nv2, nt2) == (nv, nt)
    r = finish(args, ctx, prof, ms_max, launches, V, X, R, nv, nt, e2e_ms, clk, world, rank, res, value, desc)
    if r is not None and "e2e" in r:
        r["e2e"].update(e2e_extra)
    r["voxelize"] = {"ms": round(inp["voxelize_ms"], 3), "input_triangles": int(inp["T"].shape[0]),
                     "input_vertices": int(inp["P"].shape[0]), "grid": "%d^3 fine" % (2 * res),
                     "data_res": [int(v) for v in desc.data_res], "kernels_ms": vox_kernels,
                     "note": "gm_voxelize (conservative surface + parity fill), device time, median of 5; "
                             "reported apart, not part of value (GMorpho::Load runs it once per mesh)"}
    return r


def run_e2e(args, ctx, desc, X, R, nv, nt, world, dev):
    import torch
    from broxy_gb300 import api
    hX = torch.empty(X.numel(), dtype=torch.uint8, pin_memory=True)
    hR = torch.empty(R.numel(), dtype=torch.int8, pin_memory=True)
    hX.copy_(X.cpu())
    hR.copy_(R.cpu())
    gs = 0.5  # global scale in world units: gates the morphology on (GMorpho.cu:7783)
    ctx.update(desc, hX, hR, gs)
    hV = torch.empty((nv, 3), dtype=torch.float32, pin_memory=True)
    hN = torch.empty((nv, 3), dtype=torch.float32, pin_memory=True)
    hT = torch.empty((nt, 3), dtype=torch.int32, pin_memory=True)
    def e2e_step():
        # gm_update_to_host: grid and radius field up, closing + mesh, mesh
        # down into the pinned buffers, copies overlapped with the work
        return ctx.update_to_host(desc, hX, hR, gs, hV, hN, hT)

    for _ in range(max(1, args.warmup - 1)):
        e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    marks = []
    for _ in range(args.steps):
        nv2, nt2 = e2e_step()  # returns after its own stream synchronisation
        marks.append(time.perf_counter())
    torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    steps_ms = [(b - a) * 1e3 for a, b in zip([t0] + marks[:-1], marks)]
    # the host link's bandwidth on this machine (the upload bounds the step's start)
    dR = torch.empty_like(R)
    dR.copy_(hR, non_blocking=True)
    torch.cuda.synchronize()
    h0 = time.perf_counter()
    dR.copy_(hR, non_blocking=True)
    torch.cuda.synchronize()
    h2d_gbs = hR.numel() / (time.perf_counter() - h0) / 1e9
    extra = {"step_ms_min": round(min(steps_ms), 3), "step_ms_median": round(statistics.median(steps_ms), 3),
             "step_ms_max": round(max(steps_ms), 3), "h2d_gbs_pinned": round(h2d_gbs, 1)}
    return e2e_ms, nv2, nt2, extra


def finish(args, ctx, prof, ms_max, launches, V, X, R, nv, nt, e2e_ms, clk, world, rank, res, value, desc):
    # ---- roofline of the dominant kernel and of the morphology passes
    hbm, peak_kind = peaks()
    top = max(prof.items(), key=lambda kv: kv[1]["ms"]) if prof else (None, None)
    roof = None
    def kernel_roof(name, rec):
        per_launch_ms = rec["ms"] / rec["launches"]
        if name == "k_bilateral":
            # per iteration: normal in + out, row pointer and record count per vertex
            # (16 + 16 + 4 + 2 B), one 8-byte record per (vertex, neighbour) pair: three per
            # triangle on a closed mesh (each edge shared by two triangles, read from both ends)
            nbytes, model = 38 * nv + 24 * nt, "38 B/vertex + 24 B/triangle per iteration"
        elif name in KERNEL_BYTES_PER_VOXEL:
            nbytes, model = KERNEL_BYTES_PER_VOXEL[name] * V, "%.4f B/fine voxel" % KERNEL_BYTES_PER_VOXEL[name]
        else:
            return {"kernel": name, "bound": "hbm", "achieved": None, "peak": hbm, "unit": "GB/s", "frac": None,
                    "peak_kind": peak_kind, "traffic": None, "per_launch_ms": round(per_launch_ms, 4)}
        ach = nbytes / (per_launch_ms * 1e-3) / 1e9
        out = {"kernel": name, "bound": "hbm", "achieved": round(ach, 1), "peak": hbm, "unit": "GB/s",
               "frac": round(ach / hbm, 4), "peak_kind": peak_kind, "traffic": TRAFFIC.get(name) if res == RES else None,
               "algorithmic_bytes_per_launch": int(nbytes), "bytes_model": model, "limiter": LIMITER.get(name),
               "per_launch_ms": round(per_launch_ms, 4)}
        if name in ALU_PIPE_NCU:
            # HBM is the only memory roofline the peaks give; this kernel is
            # bound by the integer ALU pipe, whose measured utilisation is here
            out["alu_pipe_util_ncu"] = ALU_PIPE_NCU[name]
        if name.startswith(("k_pass_dil", "k_dil_pass", "k_pass_ero", "k_ero_pass")):
            # the operation-level bytes of a morphology pass (read X + read R
            # + write the result, V/8 + V + V/8), credited to this one kernel
            sb = 1.25 * V
            out["operation_bytes_per_launch"] = int(sb)
            out["frac_of_operation_bytes"] = round(sb / (per_launch_ms * 1e-3) / 1e9 / hbm, 4)
        return out

    if top[0] is not None:
        roof = kernel_roof(*top)
    morph_top = max(((k, v) for k, v in prof.items() if k in KERNEL_BYTES_PER_VOXEL), key=lambda kv: kv[1]["ms"],
                    default=(None, None))
    morph_roof = kernel_roof(*morph_top) if morph_top[0] is not None else None
    morph_kernels = [k for k in prof if not k.startswith(("k_mc", "k_adj", "k_scan", "k_vertex", "k_bilateral"))]
    morph_ms = sum(prof[k]["ms"] for k in morph_kernels) / args.steps
    mesh_ms = sum(prof[k]["ms"] for k in prof if k not in morph_kernels) / args.steps
    # per-pass algorithmic bytes: dilation V/8 + R + V/8, erosion V/8 + R + V/8
    morph_bytes = 2 * (V / 8 + V + V / 8)
    morph_gbs = morph_bytes / (morph_ms * 1e-3) / 1e9 if morph_ms > 0 else None

    clocks = clk.summary()
    result = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_max, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8/u16 (integer distance transforms), f32 mesh", "data": "synthetic",
        "config": {"workload": "%d^3 fine grid (res %d): 200-blob solid's triangle mesh voxelized "
                               "(data_res %s), variable radius r = 2 + floor(30 s(x)), GM_REF sphere closing + "
                               "contour MC + 20 bilateral" % (2 * res, res, list(desc.data_res)),
                   "fine_voxels": V, "parallelism": "replicas" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (1 GiB radius field + 2 GiB intermediate fields)",
                   "mesh_vertices": nv, "mesh_triangles": nt},
        "e2e": {"value": round(world * V / (e2e_ms * 1e-3) / 1e9, 3), "unit": UNIT, "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": int(X.numel() + R.numel()),
                "d2h_bytes_per_step": int(24 * nv + 12 * nt)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "roofline_morphology_top": morph_roof,
        "morphology": {"ms": round(morph_ms, 3), "algorithmic_bytes": int(morph_bytes),
                       "achieved_gbs": round(morph_gbs, 1) if morph_gbs else None,
                       "frac_of_peak": round(morph_gbs / hbm, 4) if morph_gbs else None},
        "mesh_ms": round(mesh_ms, 3),
        "kernels": {k: {"launches": v["launches"], "ms_per_step": round(v["ms"] / args.steps, 4)}
                    for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])},
        "clocks": {"sm_mhz": clocks["sm_mhz"], "sm_max_mhz": clocks["sm_max_mhz"], "reasons": clocks["reasons"]},
    }
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(X, R, res, args.cpu_res)
    if rank == 0 and not args.no_batch:
        try:
            result["batch"] = run_batch(args, ctx)
        except Exception as exc:  # reported, never hides the headline line
            result["batch"] = {"error": repr(exc)[:300]}
    if rank == 0 and not args.no_frame_field:
        try:
            result["frame_field"] = run_frame_field(args, ctx, X, R, res, desc)
        except Exception as exc:
            result["frame_field"] = {"error": repr(exc)[:300]}
    if rank == 0 and not args.no_serve:
        import torch
        torch.cuda.empty_cache()
        try:
            result["serving"] = run_serve(args)
        except Exception as exc:
            result["serving"] = {"error": repr(exc)[:300]}
    ctx.close_ctx()
    return result


def run_batch(args, ctx):
    """Batching workload: 64 uneven grids (fine edge log-uniform in [64, 512],
    padded to 32, embedded in the next power-of-two cube), own uniform radius
    U{1..24}: 64 plain gm_close + gm_mesh calls against one batched call."""
    import torch
    from broxy_gb300 import api, synth
    inst = synth.batch_instances(seed=4000, count=64, device="cuda")
    items = []
    for it in inst:
        d = api.make_desc(it["res"], it["data_res"], cell_size=1.0 / it["res"])
        items.append((d, it["X"].contiguous(), None, it["radius"], torch.empty_like(it["X"])))

    def plain():
        tris = 0
        for d, X, R, r, out in items:
            ctx.close(d, X, R, r, api.L.GM_REF, api.L.GM_SE_SPHERE, out=out)
            _, _, T = ctx.mesh(d, out, BILATERAL)
            tris += T.shape[0]
        return tris

    def batched():
        ms = ctx.batch_close_mesh(items, bilateral_iters=BILATERAL, lanes=0)
        return sum(m[2].shape[0] for m in ms)

    def timed(fn, reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            v = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3 / reps, v

    def form(lanes):
        def run():
            ms = ctx.batch_close_mesh(items, bilateral_iters=BILATERAL, lanes=lanes)
            return sum(m[2].shape[0] for m in ms)
        return run

    timed(plain, 1)
    timed(batched, 1)  # first call: autotunes the form (lane count or grouped) and captures the graph
    tuned = ctx.batch_lanes
    plain_ms, t_plain = timed(plain, 3)
    batch_ms, t_batch = timed(batched, 3)
    assert t_plain == t_batch
    forms_ms = {}
    for name, lanes in (("lanes_4", 4), ("grouped", api.L.GM_BATCH_GROUPED)):
        timed(form(lanes), 1)
        forms_ms[name], t_form = timed(form(lanes), 3)
        forms_ms[name] = round(forms_ms[name], 3)
        assert t_form == t_plain

    def kernel_time(fn):
        """Device time of the kernels of one run, by phase (events around
        each launch; the batch then runs without its graph)."""
        ctx.profile(True)
        ctx.profile_reset()
        fn()
        torch.cuda.synchronize()
        prof = ctx.profile_read()
        ctx.profile(False)
        ph = {"closing": 0.0, "mesh": 0.0, "bilateral": 0.0}
        for k, v in prof.items():
            key = "bilateral" if k.startswith("k_bilateral") else (
                "mesh" if k.startswith(("k_mc", "k_adj", "k_scan", "k_rec", "k_row0", "k_brick")) else "closing")
            ph[key] += v["ms"]
        return {k: round(v, 2) for k, v in ph.items()}, round(sum(v["ms"] for v in prof.values()), 2)

    plain_phases, plain_kernel_ms = kernel_time(plain)
    batch_phases, batch_kernel_ms = kernel_time(batched)
    # the grouped form: its min-plus passes (one launch each for all grids,
    # nothing beside them) against the rest of its kernels
    ctx.profile(True)
    ctx.profile_reset()
    form(api.L.GM_BATCH_GROUPED)()
    torch.cuda.synchronize()
    gprof = ctx.profile_read()
    ctx.profile(False)
    gpass = {k: round(v["ms"], 3) for k, v in gprof.items() if k.endswith("_group")}
    vox = sum((2 * it["res"]) ** 3 for it in inst)
    edges = [it["edge"] for it in inst]
    return {"instances": len(inst), "plain_ms": round(plain_ms, 3), "batched_ms": round(batch_ms, 3),
            "speedup": round(plain_ms / batch_ms, 3),
            "form": "grouped" if tuned == api.L.GM_BATCH_GROUPED else "lanes", "lanes": tuned,
            "forms_ms": forms_ms, "grouped_passes_ms": gpass,
            "grouped_passes_total_ms": round(sum(gpass.values()), 3),
            "edge_min": min(edges), "edge_max": max(edges), "fine_voxels": int(vox), "triangles": int(t_batch),
            "radius": "U{1..24}", "closing": "GM_REF sphere, 20 bilateral iterations",
            "batched_gvoxel_s": round(vox / (batch_ms * 1e-3) / 1e9, 3),
            "breakdown": {"plain_kernel_ms": plain_kernel_ms, "plain_phases_ms": plain_phases,
                          "batched_kernel_ms": batch_kernel_ms, "batched_phases_ms": batch_phases,
                          "note": "kernel device time summed over launches (concurrent lanes overlap in the "
                                  "batched wall time); the plain calls' kernel time is their wall time, so "
                                  "batching removes work (padding, per-grid tails), not launch overhead"}}


def run_frame_field(args, ctx, X, R, res, desc):
    """Frame-field workload on the same grid and radius field: a frame field
    of (res/16)^3 nodes over the grid's box with 4 seeded hard constraints
    (FrameField::Generate, biharmonic system), then the rotated-cube closing
    (GMorpho::Update with use_frame_field) and its mesh with the 200
    bilateral iterations of the asymmetric closing."""
    import torch
    from broxy_gb300 import api
    qres = max(2, res // 16)
    rng = np.random.default_rng(6000)
    lo, hi = np.array(desc.bbox_min, np.float64), np.array(desc.bbox_max, np.float64)
    ff = api.FrameField(ctx, tuple(lo), tuple(hi), qres)
    for _ in range(4):
        ff.add_point(lo + (hi - lo) * rng.uniform(0.1, 0.9, 3), rng.normal(size=3) * 0.6)
    t0 = time.perf_counter()
    iters = ff.generate()
    gen_ms = (time.perf_counter() - t0) * 1e3
    Q = ff.quats()
    out = torch.empty_like(X)
    st = torch.cuda.current_stream()
    ctx.close_rotcube(desc, X, Q, qres, R, 0, api.L.GM_REF, out=out)
    ctx.mesh(desc, out, 200)
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    reps = 3
    close_ms = mesh_ms = 0.0
    for _ in range(reps):
        e0.record(st)
        ctx.close_rotcube(desc, X, Q, qres, R, 0, api.L.GM_REF, out=out)
        e1.record(st)
        _, _, T = ctx.mesh(desc, out, 200)
        e2.record(st)
        torch.cuda.synchronize()
        close_ms += e0.elapsed_time(e1) / reps
        mesh_ms += e1.elapsed_time(e2) / reps
    # one more closing with per-kernel events (not part of the timings above)
    ctx.profile(True)
    ctx.profile_reset()
    ctx.close_rotcube(desc, X, Q, qres, R, 0, api.L.GM_REF, out=out)
    torch.cuda.synchronize()
    prof = ctx.profile_read()
    ctx.profile(False)
    ff.destroy()
    vox = (2 * res) ** 3
    return {"field_nodes": qres ** 3, "constraints": 4, "generate_ms": round(gen_ms, 2), "cg_iterations": iters,
            "closing_ms": round(close_ms, 3), "closing_gvoxel_s": round(vox / (close_ms * 1e-3) / 1e9, 3),
            "mesh_ms_200_bilateral": round(mesh_ms, 3), "triangles": int(T.shape[0]),
            "kernels_ms": {k: round(v["ms"], 3) for k, v in sorted(prof.items(), key=lambda kv: -kv[1]["ms"])[:8]}}


def run_serve(args):
    """Serving workload: resident 2048^3 grid with base radius 8, Poisson
    (200/s) brush edits, brush reach U[16,256] fine voxels, new local radius
    U[1,32]; exact local re-closing + re-mesh of the dirty region."""
    import torch
    from broxy_gb300 import api, synth
    res = args.serve_res
    dev = torch.device("cuda")
    # configuration 5's input: the ~8M-triangle blob mesh voxelized into the grid
    mctx = api.Context(torch.cuda.current_device())
    inp = synth.config_inputs(mctx, 5, res=res)
    X, desc = inp["X"], inp["desc"]
    mesh_triangles = int(inp["T"].shape[0])
    del inp
    mctx.close_ctx()
    torch.cuda.empty_cache()
    R = torch.full(((2 * res) ** 3,), 8, dtype=torch.int8, device=dev)
    t0 = time.perf_counter()
    srv = api.Server(desc, X, R, slots=args.serve_slots, max_crop_res=min(res, 512), rmax=32, mode=api.L.GM_REF,
                     bilateral_iters=0)
    init_ms = (time.perf_counter() - t0) * 1e3
    rng = np.random.default_rng(5001)
    n = args.serve_edits
    arrivals = np.cumsum(rng.exponential(1.0 / 200.0, size=n))
    cs = 0.5 * desc.cell_size  # fine voxel edge in world units
    lo, hi = np.array(desc.bbox_min, np.float64), np.array(desc.bbox_max, np.float64)
    edits = []
    for i in range(n):
        c = lo + (hi - lo) * rng.uniform(0.2, 0.8, size=3)
        reach = float(rng.uniform(16, 256))
        r_new = int(rng.integers(1, 33))
        core = min(r_new, reach - 1)
        scale = r_new * cs
        support = (core + (reach - core) * np.sqrt(1 - np.sqrt(0.5))) * cs
        mode = api.L.GM_BRUSH_MAX if r_new >= 8 else api.L.GM_BRUSH_MIN
        edits.append((c, scale, support, mode))
    # warm-up edit (first-touch of the slots)
    srv.submit(edits[0][0], edits[0][1], edits[0][2], 0.0, edits[0][3])
    srv.drain()
    launches0 = srv.kernel_launches
    results = []
    start = time.perf_counter()
    i = 0
    while i < n or srv.pending > 0:
        now = time.perf_counter() - start
        while i < n and arrivals[i] <= now:
            c, scale, support, mode = edits[i]
            srv.submit(c, scale, support, 0.0, mode)
            i += 1
        results += srv.poll()
    results += srv.poll()
    wall = time.perf_counter() - start
    ok = [r for r in results if r["status"] == 0]
    lat = np.array([r["latency_ms"] for r in ok])
    dev_ms = np.array([r["device_ms"] for r in ok])
    crops = np.array([r["crop_res"] for r in ok])
    out = {"grid": "%d^3 fine" % (2 * res), "input_mesh_triangles": mesh_triangles, "edits": n, "completed": len(ok), "rejected": len(results) - len(ok),
           "arrival_rate_per_s": 200, "edits_per_s": round(len(ok) / wall, 2),
           "latency_p50_ms": round(float(np.percentile(lat, 50)), 3) if len(lat) else None,
           "latency_p99_ms": round(float(np.percentile(lat, 99)), 3) if len(lat) else None,
           "device_p50_ms": round(float(np.percentile(dev_ms, 50)), 3) if len(lat) else None,
           "device_p99_ms": round(float(np.percentile(dev_ms, 99)), 3) if len(lat) else None,
           "crop_res_p50": int(np.percentile(crops, 50)) if len(ok) else None,
           "crop_res_max": int(crops.max()) if len(ok) else None,
           "slots": args.serve_slots, "initial_closing_ms": round(init_ms, 1),
           "gpu_launches": srv.kernel_launches - launches0, "target_p99_ms": 16.0}
    srv.destroy()
    return out


def cpu_crop(X, R, res, sub):
    """Centre crop of `sub` base cells per axis of the device inputs (the
    whole grid when sub >= res)."""
    sub = min(sub, res)
    Xh = X.cpu().numpy().reshape(res, res, res)
    Rh = R.cpu().numpy().reshape(2 * res, 2 * res, 2 * res)
    o = (res - sub) // 2
    Xc = np.ascontiguousarray(Xh[o:o + sub, o:o + sub, o:o + sub]).reshape(-1)
    Rc = np.ascontiguousarray(Rh[2 * o:2 * (o + sub), 2 * o:2 * (o + sub), 2 * o:2 * (o + sub)]).reshape(-1)
    return Xc, Rc


def cpu_model():
    """The host CPU's model name (lscpu), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return None


def cpu_baseline(X, R, res, sub):
    """The oracle's reference-algorithm closing + MC + normals on all host
    cores, on a centre crop of the same inputs (bounded sample)."""
    from oracle import oracle as O
    sub = min(sub, res)
    Xc, Rc = cpu_crop(X, R, res, sub)
    t0 = time.perf_counter()
    _, _, Cc = O.close(Xc, sub, [sub] * 3, Rc, 0, 0)
    Vc, Tc = O.mc(Cc, sub, np.zeros(3, np.float32), 1.0 / res)
    O.normals(Vc, Tc, BILATERAL)
    dt = time.perf_counter() - t0
    vox = (2 * sub) ** 3
    return {"value": round(vox / dt / 1e9, 6), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
            "cpu_model": cpu_model(),
            "sample": "centre crop of %d^3 fine voxels of the same grid and radius field; oracle GM_REF closing "
                      "(pyramid traversal, OpenMP) + contour MC + %d bilateral iterations; %.1f s" %
                      (2 * sub, BILATERAL, dt)}


def reference_inputs(res):
    """Configuration 3's inputs built without this library's kernels (the
    reference arm runs none of them): the blob isosurface mesh (torch), its
    grid attributes and conservative voxelization by the oracle, which
    restates this library's voxelizer bit for bit (tests), and the radius
    field."""
    import torch
    from broxy_gb300 import synth
    from oracle import oracle as O
    c = synth.CONFIGS[3]
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    P, T = synth.blob_mesh(synth.mesh_samples(3, res), c["seed"], count=BLOBS, device=dev)
    P, T = P.cpu().numpy(), T.cpu().numpy().astype(np.uint32)
    bmin, _, cell, _ = O.grid_attributes(P, res, synth.MESH_MARGIN)
    X = O.voxelize(P, T, res, bmin, cell)
    R = synth.radius_field(res, c["seed"], base=2, span=30, device=dev)
    return X, (R.cpu().numpy() if dev else R)


def run_reference(args, rank, world):
    """Reference arm: the reference's algorithm on the host cores (the oracle
    port; the reference itself cannot be built here), same metric."""
    if rank != 0:
        return None
    import torch
    from broxy_gb300 import synth
    from oracle import oracle as O
    res, sub = args.res, min(args.cpu_res, args.res)
    X, R = reference_inputs(res)
    times = []
    Xc, Rc = cpu_crop(torch.as_tensor(X), torch.as_tensor(R), res, sub)
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, _, Cc = O.close(Xc, sub, [sub] * 3, Rc, 0, 0)
        Vc, Tc = O.mc(Cc, sub, np.zeros(3, np.float32), 1.0 / res)
        O.normals(Vc, Tc, BILATERAL)
        if i >= args.warmup:
            times.append(time.perf_counter() - t0)
    vox = (2 * sub) ** 3
    val = vox / statistics.mean(times) / 1e9
    return {"metric": METRIC, "value": round(val, 6), "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * statistics.mean(times), 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int (CPU)",
            "data": "synthetic",
            "config": {"workload": "crop: %d^3 fine voxels of the %d^3 grid, same radius field" % (2 * sub, 2 * res)},
            "cpu_baseline": {"value": round(val, 6), "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": "centre crop of %d^3 fine voxels per step" % (2 * sub)},
            "e2e": {"value": round(val, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--res", type=int, default=RES)
    ap.add_argument("--cpu-res", type=int, default=256, help="base cells per axis of the CPU crop")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer leg (profiling runs)")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-grid batching comparison")
    ap.add_argument("--no-serve", action="store_true", help="skip the edit-server measurement")
    ap.add_argument("--no-frame-field", action="store_true", help="skip the frame-field closing measurement")
    ap.add_argument("--serve-res", type=int, default=1024, help="base cells of the resident grid (1024 = 2048^3)")
    ap.add_argument("--serve-slots", type=int, default=4)
    ap.add_argument("--serve-edits", type=int, default=200)
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        r = run_reference(args, rank, world)
    else:
        r = run_ours(args, rank, world)
    if rank == 0 and r is not None:
        print(json.dumps(r))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
