"""Benchmark of the screen-space NL-PF pass on the synthetic 1920x1080 x 4 spp x 5 depth records.

One step = one full NL-PF pass: the 5 depths filtered deepest-first through the C ABI
(sty_pf_screen_filter_depth), each depth's styled output feeding the parent depth.
  value : Mpath-vertices/s with the records already resident in HBM (valid records filtered per
          second; 41.47 M records, ~90 % valid, per step). Inputs (2.2 GB) exceed the 129 MB L2,
          so no explicit flush is needed between steps.
  e2e   : the same metric through the public API with HOST buffers: every step copies the
          records from pinned host memory (per depth, deepest first, on a copy stream; a depth's
          upload waits only for the previous step's filter of that depth, so uploads overlap the
          filters), runs the pass and reads the depth-0 result back on a third stream; the result
          is checked equal to the resident pass's.
  roofline: the dominant kernel (k_pf_screen4) against measured HBM bandwidth, from CUDA events
          around each launch on the launching stream; `alu_roofline` gives the binding FP32 roof
          (FMAs per pair by the exponent form the tiles take).
  cpu_baseline: the FP32 CPU restatement (oracle, all host cores) on a bounded band of rows.
`--impl reference` times the reference's CPU path (the restatement; the reference's own Rust /
LuisaCompute CPU backend cannot be built on these machines) and prints the same metric.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import tempfile
import pathlib
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "NL-PF Mpath-vertices/s; NL-NRC BF16 vs FP32 Msamples/s at equal image MSE"
W_, H_, S_, D_ = 1920, 1080, 4, 5
WORKLOAD = "NL-PF screen-space filter, synthetic records 1920x1080 x 4 spp x 5 depths, radius 16 px"
# HBM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of one k_pf_screen4 launch at this
# size (1080p x 4 spp, child input present), from the ncu capture summarised in
# profiles/k_pf_screen_1080p_x4spp.md
NCU_TRAFFIC_PER_LAUNCH = 535.2e6 + 90.8e6


def _rank_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.gpu = gpu_index
        # the raw samples (the JSON line carries their summary); STY_CLOCKS_DIR keeps them
        out_dir = os.environ.get("STY_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = pathlib.Path(out_dir) / f"clocks_rank{gpu_index}.csv"

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def expanded_fraction(planes, valid, W, H, S, D, sigma_pos, tw=32, th=16, lim=16.0):
    """Fraction of the filter's (tile, depth) launches units that take the expanded exponent form:
    every valid query of a 32 x 16 tile within |p * pscale - c|^2 <= 16 of the tile's mean c
    (the kernel's own test, done here in FP64 on the host)."""
    pscale = math.sqrt(1.4426950408889634 / (2.0 * sigma_pos * sigma_pos))
    hp, wp = -(-H // th) * th, -(-W // tw) * tw
    exp_tiles = tiles = 0
    for d in range(D):
        sl = slice(d * W * H * S, (d + 1) * W * H * S)
        v = np.zeros((hp, wp, S), bool)
        v[:H, :W] = valid[sl].reshape(H, W, S) != 0
        p = np.zeros((3, hp, wp, S))
        p[:, :H, :W] = planes[0:3, sl].reshape(3, H, W, S) * pscale
        v = v.reshape(hp // th, th, wp // tw, tw, S).transpose(0, 2, 1, 3, 4).reshape(hp // th, wp // tw, -1)
        p = p.reshape(3, hp // th, th, wp // tw, tw, S).transpose(0, 1, 3, 2, 4, 5).reshape(3, hp // th, wp // tw, -1)
        cnt = v.sum(-1)
        c = (p * v).sum(-1) / np.maximum(cnt, 1)
        q = (((p - c[..., None]) ** 2).sum(0) * v).max(-1)
        live = cnt > 0
        tiles += int(live.sum())
        exp_tiles += int((live & (q <= lim)).sum())
    return exp_tiles / max(tiles, 1)


def cpu_baseline(sty, orc, planes, valid, depths: int = D_, budget_s: float = 12.0):
    """FP32 CPU restatement on all host threads over a band of query rows at every depth, deepest
    first, each depth's band reading the deeper depth's band output as its incoming radiance (the
    same pass shape as the GPU step; the same rows at every depth). The band height is set on
    depth 1 so that the five bands take about budget_s / 4 together; Mpath-vertices/s = the bands'
    valid vertices / their total time."""
    n = W_ * H_ * S_
    assert planes.shape[1] == n * depths
    rec = sty.pf.host_records(planes, valid, W_, H_, S_, depths)
    prm = sty.c2_params().c()
    style = sty.c2_style()
    target = budget_s / 4 / depths
    rows = 2 * max(8, orc.num_threads())  # the restatement splits the band's rows over the host threads
    while True:  # band height: depth 1 (the styled depth) alone takes about target seconds
        t0 = time.perf_counter()
        orc.pf_screen_filter_depth_f32(rec, min(1, depths - 1), prm, style, out_next=None, y0=540, y1=540 + rows)
        elapsed = time.perf_counter() - t0
        if elapsed >= target or rows >= 256:
            break
        rows = min(256, max(rows * 2, int(rows * target / max(elapsed, 1e-3))))
    total_t, total_v = 0.0, 0
    nxt = None
    y0 = H_ // 2 - rows // 2
    for d in range(depths - 1, -1, -1):
        t0 = time.perf_counter()
        out = orc.pf_screen_filter_depth_f32(rec, d, prm, style, out_next=nxt, y0=y0, y1=y0 + rows)
        total_t += time.perf_counter() - t0
        total_v += int(valid[d * n + y0 * W_ * S_: d * n + (y0 + rows) * W_ * S_].sum())
        nxt = out
    return {"value": total_v / total_t / 1e6, "unit": "Mpath-vertices/s", "cores": orc.num_threads(),
            "kind": "port",
            "sample": f"query rows {y0}..{y0 + rows - 1} of 1080 at each of the {depths} depths (x 1920 px x 4 spp, "
                      f"radius 16, toon at depth 1, each depth's input the deeper depth's output), {total_v} valid "
                      f"vertices in {total_t:.2f} s, FP32 restatement of the filter"}


def nrc_bench(sty, frames: int, warmup: int, dev, bf16_peak: float):
    """NL-NRC on the neural-cache workload scene (10 x 10 icospheres of subdivision 3 = 128 000
    triangles on a ground quad, GGX alpha ~ U[0.05, 0.5], albedo ~ U[0.2, 0.9], one area light);
    network: frequency encoding of 11 inputs to 64, 5 x 64 ReLU, RGB; relative L2, Adam lr 1e-2.
    Per frame: one training step on a batch of 2^16 rows drawn from that frame's tracer rows (1 path
    per pixel of a 192 x 108 view, depths 0..4) and inference of the 1920 x 1080 first-hit queries
    (2 073 600 rows); `frames` frames (1 spp each) for the BF16 tcgen05 path and the FP32
    CUDA-core path on the same rows. Msamples/s = (2^16 + queries) per frame / NRC time (rows
    resident in HBM; the tracer is not timed). Image quality: after training, the cache read at
    the first hit of a 240 x 135 view (4 rays per pixel) against a 1024-spp self-reuse render of
    that view, beside the 1-spp cache-free render."""
    import numpy as np
    import torch
    D, nt = 4, 1 << 16
    stream = torch.cuda.current_stream(dev)
    pos, mids, mats, cam = sty.scene.icosphere_grid(1920, 1080)
    view = lambda w, h: sty.scene.camera(tuple(cam.eye), tuple(cam.target), fov_y=cam.fov_y, width=w, height=h)  # noqa: E731
    q_scene = sty.scene.Scene(pos, mids, mats, cam)
    t_scene = sty.scene.Scene(pos, mids, mats, view(192, 108))
    e_scene = sty.scene.Scene(pos, mids, mats, view(240, 135))
    t0 = time.perf_counter()
    qx, _ = q_scene.nrc_samples(sty.scene.NRC_SAMPLES_QUERY, 1, D, seed=99)
    rows = [t_scene.nrc_samples(sty.scene.NRC_SAMPLES_TRAIN, 1, D, seed=1000 + f) for f in range(frames + warmup)]
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    nq = qx.shape[0]
    out = torch.empty((nq, 3), device=dev)
    # reference image and the cache-free render of the evaluation view
    self_only = lambda seed, b, r=1: sty.scene.render_config(max_depth=D, branch=b, repeats=r, radius_scale=(1e-4,),  # noqa: E731
                                                              reuse=(8,), smis=False, seed=seed)
    gt = e_scene.render(self_only(4242, 256, 4))[0].cpu().numpy()
    ex, ele = e_scene.nrc_samples(sty.scene.NRC_SAMPLES_QUERY, 4, D, seed=5)
    lit = (ele.reshape(4, 135, 240, 3).amax((0, 3)) > 0).cpu().numpy()

    def mse(im):
        e = ((im - gt) ** 2).mean(2)
        return float(e.mean()), float(e[~lit].mean())

    pt = [mse(e_scene.render(self_only(10 + k, 1))[0].cpu().numpy()) for k in range(4)]
    res = {"cache_free_1spp_mse": float(np.mean([m[0] for m in pt])),
           "cache_free_1spp_mse_unlit": float(np.mean([m[1] for m in pt]))}
    for name, prec in (("fp32", sty.nrc.STY_NRC_FP32), ("bf16", sty.nrc.STY_NRC_BF16)):
        cfg = lambda: sty.nrc.config(sty.nrc.C4_FREQS, 3, nt, 5, prec, learning_rate=1e-2, seed=1)  # noqa: E731
        warm = sty.nrc.NRC(cfg())
        for f in range(warmup):
            warm.train(rows[frames + f][0], rows[frames + f][1], 1, stream=stream, want_loss=False)
            warm.inference(qx, out, stream=stream)
        warm.close()
        net = sty.nrc.NRC(cfg())
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for f in range(frames):
            net.train(rows[f][0], rows[f][1], 1, stream=stream, want_loss=False)
            net.inference(qx, out, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / frames
        # inference alone (the tensor-core kernel for bf16), for the roofline
        i0, i1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        i0.record(stream)
        for _ in range(frames):
            net.inference(qx, out, stream=stream)
        i1.record(stream)
        torch.cuda.synchronize()
        inf_ms = i0.elapsed_time(i1) / frames
        def image_mse(n_):
            pe = n_.inference(ex)
            pe = torch.where((ex[:, 7] > 0)[:, None], pe, torch.zeros_like(pe))
            return mse(pe.reshape(4, 135, 240, 3).mean(0).double().cpu().numpy())

        # image quality: the timed network and three more network seeds on the same rows (one
        # training's MSE varies by ~15 % from seed to seed, more than the precisions differ)
        per_seed = [image_mse(net)]
        net.close()
        for seed in (2, 3, 4):
            n2 = sty.nrc.NRC(sty.nrc.config(sty.nrc.C4_FREQS, 3, nt, 5, prec, learning_rate=1e-2, seed=seed))
            for f in range(frames):
                n2.train(rows[f][0], rows[f][1], 1, stream=stream, want_loss=False)
            per_seed.append(image_mse(n2))
            n2.close()
        m_all = float(np.mean([m[0] for m in per_seed]))
        m_unlit = float(np.mean([m[1] for m in per_seed]))
        # algorithmic FLOPs: the 3-wide output layer at N = 3 (the MMAs pad it to 16); training per
        # sample = forward + weight gradients + input gradients of every layer but the first
        flops_q = 2.0 * (5 * 64 * 64 + 3 * 64)
        flops_t = 3.0 * flops_q - 2.0 * 64 * 64
        res[name] = {"ms_per_frame": ms, "msamples_per_s": (nq + nt) / ms / 1e3,
                     "inference_ms": inf_ms, "train_ms": ms - inf_ms,
                     "inference_tflops": nq * flops_q / (inf_ms / 1e3) / 1e12,
                     "train_tflops": nt * flops_t / ((ms - inf_ms) / 1e3) / 1e12,
                     "image_mse": m_all, "image_mse_unlit": m_unlit,
                     "image_mse_per_seed": [round(m[0], 7) for m in per_seed], "frames": frames}
    res["speedup_bf16_over_fp32"] = res["bf16"]["msamples_per_s"] / res["fp32"]["msamples_per_s"]
    res["image_mse_ratio_bf16_over_fp32"] = res["bf16"]["image_mse"] / res["fp32"]["image_mse"]
    res["image_mse_unlit_ratio_bf16_over_fp32"] = res["bf16"]["image_mse_unlit"] / res["fp32"]["image_mse_unlit"]
    ach = res["bf16"]["inference_tflops"]
    res["roofline"] = {"bound": "tensor", "kernel": "k_nrc_fwd_tc", "achieved": ach, "peak": bf16_peak,
                       "unit": "TFLOP/s", "frac": ach / bf16_peak, "peak_source": "measured (bf16 burst)"}
    res["config"] = {"workload": "NRC on 10x10 subdivision-3 icospheres (128k tris), GGX, one area light",
                     "queries_per_frame": nq, "train_batch_per_frame": nt,
                     "train_rows_per_frame": int(np.mean([r[0].shape[0] for r in rows[:frames]])),
                     "network": "freq-enc 11->64, 5x64 ReLU, 3", "lr": 1e-2, "loss": "relative L2",
                     "eval": "240x135, cache at first hit (4 rays/px) vs 1024-spp self-reuse render, mean of 4 network seeds",
                     "tracer_seconds_for_rows": gen_s}
    for s_ in (q_scene, t_scene, e_scene):
        s_.close()
    return res


def grid_nrc_bench(sty, frames: int, warmup: int, dev, bf16_peak: float):
    """The reference's NL-NRC network (hash grid 22 x 4 levels on 2^19-entry FP16 tables, one-blob 7 x
    4, identity; 144 -> 5 x 128 ReLU -> 3; the teaser's configuration with max depth 12, so 32 inputs
    per row in the reference's row layout) on the interior workload scene. Per frame: one training
    step on a 2^16 batch from that frame's tracer rows (1 path per pixel of a 192 x 108 view) and
    inference of the 1920 x 1080 first-hit queries (2 073 600 rows), as in the NL-NRC frames of the
    spherical network. Training runs layer by layer on the tcgen05 GEMMs of gemm_tc.cu (BF16
    operands; FP16, tiny-cuda-nn's precision, timed beside it); inference runs the fused tensor-core
    path (k_grid_tiles + k_grid_mlp_tc), the layer-by-layer GEMM path timed beside it on the same
    rows."""
    import numpy as np
    import torch
    D, nt = 12, 1 << 16
    stream = torch.cuda.current_stream(dev)
    pos, mids, mats, cam = sty.scene.room_with_door(1920, 1080)
    view = sty.scene.camera(tuple(cam.eye), tuple(cam.target), fov_y=cam.fov_y, width=192, height=108)
    q_scene = sty.scene.Scene(pos, mids, mats, cam)
    t_scene = sty.scene.Scene(pos, mids, mats, view)
    ref_rows = sty.scene.NRC_ROWS_REF
    qx, _ = q_scene.nrc_samples(sty.scene.NRC_SAMPLES_QUERY, 1, D, layout=ref_rows, seed=99)
    rows = [t_scene.nrc_samples(sty.scene.NRC_SAMPLES_TRAIN, 1, D, layout=ref_rows, seed=1000 + f)
            for f in range(frames + warmup)]
    nq = qx.shape[0]
    out = torch.empty((nq, 3), device=dev)
    res = {}
    for name, layered, fp16 in (("tensor_core", False, False), ("layered", True, False), ("fp16", False, True)):
        net = sty.nrc.NRC(sty.nrc.grid_config(max_depth=D, batch_size=nt, learning_rate=1e-2, seed=1,
                                              layered=layered, fp16=fp16))
        for f in range(warmup):
            net.train(rows[frames + f][0], rows[frames + f][1], 1, stream=stream, want_loss=False)
            net.inference(qx, out, stream=stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for f in range(frames):
            net.train(rows[f][0], rows[f][1], 1, stream=stream, want_loss=False)
            net.inference(qx, out, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / frames
        i0, i1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        i0.record(stream)
        for _ in range(frames):
            net.inference(qx, out, stream=stream)
        i1.record(stream)
        torch.cuda.synchronize()
        inf_ms = i0.elapsed_time(i1) / frames
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for f in range(frames):
            net.train(rows[f][0], rows[f][1], 1, stream=stream, want_loss=False)
        t1.record(stream)
        torch.cuda.synchronize()
        res[name] = {"ms_per_frame": ms, "msamples_per_s": (nq + nt) / ms / 1e3, "inference_ms": inf_ms,
                     "inference_mqueries_per_s": nq / inf_ms / 1e3, "train_ms": t0.elapsed_time(t1) / frames,
                     "params": net.param_count(), "frames": frames,
                     "operands": "FP16 (loss scale 128)" if fp16 else "BF16",
                     "inference_path": "layer by layer" if (layered or fp16) else "fused tensor-core"}
        net.close()
    mlp_flops = 2.0 * (144 * 128 + 4 * 128 * 128 + 3 * 128)  # algorithmic MLP FLOPs per query (output at N = 3)
    tc = res["tensor_core"]
    res["inference_speedup_tc_over_layered"] = res["layered"]["inference_ms"] / tc["inference_ms"]
    res["inference_mlp_tflops"] = nq * mlp_flops / (tc["inference_ms"] / 1e3) / 1e12
    res["inference_mlp_frac_of_bf16_peak"] = res["inference_mlp_tflops"] / bf16_peak
    res["config"] = {"workload": "interior room (~377k tris), 1920x1080 first-hit queries, rows in the reference layout",
                     "queries_per_frame": nq, "train_batch_per_frame": nt,
                     "train_rows_per_frame": int(np.mean([r[0].shape[0] for r in rows[:frames]])),
                     "network": "hash grid 22x4 (2^19, FP16) + one-blob 7x4 + identity -> 144, 5x128 ReLU, 3",
                     "lr": 1e-2, "loss": "relative L2",
                     "note": "inference is bound by the encoder's random table gathers (L2 sectors)"}
    q_scene.close()
    t_scene.close()
    return res


def c1_bench(sty, repeats: int = 3):
    """End-to-end NL-PF render of the Cornell box workload: 256x256 px, 16 paths per pixel, vertex
    depths 0..5, reference-mode filter (radius 0.05 = 1 % of the box x 5, reuse 64, SMIS, clusters
    off), reference toon (band width 0.2) on every surface. Mpath-vertices/s = traced and filtered
    vertices / wall time of sty_pf_render (trace + grid + filter + splat)."""
    import torch
    a = sty.abi
    pos, mids, mats, cam = sty.scene.cornell_box(256, 256, style=(0, -1, -1, -1))
    sc = sty.scene.Scene(pos, mids, mats, cam)
    progs = [a.style_program([a.toon(0.2)])]
    cfg = sty.scene.render_config(max_depth=5, branch=16, radius_scale=(5.0,), reuse=(64,), seed=0)
    sc.render(cfg, progs)  # warm-up (module load, allocator)
    torch.cuda.synchronize()
    times, nv = [], 0
    for r in range(repeats):
        cfg.seed = r + 1
        t0 = time.perf_counter()
        film, nv = sc.render(cfg, progs)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    sc.close()
    return {"workload": "Cornell box 256x256, 16 paths/px, depth 5, reference-mode NL-PF (r=0.05, reuse 64, SMIS)",
            "mpath_vertices_per_s": nv / t / 1e6, "vertices": nv, "seconds_per_render": t,
            "image_mean": float(film.mean())}


def c1_screen_setup(sty, W: int = 256, H: int = 256):
    """The plain NL-PF workload with the screen-space bilateral filter on traced vertices: the Cornell
    box at W x H, 16 paths per pixel, vertex depths 0..5, radius 8 px, sigma_pos 0.05, sigma_nrm 0.2
    (no pixel-distance term), 4-level toon (0.1 / 0.3 / 0.6) of the first-bounce radiance."""
    a = sty.abi
    pos, mids, mats, cam = sty.scene.cornell_box(W, H)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    progs = [a.style_program([a.toon_steps([0.1, 0.3, 0.6], [0.05, 0.2, 0.45, 1.0], depth_mask=1 << 1)])]
    cfg = sty.scene.screen_render_config(max_depth=5, branch=16, radius=8, sigma_pixel=0.0, sigma_pos=0.05,
                                         sigma_nrm=0.2, screen_style=0, seed=0)
    return sc, progs, cfg


def c1_bilateral_bench(sty, repeats: int = 5):
    """End-to-end NL-PF render of the Cornell box workload with the screen-space bilateral filter
    (STY_PF_MODE_SCREEN, c1_screen_setup): trace (the tracer writes the screen records) + filter
    from depth 5 down to 0 + splat into the FP64 film. Mpath-vertices/s = traced and filtered
    vertices / time of sty_pf_render (CUDA events on its stream, after an untimed warm-up render);
    the breakdown times the trace (sty_pf_trace_records) and the filter pass apart."""
    import torch
    sc, progs, cfg = c1_screen_setup(sty)
    stream = torch.cuda.current_stream()
    sc.render(cfg, progs)  # warm-up (module load, render buffers)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times, nv, film = [], 0, None
    for r in range(repeats):
        cfg.seed = r + 1
        e0.record(stream)
        film, nv = sc.render(cfg, progs)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t = statistics.median(times)
    rs, _, nvr = sc.trace_records(cfg, progs)
    torch.cuda.synchronize()
    e0.record(stream)
    sc.trace_records(cfg, progs)
    e1.record(stream)
    torch.cuda.synchronize()
    t_trace = e0.elapsed_time(e1) / 1e3
    prm = sty.ScreenParams(radius=8, sigma_pixel=0.0, sigma_pos=0.05, sigma_nrm=0.2)
    out = sty.pf_screen_filter(rs, prm, progs[0])
    torch.cuda.synchronize()
    e0.record(stream)
    sty.pf_screen_filter(rs, prm, progs[0], out=out)
    e1.record(stream)
    torch.cuda.synchronize()
    t_filter = e0.elapsed_time(e1) / 1e3
    n_q = rs.width * rs.height * rs.spp * rs.depths
    pairs = n_q * (2 * prm.radius + 1) ** 2 * rs.spp
    res = {"workload": "Cornell box 256x256, 16 paths/px, depth 5, traced vertices -> screen-space bilateral "
                       "filter (radius 8 px, sigma_pos 0.05, sigma_nrm 0.2), toon 0.1/0.3/0.6 at depth 1",
           "mpath_vertices_per_s": nv / t / 1e6, "vertices": nv, "seconds_per_render": t,
           "trace_ms": t_trace * 1e3, "filter_ms": t_filter * 1e3,
           "filter_pair_evaluations": pairs, "filter_gpairs_per_s": pairs / t_filter / 1e9,
           "image_mean": float(film.mean())}
    sc.close()
    return res, rs


def c1_bilateral_cpu_baseline(sty, orc, rs, budget_s: float = 8.0):
    """The FP32 restatement of the filter (oracle, all host threads) on a band of depth-1 query rows
    of the traced Cornell records (depth-2 input zero): the filter stage of the render on the CPU,
    tracing not included (a lower bound of the CPU time per vertex)."""
    import torch
    torch.cuda.synchronize()
    planes = rs.planes.cpu().numpy()
    valid = rs.valid.cpu().numpy()
    W, H, S, D = rs.width, rs.height, rs.spp, rs.depths
    n = W * H * S
    rec = sty.pf.host_records(planes, valid, W, H, S, D)
    prm = sty.ScreenParams(radius=8, sigma_pixel=0.0, sigma_pos=0.05, sigma_nrm=0.2).c()
    a = sty.abi
    style = a.style_program([a.toon_steps([0.1, 0.3, 0.6], [0.05, 0.2, 0.45, 1.0], depth_mask=1 << 1)])
    nxt = np.zeros((3, n), dtype=np.float32)
    rows, y0 = 2, H // 2 - 16
    while True:
        t0 = time.perf_counter()
        orc.pf_screen_filter_depth_f32(rec, 1, prm, style, out_next=nxt, y0=y0, y1=y0 + rows)
        elapsed = time.perf_counter() - t0
        if elapsed >= budget_s / 4 or rows >= 64:
            break
        rows = min(64, max(rows * 2, int(rows * (budget_s / 4) / max(elapsed, 1e-3))))
    nvalid = int(valid[n + y0 * W * S: n + (y0 + rows) * W * S].sum())
    return {"value": nvalid / elapsed / 1e6, "unit": "Mpath-vertices/s", "cores": orc.num_threads(), "kind": "port",
            "sample": f"depth-1 query rows {y0}..{y0 + rows - 1} of {H} of the traced records (x {W} px x {S} "
                      f"paths, radius 8), {nvalid} valid vertices in {elapsed:.2f} s, FP32 restatement of the "
                      f"filter; tracing not timed"}


def c3_bench(sty, reps: int = 20):
    """Adjoint of the screen-space filter + smoothed ramp (36 parameters: sharpness 50, 8
    thresholds, 8 RGB ramp colours, sigma_pixel / sigma_pos / sigma_nrm) on the plain NL-PF
    workload's traced buffers at 512 x 512 x 4 paths per pixel (the Cornell box, depth 5): the
    depth-0 records with the filtered depth-1 result (radius 8, sigma_pos 0.05, sigma_nrm 0.2, toon
    0.1 / 0.3 / 0.6) as child input, radius 8, bandwidths (4, 0.05, 0.2). The loss target is the
    image the forward renders from the parameters perturbed by N(0, 0.05^2) (relative, seed 1). One
    gradient = forward + loss + backward (weights recomputed, two sweeps), timed with CUDA events
    over `reps` gradients; correctness against FP64 central differences is in the tests."""
    import ctypes as C
    import torch
    a = sty.abi
    W, H, S, R = 512, 512, 4, 8
    pos, mids, mats, cam = sty.scene.cornell_box(W, H)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    cfg = sty.scene.screen_render_config(max_depth=5, branch=S, radius=R, sigma_pixel=0.0, sigma_pos=0.05,
                                         sigma_nrm=0.2, screen_style=0, seed=0)
    toon = a.style_program([a.toon_steps([0.1, 0.3, 0.6], [0.05, 0.2, 0.45, 1.0], depth_mask=1 << 1)])
    rs_all, _, _ = sc.trace_records(cfg, [toon])
    out = sty.pf_screen_filter(rs_all, sty.ScreenParams(R, 0.0, 0.05, 0.2), toon)
    n = W * H * S
    rs = sty.RecordSet(rs_all.planes[:, :n].contiguous(), rs_all.valid[:n].contiguous(), W, H, S, 1)
    child = out[1].contiguous()
    del rs_all, out
    rng = np.random.default_rng(4)
    p = np.zeros(36, np.float64)
    p[0] = 50.0
    p[1:9] = np.sort(rng.uniform(0.02, 0.8, 8))
    p[9:33] = np.sort(rng.uniform(0.0, 1.0, 24))
    p[33:36] = [4.0, 0.05, 0.2]
    pt = p + np.random.default_rng(1).normal(0.0, 0.05, 36) * np.abs(p)
    pt[33:36] = np.abs(pt[33:36])
    # the target image: the forward (filter + ramp at depth 0, pixel mean over the paths) at pt
    ramp = a.style_program([a.ramp_smooth(float(pt[0]), pt[1:9].tolist(), pt[9:33].reshape(8, 3).tolist(),
                                          depth_mask=1)])
    tout = sty.pf_screen_filter_depth(rs, 0, sty.ScreenParams(R, float(pt[33]), float(pt[34]), float(pt[35])), ramp,
                                      out_next=child)
    target = tout.reshape(3, H, W, S).mean(-1).permute(1, 2, 0).contiguous()
    grad = torch.zeros(36, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    prm = (C.c_float * 36)(*p.astype(np.float32))

    def one():
        sty.check(sty.lib().sty_pf_adjoint(C.byref(rs.c()), 0, R, prm, 8, C.c_void_p(child.data_ptr()),
                                           C.c_void_p(target.data_ptr()), C.c_void_p(grad.data_ptr()), None,
                                           C.c_void_p(sp)))

    for _ in range(3):
        one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        one()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    loss = C.c_float()
    sty.check(sty.lib().sty_pf_adjoint(C.byref(rs.c()), 0, R, prm, 8, C.c_void_p(child.data_ptr()),
                                       C.c_void_p(target.data_ptr()), C.c_void_p(grad.data_ptr()), C.byref(loss),
                                       C.c_void_p(sp)))
    sc.close()
    return {"workload": "adjoint on the traced Cornell records 512x512 x 4 paths (depth 0, child = filtered "
                        "depth 1), radius 8, 36 parameters (filter bandwidths + smoothed ramp, sharpness 50), "
                        "target rendered from parameters perturbed by N(0, 0.05^2), seed 1",
            "ms_per_gradient": ms, "gradients_per_s": 1e3 / ms, "mrecords_per_s": n / ms / 1e3,
            "valid_records": int(rs.valid.sum().item()), "loss": loss.value,
            "grad_finite": bool(torch.isfinite(grad).all().item())}


def brpt_bench(sty, W: int = 160, H: int = 90):
    """One branching path tracer render of the interior workload at the teaser's branching
    (32, 14, 8, 6), after an untimed warm-up render (the `brpt` entry of c5_bench without the
    reference image)."""
    import torch
    a = sty.abi
    pos, mids, mats, cam = sty.scene.room_with_door(W, H)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    progs = [a.style_program([a.toon(0.2, depth_mask=0b11),
                              a.ramp_smooth(30.0, [0.02, 0.15, 0.6],
                                            [(0.08, 0.1, 0.2), (0.55, 0.45, 0.35), (1.3, 1.2, 1.0)],
                                            depth_mask=0b11)])]
    sc.brpt_render(sty.scene.brpt_config(max_depth=8, inner_samples=(4, 2), repeats=1, seed=2), progs)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, st = sc.brpt_render(sty.scene.brpt_config(max_depth=8, inner_samples=(32, 14, 8, 6), repeats=1, seed=5), progs)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    sc.close()
    return {"seconds": t, "vertices": int(st.vertices), "mvertices_per_s": st.vertices / t / 1e6,
            "passes": int(st.passes)}


def c5_bench(sty, W: int = 160, H: int = 90):
    """Full stylized render of the interior workload (6 x 3 x 4 m room of ~377 k triangles, door
    open 20 degrees, the only emitter behind it; GGX + diffuse; toon (band 0.2) and a 3-colour
    luminance ramp at bounces 0 and 1; max depth 8) at a reduced scale: W x H px. Methods, each
    timed (CUDA-synchronised wall time) and scored by image MSE against a 1024-spp
    FP64-accumulated NL-PF render of the same view:
      nl_pf      reference-mode NL-PF at 64 spp (16 paths x 4 repeats, radius 1 % of the scene
                 extent, reuse 32, SMIS);
      nl_nrc_*   the NL-NRC loop (128 training iterations of 4 batches of 2^14, 16 first-hit
                 passes) with the BF16 tcgen05 cache and with the FP32 cache (spherical-frequency
                 network), and with the reference's own network (hash grid 22 x 4 on 2^19 tables +
                 one-blob + identity, 5 x 128; rows in the reference layout);
      brpt       the branching path tracer at the teaser's branching (32, 14, 8, 6), 1 repeat;
      pt_64spp   the plain stylized path tracer (branching 1), 64 repeats."""
    import numpy as np
    import torch
    a = sty.abi
    pos, mids, mats, cam = sty.scene.room_with_door(W, H)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    progs = [a.style_program([a.toon(0.2, depth_mask=0b11),
                              a.ramp_smooth(30.0, [0.02, 0.15, 0.6],
                                            [(0.08, 0.1, 0.2), (0.55, 0.45, 0.35), (1.3, 1.2, 1.0)],
                                            depth_mask=0b11)])]

    def pf(branch, repeats, seed):
        cfg = sty.scene.render_config(max_depth=8, branch=branch, repeats=repeats, radius_scale=(1.0,),
                                      reuse=(32,), seed=seed)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        film, nv = sc.render(cfg, progs)
        torch.cuda.synchronize()
        return film.cpu().numpy(), time.perf_counter() - t0, nv

    pf(4, 1, 99)  # warm-up
    ref, t_ref, nv_ref = pf(64, 16, 4242)
    res = {"workload": f"interior room {pos.shape[0]} tris, door 20 deg, {W}x{H}, max depth 8, toon + "
                       "3-colour ramp at bounces 0-1",
           "reference": {"spp": 1024, "seconds": t_ref, "vertices": nv_ref}}
    img, t, nv = pf(16, 4, 7)
    res["nl_pf"] = {"spp": 64, "seconds": t, "mpath_vertices_per_s": nv / t / 1e6,
                    "image_mse": float(((img - ref) ** 2).mean())}
    def nrc_warmup(make):
        # untimed short render: the first use of a code path in a process loads its kernels (and,
        # on a fresh machine, cuBLAS from disk: seconds)
        w = make()
        sc.nrc_render(w, sty.scene.nrc_render_config(max_depth=8, training_iters=2, batches_per_iter=1, repeats=1,
                                                     seed=1), progs)
        torch.cuda.synchronize()
        w.close()

    for name, prec in (("nl_nrc_bf16", sty.nrc.STY_NRC_BF16), ("nl_nrc_fp32", sty.nrc.STY_NRC_FP32)):
        make = lambda: sty.nrc.NRC(sty.nrc.config(sty.nrc.C4_FREQS, 3, 1 << 14, 5, prec, learning_rate=1e-2,  # noqa: E731
                                                  seed=1))
        nrc_warmup(make)
        net = make()
        cfg = sty.scene.nrc_render_config(max_depth=8, training_iters=128, batches_per_iter=4, repeats=16, seed=3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        film, st = sc.nrc_render(net, cfg, progs)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        img = film.cpu().numpy()
        res[name] = {"seconds": t, "training_rows": int(st.training_rows), "queries": int(st.inference_queries),
                     "image_mse": float(((img - ref) ** 2).mean())}
        net.close()
    make = lambda: sty.nrc.NRC(sty.nrc.grid_config(max_depth=8, batch_size=1 << 14, learning_rate=1e-2, seed=1))  # noqa: E731
    nrc_warmup(make)
    net = make()
    cfg = sty.scene.nrc_render_config(max_depth=8, training_iters=128, batches_per_iter=4, repeats=16, seed=3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    film, st = sc.nrc_render(net, cfg, progs)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    img = film.cpu().numpy()
    res["nl_nrc_ref_network"] = {"seconds": t, "training_rows": int(st.training_rows),
                                 "queries": int(st.inference_queries), "params": net.param_count(),
                                 "image_mse": float(((img - ref) ** 2).mean())}
    net.close()
    # the branching path tracer at the teaser's branching (configs/teaser/brpt.json: inner samples
    # 32, 14, 8, 6) and the plain stylized path tracer of configs/teaser/pt.json (inner samples 1)
    sc.brpt_render(sty.scene.brpt_config(max_depth=8, inner_samples=(2,), repeats=1, seed=1), progs)  # warm-up
    for name, inner, reps in (("brpt", (32, 14, 8, 6), 1), ("pt_64spp", (1,), 64)):
        cfg = sty.scene.brpt_config(max_depth=8, inner_samples=inner, repeats=reps, vram_mb=16384, seed=5)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        film, st = sc.brpt_render(cfg, progs)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        img = film.cpu().numpy()
        res[name] = {"seconds": t, "inner_samples": list(inner), "repeats": reps, "vertices": int(st.vertices),
                     "mvertices_per_s": st.vertices / t / 1e6, "passes": int(st.passes),
                     "image_mse": float(((img - ref) ** 2).mean())}
    res["reference_mean"] = float(ref.mean())
    sc.close()
    return res


def c5_full_bench(sty, W: int = 1920, H: int = 1080, ref_spp: int = 1024):
    """The full stylized render at its stated scale: the interior workload (6 x 3 x 4 m room of ~377 k
    triangles, door open 20 degrees, the only emitter behind it; GGX + diffuse; toon (band 0.2) + a
    3-colour luminance ramp at bounces 0-1) at 1920 x 1080, 64 spp (16 paths per pixel x 4
    repeats), max depth 8, the screen-space NL-PF filter (radius 8 px, sigma_pos 0.05 m, sigma_nrm
    0.2, program 0 by its depth mask). Each method is timed (CUDA-synchronised wall time, cache
    training included) and scored by image MSE against a `ref_spp`-spp FP64-accumulated plain
    NL-PF render of the same view (the same filter, max depth 8):
      nl_pf_fp32             plain NL-PF: every path traced to depth 8 and filtered at every depth;
      nl_pf_nrc_ref_network  NL-PF and NL-NRC together (sty_pf_nrc_render): paths traced to depth 3,
                             the cache's prediction there standing in for the rest of each path,
                             the filter on depths 2 .. 0; the cache is the reference's network (hash
                             grid 22 x 4 on 2^19 tables + one-blob + identity, 5 x 128, BF16 tcgen05)
                             trained online by the NL-NRC loop (128 iterations x 4 batches of 2^14);
      nl_pf_nrc_bf16 / fp32  the same at cache depth 2 with the spherical-frequency cache (BF16
                             tcgen05 / FP32 CUDA cores): the BF16-vs-FP32 comparison at equal MSE;
      cut_at_depth_K         the paths simply ended at depth K (no cache): what the cache buys."""
    import numpy as np
    import torch
    a = sty.abi
    pos, mids, mats, cam = sty.scene.room_with_door(W, H)
    sc = sty.scene.Scene(pos, mids, mats, cam)
    progs = [a.style_program([a.toon(0.2, depth_mask=0b11),
                              a.ramp_smooth(30.0, [0.02, 0.15, 0.6],
                                            [(0.08, 0.1, 0.2), (0.55, 0.45, 0.35), (1.3, 1.2, 1.0)],
                                            depth_mask=0b11)])]
    scr = dict(radius=8, sigma_pixel=0.0, sigma_pos=0.05, sigma_nrm=0.2, screen_style=0)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        film, extra = fn()
        torch.cuda.synchronize()
        return film.cpu().numpy(), time.perf_counter() - t0, extra

    def pf_cfg(depth, repeats, seed):
        return sty.scene.screen_render_config(max_depth=depth, branch=16, repeats=repeats, seed=seed, **scr)

    sc.render(pf_cfg(8, 1, 99), progs)  # warm-up
    ref, t_ref, nv_ref = timed(lambda: sc.render(pf_cfg(8, ref_spp // 16, 4242), progs))
    mse = lambda im: float(((im - ref) ** 2).mean())  # noqa: E731
    res = {"workload": f"interior room {pos.shape[0]} tris, door 20 deg, {W}x{H}, 64 spp, max depth 8, toon + "
                       "3-colour ramp at bounces 0-1, screen-space NL-PF radius 8 px",
           "reference": {"spp": ref_spp, "seconds": t_ref, "vertices": nv_ref, "image_mean": float(ref.mean())}}
    img, t, nv = timed(lambda: sc.render(pf_cfg(8, 4, 7), progs))
    res["nl_pf_fp32"] = {"spp": 64, "seconds": t, "mpath_vertices_per_s": nv / t / 1e6, "image_mse": mse(img)}
    for K in (2, 3):
        img, t, _ = timed(lambda: sc.render(pf_cfg(K, 4, 7), progs))
        res[f"cut_at_depth_{K}"] = {"spp": 64, "seconds": t, "image_mse": mse(img), "image_mean": float(img.mean())}
    caches = (("nl_pf_nrc_ref_network", 3, lambda: sty.nrc.NRC(sty.nrc.grid_config(
                  max_depth=8, batch_size=1 << 14, learning_rate=1e-2, seed=1))),
              ("nl_pf_nrc_bf16", 2, lambda: sty.nrc.NRC(sty.nrc.config(
                  sty.nrc.C4_FREQS, 3, 1 << 14, 5, sty.nrc.STY_NRC_BF16, learning_rate=1e-2, seed=1))),
              ("nl_pf_nrc_fp32", 2, lambda: sty.nrc.NRC(sty.nrc.config(
                  sty.nrc.C4_FREQS, 3, 1 << 14, 5, sty.nrc.STY_NRC_FP32, learning_rate=1e-2, seed=1))))
    for name, K, make in caches:
        w = make()  # untimed warm-up (the first use of a path loads its kernels)
        sc.pf_nrc_render(w, sty.scene.screen_render_config(max_depth=8, branch=1, repeats=1, seed=1, **scr),
                         sty.scene.nrc_render_config(max_depth=8, training_iters=2, batches_per_iter=1, seed=1), K,
                         progs)
        torch.cuda.synchronize()
        w.close()
        net = make()
        nc = sty.scene.nrc_render_config(max_depth=8, training_iters=128, batches_per_iter=4, seed=3)
        img, t, st = timed(lambda: sc.pf_nrc_render(net, pf_cfg(8, 4, 7), nc, K, progs))
        res[name] = {"spp": 64, "cache_depth": K, "seconds": t, "training_rows": int(st.training_rows),
                     "queries": int(st.inference_queries), "image_mse": mse(img), "image_mean": float(img.mean())}
        net.close()
    res["speedup_ref_network_over_plain"] = res["nl_pf_fp32"]["seconds"] / res["nl_pf_nrc_ref_network"]["seconds"]
    res["speedup_bf16_over_fp32_cache"] = res["nl_pf_nrc_fp32"]["seconds"] / res["nl_pf_nrc_bf16"]["seconds"]
    res["mse_ratio_bf16_over_fp32_cache"] = res["nl_pf_nrc_bf16"]["image_mse"] / res["nl_pf_nrc_fp32"]["image_mse"]
    sc.close()
    return res


def c2_alt_kernel(sty, rs, prm, style, out, D, steps, kernel, stream):
    """The resident C2 pass on another screen-filter kernel (`kernel`: sty.SCREEN_KERNEL_*): mean ms per
    depth launch from CUDA events on the launching stream, Mpath-vertices/s, and the largest relative
    difference of its deepest-depth output (pure filter, no style node) from `out` (the headline run's)."""
    import torch
    sty.set_screen_kernel(kernel)
    try:
        alt = torch.empty_like(out)

        def one_pass(evs=None):
            for d in range(D - 1, -1, -1):
                nxt = alt[d + 1] if d + 1 < D else None
                if evs is not None:
                    evs[d][0].record(stream)
                sty.pf_screen_filter_depth(rs, d, prm, style, out_next=nxt, out=alt[d], stream=stream)
                if evs is not None:
                    evs[d][1].record(stream)

        for _ in range(3):
            one_pass()
        torch.cuda.synchronize()
        evs = [[[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(D)] for _ in range(steps)]
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for k in range(steps):
            one_pass(evs[k])
        t1.record(stream)
        torch.cuda.synchronize()
        launch_ms = statistics.mean(evs[k][d][0].elapsed_time(evs[k][d][1]) for k in range(steps) for d in range(D))
        ms_pass = t0.elapsed_time(t1) / steps
        m = rs.valid[(D - 1) * rs.n_per_depth:D * rs.n_per_depth].bool()
        a, b = alt[D - 1][:, m], out[D - 1][:, m]
        diff = ((a - b).abs() / b.abs().clamp_min(1e-6)).max().item()
        nvalid = int(rs.valid.sum().item())
        return {"ms_per_launch": launch_ms, "ms_per_pass": ms_pass,
                "mpath_vertices_per_s": nvalid / (ms_pass / 1e3) / 1e6,
                "max_rel_diff_deepest_vs_headline": diff}
    finally:
        sty.set_screen_kernel(sty.SCREEN_KERNEL_AUTO)


def run_reference(args):
    rank, world, _ = _rank_env()
    if rank != 0:
        return
    import __graft_entry__ as g
    sty = g.package()
    import oracle as orc
    planes, valid = sty.synth.records(W_, H_, S_, D_, seed=0)
    vals = []
    last = None
    for i in range(args.warmup + args.steps):
        last = cpu_baseline(sty, orc, planes, valid, budget_s=args.ref_budget)
        if i >= args.warmup:
            vals.append(last["value"])
    v = statistics.median(vals)
    last["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mpath-vertices/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": WORKLOAD, "records": W_ * H_ * S_ * D_, "l2": "inputs > L2"},
            "cpu_baseline": last,
            "note": "reference CPU backend (Rust + LuisaCompute LLVM) cannot be built here; "
                    "timed path is the oracle's FP32 restatement of the same filter",
            "e2e": {"value": v, "unit": "Mpath-vertices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run(args):
    import torch
    rank, world, local = _rank_env()
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import __graft_entry__ as g
    sty = g.package()
    lib = sty.abi.lib()
    if args.nrc_only:  # profiling case: the NL-NRC frames alone
        print(json.dumps({"nrc": nrc_bench(sty, args.nrc_frames, max(3, args.warmup), dev, 1943.8)}), flush=True)
        return
    if args.c1_only:  # profiling case: the end-to-end render alone
        print(json.dumps({"c1_render": c1_bench(sty, repeats=max(1, args.steps))}), flush=True)
        return
    if args.c1b_only:  # profiling case: the traced Cornell render with the screen-space filter alone
        print(json.dumps({"c1_bilateral": c1_bilateral_bench(sty, repeats=max(1, args.steps))[0]}), flush=True)
        return
    if args.grid_only:  # the reference's NL-NRC network alone
        print(json.dumps({"nrc_ref_network": grid_nrc_bench(sty, args.grid_frames, max(3, args.warmup), dev, 1943.8)}),
              flush=True)
        return
    if args.c5_only:  # the full stylized render alone
        print(json.dumps({"c5_render": c5_bench(sty)}), flush=True)
        return
    if args.c5_full:  # the full stylized render at 1920 x 1080 x 64 spp (minutes: not in the default run)
        print(json.dumps({"c5_full": c5_full_bench(sty, ref_spp=args.c5_ref_spp)}), flush=True)
        return
    if args.c3_only:  # profiling case: the adjoint alone
        print(json.dumps({"c3_adjoint": c3_bench(sty, reps=max(1, args.steps))}), flush=True)
        return
    if args.brpt_only:  # profiling case: one branching path tracer render of the interior workload
        print(json.dumps({"brpt": brpt_bench(sty)}), flush=True)
        return

    kernels = {"auto": sty.SCREEN_KERNEL_AUTO, "fp32": sty.SCREEN_KERNEL_FP32, "tensor": sty.SCREEN_KERNEL_TENSOR}
    sty.set_screen_kernel(kernels[args.kernel])
    D_ = args.depths
    planes, valid = sty.synth.records(W_, H_, S_, D_, seed=rank)
    rs = sty.RecordSet.from_numpy(planes, valid, W_, H_, S_, D_, device=dev)
    n = rs.n_per_depth
    prm = sty.c2_params()
    style = sty.c2_style()
    nvalid = int(valid.sum())
    stream = torch.cuda.current_stream(dev)
    out = torch.empty((D_, 3, n), dtype=torch.float32, device=dev)

    def barrier():
        if dist:
            torch.distributed.barrier()

    def one_pass(evs=None):
        for d in range(D_ - 1, -1, -1):
            nxt = out[d + 1] if d + 1 < D_ else None
            if evs is not None:
                evs[d][0].record(stream)
            sty.pf_screen_filter_depth(rs, d, prm, style, out_next=nxt, out=out[d], stream=stream)
            if evs is not None:
                evs[d][1].record(stream)

    for _ in range(args.warmup):
        one_pass()
    torch.cuda.synchronize()

    # ---- device-resident timed region
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lib.sty_launch_count()
    kev = [[[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(D_)] for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    t_start.record(stream)
    for k in range(args.steps):
        one_pass(kev[k])
    t_end.record(stream)
    torch.cuda.synchronize()
    barrier()
    launches = lib.sty_launch_count() - launches0
    ms_total = t_start.elapsed_time(t_end)
    launch_ms = [kev[k][d][0].elapsed_time(kev[k][d][1]) for k in range(args.steps) for d in range(D_)]
    clk = clocks.stop()

    # ---- end-to-end through the public API with host buffers
    if args.no_e2e:
        e2e_step = None
    h_planes = torch.from_numpy(planes).pin_memory()
    h_valid = torch.from_numpy(valid).pin_memory()
    h_out = torch.empty((3, n), dtype=torch.float32).pin_memory()
    d_planes, d_valid = rs.planes, rs.valid

    # per depth (deepest first, the order of the backward loop) the depth's 13 record slices go up on
    # a copy stream; the filter of a depth waits only for its own records, and a depth's slice is
    # overwritten by the next step's upload as soon as this step's filter of that depth is done, so
    # uploads overlap the filters of the other depths (also across steps). The result (depth 0) goes
    # down on its own stream (on the upload stream it would hold the next step's uploads behind the
    # end of this step); the next step's depth-0 filter waits for that copy.
    copy_stream = torch.cuda.Stream(dev)
    down_stream = torch.cuda.Stream(dev)
    ev_filtered = [torch.cuda.Event() for _ in range(D_)]
    ev_copied = [torch.cuda.Event() for _ in range(D_)]
    ev_out_read = torch.cuda.Event()
    first = [True]

    def e2e_step():
        with torch.cuda.stream(copy_stream):
            for d in range(D_ - 1, -1, -1):
                if not first[0]:
                    copy_stream.wait_event(ev_filtered[d])  # the previous step's filter of depth d
                sl = slice(d * n, (d + 1) * n)
                for f in range(d_planes.shape[0]):
                    d_planes[f, sl].copy_(h_planes[f, sl], non_blocking=True)
                d_valid[sl].copy_(h_valid[sl], non_blocking=True)
                ev_copied[d].record(copy_stream)
        for d in range(D_ - 1, -1, -1):
            stream.wait_event(ev_copied[d])
            if d == 0 and not first[0]:
                stream.wait_event(ev_out_read)  # the previous step's result has reached the host
            nxt = out[d + 1] if d + 1 < D_ else None
            sty.pf_screen_filter_depth(rs, d, prm, style, out_next=nxt, out=out[d], stream=stream)
            ev_filtered[d].record(stream)
        with torch.cuda.stream(down_stream):
            down_stream.wait_event(ev_filtered[0])
            h_out.copy_(out[0], non_blocking=True)
            ev_out_read.record(down_stream)
        first[0] = False

    e2e_ms = float("nan")
    e2e_same = None
    if not args.no_e2e:
        resident0 = out[0].clone()  # the resident pass's result, for the host round trip to match
        for _ in range(max(1, args.warmup)):
            e2e_step()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        copy_stream.wait_event(e0)  # the first upload starts inside the timed region
        for _ in range(args.steps):
            e2e_step()
        stream.wait_event(ev_out_read)  # ... and the last result's download ends inside it
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        e2e_ms = e0.elapsed_time(e1)
        e2e_same = bool(torch.equal(h_out, resident0.cpu()))
        del resident0

    # ---- max over ranks (replicas: the job's time is its slowest rank's)
    ms_total = sty.replicas.max_over_ranks(ms_total, device=dev)
    e2e_ms = sty.replicas.max_over_ranks(e2e_ms, device=dev)
    ms_step = ms_total / args.steps
    value = nvalid * world * args.steps / (ms_total / 1e3) / 1e6
    e2e_value = nvalid * world * args.steps / (e2e_ms / 1e3) / 1e6

    # ---- roofline of k_pf_screen (algorithmic bytes per launch / mean launch time)
    bytes_step = (52 * D_ + 12 * (D_ - 1) + 12 * D_) * n
    bytes_launch = bytes_step / D_
    mean_launch_s = statistics.mean(launch_ms) / 1e3
    hbm_peak, peak_kind = _load_peaks()
    achieved = bytes_launch / mean_launch_s / 1e9
    pairs_launch = n * (2 * prm.radius + 1) ** 2 * S_
    sm_clock = (clk or {}).get("sm_mhz") or 1900.0
    fp32_peak = 152 * 128 * 2 * sm_clock * 1e6 / 1e12  # TFLOP/s, FFMA = 2 FLOP, at the sampled clock
    # FP32-pipe instructions per pair: expanded exponent 6 FFMA + 4 FFMA accumulate; direct form
    # 3 FADD + 6 FFMA + 4 FFMA. The tile's form depends on its positions (see expanded_fraction).
    f_exp = expanded_fraction(planes, valid, W_, H_, S_, D_, prm.sigma_pos)
    flops_pair = 2 * (10 * f_exp + 13 * (1 - f_exp))
    alu_achieved = pairs_launch * flops_pair / mean_launch_s / 1e12

    if rank != 0:
        if dist:
            torch.distributed.destroy_process_group()
        return
    line = {
        "metric": METRIC, "value": value, "unit": "Mpath-vertices/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded records, distributions of the workload)",
        "config": {"workload": WORKLOAD, "width": W_, "height": H_, "spp": S_, "depths": D_,
                   "radius": prm.radius, "sigma_pixel": prm.sigma_pixel, "sigma_pos": prm.sigma_pos,
                   "sigma_nrm": prm.sigma_nrm, "style": "toon 0.1/0.3/0.6 at depth 1",
                   "records_per_step": W_ * H_ * S_ * D_, "valid_vertices_per_step": nvalid,
                   "l2": "inputs (2.2 GB) larger than L2; no flush", "parallelism": f"replicas x{world}"},
        "gpu_launches": int(launches),
        "e2e": {"value": e2e_value, "unit": "Mpath-vertices/s",
                "h2d_bytes_per_step": int(planes.nbytes + valid.nbytes), "d2h_bytes_per_step": int(3 * n * 4),
                "result_matches_resident": e2e_same},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "traffic": NCU_TRAFFIC_PER_LAUNCH,
                     "kernel": "k_pf_screen4", "peak_source": peak_kind,
                     "algorithmic_bytes_per_launch": bytes_launch, "mean_launch_ms": mean_launch_s * 1e3},
        "alu_roofline": {"bound": "fp32", "achieved": alu_achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                         "frac": alu_achieved / fp32_peak, "pairs_per_launch": pairs_launch,
                         "flops_per_pair": flops_pair, "expanded_tile_fraction": f_exp,
                         "mufu_ex2_per_s": pairs_launch / mean_launch_s,
                         "peak_source": "nominal 152 SM x 128 FP32 lanes x 2 at the sampled SM clock",
                         "note": "the binding roof of this kernel (pair arithmetic); HBM traffic is ~0.6 % of it"},
        "clocks": clk,
    }
    if world == 1 and not args.no_alt_kernel:
        # the other screen-filter kernel family on the same resident records
        alt = sty.SCREEN_KERNEL_FP32 if args.kernel == "tensor" else sty.SCREEN_KERNEL_TENSOR
        line["c2_alt_kernel"] = {"kernel": "k_pf_screen4 (CUDA cores)" if alt == sty.SCREEN_KERNEL_FP32
                                 else "k_pf_screen_tc (tcgen05 split-TF32)",
                                 **c2_alt_kernel(sty, rs, prm, style, out, D_, max(3, args.steps), alt, stream)}
        sty.set_screen_kernel(kernels[args.kernel])
    if world == 1 and not args.no_c1:
        line["c1_render"] = c1_bench(sty)
        line["c1_bilateral"], c1_rs = c1_bilateral_bench(sty)
        if not args.no_cpu_baseline:
            import oracle as orc
            line["c1_bilateral"]["cpu_baseline"] = c1_bilateral_cpu_baseline(sty, orc, c1_rs)
        del c1_rs
        line["c3_adjoint"] = c3_bench(sty)
        line["c5_render"] = c5_bench(sty)
    if world == 1 and not args.no_nrc:
        bf16_peak = 1943.8
        p = ROOT / "MEASURED_PEAKS.json"
        if p.exists():
            bf16_peak = float(json.loads(p.read_text())["bf16_tflops"])
        line["nrc"] = nrc_bench(sty, args.nrc_frames, max(3, args.warmup), dev, bf16_peak)
        line["nrc_ref_network"] = grid_nrc_bench(sty, args.grid_frames, max(3, args.warmup), dev, bf16_peak)
    if world == 1 and not args.no_cpu_baseline:
        import oracle as orc
        line["cpu_baseline"] = cpu_baseline(sty, orc, planes, valid, D_)
    print(json.dumps(line), flush=True)
    if dist:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-budget", type=float, default=8.0)
    ap.add_argument("--depths", type=int, default=D_, help="path depths (profiling cases use fewer)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer pass (profiling cases)")
    ap.add_argument("--kernel", default="auto", choices=["auto", "fp32", "tensor"],
                    help="screen-filter kernel of the headline pass (sty_pf_screen_set_kernel)")
    ap.add_argument("--no-alt-kernel", action="store_true",
                    help="skip timing the other screen-filter kernel on the same records")
    ap.add_argument("--no-nrc", action="store_true", help="skip the NL-NRC frames")
    ap.add_argument("--nrc-frames", type=int, default=256)
    ap.add_argument("--no-c1", action="store_true", help="skip the end-to-end Cornell box render")
    ap.add_argument("--nrc-only", action="store_true", help="profiling case: only the NL-NRC frames")
    ap.add_argument("--c1-only", action="store_true", help="profiling case: only the end-to-end Cornell box render")
    ap.add_argument("--c1b-only", action="store_true",
                    help="profiling case: only the traced Cornell render with the screen-space filter")
    ap.add_argument("--c5-only", action="store_true", help="only the full stylized interior render")
    ap.add_argument("--c5-full", action="store_true",
                    help="the full stylized render at 1920x1080 x 64 spp against a high-spp NL-PF reference")
    ap.add_argument("--c5-ref-spp", type=int, default=1024, help="spp of the --c5-full reference (multiple of 16)")
    ap.add_argument("--c3-only", action="store_true", help="profiling case: only the adjoint")
    ap.add_argument("--brpt-only", action="store_true",
                    help="profiling case: one branching path tracer render of the interior workload")
    ap.add_argument("--grid-only", action="store_true", help="only the reference's NL-NRC network frames")
    ap.add_argument("--grid-frames", type=int, default=32, help="frames of the reference's NL-NRC network")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run(args)


if __name__ == "__main__":
    main()
