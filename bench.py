"""Benchmark: the procedural material scene (327,690 triangles, 1920x1080,
64 spp, max depth 16) rendered by the GB300 wavefront path tracer.

One step = one full frame: 1920*1080*64 = 132.7M camera paths.  The scene
(geometry, BVH, materials, lights) is resident on the device before timing.

  value      samples/s of the whole job (device time from CUDA events on the
             library's stream, summed over the K timed steps; L2 flushed
             between steps)
  e2e        the same metric through dl_render with a host output buffer
             (film resolve + device-to-host copy of the image inside the call)
  roofline   closest-hit traversal kernel: algorithmic fetch bytes (node and
             triangle fetches counted by a counting replay of the same frame,
             plus ray in / hit out) / its summed launch time, against the L2
             read bandwidth measured live by the library's probe (the BVH
             stays in L2); beside it the L2 -> L1 and DRAM bytes it really
             moves (per ray, from an ncu capture) against the L2 and HBM
             peaks
  cpu_baseline  the CPU restatement of the reference renderer (spiral 32x32
             blocks, per-block pcg32) on 64 blocks of the same frame drawn
             uniformly with a fixed seed, all host cores
  c4_batch   the batched workload (64 requests, autotuned launch shape)
  c5_guided  learned guiding vs plain at equal time (relMSE at 480x270
             against a 64k-spp reference), the guided 1080p rate and the
             network kernels against the tensor-core peak

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                 [--workload batch|guided|network] [--no-extras] [--profile-frame --spp S]

Multi-GPU (torchrun, one rank per GPU): replicas render disjoint sample ranges
(weak scaling), no collective on the data path.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOAD = dict(workload="material_spheres", width=1920, height=1080, spp=64, max_depth=16,
                triangles=327690, spheres=64, sphere_level=4, area_lights=4, point_lights=1,
                triangles_note="64 x 5120 sphere + 2 ground + 8 light-quad triangles")
METRIC = "samples/s (material-sphere scene 1920x1080, 64 spp, depth 16)"

# algorithmic bytes per closest-hit ray: node = 64 B (both child boxes + refs),
# triangle = 48 B (3 x float4), ray in 32 B, hit out 16 B
NODE_BYTES, TRI_BYTES, RAY_IN, HIT_OUT = 64, 48, 32, 16
# Per-ray cache and DRAM traffic of the traversal kernels, from one ncu
# capture of every k_traverse launch of a 4-spp frame of this scene
# (python bench.py --profile-frame --spp 4; profiles/k_traverse_l2_dram_material_spheres_1080p_4spp.md):
# L2 -> L1 bytes (lts__t_sectors_srcunit_tex_op_read.sum x 32) and DRAM
# bytes (dram__bytes_read.sum + dram__bytes_write.sum) summed over the
# frame's launches of each kernel, divided by the frame's extension / shadow
# rays.  Profile measurements, scaled here by the rays of the timed frames.
EXT_L2_BYTES_PER_RAY = 158925079 * 32 / 14984872            # 339.4 B
EXT_DRAM_BYTES_PER_RAY = (2181426688 + 471964416) / 14984872  # 177.1 B
SH_L2_BYTES_PER_RAY = 63489526 * 32 / 5484823                 # 370.4 B
SH_DRAM_BYTES_PER_RAY = (954967296 + 120330240) / 5484823     # 196.1 B


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def tensor_peak():
    """Dense fp16/bf16 tensor peak (TFLOP/s) for a kernel timed alone."""
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        if "bf16_tflops" in d:
            return d["bf16_tflops"], "measured"
    return 1900.0, "fallback"


# Multiply-adds per row of the guiding network: 144x64 + 64x64 + 64x48
# (forward), 48x64 + 64x64 (backward through layers 3 and 2), and the
# weight gradients (as many as the forward).
NET_MAC_FWD = 144 * 64 + 64 * 64 + 64 * 48
NET_MAC_TRAIN = NET_MAC_FWD + (48 * 64 + 64 * 64) + NET_MAC_FWD


def network_roofline(ctx, api, train_rows=(131072, 32768)):
    """Device time of the network kernels alone (dl_guide_forward on 4M rows;
    dl_guide_gradient on training batches of train_rows records, the first
    the renderer's default batch, 131072), as FLOP/s against the measured
    tensor peak and as bytes/s against HBM."""
    tpk, tkind = tensor_peak()
    hbm, hkind = peaks()
    rng = np.random.default_rng(3)
    g = api.Guide(ctx, seed=5)
    n = 1 << 22
    inp = np.concatenate([rng.uniform(0, 1, (n, 3)), rng.normal(size=(n, 3))], axis=1).astype(np.float32)
    inp[:, 3:] /= np.linalg.norm(inp[:, 3:], axis=1, keepdims=True)
    times = []
    for _ in range(4):
        g.forward(inp)
        times.append(ctx.stats().guide_ms)
    t_inf = float(np.median(times[1:]))
    train = []
    for nb in train_rows:
        rec = np.zeros((nb, 12), np.float32)
        rec[:, :6] = inp[:nb]
        w = rng.normal(size=(nb, 3))
        rec[:, 6:9] = w / np.linalg.norm(w, axis=1, keepdims=True)
        rec[:, 9] = rng.uniform(0.05, 2.0, nb)
        rec[:, 10] = rng.uniform(0.0, 3.0, nb)
        times = []
        for _ in range(16):
            g.gradient(rec)
            times.append(ctx.stats().guide_ms)
        t_tr = float(np.median(times[1:]))
        tr_tf = 2.0 * NET_MAC_TRAIN * nb / (t_tr * 1e-3) / 1e12
        train.append({"kernels": "k_guide_weight_sum + k_guide_train + k_guide_grad_reduce (tcgen05)", "rows": nb, "ms": t_tr, "tflops": tr_tf, "frac_tensor": tr_tf / tpk,
                      "flop_per_row": 2 * NET_MAC_TRAIN})
    inf_tf = 2.0 * NET_MAC_FWD * n / (t_inf * 1e-3) / 1e12
    inf_gbs = (24 + 160) * n / (t_inf * 1e-3) / 1e9
    return {"inference": {"kernel": "k_guide_infer (tcgen05)", "rows": n, "ms": t_inf, "tflops": inf_tf,
                          "frac_tensor": inf_tf / tpk, "gbs": inf_gbs, "frac_hbm": inf_gbs / hbm,
                          "bytes_per_row": 184, "flop_per_row": 2 * NET_MAC_FWD},
            "training_batch": train[0], "training_batches": train,
            "peak_tflops": tpk, "peak_kind": tkind, "hbm_peak": hbm, "hbm_kind": hkind}


def run_network(args):
    """The network kernels alone (the command under ncu for their launch list)."""
    local = _device_setup()
    if local is None:
        return
    from drawlab_gb300 import api
    ctx = api.Context(local)
    print(json.dumps({"network": network_roofline(ctx, api)}))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        try:
            rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
            os.unlink(self.path)
        except Exception:
            return out
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except Exception:
                continue
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(n)
        if sm:
            out["sm_mhz"] = statistics.median(sm)
            out["sm_max_mhz"] = max(mx)
        out["reasons"] = sorted(reasons)
        out["samples"] = len(sm)
        return out


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# The CPU sample: 64 of the frame's 2040 32x32 blocks drawn uniformly (seed
# 0) from the spiral order, each at the full 64 spp and depth 16.
CPU_BLOCKS = 64
CPU_BLOCK_SEED = 0


def cpu_block_subset(n_blocks_total):
    rng = np.random.default_rng(CPU_BLOCK_SEED)
    return np.sort(rng.choice(n_blocks_total, size=CPU_BLOCKS, replace=False)).astype(np.int32)


def cpu_baseline(scene_data):
    """Oracle block renderer (reference semantics: per-block pcg32, spiral
    order, Gaussian film) on the seeded 64-block subset of the frame, every
    host core: samples/s."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle as po
    from drawlab_gb300 import abi

    orc = po.OracleScene(scene_data)
    cores = os.cpu_count() or 1
    opts = abi.make_opts(spp=WORKLOAD["spp"], max_depth=WORKLOAD["max_depth"])
    blocks = cpu_block_subset(orc.num_blocks())
    _, sec = orc.render_block_subset(opts, blocks, threads=cores)
    samples = len(blocks) * 32 * 32 * WORKLOAD["spp"]
    return {"value": samples / sec, "unit": "samples/s", "cores": cores, "kind": "port",
            "sample": "%d of the %d 32x32 blocks drawn uniformly (seed %d), 64 spp, depth 16, %.1f s"
                      % (len(blocks), orc.num_blocks(), CPU_BLOCK_SEED, sec)}, orc


def ref_blocks_per_step(cores, steps):
    """Blocks of the 64-block subset one reference step renders: at least one
    per host core (so no core idles), up to four per core while K steps stay
    within a few minutes (a block at 64 spp and depth 16 takes about 8 s of
    one core)."""
    per_core = max(1, min(4, 16 // max(1, steps)))
    return max(1, min(CPU_BLOCKS, cores * per_core))


def run_reference(args):
    """The reference's CPU renderer on the bench's frame: each step renders
    a chunk of the seeded 64-block subset (steps cycle through it) on all
    host cores, one or more blocks per core.  The reference sources do not
    travel to the GPU host, so its CPU restatement (bit-exact with the
    reference on the golden vectors) runs."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle as po
    from drawlab_gb300 import abi, scenes
    sc = scenes.material_spheres()
    orc = po.OracleScene(sc)
    cores = os.cpu_count() or 1
    opts = abi.make_opts(spp=WORKLOAD["spp"], max_depth=WORKLOAD["max_depth"])
    subset = cpu_block_subset(orc.num_blocks())
    per_step = ref_blocks_per_step(cores, args.steps)
    chunks = [np.resize(np.roll(subset, -k), per_step) for k in range(0, len(subset), per_step)]
    for w in range(args.warmup):
        orc.render_block_subset(opts, chunks[w % len(chunks)][:2], threads=cores)
    tot_s = 0.0
    for k in range(args.steps):
        _, s = orc.render_block_subset(opts, chunks[k % len(chunks)], threads=cores)
        tot_s += s
    samples = per_step * 32 * 32 * WORKLOAD["spp"] * args.steps
    value = samples / tot_s
    sample = ("%d blocks per step, cycling through %d of the frame's %d 32x32 blocks drawn uniformly (seed %d); "
              "64 spp, depth 16; the reference sources do not travel to this host, so the CPU restatement "
              "(bit-exact with the reference on its golden vectors) runs"
              % (per_step, len(subset), orc.num_blocks(), CPU_BLOCK_SEED))
    line = {"metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * tot_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (procedural scene, seed 2)",
            "impl": "reference",
            "config": dict(WORKLOAD, step="%d blocks of 32x32 pixels at 64 spp" % per_step),
            "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--spp", type=int, default=WORKLOAD["spp"])
    ap.add_argument("--workload", default="material_spheres",
                    choices=["material_spheres", "batch", "guided", "network"],
                    help="material_spheres: the headline frame; batch: 64 requests in one wavefront; "
                         "guided: learned proposal vs plain at equal time; network: the guiding network's "
                         "kernels alone")
    ap.add_argument("--guided-res", default="480x270", help="guided workload: resolution of the relMSE comparison")
    ap.add_argument("--ref-spp", type=int, default=REF_SPP, help="guided workload: spp of the plain reference")
    ap.add_argument("--no-extras", action="store_true", help="headline line without the c4_batch / c5_guided keys")
    ap.add_argument("--profile-frame", action="store_true",
                    help="render one frame of the headline scene at --spp and print its ray counts (for ncu)")
    args = ap.parse_args()
    if args.profile_frame:
        return run_profile_frame(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "guided":
        return run_guided(args)
    if args.workload == "network":
        return run_network(args)

    ws, rank, local = dist_env()
    import torch
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    import __graft_entry__ as ge
    ge.build()
    from drawlab_gb300 import abi, api, scenes

    sc = scenes.material_spheres()
    ctx = api.Context(local)
    gs = api.Scene.from_data(ctx, sc)
    info = gs.info()
    W, H, spp = sc.camera.width, sc.camera.height, args.spp
    opts = abi.make_opts(spp=spp, max_depth=WORKLOAD["max_depth"], seed=0, spp_offset=rank * spp)
    b = 2
    film = torch.empty(((H + 2 * b) * (W + 2 * b) * 4,), dtype=torch.float32, device="cuda")
    flush = torch.empty((256 << 20) // 4, dtype=torch.float32, device="cuda")  # 256 MB > 129 MB L2

    def step():
        ctx.check(ctx.lib.dl_render_film_device(gs.h, abi.C.byref(opts), abi.C.c_void_p(film.data_ptr())))

    ctx.set_kernel_timing(False)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    # timed frames: the production path (graph replay, concurrent material
    # kernels); device time from CUDA events on the library stream
    dev_ms = 0.0
    ext_rays = sh_rays = cam_rays = launches = 0
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            step()
            st = ctx.stats()
            dev_ms += st.render_ms
            ext_rays += st.extension_rays
            sh_rays += st.shadow_rays
            cam_rays += st.camera_rays
            launches += st.kernel_launches
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    ck = clocks.summary()
    # one more frame with per-kernel events (kernels serialised) for the
    # kernel split and the traversal roofline
    ctx.set_kernel_timing(True)
    flush.zero_()
    torch.cuda.synchronize()
    step()
    st = ctx.stats()
    ctx.set_kernel_timing(False)
    ext_ms, sh_ms, shade_ms, ret_ms = st.extend_ms, st.shadow_ms, st.shade_ms, st.retire_ms
    timed_frame_ms = st.render_ms
    t_ext_rays, t_sh_rays = st.extension_rays, st.shadow_rays
    ext_launches = st.iterations  # one closest-hit launch per wavefront iteration
    t = torch.tensor([dev_ms], dtype=torch.float64, device="cuda")
    if dist:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dev_ms_max = float(t.item())
    samples = W * H * spp * args.steps * ws
    value = samples / (dev_ms_max / 1000.0)
    mrays = (ext_rays + sh_rays) * ws / (dev_ms_max / 1000.0) / 1e6

    # e2e: public C-ABI render into a host buffer
    rgb = np.empty((H, W, 3), np.float32)
    gs.render(opts)
    e2e_s = 0.0
    for _ in range(max(1, min(args.steps, 3))):
        t1 = time.perf_counter()
        gs.render(opts)
        e2e_s += time.perf_counter() - t1
    e2e_steps = max(1, min(args.steps, 3))
    e2e_value = W * H * spp * e2e_steps / e2e_s

    # roofline of the closest-hit kernel
    counts = gs.traversal_counts(opts)
    hbm, peak_kind = peaks()
    n_node = counts.extension_node_visits / max(1, counts.extension_rays)
    n_tri = counts.extension_triangle_tests / max(1, counts.extension_rays)
    bytes_per_ray = n_node * NODE_BYTES + n_tri * TRI_BYTES + RAY_IN + HIT_OUT
    achieved = t_ext_rays * bytes_per_ray / (ext_ms / 1000.0) / 1e9 if ext_ms > 0 else 0.0
    sh_node = counts.shadow_node_visits / max(1, counts.shadow_rays)
    sh_tri = counts.shadow_triangle_tests / max(1, counts.shadow_rays)
    sh_bytes = sh_node * NODE_BYTES + sh_tri * TRI_BYTES + 48 + 1
    sh_achieved = t_sh_rays * sh_bytes / (sh_ms / 1000.0) / 1e9 if sh_ms > 0 else 0.0
    l2_peak = ctx.l2_read_gbs(64 << 20, 200)
    roofline = traversal_roofline(hbm, peak_kind, l2_peak, ext_ms, sh_ms, t_ext_rays, t_sh_rays, ext_launches,
                                  bytes_per_ray, n_node, n_tri, achieved, sh_bytes, sh_node, sh_tri, sh_achieved)

    if rank == 0:
        base = None
        if not args.no_cpu_baseline:
            base, _ = cpu_baseline(sc)
        line = {
            "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (procedural scene, seed 2; no scene files ship with the reference)",
            "config": dict(WORKLOAD, spp=spp, l2_flush="256 MB buffer written between timed steps",
                           paths_in_flight=min(ctx.get_tune().paths_in_flight, W * H * spp),
                           parallelism="replicas" if ws > 1 else "single"),
            "mrays_per_s": mrays,
            "rays": {"camera": cam_rays, "extension": ext_rays, "shadow": sh_rays},
            "wall_s": wall,
            "kernel_ms": {"frame": "one extra frame with per-kernel events (serialised kernels)",
                          "extend": ext_ms, "shadow": sh_ms, "materials": shade_ms, "miss": ret_ms,
                          "frame_total": timed_frame_ms, "timed_steps_device": dev_ms},
            "gpu_launches": launches,
            "e2e": {"value": e2e_value, "unit": "samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": W * H * 3 * 4,
                    "call": "dl_render (render options by value; image returned to host memory)"},
            "roofline": roofline,
            "clocks": ck,
            "scene": {"triangles": info.num_triangles, "bvh_nodes": info.num_bvh_nodes,
                      "bvh_depth": info.bvh_depth, "bvh_build_s": info.bvh_build_seconds,
                      "sah_cost": info.bvh_sah_cost},
            "cpu_baseline": base,
        }
        if ws == 1 and not args.no_extras:
            gs.close()
            line["c4_batch"] = batch_measure(ctx, steps=2, warmup=1)
            line["c5_guided"] = guided_measure(ctx, reps=9, warmup=1)
            line["c5_guided"]["config"]["relmse_resolution_note"] = (
                "480x270: a 64k-spp plain reference at 1920x1080 is 136 G samples (about 2 minutes of GPU time "
                "per bench run); the 1080p throughput is measured on the full frame (guided_1080p)")
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def traversal_roofline(hbm, peak_kind, l2_peak, ext_ms, sh_ms, ext_rays, sh_rays, ext_launches, bytes_per_ray,
                       n_node, n_tri, alg_gbs, sh_bytes, sh_node, sh_tri, sh_alg_gbs):
    """The closest-hit traversal against the memory level that bounds it.
    The BVH of this scene (~28 MB) stays in L2, so every node and triangle
    fetch is served by L1 or L2, not DRAM: achieved = the kernel's
    algorithmic fetch bytes (counted node visits and triangle tests of the
    same frame) over its launch time, against the L2 read bandwidth measured
    live.  Beside it: the L2 -> L1 bytes the kernel really moves and its
    DRAM bytes (per ray, from the profile), against the same L2 peak and the
    measured HBM bandwidth."""
    ext_s, sh_s = ext_ms / 1e3, sh_ms / 1e3
    l2_gbs = ext_rays * EXT_L2_BYTES_PER_RAY / ext_s / 1e9 if ext_s > 0 else 0.0
    dram_gbs = ext_rays * EXT_DRAM_BYTES_PER_RAY / ext_s / 1e9 if ext_s > 0 else 0.0
    r = {"bound": "l2", "kernel": "k_traverse<extension> (closest-hit traversal)", "unit": "GB/s",
         "achieved": alg_gbs, "peak": l2_peak, "frac": alg_gbs / l2_peak,
         "peak_kind": "measured live (dl_measure_l2_read_bandwidth: 64 MiB L2-resident buffer, L2-only loads, "
                      "200 passes)",
         "achieved_note": "algorithmic bytes per ray (64 B per node visit, 48 B per triangle test, 32 B ray, "
                          "16 B hit) x rays / summed launch time",
         "bytes_per_ray": bytes_per_ray, "node_visits_per_ray": n_node, "tri_tests_per_ray": n_tri,
         "algorithmic_bytes_per_launch": bytes_per_ray * ext_rays / max(1, ext_launches),
         "traffic": EXT_DRAM_BYTES_PER_RAY * ext_rays / max(1, ext_launches),
         "traffic_note": "DRAM bytes per launch: the profile's DRAM bytes per ray (177 B) x this frame's rays per "
                         "launch",
         "l2_traffic": {"bytes_per_ray": EXT_L2_BYTES_PER_RAY, "achieved": l2_gbs, "frac": l2_gbs / l2_peak,
                        "l1_served_fraction": 1.0 - EXT_L2_BYTES_PER_RAY / bytes_per_ray,
                        "note": "L2 -> L1 bytes the kernel moves (lts__t_sectors_srcunit_tex_op_read x 32 per ray)"},
         "dram": {"bytes_per_ray": EXT_DRAM_BYTES_PER_RAY, "achieved": dram_gbs, "peak": hbm,
                  "frac": dram_gbs / hbm, "peak_kind": peak_kind}}
    sh = {"achieved": sh_alg_gbs, "frac": sh_alg_gbs / l2_peak, "bytes_per_ray": sh_bytes,
          "node_visits_per_ray": sh_node, "tri_tests_per_ray": sh_tri}
    if sh_s > 0:
        sh_l2 = sh_rays * SH_L2_BYTES_PER_RAY / sh_s / 1e9
        sh_dram = sh_rays * SH_DRAM_BYTES_PER_RAY / sh_s / 1e9
        sh.update({"l2_traffic": {"bytes_per_ray": SH_L2_BYTES_PER_RAY, "achieved": sh_l2, "frac": sh_l2 / l2_peak},
                   "dram": {"bytes_per_ray": SH_DRAM_BYTES_PER_RAY, "achieved": sh_dram, "frac": sh_dram / hbm}})
    r["shadow"] = sh
    return r


def _device_setup():
    ws, rank, local = dist_env()
    if ws > 1 and rank != 0:
        return None
    import torch
    torch.cuda.set_device(local)
    import __graft_entry__ as ge
    ge.build()
    return local


def batch_measure(ctx, steps, warmup):
    """64 requests (seed 4) of 1k-2M-triangle scenes, 128^2..1080p, 4..256
    spp, half under the 2048x1024 sky, rendered by one dl_render_batch call
    per step (images to host memory).  The launch shape comes from
    dl_autotune on an eighth of the samples, outside the timed region."""
    from drawlab_gb300 import abi, api, scenes
    scene_list, reqs = scenes.batch_workload(seed=4)
    gscenes = [api.Scene.from_data(ctx, s) for s in scene_list]
    items = [(gscenes[si], abi.make_opts(spp=spp, max_depth=8, seed=17 + k), cam)
             for k, (si, spp, cam) in enumerate(reqs)]
    samples = sum(c.width * c.height * spp for _, spp, c in reqs)
    t_tune = time.perf_counter()
    tune, trials = ctx.autotune(items, trial_spp=0)
    t_tune = time.perf_counter() - t_tune
    for _ in range(warmup):
        ctx.render_batch(items)
    dev_ms, wall, launches = 0.0, 0.0, 0
    with ClockSampler(ctx_device(ctx)) as clocks:
        for _ in range(steps):
            t0 = time.perf_counter()
            ctx.render_batch(items)
            wall += time.perf_counter() - t0
            st = ctx.stats()
            dev_ms += st.render_ms
            launches += st.kernel_launches
    ck = clocks.summary()
    tris = [int(sum(m.indices.shape[0] for m in s.meshes)) for s in scene_list]
    for gsc in gscenes:
        gsc.close()
    return {"metric": "samples/s (64 batched requests, seed 4)", "value": samples * steps / (dev_ms / 1e3),
            "unit": "samples/s", "steps": steps, "warmup": warmup, "ms_per_step": dev_ms / steps,
            "config": {"workload": "batch", "requests": len(reqs), "samples_per_step": samples,
                       "scene_triangles": tris, "resolutions": "128^2..1920x1080", "spp": "4..256",
                       "max_depth": 8, "l2_flush": "inputs larger than L2 (BVHs 2.6 GB, samples 4 GB)"},
            "gpu_launches": launches,
            "autotune": {"paths_in_flight": tune.paths_in_flight, "traverse_ctas_per_sm": tune.traverse_ctas_per_sm,
                         "shade_ctas_per_sm": tune.shade_ctas_per_sm, "shade_threads": tune.shade_threads,
                         "iterations_per_graph": tune.iterations_per_graph, "trials": trials, "seconds": t_tune},
            "e2e": {"value": samples * steps / wall, "unit": "samples/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": sum(c.width * c.height * 12 for _, _, c in reqs),
                    "call": "dl_render_batch (64 requests; images returned to host memory)"},
            "clocks": ck}


def ctx_device(ctx):
    import torch
    return torch.cuda.current_device()


def run_batch(args):
    local = _device_setup()
    if local is None:
        return
    from drawlab_gb300 import api
    ctx = api.Context(local)
    r = batch_measure(ctx, args.steps, args.warmup)
    line = dict(r, n_gpus=1, higher_is_better=True, scaling="weak", vs_baseline=None, dtype="f32",
                data="synthetic (procedural scenes and sky, seed 4)")
    print(json.dumps(line))


REF_SPP = 65536  # plain reference of the equal-time comparison


def guided_measure(ctx, reps, warmup, width=480, height=270, ref_spp=REF_SPP, spp_g=256, big=True):
    """Learned guiding at equal time on the window-lit room (2M triangles,
    depth 12): relMSE of guided vs plain against a ref_spp plain reference
    at width x height (median over `reps` runs); throughput of the guided
    render at 1920x1080 (big=True); the network kernels against the
    tensor-core peak."""
    from drawlab_gb300 import abi, api, metrics, scenes
    small = api.Scene.from_data(ctx, scenes.guiding_room(width=width, height=height))
    t0 = time.perf_counter()
    ref = small.render(abi.make_opts(spp=ref_spp, max_depth=12, seed=1000))
    ref_s = time.perf_counter() - t0
    results = []
    for rep in range(max(1, reps)):
        g = api.Guide(ctx, seed=40 + rep)
        img_g = small.render_guided(abi.make_opts(spp=spp_g, max_depth=12, seed=50 + rep), g)
        st = ctx.stats()
        t_g, train_ms = st.render_ms, st.guide_train_ms
        small.render(abi.make_opts(spp=64, max_depth=12, seed=60 + rep))
        t_p64 = ctx.stats().render_ms
        spp_p = max(1, int(round(64 * t_g / t_p64)))
        img_p = small.render(abi.make_opts(spp=spp_p, max_depth=12, seed=70 + rep))
        t_p = ctx.stats().render_ms
        results.append((metrics.relmse(img_g, ref), metrics.relmse(img_p, ref), t_g, t_p, spp_p, train_ms,
                        metrics.relmse_robust(img_g, ref), metrics.relmse_robust(img_p, ref)))
    small.close()
    e_g = float(np.median([r[0] for r in results]))
    e_p = float(np.median([r[1] for r in results]))
    r_g = float(np.median([r[6] for r in results]))
    r_p = float(np.median([r[7] for r in results]))
    out = {"metric": "relMSE ratio plain/guided at equal time (window-lit room, 2M triangles)",
           "value": e_p / e_g, "unit": "x (median over runs)", "steps": len(results),
           "ms_per_step": float(np.mean([r[2] for r in results])),
           "config": {"workload": "guided", "triangles": 1960090, "relmse_resolution": "%dx%d" % (width, height),
                      "reference": "plain, %d spp (%.1f s)" % (ref_spp, ref_s), "guided_spp": spp_g,
                      "max_depth": 12, "l2_flush": "inputs larger than L2 (BVH + samples)"},
           "relmse": {"guided": e_g, "plain": e_p, "runs": [
               {"guided": r[0], "plain": r[1], "guided_ms": r[2], "plain_ms": r[3], "plain_spp": r[4],
                "train_ms": r[5], "robust_guided": r[6], "robust_plain": r[7]} for r in results]},
           "relmse_robust": {"guided": r_g, "plain": r_p, "ratio": r_p / r_g,
                             "note": "relMSE without the 0.1 % largest per-pixel errors (sun-edge fireflies)"}}
    if big:
        bigs = api.Scene.from_data(ctx, scenes.guiding_room())
        g = api.Guide(ctx, seed=99)
        for _ in range(warmup):
            bigs.render_guided(abi.make_opts(spp=4, max_depth=12, seed=5), g)
        with ClockSampler(ctx_device(ctx)) as clocks:
            t0 = time.perf_counter()
            bigs.render_guided(abi.make_opts(spp=16, max_depth=12, seed=6), g)
            wall = time.perf_counter() - t0
            st = ctx.stats()
        bigs.close()
        samples = 1920 * 1080 * 16
        out["guided_1080p"] = {"samples_per_s": samples / (st.render_ms / 1e3), "ms": st.render_ms,
                               "records": st.guide_records, "train_ms": st.guide_train_ms}
        out["gpu_launches"] = st.kernel_launches
        out["e2e"] = {"value": samples / wall, "unit": "samples/s (guided 1080p, 16 spp)", "h2d_bytes_per_step": 0,
                      "d2h_bytes_per_step": 1920 * 1080 * 12, "call": "dl_render_guided"}
        out["clocks"] = clocks.summary()
    out["network"] = network_roofline(ctx, api)
    return out


def run_guided(args):
    local = _device_setup()
    if local is None:
        return
    from drawlab_gb300 import api
    ctx = api.Context(local)
    w, h = (int(v) for v in args.guided_res.split("x"))
    r = guided_measure(ctx, max(1, args.steps), args.warmup, w, h, args.ref_spp)
    line = dict(r, n_gpus=1, warmup=args.warmup, higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="f32 (network fp16 in, fp32 accumulate)", data="synthetic (procedural room and sky)")
    print(json.dumps(line))


def run_profile_frame(args):
    """One frame of the headline scene at --spp samples per pixel and nothing
    else (no warm-up, no extra frames): the command under ncu for the
    traversal kernels' cache and DRAM counters.  Prints the frame's ray
    counts, which turn the counters into per-ray figures."""
    local = _device_setup()
    if local is None:
        return
    from drawlab_gb300 import abi, api, scenes
    sc = scenes.material_spheres()
    ctx = api.Context(local)
    gs = api.Scene.from_data(ctx, sc)
    gs.render(abi.make_opts(spp=args.spp, max_depth=WORKLOAD["max_depth"], seed=0))
    st = ctx.stats()
    print(json.dumps({"profile_frame": {"spp": args.spp, "camera_rays": st.camera_rays,
                                        "extension_rays": st.extension_rays, "shadow_rays": st.shadow_rays,
                                        "iterations": st.iterations, "render_ms": st.render_ms}}))


if __name__ == "__main__":
    main()
