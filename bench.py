"""VBM3D throughput benchmark (both steps, run_vbm3d semantics).

Workload: 1920x1080 x 30 frames RGB, AWGN sigma = 30, reference default
parameters for both steps, colour transform on (the reference CLI's
default), no flow; seeded synthetic clip (vbm3d_gb300.synth, seed 3000,
motion <= 6 px/frame) in place of a dataset.

Metric: denoised Mpix-frames/s = W*H*F / 1e6 / time of (step 1 + step 2).
  value : device-resident (inputs already in HBM; every step restores the
          noisy input on the device, runs both passes, and leaves basic and
          final estimates in HBM).  The clip (746 MB) is larger than L2.
  e2e   : the same work through vbm3d_run_host (the C-ABI call a CPU caller
          makes) from pinned host memory: H2D of the noisy clip and D2H of
          the basic and final estimates inside every timed step.
Multi-GPU: the path has no exchange step; --gpus N runs N independent
replicas (one per rank) and value = total clip frames / max time.

--impl reference times the reference's CPU implementation of the path on
the host cores instead: the oracle port (oracle/vbm3d_oracle.c) with all
host threads, each step a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, F, C = 1920, 1080, 30, 3
SIGMA = 30.0
SEED = 3000
COLOR = True
# CPU sample: a centre crop of the same clip with all 30 frames
CROP_W, CROP_H = 480, 270
METRIC = "denoised Mpix-frames/s (both steps)"
UNIT = "Mpix-frames/s"
WORKLOAD = "plain VBM3D, RGB 1920x1080x30, sigma=30, reference default parameters, colour transform on, no flow"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def make_workload():
    from vbm3d_gb300.synth import make_clip
    clean, noisy, _, _ = make_clip(W, H, F, C, SIGMA, SEED, vmax=6.0)
    return clean, noisy


def crop(noisy):
    import numpy as np
    y0, x0 = (H - CROP_H) // 2, (W - CROP_W) // 2
    return np.ascontiguousarray(noisy[:, :, y0:y0 + CROP_H, x0:x0 + CROP_W])


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_cpu_sample(noisy_crop, steps=1):
    """Oracle port on the crop with all host threads; returns (Mpix-frames/s, threads)."""
    from oracle.pyoracle import Oracle
    o = Oracle()
    th = cpu_threads()
    p1, p2 = o.default_params(1, SIGMA), o.default_params(2, SIGMA)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.run(SIGMA, noisy_crop, p1, p2, color_space=COLOR, threads=th)
    dt = time.perf_counter() - t0
    f, _, h, w = noisy_crop.shape
    return w * h * f * steps / 1e6 / dt, th


class ClockSampler:
    """nvidia-smi samples during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n):
    if n <= 1:
        return 0, 1
    import torch.distributed as dist
    dist.init_process_group("nccl")
    return dist.get_rank(), dist.get_world_size()


def reduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_reference(args):
    """CPU arm: the oracle port on the host cores, each step a bounded sample."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    _, noisy = make_workload()
    sample = crop(noisy)
    time_cpu_sample(sample[:4], steps=1) if args.warmup > 0 else None
    value, th = time_cpu_sample(sample, steps=args.steps)
    f, _, h, w = sample.shape
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "ms_per_step": round(w * h * f / 1e6 / value * 1e3, 1), "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded blobs/gratings/translation + AWGN)",
        "config": {"workload": WORKLOAD, "sample": "%dx%dx%d centre crop" % (w, h, f)},
        "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": th, "kind": "port",
                         "sample": "%dx%dx%d centre crop of the workload, both steps, %d OpenMP threads"
                                   % (w, h, f, th)},
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bm_flops(p, dims_video, n_dist):
    return float(n_dist) * p.k * p.k * p.kt * dims_video.channels * 3.0  # sub, mul, add per term


def run_gpu(args):
    import numpy as np
    import torch

    import vbm3d_gb300 as vb

    rank, world = dist_setup(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    vb.load()

    clean, noisy = make_workload()
    p1, p2 = vb.default_params(1, SIGMA), vb.default_params(2, SIGMA)
    x0 = torch.from_numpy(noisy).to(dev)
    x = torch.empty_like(x0)
    stream = torch.cuda.current_stream()

    def one_step():
        x.copy_(x0)
        return vb.run(x, SIGMA, p1, p2, color_space=COLOR)

    for _ in range(max(args.warmup, 0)):
        basic, final = one_step()
    torch.cuda.synchronize()

    # timed region: K steps, barrier + synchronize on both sides
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        basic, final = one_step()
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    barrier(world)
    ms = ev0.elapsed_time(ev1) / args.steps
    ms = reduce_max(ms, world)
    mpf = W * H * F / 1e6
    value = mpf * world / (ms / 1e3)
    launches_per_step = 2 + 2 + 2 + (4 if COLOR else 0)  # bm, filter, normalize per step; colour transforms

    # quality of this run (not part of the timed region)
    from vbm3d_gb300.synth import psnr
    final_np = final.cpu().numpy()
    q = {"psnr_noisy": round(psnr(clean, noisy), 3), "psnr_final": round(psnr(clean, final_np), 3)}

    # roofline of the dominant kernel: step-2 block matching on the basic
    # estimate (in the colour space the step sees), timed alone on the stream
    xb = torch.from_numpy(noisy).to(dev)
    vb.color_transform(xb, True)
    b_ws = basic.clone()
    vb.color_transform(b_ws, True)
    n_dist = vb.bm_distance_count(b_ws, p2)
    d_video = vb.Dims(W, H, F, C)
    flops = bm_flops(p2, d_video, n_dist)
    reps = 3
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    vb.similar_patches(b_ws, p2)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        vb.similar_patches(b_ws, p2)
    e1.record(stream)
    torch.cuda.synchronize()
    bm_ms = e0.elapsed_time(e1) / reps
    sm_max = clocks.get("sm_max_mhz") or 2070.0
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        sm_max = peaks.get("sm_max_mhz", sm_max)
    except (OSError, ValueError):
        pass
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_max * 1e6 / 1e12  # TFLOP/s, FMA = 2 flops
    achieved = flops / (bm_ms / 1e3) / 1e12
    roofline = {"kernel": "bm_kernel (step-2 block matching)", "bound": "fp32", "achieved": round(achieved, 3),
                "peak": round(fp32_peak, 1), "unit": "TFLOP/s", "frac": round(achieved / fp32_peak, 4),
                "traffic": None, "peak_source": "nominal FP32 FMA rate: %d SMs x 128 lanes x 2 x %.0f MHz" % (n_sm, sm_max),
                "algorithmic_flops": flops, "distances": n_dist, "ms": round(bm_ms, 3)}

    # end to end through the host C-ABI call, pinned host buffers
    e2e = None
    if args.e2e_steps > 0:
        hn = torch.from_numpy(noisy).pin_memory().numpy()
        hb = torch.empty(noisy.shape, dtype=torch.float32).pin_memory().numpy()
        hf = torch.empty(noisy.shape, dtype=torch.float32).pin_memory().numpy()
        vb.run_host(hn, SIGMA, p1, p2, color_space=COLOR, basic=hb, out=hf)
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            vb.run_host(hn, SIGMA, p1, p2, color_space=COLOR, basic=hb, out=hf)
        dt = (time.perf_counter() - t0) / args.e2e_steps
        dt = reduce_max(dt, world)
        e2e = {"value": round(mpf * world / dt, 3), "unit": UNIT, "h2d_bytes_per_step": int(hn.nbytes),
               "d2h_bytes_per_step": int(hb.nbytes + hf.nbytes), "ms_per_step": round(dt * 1e3, 1)}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        sample = crop(noisy)
        val, th = time_cpu_sample(sample, steps=1)
        f, _, h, w = sample.shape
        cpu = {"value": round(val, 4), "unit": UNIT, "cores": th, "kind": "port",
               "sample": "%dx%dx%d centre crop of the workload, both steps, %d OpenMP threads" % (w, h, f, th)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded blobs/gratings/translation + AWGN)",
            "config": {"workload": WORKLOAD, "global_batch": world, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (746 MB clip)", "quality": q},
            "clocks": clocks, "e2e": e2e, "gpu_launches": launches_per_step * args.steps,
            "roofline": roofline, "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
