"""VBM3D throughput benchmark (both steps, run_vbm3d semantics).

Default workload (--workload batch64): the batched form on 64 clips of
uneven size, width uniform in 160-1280, height in 120-720, 5-40 frames, 1
or 3 channels, sigma in {5, 10, 20, 30, 50}; shapes drawn from numpy
PCG64(4000), each clip from the seeded synthetic generator
(vbm3d_gb300.synth, seed 4000 + clip) in place of a dataset; reference
default parameters for both steps, colour transform on, no flow.
--workload 1080p30: the plain path on one RGB 1920x1080 x 30 clip, sigma 30
(seed 3000, motion <= 6 px/frame).

Metric: denoised Mpix-frames/s = sum of W*H*F / 1e6 / time of (step 1 +
step 2) over every clip.
  value : device-resident (inputs already in HBM, 2.7 GB for batch64 and
          0.75 GB for 1080p30, both larger than L2): one CUDA-graph launch
          of the whole batch per step (batch64), one vbm3d_gpu_run per step
          (1080p30).
  plain : (batch64) the same clips looped through vbm3d_gpu_run, and the
          largest PSNR difference between the two forms.
  e2e   : the same work from pinned host memory through the public API:
          H2D of every noisy clip, the run, D2H of the basic and final
          estimates, all inside every timed step.
Multi-GPU: the path has no exchange step; --gpus N runs N independent
replicas (one per rank) and value = total clip frames / max time.

--impl reference times the reference's CPU implementation of the path on
the host cores instead: the oracle port (oracle/vbm3d_oracle.c) built with
the reference's own flags (-O3 -ffast-math -fomit-frame-pointer, OpenMP;
oracle/_build/liboracle_fast.so), each step a bounded sample of the same
workload.  The reference's sources are not on the GPU host; where they are,
oracle/time_ref_vs_port.py times this build against the reference's own
build on the same sample, and the line carries that measured ratio
(profiles/cpu_reference_vs_port.json) as port_vs_reference.  The CPU figure (that line's value and
the GPU line's cpu_baseline) is the higher of two modes: all host threads
on one clip at a time (OpenMP), and independent clips of at most 8 frames
as concurrent single-threaded processes, one per host thread, with at
least four clips queued per process.
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

METRIC = "denoised Mpix-frames/s (both steps), batched vs plain at <=0.01 dB PSNR delta"
UNIT = "Mpix-frames/s"
COLOR = True
DATA = "synthetic (seeded blobs/gratings/translation + AWGN)"

# 1080p30 plain workload
W, H, F, C = 1920, 1080, 30, 3
SIGMA = 30.0
SEED = 3000
WORKLOAD_1080 = "plain VBM3D, RGB 1920x1080x30, sigma=30, reference default parameters, colour transform on, no flow"
WORKLOAD_MS = ("multiscaler DCT pyramid of an RGB 1920x1080x30 clip, 3 levels: decompose, then recompose with "
               "ratio 0.7 (the multiscale script's pre- and post-processing)")
WORKLOAD_BATCH = ("batched VBM3D, 64 clips: width U[160,1280], height U[120,720], 5-40 frames, 1 or 3 channels, "
                  "sigma in {5,10,20,30,50}; reference default parameters, colour transform on, no flow")

# CPU sample: centre crops of this size (at most) of every 8th clip
SAMPLE_W, SAMPLE_H, SAMPLE_F = 256, 144, 8
# 1080p30 CPU sample: a centre crop with all 30 frames
CROP_W, CROP_H = 480, 270


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batch64", choices=["batch64", "1080p30"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-1080p", action="store_true", help="batch64: skip the extra 1080p30 plain figure")
    return ap.parse_args()


def make_batch():
    from vbm3d_gb300.synth import batch_specs, make_clip
    clips = []
    for i, (w, h, f, c, s) in enumerate(batch_specs()):
        clean, noisy, _, _ = make_clip(w, h, f, c, s, 4000 + i)
        clips.append(dict(clean=clean, noisy=noisy, sigma=s))
    return clips


def make_1080():
    from vbm3d_gb300.synth import make_clip
    clean, noisy, _, _ = make_clip(W, H, F, C, SIGMA, SEED, vmax=6.0)
    return clean, noisy


def crop(v, w, h, f):
    import numpy as np
    F_, _, H_, W_ = v.shape
    w, h, f = min(w, W_), min(h, H_), min(f, F_)
    y0, x0 = (H_ - h) // 2, (W_ - w) // 2
    return np.ascontiguousarray(v[:f, :, y0:y0 + h, x0:x0 + w])


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_cpu(samples, steps=1):
    """Oracle port (reference flags) over [(noisy, sigma)] with all host
    threads; returns (Mpix-frames/s, threads)."""
    from oracle.pyoracle import ORACLE_FAST_SO, Oracle
    o = Oracle(ORACLE_FAST_SO)
    th = cpu_threads()
    mpf = 0.0
    t0 = time.perf_counter()
    for _ in range(steps):
        for noisy, sigma in samples:
            o.run(sigma, noisy, o.default_params(1, sigma), o.default_params(2, sigma), color_space=COLOR,
                  threads=th)
            f, _, h, w = noisy.shape
            mpf += w * h * f / 1e6
    return mpf / (time.perf_counter() - t0), th


def _port_warm(_):
    from oracle.pyoracle import ORACLE_FAST_SO, Oracle
    Oracle(ORACLE_FAST_SO)
    return 0


def _port_job(job):
    """One clip through the oracle port on one thread (a worker process)."""
    noisy, sigma = job
    from oracle.pyoracle import ORACLE_FAST_SO, Oracle
    o = Oracle(ORACLE_FAST_SO)
    o.run(sigma, noisy, o.default_params(1, sigma), o.default_params(2, sigma), color_space=COLOR, threads=1)
    f, _, h, w = noisy.shape
    return w * h * f / 1e6


PROC_CHUNK_F = 8    # process mode: a sample clip runs as independent clips of at most 8 frames
PROC_JOBS_PER = 4   # and at least this many jobs per worker, so that the last jobs' tail stays short


def proc_jobs(samples, th):
    """Jobs of the process mode: each sample clip cut into clips of at most
    PROC_CHUNK_F frames, repeated until there are PROC_JOBS_PER jobs per
    worker, largest first (a steady stream of clips keeps every core busy,
    as a serving loop would); returns (jobs, repeats)."""
    chunks = [(a[t:t + PROC_CHUNK_F], s) for a, s in samples for t in range(0, a.shape[0], PROC_CHUNK_F)]
    reps = max(1, -(-PROC_JOBS_PER * th // len(chunks)))
    return sorted([c for c in chunks for _ in range(reps)], key=lambda c: -c[0].size), reps


def time_cpu_procs(samples, steps=1):
    """The same sample as independent single-threaded runs, one worker
    process per host thread; returns (Mpix-frames/s, processes, repeats).
    The workers are spawned (the parent may hold a CUDA context) and have
    loaded the oracle before the clock starts."""
    import multiprocessing as mp
    th = cpu_threads()
    jobs, reps = proc_jobs(samples, th)
    with mp.get_context("spawn").Pool(th) as pool:
        pool.map(_port_warm, range(th), chunksize=1)
        t0 = time.perf_counter()
        mpf = sum(pool.map(_port_job, jobs * steps, chunksize=1))
        dt = time.perf_counter() - t0
    return mpf / dt, th, reps


def port_vs_reference():
    """The measured ratio of this port build to the reference's own build on
    the same samples and threads (oracle/time_ref_vs_port.py, committed in
    profiles/cpu_reference_vs_port.json), or None."""
    path = os.path.join(ROOT, "profiles", "cpu_reference_vs_port.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        m = json.load(f)
    return {"host": m["host"], "source": "profiles/cpu_reference_vs_port.json",
            "port_fast_over_reference": {w: r["port_fast_over_reference"] for w, r in m["workloads"].items()}}


def cpu_baseline(samples, desc, steps=1):
    """cpu_baseline of the JSON line: the oracle port on the host cores in
    two modes, all threads on one clip at a time (OpenMP) and independent
    clips as concurrent single-threaded processes; value = the higher."""
    v_omp, th = time_cpu(samples, steps)
    v_proc, npr, reps = time_cpu_procs(samples, steps)
    return {"value": round(max(v_omp, v_proc), 4), "unit": UNIT, "cores": th, "kind": "port",
            "build": "oracle/vbm3d_oracle.c with the reference's flags (-O3 -ffast-math -fomit-frame-pointer "
                     "-fopenmp)",
            "port_vs_reference": port_vs_reference(),
            "sample": desc + "; the higher of two modes",
            "modes": {"openmp": {"value": round(v_omp, 4), "threads": th},
                      "processes": {"value": round(v_proc, 4), "processes": npr,
                                    "jobs": "the sample in clips of at most %d frames, x %d, one thread each"
                                            % (PROC_CHUNK_F, reps)}}}


def cpu_sample(workload, clips=None, noisy=None):
    """The bounded CPU sample of a workload and its description."""
    if workload == "batch64":
        picks = list(range(0, 64, 8))
        samples = [(crop(clips[i]["noisy"], SAMPLE_W, SAMPLE_H, SAMPLE_F), clips[i]["sigma"]) for i in picks]
        mpf = sum(a.shape[0] * a.shape[2] * a.shape[3] for a, _ in samples) / 1e6
        return samples, ("centre crops (at most %dx%dx%d) of clips %s, %.2f Mpix-frames, both steps"
                         % (SAMPLE_W, SAMPLE_H, SAMPLE_F, picks, mpf))
    c = crop(noisy, CROP_W, CROP_H, F)
    return [(c, SIGMA)], "%dx%dx%d centre crop of the workload, both steps" % (CROP_W, CROP_H, F)


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
    """One process per GPU (torchrun's RANK / WORLD_SIZE / MASTER_*): NCCL on
    GPUs, gloo where there is none (the CPU tests of the replica path)."""
    if n <= 1:
        return 0, 1
    import torch
    import torch.distributed as dist
    dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return dist.get_rank(), dist.get_world_size()


def reduce_max(x, world):
    """The largest of the ranks' values (timings: the slowest replica)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
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
    if args.workload == "batch64":
        samples, desc = cpu_sample("batch64", clips=make_batch())
        workload = WORKLOAD_BATCH
    else:
        _, noisy = make_1080()
        samples, desc = cpu_sample("1080p30", noisy=noisy)
        workload = WORKLOAD_1080
    if args.warmup > 0:
        time_cpu([(a[:2], s) for a, s in samples[:2]])
    cpu = cpu_baseline(samples, desc, steps=args.steps)
    value = cpu["value"]
    mpf = sum(a.shape[0] * a.shape[2] * a.shape[3] for a, _ in samples) / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "ms_per_step": round(mpf / value * 1e3, 1), "vs_baseline": None, "dtype": "f32", "data": DATA,
        "config": {"workload": workload, "sample": desc},
        "cpu_baseline": cpu,
        "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bm_flops(k, channels, n_dist):
    return float(n_dist) * k * k * channels * 3.0  # sub, mul, add per term (kt = 1)


def fp32_peak(dev, clocks):
    import torch
    sm_max = clocks.get("sm_max_mhz") or 2070.0
    try:
        sm_max = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("sm_max_mhz", sm_max)
    except (OSError, ValueError):
        pass
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    return n_sm * 128 * 2 * sm_max * 1e6 / 1e12, "nominal FP32 FMA rate: %d SMs x 128 lanes x 2 x %.0f MHz" % (
        n_sm, sm_max)


# DRAM bytes (read + write) per reference patch of the batched step-2 block
# matching of the RGB k = 7 clips: ncu dram__bytes_read.sum +
# dram__bytes_write.sum of batch_bm_kernel<2, 7, 3, 32> on the small case
# (python -m vbm3d_gb300.profile_case --batch 16 --scale 0.5: 111.7 MB +
# 24.2 MB for 973 383 reference patches), scaled by the launch's reference
# patches.
BM2_DRAM_BYTES_PER_REF = 139.7


def timed(stream, fn, steps):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def measure_multiscaler(vb, dev, stream, clocks, with_cpu):
    """The multiscaler DCT pyramid (vbm3d_gpu_ms_decompose / _recompose) of an
    RGB 1080p30 clip, 3 levels; its float products against the nominal FP32
    FMA rate; optionally the restatement (scipy, double) on one frame."""
    import torch
    F_, C_, H_, W_, L_ = 30, 3, 1080, 1920, 3
    g = torch.Generator(device=dev).manual_seed(5)
    x = torch.rand((F_, C_, H_, W_), device=dev, generator=g) * 255
    lv = vb.ms_decompose(x, L_)
    for _ in range(3):
        vb.ms_recompose(vb.ms_decompose(x, L_), 0.7)
    t_dec = timed(stream, lambda: vb.ms_decompose(x, L_), 3)
    t_rec = timed(stream, lambda: vb.ms_recompose(lv, 0.7), 3)
    P_ = F_ * C_
    # multiply-adds of the products: every transform is split into its even
    # and odd halves (ne = ceil(n / 2), no = n / 2): a forward 2D transform
    # of R x W costs R (ne_W^2 + no_W^2) + W (ne_R^2 + no_R^2) per plane, an
    # inverse one R ne_W W + W ne_R R; decompose runs one full-size forward
    # transform and one inverse per level, recompose one forward per level
    # and one full-size inverse
    def fwd(r, w):
        return P_ * (r * (((w + 1) // 2) ** 2 + (w // 2) ** 2) + w * (((r + 1) // 2) ** 2 + (r // 2) ** 2))

    def inv(r, w):
        return P_ * (r * ((w + 1) // 2) * w + w * ((r + 1) // 2) * r)

    lv = [(H_ >> i, W_ >> i) for i in range(L_)]
    macs = float(fwd(H_, W_) + sum(inv(r, w) for r, w in lv) + sum(fwd(r, w) for r, w in lv) + inv(H_, W_))
    ms = t_dec + t_rec
    peak, src = fp32_peak(dev, clocks)
    tf = 2 * macs / (ms / 1e3) / 1e12
    out = {"workload": WORKLOAD_MS, "value": round(F_ * H_ * W_ / 1e6 / (ms / 1e3), 3), "unit": "Mpix-frames/s",
           "decompose_ms": round(t_dec, 2), "recompose_ms": round(t_rec, 2), "tflops": round(tf, 1),
           "fp32_frac": round(tf / peak, 3), "fp32_peak_source": src}
    if with_cpu:
        from oracle import ms_oracle
        img = x[0].cpu().numpy()
        t0 = time.perf_counter()
        ms_oracle.recompose(ms_oracle.decompose(img, L_), 0.7)
        dt = time.perf_counter() - t0
        out["cpu_port"] = {"value": round(H_ * W_ / 1e6 / dt, 3), "unit": "Mpix-frames/s", "cores": 1,
                           "kind": "port", "sample": "one RGB frame through oracle/ms_oracle.py (scipy FFT DCTs "
                                                     "in double)"}
    return out


def measure_1080(vb, dev, steps, warmup, full):
    """The plain 1080p30 workload; with full, also the roofline inputs."""
    import torch
    clean, noisy = make_1080()
    p1, p2 = vb.default_params(1, SIGMA), vb.default_params(2, SIGMA)
    x0 = torch.from_numpy(noisy).to(dev)
    x = torch.empty_like(x0)
    out = {}

    def one_step():
        x.copy_(x0)
        out["bf"] = vb.run(x, SIGMA, p1, p2, color_space=COLOR)

    for _ in range(max(warmup, 0)):
        one_step()
    torch.cuda.synchronize()
    return clean, noisy, x0, one_step, out, p1, p2


def run_gpu(args):
    import numpy as np
    import torch

    import vbm3d_gb300 as vb
    from vbm3d_gb300.synth import psnr

    rank, world = dist_setup(args.gpus)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream()
    vb.load()
    line = {}

    if args.workload == "batch64":
        clips = make_batch()
        mpf = sum(c["noisy"].shape[0] * c["noisy"].shape[2] * c["noisy"].shape[3] for c in clips) / 1e6
        x0 = [torch.from_numpy(c["noisy"]).to(dev) for c in clips]
        t0 = time.perf_counter()
        b = vb.Batch([dict(noisy=x, sigma=c["sigma"]) for x, c in zip(x0, clips)], color_space=COLOR)
        torch.cuda.synchronize()
        create_s = time.perf_counter() - t0
        cfg = b.config()
        for _ in range(max(args.warmup, 0)):
            b.run()
        torch.cuda.synchronize()
        sampler = ClockSampler(local)
        barrier(world)
        torch.cuda.synchronize()
        sampler.start()
        ms = timed(stream, b.run, args.steps)
        clocks = sampler.stop()
        barrier(world)
        ms = reduce_max(ms, world)
        value = mpf * world / (ms / 1e3)
        launches = b.profile()
        gpu_launches = (len(launches) + 3) * args.steps  # work launches + prep, mid, final
        batched_final = [d.cpu().numpy() for d in b.denoised]

        # the plain path looped over the same clips (vbm3d_gpu_run transforms
        # its input in place and back, so every step restores it first)
        xs = [torch.empty_like(x) for x in x0]
        outs = []

        def plain_step():
            outs.clear()
            for x, xi, c in zip(xs, x0, clips):
                x.copy_(xi)
                outs.append(vb.run(x, c["sigma"], color_space=COLOR))

        plain_step()
        torch.cuda.synchronize()
        plain_ms = timed(stream, plain_step, 2)
        dps, gain = 0.0, []
        for c, bf, (_, pf) in zip(clips, batched_final, outs):
            pb = psnr(c["clean"], bf)
            dps = max(dps, abs(pb - psnr(c["clean"], pf.cpu().numpy())))
            gain.append(pb - psnr(c["clean"], c["noisy"]))
        plain = {"value": round(mpf * world / (plain_ms / 1e3), 3), "unit": UNIT, "ms_per_step": round(plain_ms, 1),
                 "psnr_delta_max_db": round(dps, 5), "what": "the same clips looped through vbm3d_gpu_run"}

        # roofline: the dominant block-matching launch of the batch
        bm = max((l for l in launches if l["phase"] in (0, 2)), key=lambda l: l["ms"])
        top = max(launches, key=lambda l: l["ms"])
        step = bm["phase"] // 2 + 1
        members = [i for i, c in enumerate(clips)
                   if vb.default_params(step, c["sigma"]).k == bm["k"] and c["noisy"].shape[1] == bm["channels"]]
        n_dist = 0
        for i in members:
            c = clips[i]
            p1, p2 = vb.default_params(1, c["sigma"]), vb.default_params(2, c["sigma"])
            x = x0[i].clone()
            vb.color_transform(x, COLOR)
            if step == 1:
                n_dist += vb.bm_distance_count(x, p1)
            else:
                num, den = vb.step1(x, p1, c["sigma"], color_space=COLOR)
                n_dist += vb.bm_distance_count(vb.normalize(num, den, x), p2)
        flops = bm_flops(bm["k"], bm["channels"], n_dist)
        peak, peak_src = fp32_peak(dev, clocks)
        achieved = flops / (bm["ms"] / 1e3) / 1e12
        traffic = BM2_DRAM_BYTES_PER_REF * bm["refs"] if (step, bm["k"], bm["channels"]) == (2, 7, 3) else None
        roofline = {"kernel": "batch_bm_kernel<%d, %d, %d, %d> (step-%d block matching, %d clips)"
                              % (step, bm["k"], bm["channels"], 16 if bm["channels"] == 1 else 32, step,
                                 bm["clips"]),
                    "bound": "fp32", "achieved": round(achieved, 3), "peak": round(peak, 1), "unit": "TFLOP/s",
                    "frac": round(achieved / peak, 4), "traffic": traffic,
                    "traffic_source": "ncu DRAM bytes (read + write) of this kernel per reference patch on "
                                      "the small case (profile_case --batch 16 --scale 0.5), x the launch's "
                                      "reference patches",
                    "peak_source": peak_src,
                    # the exact-order sums issue a packed subtract, FMA square and add per two
                    # candidate-terms: their issue ceiling is half the FMA peak
                    "exact_order_ceiling": {"peak": round(peak / 2, 1), "frac": round(2 * achieved / peak, 4),
                                            "what": "3 packed f32x2 ops per 2 candidate-terms (sub, fma square, "
                                                    "add in the reference's order): half the FMA rate"},
                    "algorithmic_flops": flops, "distances": n_dist, "refs": bm["refs"], "ms": round(bm["ms"], 2),
                    "share_of_run": round(bm["ms"] / sum(l["ms"] for l in launches), 3),
                    "largest_launch": "phase %d k=%d C=%d, %.1f ms" % (top["phase"], top["k"], top["channels"],
                                                                      top["ms"])}

        # end to end through the public API from pinned host memory
        e2e = None
        if args.e2e_steps > 0:
            hin = [torch.from_numpy(c["noisy"]).pin_memory() for c in clips]
            hb = [torch.empty(c["noisy"].shape, dtype=torch.float32).pin_memory() for c in clips]
            hd = [torch.empty(c["noisy"].shape, dtype=torch.float32).pin_memory() for c in clips]

            def e2e_step():
                for x, h in zip(x0, hin):
                    x.copy_(h, non_blocking=True)
                b.run()
                for ob, od, db, dd in zip(hb, hd, b.basic, b.denoised):
                    ob.copy_(db, non_blocking=True)
                    od.copy_(dd, non_blocking=True)
                torch.cuda.synchronize()

            e2e_step()
            barrier(world)
            t0 = time.perf_counter()
            for _ in range(args.e2e_steps):
                e2e_step()
            dt_serial = reduce_max((time.perf_counter() - t0) / args.e2e_steps, world)

            # Pipelined, as a serving loop runs it: two batches over their own
            # device inputs (same clips, same configuration), so that while one
            # batch computes, the next step's inputs upload into the other and
            # the previous step's estimates download.  Every step still moves
            # its 2.8 GB in and 5.6 GB out over the host link (about 200 GB/s
            # each way on this machine) inside the timed region.
            x1 = [torch.empty_like(x) for x in x0]
            b1 = vb.Batch([dict(noisy=x, sigma=c["sigma"]) for x, c in zip(x1, clips)], color_space=COLOR,
                          config={k: cfg[k] for k in cfg if k.endswith(("tile", "warps"))})
            pair = [(b, x0), (b1, x1)]
            s_comp, s_up, s_down = torch.cuda.current_stream(), torch.cuda.Stream(), torch.cuda.Stream()
            ran, down = [None, None], [None, None]  # per batch: last run done, its outputs copied out

            def e2e_pipelined(nsteps):
                for i in range(nsteps):
                    j = i % 2
                    bj, xj = pair[j]
                    with torch.cuda.stream(s_up):
                        if ran[j] is not None:
                            s_up.wait_event(ran[j])  # the batch's previous run has read its inputs
                        for x, h in zip(xj, hin):
                            x.copy_(h, non_blocking=True)
                        up = torch.cuda.Event()
                        up.record(s_up)
                    s_comp.wait_event(up)
                    if down[j] is not None:
                        s_comp.wait_event(down[j])  # its previous estimates are out
                    bj.run(stream=s_comp)
                    ran[j] = torch.cuda.Event()
                    ran[j].record(s_comp)
                    with torch.cuda.stream(s_down):
                        s_down.wait_event(ran[j])
                        for ob, od, db, dd in zip(hb, hd, bj.basic, bj.denoised):
                            ob.copy_(db, non_blocking=True)
                            od.copy_(dd, non_blocking=True)
                        down[j] = torch.cuda.Event()
                        down[j].record(s_down)
                torch.cuda.synchronize()

            e2e_pipelined(2)
            barrier(world)
            t0 = time.perf_counter()
            e2e_pipelined(args.e2e_steps)
            dt = reduce_max((time.perf_counter() - t0) / args.e2e_steps, world)
            b1.close()
            del x1
            nb = sum(h.numel() * 4 for h in hin)
            e2e = {"value": round(mpf * world / dt, 3), "unit": UNIT, "h2d_bytes_per_step": nb,
                   "d2h_bytes_per_step": 2 * nb, "ms_per_step": round(dt * 1e3, 1), "steps": args.e2e_steps,
                   "what": "every step: pinned host -> device copies of the 64 noisy clips, one batch run, "
                           "device -> pinned host copies of the basic and final estimates; two batches "
                           "alternate so that a step's copies overlap the other batch's run (wall clock over "
                           "all steps, first upload and last download included)",
                   "serial": {"value": round(mpf * world / dt_serial, 3), "ms_per_step": round(dt_serial * 1e3, 1),
                              "what": "the same step with copies and run one after the other on one stream"}}

        extra_1080 = None
        if not args.no_1080p:
            clean, noisy, _, one_step, out, _, _ = measure_1080(vb, dev, 2, 2, False)
            ms1080 = timed(stream, one_step, 3)
            extra_1080 = {"workload": WORKLOAD_1080, "value": round(W * H * F / 1e6 / (ms1080 / 1e3), 3),
                          "unit": UNIT, "ms_per_step": round(ms1080, 1),
                          "psnr_final": round(psnr(clean, out["bf"][1].cpu().numpy()), 3)}

        extra_ms = None
        if not args.no_1080p:
            extra_ms = measure_multiscaler(vb, dev, stream, clocks, rank == 0 and not args.no_cpu_baseline)

        cpu = None
        if rank == 0 and not args.no_cpu_baseline:
            samples, desc = cpu_sample("batch64", clips=clips)
            cpu = cpu_baseline(samples, desc)
            if extra_1080 is not None:
                # the 1080p30 clip's own CPU sample (a 480x270x30 centre crop)
                samples, desc = cpu_sample("1080p30", noisy=noisy)
                c1080 = cpu_baseline(samples, desc)
                extra_1080["cpu_baseline"] = c1080
                extra_1080["vs_cpu"] = round(extra_1080["value"] / c1080["value"], 1)
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": DATA,
            "config": {"workload": WORKLOAD_BATCH, "clips": len(clips), "mpix_frames": round(mpf, 2),
                       "global_batch": world, "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (%.1f GB)" % (sum(x.numel() for x in x0) * 4 / 1e9),
                       "graph": "one CUDA-graph launch per step", "tuned": {k: cfg[k] for k in cfg
                                                                            if k.endswith(("tile", "warps"))},
                       "create_s": round(create_s, 2),
                       "psnr_gain_db": {"min": round(min(gain), 3), "mean": round(float(np.mean(gain)), 3)}},
            "plain": plain, "clocks": clocks, "e2e": e2e, "gpu_launches": gpu_launches, "roofline": roofline,
            "cpu_baseline": cpu, "plain_1080p30": extra_1080, "multiscaler_1080p30": extra_ms,
            "launches": [{k: (round(v, 2) if isinstance(v, float) else v) for k, v in l.items()
                          if k in ("phase", "k", "channels", "clips", "refs", "ms")} for l in launches],
        }
    else:
        clean, noisy, x0, one_step, out, p1, p2 = measure_1080(vb, dev, args.steps, args.warmup, True)
        sampler = ClockSampler(local)
        barrier(world)
        torch.cuda.synchronize()
        sampler.start()
        ms = timed(stream, one_step, args.steps)
        clocks = sampler.stop()
        barrier(world)
        ms = reduce_max(ms, world)
        mpf = W * H * F / 1e6
        value = mpf * world / (ms / 1e3)
        basic, final = out["bf"]
        q = {"psnr_noisy": round(psnr(clean, noisy), 3), "psnr_final": round(psnr(clean, final.cpu().numpy()), 3)}
        # roofline of the dominant kernel: step-2 block matching on the basic
        # estimate (in the colour space the step sees), timed alone
        b_ws = basic.clone()
        vb.color_transform(b_ws, True)
        n_dist = vb.bm_distance_count(b_ws, p2)
        flops = bm_flops(p2.k, C, n_dist)
        vb.similar_patches(b_ws, p2)
        torch.cuda.synchronize()
        bm_ms = timed(stream, lambda: vb.similar_patches(b_ws, p2), 3)
        peak, peak_src = fp32_peak(dev, clocks)
        achieved = flops / (bm_ms / 1e3) / 1e12
        roofline = {"kernel": "bm2_kernel<7, 3> (step-2 block matching)", "bound": "fp32",
                    "achieved": round(achieved, 3), "peak": round(peak, 1), "unit": "TFLOP/s",
                    "frac": round(achieved / peak, 4), "traffic": None, "peak_source": peak_src,
                    "algorithmic_flops": flops, "distances": n_dist, "ms": round(bm_ms, 3)}
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
            dt = reduce_max((time.perf_counter() - t0) / args.e2e_steps, world)
            e2e = {"value": round(mpf * world / dt, 3), "unit": UNIT, "h2d_bytes_per_step": int(hn.nbytes),
                   "d2h_bytes_per_step": int(hb.nbytes + hf.nbytes), "ms_per_step": round(dt * 1e3, 1)}
        cpu = None
        if rank == 0 and not args.no_cpu_baseline:
            samples, desc = cpu_sample("1080p30", noisy=noisy)
            cpu = cpu_baseline(samples, desc)
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": DATA,
            "config": {"workload": WORKLOAD_1080, "global_batch": world,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (746 MB clip)", "quality": q},
            "clocks": clocks, "e2e": e2e, "gpu_launches": 10 * args.steps, "roofline": roofline,
            "cpu_baseline": cpu,
        }
    if rank == 0:
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
