"""bench.py's CPU baseline (the oracle port on the host cores): both modes,
all threads on one clip at a time and independent clips as concurrent
single-threaded worker processes (spawned), the higher one reported."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from vbm3d_gb300.synth import make_clip  # noqa: E402


def tiny_samples():
    out = []
    for i, (w, h, f, c, s) in enumerate([(40, 32, 5, 3, 20.0), (36, 30, 11, 1, 10.0)]):
        _, noisy, _, _ = make_clip(w, h, f, c, s, 4300 + i)
        out.append((noisy, s))
    return out


def test_process_jobs_cover_the_sample():
    samples = tiny_samples()
    jobs, reps = bench.proc_jobs(samples, 8)
    # clips of at most 8 frames: 5 | 8 + 3 frames -> 3 chunks, 11 copies for 4 jobs per worker
    assert bench.PROC_JOBS_PER == 4 and reps == 11 and len(jobs) == 33
    assert all(a.shape[0] <= bench.PROC_CHUNK_F for a, _ in jobs)
    frames = sum(a.shape[0] for a, _ in jobs)
    assert frames == reps * sum(a.shape[0] for a, _ in samples)
    sizes = [a.size for a, _ in jobs]
    assert sizes == sorted(sizes, reverse=True)


def test_cpu_baseline_reports_the_higher_mode():
    cpu = bench.cpu_baseline(tiny_samples(), "two tiny clips")
    omp, proc = cpu["modes"]["openmp"], cpu["modes"]["processes"]
    assert omp["value"] > 0 and proc["value"] > 0
    assert cpu["value"] == max(omp["value"], proc["value"])
    assert cpu["kind"] == "port" and cpu["cores"] == omp["threads"] == proc["processes"] >= 1
    assert np.isfinite(cpu["value"])
