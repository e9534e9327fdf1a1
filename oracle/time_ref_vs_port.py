"""Times the reference's own CPU build against the oracle port on the same
sample and thread count (test infrastructure: it measures the checker, it
is never on the product path).

The reference's own code (src/vbm3d.cpp run_vbm3d with its OpenMP tiling,
built with the reference's CMake flags -O3 -ffast-math by
oracle/build_ref.sh into oracle/_ref/libvbm3d_ref_fast.so) only exists
where the reference sources were present at build time, so this runs there;
the GPU host, which lacks the sources, times the port built with the same
flags (oracle/_build/liboracle_fast.so).  Timed: that fast build of the
port (what bench.py times), the reference's build, and the parity build
of the port (-O2, IEEE order) for comparison; the result is the ratio that
turns the port's figure into the reference's.

Samples: the CPU samples bench.py times (centre crops of every 8th clip of
the 64-clip batch; a 480x270x30 centre crop of the 1080p30 RGB clip), both
steps, colour transform on.  Modes, as in bench.py: all host threads on one
clip at a time (OpenMP; the reference caps itself at the largest power of
two <= min(cores, 32), src/vbm3d.cpp:121-127), and independent clips as
concurrent single-threaded processes.

    python oracle/time_ref_vs_port.py [out.json]
"""
import json
import multiprocessing as mp
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def _lib(impl):
    from oracle.pyoracle import ORACLE_FAST_SO, Oracle, RefLib
    if impl == "port":
        return Oracle()
    if impl == "port_fast":
        return Oracle(ORACLE_FAST_SO)
    return RefLib(exact=False)


def _run(impl, noisy, sigma, threads):
    from oracle.pyoracle import Oracle
    o = Oracle()
    p1, p2 = o.default_params(1, sigma), o.default_params(2, sigma)
    lib = _lib(impl)
    lib.run(sigma, noisy, p1, p2, color_space=True, threads=threads)
    f, _, h, w = noisy.shape
    return w * h * f / 1e6


def _job(args):
    impl, noisy, sigma = args
    return _run(impl, noisy, sigma, 1)


def _warm(impl):
    _lib(impl)
    return 0


def time_openmp(impl, samples, threads):
    t0 = time.perf_counter()
    mpf = sum(_run(impl, a, s, threads) for a, s in samples)
    return mpf / (time.perf_counter() - t0)


def time_processes(impl, samples, threads):
    import bench
    jobs, reps = bench.proc_jobs(samples, threads)
    with mp.get_context("spawn").Pool(threads) as pool:
        pool.map(_warm, [impl] * threads, chunksize=1)
        t0 = time.perf_counter()
        mpf = sum(pool.map(_job, [(impl, a, s) for a, s in jobs], chunksize=1))
        dt = time.perf_counter() - t0
    return mpf / dt, reps


def samples_of(workload):
    import bench
    from vbm3d_gb300.synth import batch_specs, make_clip
    if workload == "batch64":
        specs = batch_specs()
        clips = {i: dict(noisy=make_clip(*specs[i][:5], 4000 + i)[1], sigma=specs[i][4]) for i in range(0, 64, 8)}
        full = [clips.get(i, dict(noisy=None, sigma=None)) for i in range(64)]
        return bench.cpu_sample("batch64", clips=full)
    _, noisy = bench.make_1080()
    return bench.cpu_sample("1080p30", noisy=noisy)


def main():
    import bench
    from oracle.pyoracle import RefLib
    if not RefLib.available(exact=False):
        sys.exit("oracle/_ref/libvbm3d_ref_fast.so is not built (oracle/build_ref.sh needs the reference sources)")
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "profiles", "cpu_reference_vs_port.json")
    th = bench.cpu_threads()
    res = {"host": {"machine": platform.machine(), "processor": platform.processor() or platform.machine(),
                    "threads": th},
           "reference_build": "oracle/_ref/libvbm3d_ref_fast.so: src/vbm3d.cpp, src/lib_transforms.cpp, "
                              "src/Utilities/Utilities.cpp with -O3 -ffast-math -fomit-frame-pointer -fopenmp "
                              "(CMakeLists.txt:15), FFTW replaced by oracle/fftw_shim",
           "port_fast": "oracle/_build/liboracle_fast.so (oracle/vbm3d_oracle.c with the reference's flags, "
                        "-O3 -ffast-math -fomit-frame-pointer -fopenmp): the build bench.py times",
           "port": "oracle/_build/liboracle.so (oracle/vbm3d_oracle.c, -O2 -ffp-contract=off -fopenmp): the "
                   "parity build",
           "workloads": {}}
    for workload in ("batch64", "1080p30"):
        samples, desc = samples_of(workload)
        for impl in ("port_fast", "reference", "port"):  # page in the libraries
            _run(impl, samples[0][0][:2], samples[0][1], th)
        r = {"sample": desc}
        for impl in ("port_fast", "reference", "port"):
            v_omp = time_openmp(impl, samples, th)
            v_proc, reps = time_processes(impl, samples, th)
            r[impl] = {"openmp": round(v_omp, 4), "processes": round(v_proc, 4), "best": round(max(v_omp, v_proc), 4)}
            print(workload, impl, r[impl], flush=True)
        for impl in ("port_fast", "port"):
            r[impl + "_over_reference"] = {m: round(r[impl][m] / r["reference"][m], 3)
                                           for m in ("openmp", "processes", "best")}
        res["workloads"][workload] = r
    with open(out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps(res["workloads"], indent=1))


if __name__ == "__main__":
    main()
