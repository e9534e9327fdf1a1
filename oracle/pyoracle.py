"""ctypes wrappers of the CPU oracles — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker; the product path never imports it.

* `Oracle`   : the C restatement in oracle/vbm3d_oracle.c (oracle/_build);
               Oracle(ORACLE_FAST_SO) is the same code built with the
               reference's -O3 -ffast-math flags, for CPU timing only.
* `RefLib`   : the reference's own sources compiled by oracle/build_ref.sh
               into oracle/_ref (present only where the reference sources
               were available at build time).
"""
import ctypes as C
import os
import subprocess

import numpy as np

from vbm3d_gb300._abi import Dims, Params, dims_of

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
ORACLE_FAST_SO = os.path.join(HERE, "_build", "liboracle_fast.so")
REF_EXACT_SO = os.path.join(HERE, "_ref", "libvbm3d_ref_exact.so")
REF_FAST_SO = os.path.join(HERE, "_ref", "libvbm3d_ref_fast.so")

_fp = C.POINTER(C.c_float)
_up = C.POINTER(C.c_uint)


def _f(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_fp)


def _u(a):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(_up)


def build_oracle():
    subprocess.check_call(["sh", os.path.join(HERE, "build_oracle.sh")])


class Oracle:
    """The C restatement of the reference's hot path."""

    def __init__(self, path=ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        self.lib = C.CDLL(path)
        L = self.lib
        L.oracle_default_params.argtypes = [C.c_int, C.c_float, C.POINTER(Params)]
        L.oracle_sigma_table.argtypes = [C.c_float, C.c_uint, C.c_int, _fp]
        L.oracle_grid.argtypes = [C.POINTER(Params), Dims, _up, _up, _up, _up]
        L.oracle_kaiser.argtypes = [C.c_uint, _fp]
        L.oracle_similar_batch.argtypes = [C.POINTER(Params), _fp, _fp, _fp, Dims, _up,
                                           C.c_size_t, _fp, _up, _up, _up]
        L.oracle_step.argtypes = [C.c_int, C.POINTER(Params), _fp, _fp, _fp, _fp, Dims,
                                  C.c_float, C.c_int, _fp, _fp, C.c_int]
        L.oracle_run.argtypes = [C.c_float, _fp, _fp, _fp, _fp, _fp, C.POINTER(Params),
                                 C.POINTER(Params), C.c_int, Dims, C.c_int]
        L.oracle_color_transform.argtypes = [_fp, Dims, C.c_int]
        L.oracle_linear_apply.argtypes = [C.c_int, C.POINTER(Params), _fp, _fp, _fp, _fp, Dims, C.c_float, C.c_int,
                                          _fp, C.POINTER(C.c_double), C.c_int]
        for name in ("oracle_dct2d_forward", "oracle_dct2d_inverse"):
            getattr(L, name).argtypes = [_fp, _fp, C.c_uint]
        for name in ("oracle_bior2d_forward", "oracle_bior2d_inverse"):
            getattr(L, name).argtypes = [_fp, _fp]
        for name in ("oracle_haar_forward", "oracle_haar_inverse"):
            getattr(L, name).argtypes = [_fp, C.c_uint]

    def default_params(self, step, sigma):
        p = Params()
        assert self.lib.oracle_default_params(step, sigma, C.byref(p)) == 0
        return p

    def sigma_table(self, sigma, chnls, color_space):
        out = np.zeros(3, np.float32)
        rc = self.lib.oracle_sigma_table(sigma, chnls, int(color_space), _f(out))
        return None if rc else out[:chnls]

    def grid(self, p, dims):
        rows = np.zeros(dims.height + 2, np.uint32)
        cols = np.zeros(dims.width + 2, np.uint32)
        nr, nc = C.c_uint(), C.c_uint()
        assert self.lib.oracle_grid(C.byref(p), dims, C.byref(nr), C.byref(nc), _u(rows), _u(cols)) == 0
        return rows[:nr.value].copy(), cols[:nc.value].copy()

    def ref_indices(self, p, dims):
        """Patch indices of every reference patch, in the reference's loop order."""
        rows, cols = self.grid(p, dims)
        wh, whc = dims.width * dims.height, dims.width * dims.height * dims.channels
        t = np.arange(dims.frames - p.kt + 1, dtype=np.int64)
        idx = t[:, None, None] * whc + rows[None, :, None].astype(np.int64) * dims.width + cols[None, None, :]
        return idx.reshape(-1).astype(np.uint32)

    def kaiser(self, k):
        out = np.zeros(k * k, np.float32)
        self.lib.oracle_kaiser(k, _f(out))
        return out.reshape(k, k)

    def similar(self, p, video, fflow=None, bflow=None, pidx=None):
        video = np.ascontiguousarray(video, np.float32)
        d = dims_of(video)
        if pidx is None:
            pidx = self.ref_indices(p, d)
        pidx = np.ascontiguousarray(pidx, np.uint32)
        n = len(pidx)
        dist = np.zeros((n, p.N), np.float32)
        idx = np.zeros((n, p.N), np.uint32)
        nsimp = np.zeros(n, np.uint32)
        nsx = np.zeros(n, np.uint32)
        rc = self.lib.oracle_similar_batch(C.byref(p), _f(video), _f(fflow), _f(bflow), d, _u(pidx), n,
                                           _f(dist), _u(idx), _u(nsimp), _u(nsx))
        assert rc == 0, rc
        return dict(dist=dist, idx=idx, nsimp=nsimp, nsx=nsx)

    def step(self, step, p, sigma, noisy, basic=None, fflow=None, bflow=None, color_space=False, threads=1):
        noisy = np.ascontiguousarray(noisy, np.float32)
        d = dims_of(noisy)
        num = np.zeros_like(noisy)
        den = np.zeros_like(noisy)
        rc = self.lib.oracle_step(step, C.byref(p), _f(noisy), _f(basic), _f(fflow), _f(bflow), d,
                                  sigma, int(color_space), _f(num), _f(den), threads)
        assert rc == 0, rc
        return num, den

    def run(self, sigma, noisy, p1, p2, fflow=None, bflow=None, color_space=False, threads=1):
        nz = np.array(noisy, np.float32, copy=True, order="C")
        basic = np.zeros_like(nz)
        den = np.zeros_like(nz)
        rc = self.lib.oracle_run(sigma, _f(nz), _f(fflow), _f(bflow), _f(basic), _f(den),
                                 C.byref(p1), C.byref(p2), int(color_space), dims_of(nz), threads)
        assert rc == 0, rc
        return basic, den

    def linear(self, step, p, sigma, noisy, x, basic=None, fflow=None, bflow=None, color_space=False, threads=4):
        """FP64 frozen linearised step applied to x."""
        noisy = np.ascontiguousarray(noisy, np.float32)
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros(noisy.shape, np.float64)
        rc = self.lib.oracle_linear_apply(step, C.byref(p), _f(noisy), _f(basic), _f(fflow), _f(bflow), dims_of(noisy),
                                          sigma, int(color_space), _f(x), out.ctypes.data_as(C.POINTER(C.c_double)),
                                          threads)
        assert rc == 0, rc
        return out

    def color_transform(self, video, forward):
        v = np.array(video, np.float32, copy=True, order="C")
        self.lib.oracle_color_transform(_f(v), dims_of(v), int(forward))
        return v

    def block(self, name, block, k=None):
        inp = np.ascontiguousarray(block, np.float32)
        out = np.zeros_like(inp)
        fn = getattr(self.lib, "oracle_" + name)
        if k is None:
            fn(_f(inp), _f(out))
        else:
            fn(_f(inp), _f(out), k)
        return out

    def haar(self, vec, inverse=False):
        v = np.array(vec, np.float32, copy=True)
        fn = self.lib.oracle_haar_inverse if inverse else self.lib.oracle_haar_forward
        fn(_f(v), len(v))
        return v


class RefLib:
    """The reference's own code compiled from its sources (oracle/_ref)."""

    def __init__(self, exact=True):
        path = REF_EXACT_SO if exact else REF_FAST_SO
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_step.argtypes = [C.c_int, C.POINTER(Params), _fp, _fp, _fp, _fp, Dims, C.c_float,
                               C.c_int, _fp, _fp]
        L.ref_similar_batch.argtypes = [C.POINTER(Params), _fp, _fp, _fp, Dims, _up, C.c_size_t,
                                        _fp, _up, _up, _up]
        L.ref_run.argtypes = [C.c_float, _fp, _fp, _fp, _fp, _fp, C.POINTER(Params),
                              C.POINTER(Params), C.c_int, Dims, C.c_int]

    @staticmethod
    def available(exact=True):
        return os.path.exists(REF_EXACT_SO if exact else REF_FAST_SO)

    def similar(self, p, video, pidx, fflow=None, bflow=None):
        video = np.ascontiguousarray(video, np.float32)
        pidx = np.ascontiguousarray(pidx, np.uint32)
        n = len(pidx)
        dist = np.zeros((n, p.N), np.float32)
        idx = np.zeros((n, p.N), np.uint32)
        nsimp = np.zeros(n, np.uint32)
        nsx = np.zeros(n, np.uint32)
        self.lib.ref_similar_batch(C.byref(p), _f(video), _f(fflow), _f(bflow), dims_of(video), _u(pidx), n,
                                   _f(dist), _u(idx), _u(nsimp), _u(nsx))
        return dict(dist=dist, idx=idx, nsimp=nsimp, nsx=nsx)

    def step(self, step, p, sigma, noisy, basic=None, fflow=None, bflow=None, color_space=False):
        noisy = np.ascontiguousarray(noisy, np.float32)
        num = np.zeros_like(noisy)
        den = np.zeros_like(noisy)
        rc = self.lib.ref_step(step, C.byref(p), _f(noisy), _f(basic), _f(fflow), _f(bflow), dims_of(noisy),
                               sigma, int(color_space), _f(num), _f(den))
        assert rc == 0, rc
        return num, den

    def run(self, sigma, noisy, p1, p2, fflow=None, bflow=None, color_space=False, threads=1):
        nz = np.array(noisy, np.float32, copy=True, order="C")
        basic = np.zeros_like(nz)
        den = np.zeros_like(nz)
        rc = self.lib.ref_run(sigma, _f(nz), _f(fflow), _f(bflow), _f(basic), _f(den), C.byref(p1), C.byref(p2),
                              int(color_space), dims_of(nz), threads)
        assert rc == 0, rc
        return basic, den


TVL1_ORACLE_SO = os.path.join(HERE, "_build", "libtvl1_oracle.so")
TVL1_REF_SO = os.path.join(HERE, "_ref", "libtvl1_ref.so")


class TvParams(C.Structure):
    """tv_params of oracle/tvl1_oracle.h (the reference's TV-L1 options)."""
    _fields_ = [("tau", C.c_float), ("lambda_", C.c_float), ("theta", C.c_float), ("nscales", C.c_int),
                ("fscale", C.c_int), ("zfactor", C.c_float), ("nwarps", C.c_int), ("epsilon", C.c_float)]


class TvlOracle:
    """The C restatement of the reference's TV-L1 optical flow
    (oracle/tvl1_oracle.c)."""

    def __init__(self, path=TVL1_ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        self.lib = C.CDLL(path)
        L = self.lib
        L.tv_default_params.argtypes = [C.POINTER(TvParams)]
        L.tv_flow.argtypes = [_fp, _fp, C.c_int, C.c_int, C.POINTER(TvParams), _fp, C.POINTER(C.c_int)]
        L.tv_scales.argtypes = [C.c_int, C.c_int, C.POINTER(TvParams), C.POINTER(C.c_int)]

    def default_params(self, **kw):
        p = TvParams()
        self.lib.tv_default_params(C.byref(p))
        for k, v in kw.items():
            setattr(p, "lambda_" if k == "lambda" else k, v)
        return p

    def scales(self, nx, ny, p):
        fs = C.c_int(0)
        return self.lib.tv_scales(nx, ny, C.byref(p), C.byref(fs)), fs.value

    def flow(self, I0, I1, p=None, iters=False):
        """Flow [2, H, W] from I0 to I1 ([H, W] float32); with iters, also the
        iteration counts [nscales, nwarps] (-1 below fscale)."""
        p = p or self.default_params()
        I0 = np.ascontiguousarray(I0, np.float32)
        I1 = np.ascontiguousarray(I1, np.float32)
        ny, nx = I0.shape
        out = np.zeros((2, ny, nx), np.float32)
        ns, _ = self.scales(nx, ny, p)
        it = np.zeros((max(ns, 1), p.nwarps), np.int32)
        rc = self.lib.tv_flow(_f(I0), _f(I1), nx, ny, C.byref(p), _f(out), it.ctypes.data_as(C.POINTER(C.c_int)))
        if rc:
            raise ValueError("tv_flow failed")
        return (out, it) if iters else out


class TvlRef:
    """The reference's own TV-L1 library compiled from its sources
    (oracle/_ref/libtvl1_ref.so; present only where the sources were)."""

    def __init__(self):
        if not os.path.exists(TVL1_REF_SO):
            raise FileNotFoundError(TVL1_REF_SO)
        self.lib = C.CDLL(TVL1_REF_SO)
        self.lib.ref_tvl1_flow.argtypes = [_fp, _fp, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int,
                                           C.c_int, C.c_float, C.c_int, C.c_float, _fp]

    @staticmethod
    def available():
        return os.path.exists(TVL1_REF_SO)

    def flow(self, I0, I1, p):
        I0 = np.ascontiguousarray(I0, np.float32).copy()  # the reference's signature is not const
        I1 = np.ascontiguousarray(I1, np.float32).copy()
        ny, nx = I0.shape
        out = np.zeros((2, ny, nx), np.float32)
        self.lib.ref_tvl1_flow(_f(I0), _f(I1), nx, ny, p.tau, p.lambda_, p.theta, p.nscales, p.fscale, p.zfactor,
                               p.nwarps, p.epsilon, _f(out))
        return out
