"""ctypes wrappers of the CPU oracles — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker; the product path never imports it.

* `Oracle`   : the C restatement in oracle/vbm3d_oracle.c (oracle/_build).
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
