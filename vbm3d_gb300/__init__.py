"""GB300-native VBM3D video denoising (sm_103a CUDA kernels behind a C ABI).

The library is libvbm3d_gb300.so (built in-tree by vbm3d_gb300.build); its C
ABI is include/vbm3d_gb300.h.  This module is a thin ctypes binding over that
ABI for Python callers, with torch tensors as device buffers.  There is no
CPU fallback: every call runs the CUDA kernels, and importing a missing or
stale library raises.

Entry points mirror the reference's hot path (tehret/vbm3d):
  default_params(step, sigma)        initializeParameters_1/_2 (src/main.cpp:35-207)
  step1(...), step2(...)             vbm3d_1st_step / vbm3d_2nd_step (src/vbm3d.cpp:447-928)
  normalize(...)                     run_vbm3d's num/den division (src/vbm3d.cpp:168-202)
  color_transform(...)               VideoUtils::transformColorSpace
  similar_patches(...)               computeSimilarPatches over the reference grid
  tvl1_flow(...), tvl1_video(...)    tvl1flow's TV-L1 (Dual_TVL1_optic_flow_multiscale), frame pairs / a clip
  run(...) / run_host(...)           run_vbm3d (src/vbm3d.cpp:87-376), device / host buffers
Beside them, with no reference counterpart:
  set_deterministic(on), Deterministic()  reference-order, bit-reproducible aggregation
  Batch(...)                         many uneven clips in one CUDA graph (vbm3d_batch_*)
  LinearStep(...)                    frozen linearisation and adjoint of a step (vbm3d_linear_*)
"""
import ctypes as C
import os

from ._abi import (BIOR, DCT, HAAR, HADAMARD, STATUS, BatchConfig, BatchLaunch, Clip, Dims,  # noqa: F401
                   Params, TvParams, dims_of)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libvbm3d_gb300.so")

_fp = C.POINTER(C.c_float)
_up = C.POINTER(C.c_uint)
_lib = None


class VBM3DError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("%s: %s" % (STATUS.get(status, status), message))
        self.status = status


def load(path=LIB_PATH):
    """Loads the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libvbm3d_gb300.so is not built: run `python -m vbm3d_gb300.build` "
                          "(or __graft_entry__.build())")
    L = C.CDLL(path)
    P = C.POINTER(Params)
    vp = C.c_void_p
    L.vbm3d_default_params.argtypes = [C.c_int, C.c_float, P]
    L.vbm3d_sigma_table.argtypes = [C.c_float, C.c_uint, C.c_int, _fp]
    L.vbm3d_ref_count.argtypes = [P, Dims, C.POINTER(C.c_size_t)]
    L.vbm3d_gpu_step1.argtypes = [P, vp, vp, vp, Dims, C.c_float, C.c_int, vp, vp, vp]
    L.vbm3d_gpu_step2.argtypes = [P, vp, vp, vp, vp, Dims, C.c_float, C.c_int, vp, vp, vp]
    L.vbm3d_gpu_normalize.argtypes = [vp, vp, vp, vp, C.c_size_t, vp]
    L.vbm3d_gpu_color_transform.argtypes = [vp, Dims, C.c_int, vp]
    L.vbm3d_gpu_run.argtypes = [C.c_float, vp, vp, vp, vp, vp, P, P, C.c_int, Dims, vp]
    L.vbm3d_run_host.argtypes = [C.c_float, vp, vp, vp, vp, vp, P, P, C.c_int, Dims]
    L.vbm3d_gpu_similar_patches.argtypes = [P, vp, vp, vp, Dims, vp, vp, vp, vp, C.POINTER(C.c_size_t), vp]
    L.vbm3d_gpu_bm_distance_count.argtypes = [P, vp, vp, vp, Dims, C.POINTER(C.c_ulonglong), vp]
    L.vbm3d_linear_create.argtypes = [C.c_int, P, vp, vp, vp, vp, Dims, C.c_float, C.c_int, C.POINTER(vp), vp]
    L.vbm3d_linear_apply.argtypes = [vp, vp, vp, C.c_int, vp]
    L.vbm3d_linear_den.argtypes = [vp, C.POINTER(vp)]
    L.vbm3d_linear_destroy.argtypes = [vp]
    L.vbm3d_linear_destroy.restype = None
    L.vbm3d_batch_create.argtypes = [C.POINTER(Clip), C.c_int, C.c_int, C.POINTER(BatchConfig), C.POINTER(vp), vp]
    L.vbm3d_batch_run.argtypes = [vp, vp]
    L.vbm3d_batch_get_config.argtypes = [vp, C.POINTER(BatchConfig)]
    L.vbm3d_batch_profile.argtypes = [vp, vp, C.POINTER(BatchLaunch), C.c_int, C.POINTER(C.c_int)]
    L.vbm3d_batch_destroy.argtypes = [vp]
    L.vbm3d_batch_destroy.restype = None
    T = C.POINTER(TvParams)
    L.vbm3d_tvl1_default_params.argtypes = [T]
    L.vbm3d_tvl1_scales.argtypes = [C.c_uint, C.c_uint, T, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.vbm3d_gpu_tvl1_pairs.argtypes = [vp, vp, C.c_uint, C.c_uint, C.c_uint, T, vp, C.POINTER(C.c_int), vp]
    L.vbm3d_gpu_tvl1_video.argtypes = [vp, C.c_uint, C.c_uint, C.c_uint, T, vp, vp, vp]
    L.vbm3d_gpu_ms_decompose.argtypes = [vp, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.POINTER(vp), vp]
    L.vbm3d_gpu_ms_recompose.argtypes = [C.POINTER(vp), C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_float, vp, vp]
    L.vbm3d_gpu_ms_merge_coarse.argtypes = [vp, vp, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_float,
                                            vp, vp]
    L.vbm3d_set_deterministic.argtypes = [C.c_int]
    L.vbm3d_get_deterministic.argtypes = []
    L.vbm3d_status_string.restype = C.c_char_p
    L.vbm3d_last_error.restype = C.c_char_p
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise VBM3DError(rc, load().vbm3d_last_error().decode())


def set_deterministic(on):
    """Aggregation mode of the plain path (vbm3d_set_deterministic): True
    sums every pixel's terms in the reference's order (bit-reproducible
    runs); False (the default) adds with float atomics."""
    _check(load().vbm3d_set_deterministic(int(bool(on))))


def deterministic():
    return bool(load().vbm3d_get_deterministic())


class Deterministic:
    """Context manager: the plain path in the deterministic mode inside."""

    def __init__(self, on=True):
        self.on = on

    def __enter__(self):
        self.prev = deterministic()
        set_deterministic(self.on)
        return self

    def __exit__(self, *exc):
        set_deterministic(self.prev)
        return False


def default_params(step, sigma):
    p = Params()
    _check(load().vbm3d_default_params(step, sigma, C.byref(p)))
    return p


def sigma_table(sigma, channels, color_space):
    out = (C.c_float * 3)()
    _check(load().vbm3d_sigma_table(sigma, channels, int(color_space), out))
    return list(out)[:channels]


def ref_count(params, dims):
    n = C.c_size_t()
    _check(load().vbm3d_ref_count(C.byref(params), dims, C.byref(n)))
    return n.value


# ---------------------------------------------------------------- torch ---

def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _stream(stream):
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _video(t, name):
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()
            and t.dim() == 4):
        raise TypeError("%s must be a contiguous float32 CUDA tensor [F, C, H, W]" % name)
    return t


def _dims(t):
    f, c, h, w = t.shape
    return Dims(w, h, f, c)


def step1(noisy, params, sigma, fflow=None, bflow=None, color_space=False, out=None, stream=None):
    """vbm3d_1st_step on the GPU: returns (numerator, denominator)."""
    import torch
    _video(noisy, "noisy")
    num, den = out if out is not None else (torch.empty_like(noisy), torch.empty_like(noisy))
    _check(load().vbm3d_gpu_step1(C.byref(params), _ptr(noisy), _ptr(fflow), _ptr(bflow), _dims(noisy), sigma,
                                  int(color_space), _ptr(num), _ptr(den), _stream(stream)))
    return num, den


def step2(noisy, basic, params, sigma, fflow=None, bflow=None, color_space=False, out=None, stream=None):
    """vbm3d_2nd_step on the GPU: returns (numerator, denominator)."""
    import torch
    _video(noisy, "noisy")
    _video(basic, "basic")
    num, den = out if out is not None else (torch.empty_like(noisy), torch.empty_like(noisy))
    _check(load().vbm3d_gpu_step2(C.byref(params), _ptr(noisy), _ptr(basic), _ptr(fflow), _ptr(bflow),
                                  _dims(noisy), sigma, int(color_space), _ptr(num), _ptr(den), _stream(stream)))
    return num, den


def normalize(num, den, fallback, out=None, stream=None):
    import torch
    out = torch.empty_like(num) if out is None else out
    _check(load().vbm3d_gpu_normalize(_ptr(num), _ptr(den), _ptr(fallback), _ptr(out), num.numel(),
                                      _stream(stream)))
    return out


def color_transform(video, forward, stream=None):
    """In place."""
    _video(video, "video")
    _check(load().vbm3d_gpu_color_transform(_ptr(video), _dims(video), int(forward), _stream(stream)))
    return video


def similar_patches(video, params, fflow=None, bflow=None, stream=None):
    """Block matching for every reference patch of the step's grid.
    Returns dict(idx [R, N] int32 view of u32, dist [R, N], nsimp [R], nsx [R])."""
    import torch
    _video(video, "video")
    d = _dims(video)
    n = ref_count(params, d)
    dev = video.device
    idx = torch.empty((n, params.N), dtype=torch.int32, device=dev)
    dist = torch.empty((n, params.N), dtype=torch.float32, device=dev)
    nsimp = torch.empty(n, dtype=torch.int32, device=dev)
    nsx = torch.empty(n, dtype=torch.int32, device=dev)
    _check(load().vbm3d_gpu_similar_patches(C.byref(params), _ptr(video), _ptr(fflow), _ptr(bflow), d, _ptr(idx),
                                            _ptr(dist), _ptr(nsimp), _ptr(nsx), None, _stream(stream)))
    return dict(idx=idx, dist=dist, nsimp=nsimp, nsx=nsx)


def bm_distance_count(video, params, fflow=None, bflow=None, stream=None):
    """Number of patch distances the block matching of this video evaluates."""
    _video(video, "video")
    n = C.c_ulonglong()
    _check(load().vbm3d_gpu_bm_distance_count(C.byref(params), _ptr(video), _ptr(fflow), _ptr(bflow), _dims(video),
                                              C.byref(n), _stream(stream)))
    return n.value


class LinearStep:
    """Frozen linearisation L of one step (vbm3d_linear_*): apply(x) = L x,
    apply(x, adjoint=True) = L^T x.  Keeps references to its inputs."""

    def __init__(self, step, noisy, sigma, params, basic=None, fflow=None, bflow=None, color_space=False,
                 stream=None):
        _video(noisy, "noisy")
        self._keep = (noisy, basic, fflow, bflow)
        self.shape = noisy.shape
        self._h = C.c_void_p()
        _check(load().vbm3d_linear_create(step, C.byref(params), _ptr(noisy), _ptr(basic), _ptr(fflow), _ptr(bflow),
                                          _dims(noisy), sigma, int(color_space), C.byref(self._h), _stream(stream)))

    def apply(self, x, adjoint=False, out=None, stream=None):
        import torch
        _video(x, "x")
        out = torch.empty_like(x) if out is None else out
        _check(load().vbm3d_linear_apply(self._h, _ptr(x), _ptr(out), int(adjoint), _stream(stream)))
        return out

    def den(self):
        import torch
        p = C.c_void_p()
        _check(load().vbm3d_linear_den(self._h, C.byref(p)))
        return p.value

    def close(self):
        if self._h:
            load().vbm3d_linear_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tvl1_params(**kw):
    """TV-L1 options: the reference's flow-script values, with overrides
    (tau, lambda_, theta, nscales, fscale, zfactor, nwarps, epsilon)."""
    p = TvParams()
    _check(load().vbm3d_tvl1_default_params(C.byref(p)))
    for k, v in kw.items():
        setattr(p, "lambda_" if k == "lambda" else k, v)
    return p


def tvl1_flow(I0, I1, params=None, iterations=False, stream=None):
    """TV-L1 flows from I0 to I1: CUDA float32 [P, H, W] (or [H, W]) frames;
    returns [P, 2, H, W] (or [2, H, W]); with iterations, also the host
    counts [P, nscales, nwarps]."""
    import numpy as np
    import torch
    params = params or tvl1_params()
    single = I0.dim() == 2
    if single:
        I0, I1 = I0[None], I1[None]
    if not (I0.is_cuda and I0.dtype == torch.float32 and I0.is_contiguous() and I1.shape == I0.shape
            and I1.is_contiguous() and I1.dtype == torch.float32):
        raise TypeError("I0, I1 must be contiguous float32 CUDA tensors of one shape [P, H, W]")
    npairs, h, w = I0.shape
    flow = torch.empty((npairs, 2, h, w), dtype=torch.float32, device=I0.device)
    ns, fs = C.c_int(0), C.c_int(0)
    _check(load().vbm3d_tvl1_scales(w, h, C.byref(params), C.byref(ns), C.byref(fs)))
    it = np.zeros((npairs, max(ns.value, 1), params.nwarps), np.int32) if iterations else None
    _check(load().vbm3d_gpu_tvl1_pairs(_ptr(I0), _ptr(I1), npairs, w, h, C.byref(params), _ptr(flow),
                                       None if it is None else it.ctypes.data_as(C.POINTER(C.c_int)),
                                       _stream(stream)))
    out = flow[0] if single else flow
    return (out, it) if iterations else out


def tvl1_video(video, params=None, stream=None):
    """Forward and backward TV-L1 flows of a one-channel clip (CUDA float32
    [F, H, W]) in the layout the steps read: (fflow, bflow), each
    [F, 2, H, W]."""
    import torch
    params = params or tvl1_params()
    if not (video.is_cuda and video.dtype == torch.float32 and video.is_contiguous() and video.dim() == 3):
        raise TypeError("video must be a contiguous float32 CUDA tensor [F, H, W]")
    f, h, w = video.shape
    ff = torch.empty((f, 2, h, w), dtype=torch.float32, device=video.device)
    bf = torch.empty_like(ff)
    _check(load().vbm3d_gpu_tvl1_video(_ptr(video), w, h, f, C.byref(params), _ptr(ff), _ptr(bf), _stream(stream)))
    return ff, bf


def _planes(t, name):
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()
            and t.dim() >= 2):
        raise TypeError("%s must be a contiguous float32 CUDA tensor [..., H, W]" % name)
    h, w = t.shape[-2:]
    return t.numel() // max(h * w, 1), h, w


def ms_level_shapes(shape, levels):
    """Shapes of the DCT pyramid levels of an image stack [..., H, W]:
    H and W halved by integer division per level."""
    lead, (h, w) = tuple(shape[:-2]), tuple(shape[-2:])
    out = []
    for _ in range(levels):
        out.append(lead + (h, w))
        h, w = h // 2, w // 2
    return out


def ms_decompose(x, levels, stream=None):
    """The multiscaler's DCT pyramid (`decompose ... -t 0`) of a CUDA float32
    image stack [..., H, W] (every leading index one plane): a list of
    `levels` stacks, level i halved i times."""
    import torch
    p, h, w = _planes(x, "x")
    outs = [torch.empty(sh, dtype=torch.float32, device=x.device) for sh in ms_level_shapes(x.shape, levels)]
    ptrs = (C.c_void_p * levels)(*[o.data_ptr() for o in outs])
    _check(load().vbm3d_gpu_ms_decompose(_ptr(x), w, h, p, levels, ptrs, _stream(stream)))
    return outs


def ms_recompose(levels_in, factor=0.8, stream=None):
    """`recompose ... -t 0 -c factor`: one stack [..., H, W] from the levels
    of ms_decompose (possibly denoised)."""
    import torch
    p, h, w = _planes(levels_in[0], "levels_in[0]")
    shapes = ms_level_shapes(levels_in[0].shape, len(levels_in))
    for i, (lv, sh) in enumerate(zip(levels_in, shapes)):
        _planes(lv, "levels_in[%d]" % i)
        if tuple(lv.shape) != sh:
            raise ValueError("level %d has shape %s, expected %s" % (i, tuple(lv.shape), sh))
    out = torch.empty_like(levels_in[0])
    ptrs = (C.c_void_p * len(levels_in))(*[lv.data_ptr() for lv in levels_in])
    _check(load().vbm3d_gpu_ms_recompose(ptrs, w, h, p, len(levels_in), C.c_float(factor), _ptr(out),
                                         _stream(stream)))
    return out


def ms_merge_coarse(fine, coarse, factor=0.8, stream=None):
    """`merge_coarse fine coarse out -c factor` on CUDA float32 stacks
    [..., H, W] and [..., h, w] with the same leading shape."""
    import torch
    p, h, w = _planes(fine, "fine")
    pc, ch, cw = _planes(coarse, "coarse")
    if pc != p:
        raise ValueError("fine and coarse hold different numbers of planes")
    out = torch.empty_like(fine)
    _check(load().vbm3d_gpu_ms_merge_coarse(_ptr(fine), _ptr(coarse), w, h, cw, ch, p, C.c_float(factor),
                                            _ptr(out), _stream(stream)))
    return out


def ms_level_sigma(sigma, level):
    """The noise level the multiscale script denoises a level with:
    sigma / 2^level truncated to two decimals (`bc` with scale=2,
    src/utils/VBM3Ddenoising_multiscale.sh:50)."""
    from decimal import Decimal, ROUND_DOWN
    q = Decimal(repr(float(sigma))) / (Decimal(2) ** level)
    return float(q.quantize(Decimal("0.01"), rounding=ROUND_DOWN))


def multiscale_denoise(noisy, sigma, levels=3, factor=0.7, color_space=True, stream=None):
    """The multiscale denoising of src/utils/VBM3Ddenoising_multiscale.sh on
    the GPU: every frame of `noisy` (CUDA float32 [F, C, H, W]) decomposed
    into `levels` DCT levels, each level's clip denoised by VBM3D with the
    reference's default parameters at ms_level_sigma(sigma, level), and the
    denoised levels recomposed with `factor` (the script's recomposition
    ratio, 0.7).  Returns (denoised, denoised levels)."""
    _video(noisy, "noisy")
    lv = ms_decompose(noisy, levels, stream=stream)
    den = []
    for i, x in enumerate(lv):
        _, d = run(x.contiguous(), ms_level_sigma(sigma, i), color_space=color_space, stream=stream)
        den.append(d)
    return ms_recompose(den, factor, stream=stream), den


class Batch:
    """Many clips of uneven size, channel count and sigma denoised by one CUDA
    graph launch (vbm3d_batch_*).  `clips` is a list of dicts with keys
    noisy (CUDA float32 [F, C, H, W]), sigma, and optionally fflow, bflow,
    p1, p2.  Outputs are allocated here: self.basic[i] (None when basic is
    False), self.denoised[i].  `config` (a BatchConfig or a dict of its
    fields) fixes phases instead of autotuning them.  The inputs are kept
    referenced; refill them in place between runs."""

    def __init__(self, clips, color_space=False, config=None, basic=True, stream=None):
        import torch
        self._keep = []
        self.basic, self.denoised = [], []
        arr = (Clip * len(clips))()
        for i, c in enumerate(clips):
            noisy = _video(c["noisy"], "noisy")
            sigma = float(c["sigma"])
            p1 = c.get("p1") or default_params(1, sigma)
            p2 = c.get("p2") or default_params(2, sigma)
            den = torch.empty_like(noisy)
            bas = torch.empty_like(noisy) if basic else None
            self.basic.append(bas)
            self.denoised.append(den)
            self._keep += [noisy, c.get("fflow"), c.get("bflow"), p1, p2]
            arr[i] = Clip(_dims(noisy), sigma, C.pointer(p1), C.pointer(p2), _ptr(noisy), _ptr(c.get("fflow")),
                          _ptr(c.get("bflow")), _ptr(bas), _ptr(den))
        self._clips = arr
        cfg = None
        if config is not None:
            cfg = config if isinstance(config, BatchConfig) else BatchConfig(**config)
        self._h = C.c_void_p()
        _check(load().vbm3d_batch_create(arr, len(clips), int(color_space), None if cfg is None else C.byref(cfg),
                                         C.byref(self._h), _stream(stream)))

    def run(self, stream=None):
        _check(load().vbm3d_batch_run(self._h, _stream(stream)))
        return self.basic, self.denoised

    def profile(self, stream=None):
        """One run with a CUDA event around each work launch: a list of dicts
        (phase, k, channels, clips, items, refs, tile, warps, grid, ms)."""
        n = C.c_int(0)
        buf = (BatchLaunch * 64)()
        _check(load().vbm3d_batch_profile(self._h, _stream(stream), buf, 64, C.byref(n)))
        return [buf[i].as_dict() for i in range(n.value)]

    def config(self):
        c = BatchConfig()
        _check(load().vbm3d_batch_get_config(self._h, C.byref(c)))
        return c.as_dict()

    def close(self):
        if self._h:
            load().vbm3d_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run(noisy, sigma, p1=None, p2=None, fflow=None, bflow=None, color_space=False, stream=None):
    """run_vbm3d on device buffers.  `noisy` is transformed in place and back
    (as the reference does).  Returns (basic, denoised)."""
    import torch
    _video(noisy, "noisy")
    p1 = default_params(1, sigma) if p1 is None else p1
    p2 = default_params(2, sigma) if p2 is None else p2
    basic, den = torch.empty_like(noisy), torch.empty_like(noisy)
    _check(load().vbm3d_gpu_run(sigma, _ptr(noisy), _ptr(fflow), _ptr(bflow), _ptr(basic), _ptr(den),
                                C.byref(p1), C.byref(p2), int(color_space), _dims(noisy), _stream(stream)))
    return basic, den


def run_host(noisy, sigma, p1=None, p2=None, fflow=None, bflow=None, color_space=False, basic=None, out=None):
    """run_vbm3d on host (numpy) arrays: copies in, denoises, copies out.
    Flows [frames, 2, H, W] with F or F - 1 frames (the last is never read)."""
    import numpy as np
    noisy = np.ascontiguousarray(noisy, dtype=np.float32)
    F, _, H, W = noisy.shape
    for name, fl in (("fflow", fflow), ("bflow", bflow)):
        if fl is not None and (fl.dtype != np.float32 or not fl.flags.c_contiguous or fl.shape[1:] != (2, H, W)
                               or fl.shape[0] not in (F, F - 1)):
            raise ValueError("%s: float32 C-contiguous [F or F - 1, 2, %d, %d] expected, got %s %s"
                             % (name, H, W, fl.dtype, fl.shape))
    p1 = default_params(1, sigma) if p1 is None else p1
    p2 = default_params(2, sigma) if p2 is None else p2
    basic = np.empty_like(noisy) if basic is None else basic
    out = np.empty_like(noisy) if out is None else out
    vp = lambda a: None if a is None else C.c_void_p(a.ctypes.data)  # noqa: E731
    _check(load().vbm3d_run_host(sigma, vp(noisy), vp(fflow), vp(bflow), vp(basic), vp(out), C.byref(p1),
                                 C.byref(p2), int(color_space), dims_of(noisy)))
    return basic, out
