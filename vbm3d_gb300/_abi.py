"""ctypes mirror of include/vbm3d_gb300.h (the C ABI of the GPU library).

`Params` mirrors `struct Parameters` of the reference (src/parameters.h:21-58)
field for field; `Dims` is the reference's VideoSize (width, height, frames,
channels; src/Utilities/LibVideoT.hpp:40-121).
"""
import ctypes as C

DCT = 0
BIOR = 1
HADAMARD = 2
HAAR = 4

STATUS = {
    0: "VBM3D_OK",
    1: "VBM3D_ERR_INVALID_ARGUMENT",
    2: "VBM3D_ERR_UNSUPPORTED",
    3: "VBM3D_ERR_CUDA",
    4: "VBM3D_ERR_OUT_OF_MEMORY",
    5: "VBM3D_ERR_COLOR_SPACE",
    6: "VBM3D_ERR_SIZE_MISMATCH",
}


class Params(C.Structure):
    _fields_ = [
        ("k", C.c_uint), ("kt", C.c_uint), ("p", C.c_uint), ("N", C.c_uint),
        ("tau", C.c_float), ("d", C.c_float),
        ("Nf", C.c_uint), ("Ns", C.c_uint), ("Npr", C.c_uint), ("Nb", C.c_uint),
        ("T_2D", C.c_uint), ("T_3D", C.c_uint),
        ("lambda3D", C.c_float), ("mc", C.c_int), ("n", C.c_int),
    ]

    def replace(self, **kw):
        out = Params()
        C.pointer(out)[0] = self
        for key, val in kw.items():
            setattr(out, key, val)
        return out

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}

    def __repr__(self):
        return "Params(%s)" % ", ".join("%s=%r" % kv for kv in self.as_dict().items())


class Dims(C.Structure):
    _fields_ = [("width", C.c_uint), ("height", C.c_uint),
                ("frames", C.c_uint), ("channels", C.c_uint)]


def dims_of(video):
    """Dims of a [F, C, H, W] array."""
    f, c, h, w = video.shape
    return Dims(w, h, f, c)


class Clip(C.Structure):
    """vbm3d_clip: one clip of a batch (device pointers)."""
    _fields_ = [("dims", Dims), ("sigma", C.c_float),
                ("prms_1", C.POINTER(Params)), ("prms_2", C.POINTER(Params)),
                ("noisy", C.c_void_p), ("fflow", C.c_void_p), ("bflow", C.c_void_p),
                ("basic", C.c_void_p), ("denoised", C.c_void_p)]


class BatchConfig(C.Structure):
    """vbm3d_batch_config: refs per work item and warps per block of each
    phase (0, 0 = autotune), the graph switch, and three outputs."""
    _fields_ = [("bm1_tile", C.c_int), ("bm1_warps", C.c_int),
                ("filter1_tile", C.c_int), ("filter1_warps", C.c_int),
                ("bm2_tile", C.c_int), ("bm2_warps", C.c_int),
                ("filter2_tile", C.c_int), ("filter2_warps", C.c_int),
                ("no_graph", C.c_int), ("tune_ms", C.c_float),
                ("work_items", C.c_uint), ("device_bytes", C.c_size_t)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class BatchLaunch(C.Structure):
    """vbm3d_batch_launch: one work launch measured by vbm3d_batch_profile."""
    _fields_ = [("phase", C.c_int), ("k", C.c_int), ("channels", C.c_int), ("clips", C.c_int),
                ("items", C.c_uint), ("refs", C.c_ulonglong), ("tile", C.c_int), ("warps", C.c_int),
                ("grid", C.c_int), ("ms", C.c_float)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class TvParams(C.Structure):
    """vbm3d_tvl1_params: TV-L1 options (tvl1flow's command line)."""
    _fields_ = [("tau", C.c_float), ("lambda_", C.c_float), ("theta", C.c_float), ("nscales", C.c_int),
                ("fscale", C.c_int), ("zfactor", C.c_float), ("nwarps", C.c_int), ("epsilon", C.c_float)]
