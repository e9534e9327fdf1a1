"""CPU restatement of the multiscaler's DCT pyramid — TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker; the product path never imports it.

Restates multiscaler/multiscaler.cpp:21-100 (dct_inplace, idct_inplace),
multiscaler/decompose.cpp:29-60 (type 0: the DCT pyramid),
multiscaler/recompose.cpp:27-60 (type 0) and multiscaler/merge_coarse.cpp
on planar float32 images (channels, rows, columns); the reference works on
interleaved images, one transform per channel, so the values are the same.
FFTW's REDFT10 / REDFT01 (unnormalised DCT-II / DCT-III, FFTW's documented
definitions) are scipy.fft.dct types 2 and 3 with norm=None, evaluated in
double and rounded once to float per 2D transform, as oracle/fftw_shim
does for the reference's own code (FFTW itself is not installed; real FFTW
rounds differently by a few float ulps).  Pinned against the reference's
programs built over that stand-in (oracle/_ref/libms_ref.so, class MsRef)
and against the golden vectors in tests/golden/multiscaler.
"""
import ctypes as C
import os

import numpy as np
from scipy import fft as sfft

HERE = os.path.dirname(os.path.abspath(__file__))
MS_REF_SO = os.path.join(HERE, "_ref", "libms_ref.so")


def dct_inplace(img):
    """dct_inplace (multiscaler.cpp:21-60, ISOMETRIC_DCT off): REDFT10 on
    both axes, then every value / (4 * rows * columns) in float."""
    y = sfft.dct(sfft.dct(img.astype(np.float64), type=2, axis=-1), type=2, axis=-2).astype(np.float32)
    rows, cols = img.shape[-2], img.shape[-1]
    return (y / np.float32(4 * rows * cols)).astype(np.float32)


def idct_inplace(img):
    """idct_inplace (multiscaler.cpp:62-100): REDFT01 on both axes, no
    normalisation."""
    return sfft.dct(sfft.dct(img.astype(np.float64), type=3, axis=-1), type=3, axis=-2).astype(np.float32)


def level_sizes(rows, cols, levels):
    """Level i is (rows, cols) halved i times by integer division
    (decompose.cpp:34, 56-57)."""
    out = []
    h, w = rows, cols
    for _ in range(levels):
        out.append((h, w))
        h //= 2
        w //= 2
    return out


def block_count(n, factor):
    """Rows (or columns) copied by `for (j = 0; j < n * factor; ++j)` with
    an int n and a float factor: the product is formed in float
    (recompose.cpp:45-46, merge_coarse.cpp:34-35)."""
    bound = np.float32(np.float32(n) * np.float32(factor))
    j = 0
    while np.float32(j) < bound:
        j += 1
    return j


def decompose(img, levels):
    """decompose type 0 (decompose.cpp:29-60): planar (C, rows, cols)
    float32 -> list of `levels` images (C, h_i, w_i)."""
    y = dct_inplace(img)
    return [idct_inplace(y[:, :h, :w]) for (h, w) in level_sizes(img.shape[1], img.shape[2], levels)]


def recompose(levels_in, factor=0.8):
    """recompose type 0 (recompose.cpp:27-60): the DCT of level 0, the
    low-frequency block of every coarser level's DCT written over it
    (rows j < rows_i * factor, columns k < cols_i * factor), one IDCT."""
    out = dct_inplace(levels_in[0])
    for lv in levels_in[1:]:
        y = dct_inplace(lv)
        bh, bw = block_count(lv.shape[1], factor), block_count(lv.shape[2], factor)
        out[:, :bh, :bw] = y[:, :bh, :bw]
    return idct_inplace(out)


def merge_coarse(fine, coarse, factor=0.8):
    """merge_coarse (merge_coarse.cpp:11-46): fine's DCT with the
    low-frequency block of coarse's DCT written over it, one IDCT."""
    out = dct_inplace(fine)
    y = dct_inplace(coarse)
    bh, bw = block_count(coarse.shape[1], factor), block_count(coarse.shape[2], factor)
    out[:, :bh, :bw] = y[:, :bh, :bw]
    return idct_inplace(out)


def level_sigma(sigma, lvl):
    """The noise level the multiscale script denoises level lvl with:
    `bc <<< "scale=2; $NOISE / 2^$lvl"` truncates to two decimals
    (src/utils/VBM3Ddenoising_multiscale.sh:50)."""
    from decimal import Decimal, ROUND_DOWN
    q = Decimal(repr(float(sigma))) / (Decimal(2) ** lvl)
    return float(q.quantize(Decimal("0.01"), rounding=ROUND_DOWN))


class MsRef:
    """The reference's multiscaler programs over in-memory images
    (oracle/_ref/libms_ref.so; present only where the sources were)."""

    def __init__(self):
        if not os.path.exists(MS_REF_SO):
            raise FileNotFoundError(MS_REF_SO)
        self.lib = C.CDLL(MS_REF_SO)
        fp = C.POINTER(C.c_float)
        ip = C.POINTER(C.c_int)
        self.lib.msref_put.argtypes = [C.c_char_p, fp, C.c_int, C.c_int, C.c_int]
        self.lib.msref_get.argtypes = [C.c_char_p, fp, ip, ip, ip]
        self.lib.msref_get.restype = C.c_int
        self.lib.msref_run.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_char_p)]
        self.lib.msref_run.restype = C.c_int

    @staticmethod
    def available():
        return os.path.exists(MS_REF_SO)

    def put(self, name, planar):
        """Stores a planar (C, rows, cols) image, interleaved as iio reads it."""
        c, h, w = planar.shape
        il = np.ascontiguousarray(np.transpose(planar, (1, 2, 0)).astype(np.float32))
        self.lib.msref_put(name.encode(), il.ctypes.data_as(C.POINTER(C.c_float)), w, h, c)

    def get(self, name):
        w, h, c = C.c_int(), C.c_int(), C.c_int()
        if not self.lib.msref_get(name.encode(), None, C.byref(w), C.byref(h), C.byref(c)):
            raise KeyError(name)
        il = np.empty((h.value, w.value, c.value), np.float32)
        self.lib.msref_get(name.encode(), il.ctypes.data_as(C.POINTER(C.c_float)), C.byref(w), C.byref(h), C.byref(c))
        return np.ascontiguousarray(np.transpose(il, (2, 0, 1)))

    def run(self, *argv):
        args = (C.c_char_p * len(argv))(*[a.encode() for a in argv])
        rc = self.lib.msref_run(argv[0].encode(), len(argv), args)
        if rc != 0:
            raise RuntimeError("%s returned %d" % (argv[0], rc))

    def decompose(self, img, levels):
        """`decompose in lvl_ <levels> .tiff` (decompose.cpp:14-60)."""
        self.put("in", img)
        self.run("decompose", "in", "lvl_", str(levels), ".tiff")
        return [self.get("lvl_%d.tiff" % i) for i in range(levels)]

    def recompose(self, levels_in, factor):
        """`recompose den_ <levels> .tiff out -c <factor>` (recompose.cpp:11-60)."""
        for i, lv in enumerate(levels_in):
            self.put("den_%d.tiff" % i, lv)
        self.run("recompose", "den_", str(len(levels_in)), ".tiff", "out", "-c", repr(float(factor)))
        return self.get("out")

    def merge_coarse(self, fine, coarse, factor):
        """`merge_coarse fine coarse out -c <factor>` (merge_coarse.cpp:11-46)."""
        self.put("fine", fine)
        self.put("coarse", coarse)
        self.run("merge_coarse", "fine", "coarse", "out", "-c", repr(float(factor)))
        return self.get("out")
