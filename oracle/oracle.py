"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle is a plain-C restatement of jansol/texpresso's block encoder
(lib/src/) used to check the CUDA library and to time the reference's CPU
algorithm.  Only tests, the smoke check and the CPU-baseline leg of the bench
may load it; the product path never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtexpresso_oracle.so")

BC1, BC2, BC3, BC4, BC5 = range(5)
RANGE_FIT, CLUSTER_FIT, ITERATIVE_CLUSTER_FIT = range(3)
FORMATS = {"BC1": BC1, "BC2": BC2, "BC3": BC3, "BC4": BC4, "BC5": BC5}
ALGORITHMS = {"RangeFit": RANGE_FIT, "ClusterFit": CLUSTER_FIT,
              "IterativeClusterFit": ITERATIVE_CLUSTER_FIT}


class Params(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int32), ("weights", ctypes.c_float * 3),
                ("weigh_colour_by_alpha", ctypes.c_int32)]


class BlockStats(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int32), ("path", ctypes.c_int32),
                ("iterations3", ctypes.c_int32), ("iterations4", ctypes.c_int32),
                ("candidates", ctypes.c_int64), ("alpha_mode", ctypes.c_int32 * 2)]


STATS_DTYPE = np.dtype([("count", "<i4"), ("path", "<i4"), ("iterations3", "<i4"),
                        ("iterations4", "<i4"), ("candidates", "<i8"),
                        ("alpha_mode", "<i4", (2,))])
assert STATS_DTYPE.itemsize == ctypes.sizeof(BlockStats)


def build(force=False):
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "texpresso_oracle.c")):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        L.txo_block_size.restype = ctypes.c_size_t
        L.txo_block_size.argtypes = [ctypes.c_int]
        L.txo_compressed_size.restype = ctypes.c_size_t
        L.txo_compressed_size.argtypes = [ctypes.c_int, ctypes.c_size_t, ctypes.c_size_t]
        L.txo_single_lut.argtypes = [ctypes.c_int, u8p]
        L.txo_compress_block_masked.argtypes = [ctypes.c_int, u8p, ctypes.c_uint32,
                                                ctypes.POINTER(Params), u8p, ctypes.c_void_p]
        L.txo_compress.restype = ctypes.c_int
        L.txo_compress.argtypes = [ctypes.c_int, u8p, ctypes.c_size_t, ctypes.c_size_t,
                                   ctypes.POINTER(Params), u8p, ctypes.c_size_t, ctypes.c_int]
        L.txo_compress_blocks.argtypes = [ctypes.c_int, u8p, ctypes.c_void_p, ctypes.c_size_t,
                                          ctypes.POINTER(Params), u8p, ctypes.c_void_p,
                                          ctypes.c_int]
        L.txo_decompress_block.argtypes = [ctypes.c_int, u8p, u8p]
        L.txo_decompress.restype = ctypes.c_int
        L.txo_decompress.argtypes = [ctypes.c_int, u8p, ctypes.c_size_t, ctypes.c_size_t,
                                     ctypes.c_size_t, u8p, ctypes.c_size_t]
        L.txo_online_cores.restype = ctypes.c_int
        _lib = L
    return _lib


def _u8p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def make_params(algorithm=CLUSTER_FIT, weights=(0.2126, 0.7152, 0.0722), weigh_colour_by_alpha=False):
    p = Params()
    p.algorithm = int(algorithm)
    for i in range(3):
        p.weights[i] = float(weights[i])
    p.weigh_colour_by_alpha = 1 if weigh_colour_by_alpha else 0
    return p


def block_size(fmt):
    return int(lib().txo_block_size(fmt))


def compressed_size(fmt, w, h):
    return int(lib().txo_compressed_size(fmt, w, h))


def single_lut(which):
    out = np.zeros(256 * 6, np.uint8)
    lib().txo_single_lut(which, _u8p(out))
    return out


def compress(fmt, rgba, width, height, params, out_len=None, nthreads=0):
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8).reshape(-1)
    n = compressed_size(fmt, width, height) if out_len is None else out_len
    out = np.zeros(n, np.uint8)
    rc = lib().txo_compress(fmt, _u8p(rgba), width, height, ctypes.byref(params), _u8p(out),
                            n, nthreads)
    if rc != 0:
        raise ValueError("oracle compress rejected the arguments (%d)" % rc)
    return out


def compress_block_masked(fmt, rgba64, mask, params, with_stats=False):
    rgba64 = np.ascontiguousarray(rgba64, dtype=np.uint8).reshape(64)
    out = np.zeros(block_size(fmt), np.uint8)
    st = BlockStats()
    lib().txo_compress_block_masked(fmt, _u8p(rgba64), mask, ctypes.byref(params), _u8p(out),
                                    ctypes.byref(st) if with_stats else None)
    if with_stats:
        return out, st
    return out


def compress_blocks(fmt, blocks, masks, params, nthreads=0, with_stats=False):
    """blocks: (n, 64) uint8; masks: (n,) uint32 or None (all valid)."""
    blocks = np.ascontiguousarray(blocks, dtype=np.uint8).reshape(-1, 64)
    n = blocks.shape[0]
    out = np.zeros((n, block_size(fmt)), np.uint8)
    mptr = None
    if masks is not None:
        masks = np.ascontiguousarray(masks, dtype=np.uint32)
        mptr = masks.ctypes.data_as(ctypes.c_void_p)
    stats = np.zeros(n, STATS_DTYPE) if with_stats else None
    lib().txo_compress_blocks(fmt, _u8p(blocks), mptr, n, ctypes.byref(params), _u8p(out),
                              stats.ctypes.data_as(ctypes.c_void_p) if with_stats else None,
                              nthreads)
    if with_stats:
        return out, stats
    return out


def decompress_block(fmt, block):
    block = np.ascontiguousarray(block, dtype=np.uint8)
    out = np.zeros(64, np.uint8)
    lib().txo_decompress_block(fmt, _u8p(block), _u8p(out))
    return out


def decompress(fmt, data, width, height, out_len=None):
    data = np.ascontiguousarray(data, dtype=np.uint8).reshape(-1)
    n = width * height * 4 if out_len is None else out_len
    out = np.zeros(n, np.uint8)
    rc = lib().txo_decompress(fmt, _u8p(data), data.size, width, height, _u8p(out), n)
    if rc != 0:
        raise ValueError("oracle decompress rejected the arguments (%d)" % rc)
    return out


def online_cores():
    return int(lib().txo_online_cores())
