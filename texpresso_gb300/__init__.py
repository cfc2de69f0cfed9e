"""texpresso_gb300 -- GB300-native BCn block encoder behind texpresso's API.

Python mirror of the reference crate's public interface (lib/src/lib.rs):
``Format`` with ``compress``, ``compress_block_masked``, ``decompress``,
``decompress_block``, ``block_size`` and ``compressed_size``; ``Params``;
``Algorithm``; ``COLOUR_WEIGHTS_UNIFORM`` / ``COLOUR_WEIGHTS_PERCEPTUAL``;
``num_blocks``.  Every call goes through the C ABI of
``libtexpresso_gb300.so`` (include/texpresso_gb300.h) to sm_103a kernels.
There is no CPU fallback: importing fails loudly if the library has not been
built, and compute calls raise ``TexpressoError`` without a CUDA device.

Where the reference panics (short output, zero width, partial trailing block)
these functions raise ``TexpressoError`` carrying the C status code.

Device-side entry points (``compress_device``, ``compress_blocks_device``,
``decompress_device``) take raw device pointers and a CUDA stream handle so
that callers holding GPU buffers (for example torch tensors) avoid host
copies.
"""
import ctypes
import enum
import os
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtexpresso_gb300.so")

if not os.path.exists(LIB_PATH):
    raise ImportError(
        "texpresso_gb300: %s is missing; build it first with "
        "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)" % LIB_PATH)

_SIGS = {}


def _sig(name, what, value):
    """Record a ctypes signature; applied when the library is first opened."""
    _SIGS.setdefault(name, {})[what] = value
    if _Lib.handle is not None:
        setattr(getattr(_Lib.handle, name), what, value)


class _Lib:
    """The C library, opened on first use: importing the package (or its numpy
    workload generators) maps nothing; the first call opens
    libtexpresso_gb300.so and fails loudly if it cannot."""
    handle = None

    @staticmethod
    def open():
        if _Lib.handle is None:
            h = ctypes.CDLL(LIB_PATH)
            for fn, sig in _SIGS.items():
                for what, value in sig.items():
                    setattr(getattr(h, fn), what, value)
            _Lib.handle = h
        return _Lib.handle

    def __getattr__(self, name):
        return getattr(_Lib.open(), name)


_lib = _Lib()

TX_OK = 0
STATUS = {
    -1: "TX_ERR_INVALID_FORMAT", -2: "TX_ERR_INVALID_ARGUMENT", -3: "TX_ERR_OUTPUT_TOO_SMALL",
    -4: "TX_ERR_INPUT_TOO_SMALL", -5: "TX_ERR_CUDA", -6: "TX_ERR_NO_DEVICE", -7: "TX_ERR_TIMEOUT",
    -8: "TX_ERR_OUT_OF_MEMORY", -9: "TX_ERR_MISALIGNED", -10: "TX_ERR_BUSY", -11: "TX_ERR_CANCELLED",
}


class TexpressoError(RuntimeError):
    """Raised where the reference panics, or on a CUDA failure."""

    def __init__(self, status, what=""):
        self.status = status
        msg = _lib.tx_status_string(status).decode()
        if status == -5:
            msg += " (cudaError %d)" % _lib.tx_last_cuda_error()
        super().__init__("%s: %s [%s]" % (what or "texpresso", msg, STATUS.get(status, status)))


class _CParams(ctypes.Structure):
    _fields_ = [("algorithm", ctypes.c_int32), ("weights", ctypes.c_float * 3),
                ("weigh_colour_by_alpha", ctypes.c_int32)]


_u8p = ctypes.POINTER(ctypes.c_uint8)
_sz = ctypes.c_size_t
_vp = ctypes.c_void_p
_sig("tx_status_string", "restype", ctypes.c_char_p)
_sig("tx_status_string", "argtypes", [ctypes.c_int])
_sig("tx_params_default", "argtypes", [ctypes.POINTER(_CParams)])
_sig("tx_num_blocks", "restype", _sz)
_sig("tx_num_blocks", "argtypes", [_sz])
_sig("tx_block_size", "restype", _sz)
_sig("tx_block_size", "argtypes", [ctypes.c_int])
_sig("tx_compressed_size", "restype", _sz)
_sig("tx_compressed_size", "argtypes", [ctypes.c_int, _sz, _sz])
_sig("tx_compress", "argtypes", [ctypes.c_int, _vp, _sz, _sz, _sz, ctypes.POINTER(_CParams), _vp, _sz])
_sig("tx_compress_block_masked", "argtypes", [ctypes.c_int, _vp, ctypes.c_uint32, ctypes.POINTER(_CParams), _vp, _sz])
_sig("tx_compress_device", "argtypes", [ctypes.c_int, _vp, _sz, ctypes.c_int, _sz, _sz, ctypes.POINTER(_CParams),
                                        _vp, _sz, _vp])
_sig("tx_compress_blocks_device", "argtypes", [ctypes.c_int, _vp, _vp, _sz, ctypes.POINTER(_CParams), _vp, _vp])
_sig("tx_decompress", "argtypes", [ctypes.c_int, _vp, _sz, _sz, _sz, _vp, _sz])
_sig("tx_decompress_block", "argtypes", [ctypes.c_int, _vp, _sz, _vp])
_sig("tx_decompress_device", "argtypes", [ctypes.c_int, _vp, _sz, _sz, _sz, _vp, _sz, _vp])
_sig("tx_last_cuda_error", "restype", ctypes.c_int)
_sig("tx_kernel_launch_count", "restype", ctypes.c_uint64)


def _check(rc, what):
    if rc != TX_OK:
        raise TexpressoError(rc, what)


class Algorithm(enum.IntEnum):
    """lib/src/lib.rs:49-59"""
    RangeFit = 0
    ClusterFit = 1
    IterativeClusterFit = 2


COLOUR_WEIGHTS_UNIFORM = (1.0, 1.0, 1.0)               # lib/src/lib.rs:71
COLOUR_WEIGHTS_PERCEPTUAL = (0.2126, 0.7152, 0.0722)   # lib/src/lib.rs:74


@dataclass
class Params:
    """lib/src/lib.rs:76-100 (defaults: ClusterFit, perceptual weights, no alpha weighting)."""
    algorithm: Algorithm = Algorithm.ClusterFit
    weights: Sequence[float] = field(default_factory=lambda: COLOUR_WEIGHTS_PERCEPTUAL)
    weigh_colour_by_alpha: bool = False

    def _c(self):
        p = _CParams()
        p.algorithm = int(self.algorithm)
        for i in range(3):
            p.weights[i] = float(self.weights[i])
        p.weigh_colour_by_alpha = 1 if self.weigh_colour_by_alpha else 0
        return p


def num_blocks(size):
    """lib/src/lib.rs:103-105"""
    return int(_lib.tx_num_blocks(size))


def _buffer(obj, writable):
    """(address, length) of a C-contiguous bytes-like or numpy buffer, without copying."""
    if isinstance(obj, np.ndarray):
        if not obj.flags.c_contiguous:
            raise ValueError("buffer must be C-contiguous")
        if writable and not obj.flags.writeable:
            raise TypeError("output buffer is read-only")
        return (obj.ctypes.data if obj.nbytes else None), obj.nbytes
    mv = memoryview(obj)
    if not mv.contiguous:
        raise ValueError("buffer must be contiguous")
    if writable and mv.readonly:
        raise TypeError("output buffer is read-only")
    a = np.frombuffer(mv, dtype=np.uint8)
    return (a.ctypes.data if a.size else None), a.size


class Format(enum.IntEnum):
    """lib/src/lib.rs:39-46 and the methods of impl Format (:117-336)."""
    Bc1 = 0
    Bc2 = 1
    Bc3 = 2
    Bc4 = 3
    Bc5 = 4

    def block_size(self):
        """lib/src/lib.rs:159-168"""
        return int(_lib.tx_block_size(int(self)))

    def compressed_size(self, width, height):
        """lib/src/lib.rs:175-179"""
        return int(_lib.tx_compressed_size(int(self), width, height))

    def compress(self, rgba, width, height, params, output):
        """Format::compress (lib/src/lib.rs:287-335): RGBA8 in, blocks written into output."""
        src, slen = _buffer(rgba, False)
        dst, dlen = _buffer(output, True)
        rc = _lib.tx_compress(int(self), src, slen, width, height, ctypes.byref(params._c()), dst, dlen)
        _check(rc, "Format.compress")

    def compress_block_masked(self, rgba, mask, params, output):
        """Format::compress_block_masked (lib/src/lib.rs:188-234)."""
        src, slen = _buffer(rgba, False)
        if slen < 64:
            raise TexpressoError(-4, "Format.compress_block_masked")
        dst, dlen = _buffer(output, True)
        rc = _lib.tx_compress_block_masked(int(self), src, mask & 0xFFFFFFFF, ctypes.byref(params._c()), dst, dlen)
        _check(rc, "Format.compress_block_masked")

    def decompress(self, data, width, height, output):
        """Format::decompress (lib/src/lib.rs:124-156)."""
        src, slen = _buffer(data, False)
        dst, dlen = _buffer(output, True)
        rc = _lib.tx_decompress(int(self), src, slen, width, height, dst, dlen)
        _check(rc, "Format.decompress")

    def decompress_block(self, block):
        """Format::decompress_block (lib/src/lib.rs:240-277): returns 64 RGBA8 bytes."""
        out = bytearray(64)
        src, slen = _buffer(block, False)
        dst, _ = _buffer(out, True)
        rc = _lib.tx_decompress_block(int(self), src, slen, dst)
        _check(rc, "Format.decompress_block")
        return bytes(out)


def compress_device(fmt, src_ptr, src_pitch, channels, width, height, params, out_ptr, out_len, stream=0):
    """Stream-ordered compress of a device image (tx_compress_device)."""
    _check(_lib.tx_compress_device(int(fmt), src_ptr, src_pitch, channels, width, height,
                                   ctypes.byref(params._c()), out_ptr, out_len, stream or None),
           "compress_device")


def compress_blocks_device(fmt, blocks_ptr, masks_ptr, nblocks, params, out_ptr, stream=0):
    """Stream-ordered compress of nblocks x 64-byte RGBA8 blocks (tx_compress_blocks_device)."""
    _check(_lib.tx_compress_blocks_device(int(fmt), blocks_ptr, masks_ptr or None, nblocks,
                                          ctypes.byref(params._c()), out_ptr, stream or None),
           "compress_blocks_device")


def decompress_device(fmt, data_ptr, data_len, width, height, out_ptr, out_pitch, stream=0):
    """Stream-ordered decode into a device RGBA8 image (tx_decompress_device)."""
    _check(_lib.tx_decompress_device(int(fmt), data_ptr, data_len, width, height, out_ptr, out_pitch,
                                     stream or None), "decompress_device")


def kernel_launch_count():
    """Kernels this library has launched in this process."""
    return int(_lib.tx_kernel_launch_count())


def library():
    """The loaded ctypes library (for tests of the raw C ABI)."""
    return _Lib.open()


# ---------------------------------------------------------------------------
# batched form (tx_batch_*) and mip producer (tx_mip_*)

class BatchItem(ctypes.Structure):
    """tx_batch_item: one texture level in device memory."""
    _fields_ = [("src", _vp), ("src_pitch", _sz), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("format", ctypes.c_int32), ("channels", ctypes.c_int32), ("params", _CParams), ("dst", _vp)]


class BatchTuning(ctypes.Structure):
    """tx_batch_tuning: launch shape of the persistent batch kernels."""
    _fields_ = [("team_lanes", ctypes.c_int32), ("team_threads_per_cta", ctypes.c_int32),
                ("team_ctas_per_sm", ctypes.c_int32), ("team_blocks_per_unit", ctypes.c_int32),
                ("lane_ctas_per_sm", ctypes.c_int32), ("lane_blocks_per_lane", ctypes.c_int32),
                ("team_blocks_in_flight", ctypes.c_int32)]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class MipJob(ctypes.Structure):
    """tx_mip_job: one level step of one image in device memory."""
    _fields_ = [("src", _vp), ("src_pitch", _sz), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("channels", ctypes.c_int32), ("dst", _vp), ("dst_pitch", _sz)]


_sig("tx_batch_default_tuning", "argtypes", [ctypes.POINTER(BatchTuning)])
_sig("tx_batch_create", "argtypes", [ctypes.POINTER(BatchItem), _sz, ctypes.POINTER(BatchTuning), ctypes.POINTER(_vp)])
_sig("tx_batch_launch", "argtypes", [_vp, _vp])
_sig("tx_batch_set_tuning", "argtypes", [_vp, ctypes.POINTER(BatchTuning)])
_sig("tx_batch_get_tuning", "argtypes", [_vp, ctypes.POINTER(BatchTuning)])
_sig("tx_batch_info", "argtypes", [_vp, ctypes.POINTER(_sz), ctypes.POINTER(_sz), ctypes.POINTER(_sz)])
_sig("tx_batch_autotune", "argtypes", [_vp, _vp, ctypes.c_int, ctypes.POINTER(BatchTuning)])
_sig("tx_batch_destroy", "argtypes", [_vp])
_sig("tx_batch_destroy", "restype", None)
_sig("tx_mip_count", "restype", ctypes.c_uint32)
_sig("tx_mip_count", "argtypes", [ctypes.c_uint32, ctypes.c_uint32])
_sig("tx_mip_batch_device", "argtypes", [ctypes.POINTER(MipJob), _sz, _vp])


def batch_item(fmt, src_ptr, src_pitch, width, height, params, dst_ptr, channels=4):
    it = BatchItem()
    it.src, it.src_pitch, it.width, it.height = src_ptr, src_pitch, width, height
    it.format, it.channels, it.params, it.dst = int(fmt), channels, params._c(), dst_ptr
    return it


class Batch:
    """A plan over many texture levels, launched as one stream-ordered unit."""

    def __init__(self, items, tuning=None):
        arr = (BatchItem * max(1, len(items)))(*items)
        self._items = arr
        h = _vp()
        _check(_lib.tx_batch_create(arr, len(items), ctypes.byref(tuning) if tuning else None, ctypes.byref(h)),
               "tx_batch_create")
        self._h = h

    def launch(self, stream=0):
        _check(_lib.tx_batch_launch(self._h, stream or None), "tx_batch_launch")

    def autotune(self, stream=0, repeats=3):
        t = BatchTuning()
        _check(_lib.tx_batch_autotune(self._h, stream or None, repeats, ctypes.byref(t)), "tx_batch_autotune")
        return t

    @property
    def tuning(self):
        t = BatchTuning()
        _check(_lib.tx_batch_get_tuning(self._h, ctypes.byref(t)), "tx_batch_get_tuning")
        return t

    @tuning.setter
    def tuning(self, t):
        _check(_lib.tx_batch_set_tuning(self._h, ctypes.byref(t)), "tx_batch_set_tuning")

    def info(self):
        nb, nl, nt = _sz(), _sz(), _sz()
        _check(_lib.tx_batch_info(self._h, ctypes.byref(nb), ctypes.byref(nl), ctypes.byref(nt)), "tx_batch_info")
        return {"blocks": nb.value, "lane_units": nl.value, "team_units": nt.value}

    def close(self):
        if getattr(self, "_h", None):
            _lib.tx_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_batch_tuning():
    t = BatchTuning()
    _lib.tx_batch_default_tuning(ctypes.byref(t))
    return t


def mip_count(width, height):
    return int(_lib.tx_mip_count(width, height))


def mip_batch_device(jobs, stream=0):
    """One mip level step for every (src, pitch, w, h, channels, dst, dst_pitch) job."""
    if not jobs:
        return
    arr = (MipJob * len(jobs))()
    for i, (src, sp, w, h, ch, dst, dp) in enumerate(jobs):
        arr[i].src, arr[i].src_pitch, arr[i].width, arr[i].height = src, sp, w, h
        arr[i].channels, arr[i].dst, arr[i].dst_pitch = ch, dst, dp
    _check(_lib.tx_mip_batch_device(arr, len(jobs), stream or None), "tx_mip_batch_device")


# ---------------------------------------------------------------------------
# serving form (tx_server_*)

class ServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget", _sz), ("step_blocks", ctypes.c_uint32), ("min_share", ctypes.c_uint32),
                ("tuning", BatchTuning)]


class ServerRequest(ctypes.Structure):
    _fields_ = [("rgba", _vp), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("format", ctypes.c_int32),
                ("params", _CParams), ("mips", ctypes.c_int32), ("output", _vp), ("output_len", _sz)]


class ServerResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("levels", ctypes.c_uint32), ("steps", ctypes.c_uint32),
                ("blocks", ctypes.c_uint64), ("latency_us", ctypes.c_double), ("queue_us", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("steps", ctypes.c_uint64),
                ("memory_budget", _sz), ("held_high_water", _sz), ("busy_us", ctypes.c_double),
                ("hbm_deferrals", ctypes.c_uint64)]


_sig("tx_chain_compressed_size", "restype", _sz)
_sig("tx_chain_compressed_size", "argtypes", [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int])
_sig("tx_server_default_config", "argtypes", [ctypes.POINTER(ServerConfig)])
_sig("tx_server_default_config", "restype", None)
_sig("tx_server_create", "argtypes", [ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)])
_sig("tx_server_submit", "argtypes", [_vp, ctypes.POINTER(ServerRequest), ctypes.POINTER(ctypes.c_uint64)])
_sig("tx_server_wait", "argtypes", [_vp, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ServerResult)])
_sig("tx_server_get_stats", "argtypes", [_vp, ctypes.POINTER(ServerStats)])
_sig("tx_server_cancel", "argtypes", [_vp, ctypes.c_uint64])
_sig("tx_server_destroy", "argtypes", [_vp])
_sig("tx_server_destroy", "restype", None)


def chain_compressed_size(fmt, width, height, mips=True):
    """Bytes of every compressed level of a mip chain (or of level 0 alone)."""
    return int(_lib.tx_chain_compressed_size(int(fmt), width, height, 1 if mips else 0))


class Server:
    """Request loop with admission by device memory and continuous batching."""

    def __init__(self, memory_budget=None, step_blocks=None, min_share=None, tuning=None):
        c = ServerConfig()
        _lib.tx_server_default_config(ctypes.byref(c))
        if memory_budget:
            c.memory_budget = memory_budget
        if step_blocks:
            c.step_blocks = step_blocks
        if min_share:
            c.min_share = min_share
        if tuning is not None:
            c.tuning = tuning
        h = _vp()
        _check(_lib.tx_server_create(ctypes.byref(c), ctypes.byref(h)), "tx_server_create")
        self._h = h
        self._keep = {}

    def submit(self, rgba, width, height, fmt, params, output, mips=True):
        """Queue a job; rgba (host RGBA8) and output (host) stay referenced until wait()."""
        src, slen = _buffer(rgba, False)
        dst, dlen = _buffer(output, True)
        if slen < width * height * 4:
            raise TexpressoError(-4, "Server.submit")
        r = ServerRequest()
        r.rgba, r.width, r.height, r.format = src, width, height, int(fmt)
        r.params, r.mips, r.output, r.output_len = params._c(), 1 if mips else 0, dst, dlen
        rid = ctypes.c_uint64()
        _check(_lib.tx_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid)), "tx_server_submit")
        self._keep[rid.value] = (rgba, output)
        return rid.value

    def wait(self, rid, timeout_ms=-1):
        res = ServerResult()
        rc = _lib.tx_server_wait(self._h, rid, timeout_ms, ctypes.byref(res))
        if rc != -7:
            self._keep.pop(rid, None)
        _check(rc, "tx_server_wait")
        return {"status": res.status, "levels": res.levels, "steps": res.steps, "blocks": res.blocks,
                "latency_us": res.latency_us, "queue_us": res.queue_us}

    def cancel(self, rid):
        """Drop a job not yet admitted (True), or report that it already runs (False)."""
        rc = _lib.tx_server_cancel(self._h, rid)
        if rc == -10:
            return False
        _check(rc, "tx_server_cancel")
        return True

    def stats(self):
        s = ServerStats()
        _check(_lib.tx_server_get_stats(self._h, ctypes.byref(s)), "tx_server_get_stats")
        return {f: (float if t is ctypes.c_double else int)(getattr(s, f)) for f, t in s._fields_}

    def close(self):
        if getattr(self, "_h", None):
            _lib.tx_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# DDS container (tx_dds_*)

DDS_HEADER_BYTES = 148
_sig("tx_dds_write_header", "argtypes", [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp, _sz,
                                         ctypes.POINTER(_sz)])
_sig("tx_dds_parse", "argtypes", [_vp, _sz, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint32),
                                  ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(_sz)])


def dds_header(fmt, width, height, mip_levels=0):
    """The 148 header bytes the reference CLI writes (cli/src/main.rs:143-164)."""
    out = bytearray(DDS_HEADER_BYTES)
    dst, dlen = _buffer(out, True)
    n = _sz()
    _check(_lib.tx_dds_write_header(int(fmt), width, height, mip_levels, dst, dlen, ctypes.byref(n)), "dds_header")
    return bytes(out[:n.value])


def dds_parse(data):
    """(format, width, height, mip_levels, data_offset) of a DDS file's header."""
    src, slen = _buffer(data, False)
    f, w, h, m, off = ctypes.c_int(), ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32(), _sz()
    _check(_lib.tx_dds_parse(src, slen, ctypes.byref(f), ctypes.byref(w), ctypes.byref(h), ctypes.byref(m),
                             ctypes.byref(off)), "dds_parse")
    return Format(f.value), w.value, h.value, m.value, off.value


def write_dds(path, fmt, width, height, blocks, mip_levels=0):
    """Write compressed levels as a DDS file, as the reference CLI does."""
    with open(path, "wb") as f:
        f.write(dds_header(fmt, width, height, mip_levels))
        f.write(bytes(memoryview(blocks).cast("B")) if not hasattr(blocks, "tobytes") else blocks.tobytes())


def read_dds(path):
    """(format, width, height, mip_levels, compressed bytes) of a DDS file."""
    with open(path, "rb") as f:
        data = f.read()
    fmt, w, h, m, off = dds_parse(data)
    return fmt, w, h, m, data[off:]
