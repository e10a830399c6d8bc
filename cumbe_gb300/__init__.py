"""cumbe_gb300 - Python host mirror of libmbe, the GB300-native maximal
biclique enumeration engine.

Everything here is a thin ctypes layer over the C ABI declared in
include/mbe.h; all enumeration runs in the library's sm_103a kernels.
There is no Python or CPU fallback: when the library is missing or no GPU
is present, calls raise MBEError.

The reference's interface for this path is the `mbe <graph.bi> <variant>`
command (NTUDDSNLab/cuMBE src/main.cu:9) with variants cuMBE / noRS / noES
/ noWS (src/main.cu:121-122); `Engine.enumerate(graph, variant)` is its
library form, and `cumbe_gb300/mbe` is the CLI itself.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmbe.so")
CLI_PATH = os.path.join(HERE, "mbe")

VARIANTS = {"cuMBE": 0, "noRS": 1, "noES": 2, "noWS": 3}
OPT_NO_HASH = 1
OPT_EMIT = 2
OPT_TIMING = 4
OPT_L2_PIN = 8
OPT_HOST_CHUNKS = 16

STATUS = {0: "OK", 1: "INVALID_ARG", 2: "IO", 3: "FORMAT", 4: "CUDA", 5: "OUT_OF_MEMORY",
          6: "DEVICE_TIMEOUT", 7: "CAPACITY", 8: "NO_DEVICE", 9: "BUSY"}


class MBEError(RuntimeError):
    def __init__(self, status: int, what: str, msg: str):
        super().__init__(f"{what}: {STATUS.get(status, status)}: {msg}")
        self.status = status


class _GraphInfo(ctypes.Structure):
    _fields_ = [("n_rows", ctypes.c_uint32), ("n_cols", ctypes.c_uint32), ("n_edges", ctypes.c_uint64),
                ("max_row_deg", ctypes.c_uint32), ("max_col_deg", ctypes.c_uint32),
                ("n_dup_dropped", ctypes.c_uint32), ("swapped", ctypes.c_uint32)]


class _GenParams(ctypes.Structure):
    _fields_ = [("n_rows", ctypes.c_uint32), ("n_cols", ctypes.c_uint32), ("n_edges", ctypes.c_uint64),
                ("gamma_rows", ctypes.c_double), ("gamma_cols", ctypes.c_double), ("max_deg", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("planted", ctypes.c_uint32), ("planted_rows", ctypes.c_uint32),
                ("planted_cols", ctypes.c_uint32), ("planted_density", ctypes.c_double)]


class _Opts(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_uint32), ("min_rows", ctypes.c_uint32), ("min_cols", ctypes.c_uint32),
                ("warps_per_block", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("donate_min", ctypes.c_uint32), ("stack_words", ctypes.c_uint32),
                ("emit_offsets", ctypes.POINTER(ctypes.c_uint32)), ("emit_ids", ctypes.POINTER(ctypes.c_uint32)),
                ("emit_nrows", ctypes.POINTER(ctypes.c_uint32)), ("emit_cap_bicliques", ctypes.c_uint64),
                ("emit_cap_ids", ctypes.c_uint64), ("root_begin", ctypes.c_uint32), ("root_end", ctypes.c_uint32),
                ("root_stride", ctypes.c_uint32), ("reserved0", ctypes.c_uint32),
                ("wait_timeout_ns", ctypes.c_uint64)]


class _Result(ctypes.Structure):
    _fields_ = [("count", ctypes.c_uint64), ("hash", ctypes.c_uint64), ("nodes", ctypes.c_uint64),
                ("words", ctypes.c_uint64), ("words_expand", ctypes.c_uint64), ("emitted", ctypes.c_uint64),
                ("ms", ctypes.c_float), ("ms_prep", ctypes.c_float)]


class _TuneChoice(ctypes.Structure):
    _fields_ = [("bucket", ctypes.c_uint32), ("n_graphs", ctypes.c_uint32), ("sample_graphs", ctypes.c_uint32),
                ("blocks_per_sm", ctypes.c_uint32), ("donate_min", ctypes.c_uint32), ("solve_rows", ctypes.c_uint32),
                ("chunk_mwords", ctypes.c_uint32), ("trials", ctypes.c_uint32), ("ms_default", ctypes.c_float),
                ("ms_tuned", ctypes.c_float)]


class _ServerConfig(ctypes.Structure):
    _fields_ = [("slots", ctypes.c_uint32), ("max_batch", ctypes.c_uint32), ("blocks_per_sm", ctypes.c_uint32),
                ("variant", ctypes.c_uint32), ("mem_budget", ctypes.c_uint64), ("heavy_bytes", ctypes.c_uint64)]


class _RequestResult(ctypes.Structure):
    _fields_ = [("request", ctypes.c_uint64), ("graph", ctypes.c_uint32), ("status", ctypes.c_uint32),
                ("count", ctypes.c_uint64), ("hash", ctypes.c_uint64), ("submit_s", ctypes.c_double),
                ("start_s", ctypes.c_double), ("done_s", ctypes.c_double), ("batch_size", ctypes.c_uint32),
                ("slot", ctypes.c_uint32)]


# Every symbol include/mbe.h declares, with its ctypes signature.
_VP = ctypes.c_void_p
_U64P = ctypes.POINTER(ctypes.c_uint64)
_U32P = ctypes.POINTER(ctypes.c_uint32)
SIGNATURES = {
    "mbe_graph_load_bi": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_VP)]),
    "mbe_graph_from_csr": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, _U64P, _U32P, ctypes.POINTER(_VP)]),
    "mbe_graph_generate": (ctypes.c_int, [ctypes.POINTER(_GenParams), ctypes.POINTER(_VP)]),
    "mbe_graph_write_bi": (ctypes.c_int, [_VP, ctypes.c_char_p]),
    "mbe_graph_write_bin": (ctypes.c_int, [_VP, ctypes.c_char_p]),
    "mbe_graph_load_bin": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_VP)]),
    "mbe_graph_load_cached": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_VP)]),
    "mbe_graph_load_konect": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(_VP)]),
    "mbe_graph_info_get": (ctypes.c_int, [_VP, ctypes.POINTER(_GraphInfo)]),
    "mbe_graph_copy_csr": (ctypes.c_int, [_VP, _U64P, _U32P]),
    "mbe_graph_free": (None, [_VP]),
    "mbe_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_VP)]),
    "mbe_ctx_destroy": (None, [_VP]),
    "mbe_last_error": (ctypes.c_char_p, []),
    "mbe_graph_upload": (ctypes.c_int, [_VP, _VP]),
    "mbe_graph_release": (ctypes.c_int, [_VP, _VP]),
    "mbe_enumerate": (ctypes.c_int, [_VP, _VP, ctypes.c_int, ctypes.POINTER(_Opts), ctypes.POINTER(_Result)]),
    "mbe_batch_run": (ctypes.c_int, [_VP, ctypes.POINTER(_VP), ctypes.c_uint32, ctypes.c_int,
                                     ctypes.POINTER(_Opts), ctypes.POINTER(_Result), ctypes.POINTER(ctypes.c_float)]),
    "mbe_batch_tune": (ctypes.c_int, [_VP, ctypes.POINTER(_VP), ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(_Opts),
                                      ctypes.POINTER(_TuneChoice), ctypes.c_uint32, _U32P]),
    "mbe_batch_tune_reset": (ctypes.c_int, [_VP]),
    "mbe_biclique_hash": (ctypes.c_uint64, [_U32P, ctypes.c_uint32, _U32P, ctypes.c_uint32]),
    "mbe_variant_name": (ctypes.c_char_p, [ctypes.c_int]),
    "mbe_variant_from_name": (ctypes.c_int, [ctypes.c_char_p]),
    "mbe_ctx_last_grid": (ctypes.c_int, [_VP, _U32P, _U32P, _U32P]),
    "mbe_ctx_counters": (ctypes.c_int, [_VP, _U64P, _U64P, _U64P]),
    "mbe_server_start": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_ServerConfig), ctypes.POINTER(_VP)]),
    "mbe_server_add_graph": (ctypes.c_int, [_VP, _VP, _U32P]),
    "mbe_server_estimate": (ctypes.c_int, [_VP, ctypes.c_uint32, _U64P]),
    "mbe_server_submit": (ctypes.c_int, [_VP, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _U64P]),
    "mbe_server_poll": (ctypes.c_int, [_VP, ctypes.POINTER(_RequestResult), ctypes.c_uint32, _U32P]),
    "mbe_server_clock": (ctypes.c_double, [_VP]),
    "mbe_server_warmup": (ctypes.c_int, [_VP]),
    "mbe_server_memory": (ctypes.c_int, [_VP, _U64P, _U64P, _U64P]),
    "mbe_server_stop": (ctypes.c_int, [_VP]),
    "mbe_enumerate_static": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, _VP, _VP, _VP, _VP, ctypes.c_int,
                                            _VP, _VP]),
}

_lib = None


def lib() -> ctypes.CDLL:
    """Loads the in-tree libmbe.so (built by cumbe_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MBEError(8, "load", f"{LIB_PATH} is missing; run cumbe_gb300.build.build() first")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(st: int, what: str):
    if st != 0:
        raise MBEError(st, what, lib().mbe_last_error().decode(errors="replace"))


@dataclass
class Result:
    count: int
    hash: int
    nodes: int
    words: int
    words_expand: int
    ms: float
    ms_prep: float
    bicliques: list | None = field(default=None, repr=False)


class Graph:
    """A bipartite graph in file orientation (rows x cols), host side."""

    def __init__(self, handle):
        self._h = _VP(handle) if not isinstance(handle, _VP) else handle

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value and _lib is not None:
            _lib.mbe_graph_free(h)
            self._h = _VP()

    @property
    def handle(self):
        return self._h

    @classmethod
    def load_bi(cls, path: str) -> "Graph":
        h = _VP()
        _check(lib().mbe_graph_load_bi(os.fsencode(path), ctypes.byref(h)), "mbe_graph_load_bi")
        return cls(h)

    @classmethod
    def from_csr(cls, n_rows: int, n_cols: int, row_ptr, col_idx) -> "Graph":
        rp = np.ascontiguousarray(row_ptr, dtype=np.uint64)
        ci = np.ascontiguousarray(col_idx, dtype=np.uint32)
        if ci.size == 0:
            ci = np.zeros(1, np.uint32)
        h = _VP()
        _check(lib().mbe_graph_from_csr(n_rows, n_cols, rp.ctypes.data_as(_U64P), ci.ctypes.data_as(_U32P),
                                        ctypes.byref(h)), "mbe_graph_from_csr")
        return cls(h)

    @classmethod
    def from_dense(cls, M) -> "Graph":
        M = np.asarray(M, dtype=bool)
        rp = np.zeros(M.shape[0] + 1, np.uint64)
        rp[1:] = np.cumsum(M.sum(1))
        return cls.from_csr(M.shape[0], M.shape[1], rp, np.nonzero(M)[1].astype(np.uint32))

    @classmethod
    def generate(cls, n_rows, n_cols, n_edges, gamma_rows=2.1, gamma_cols=2.1, max_deg=0, seed=1, planted=0,
                 planted_rows=0, planted_cols=0, planted_density=0.0) -> "Graph":
        p = _GenParams(n_rows, n_cols, n_edges, gamma_rows, gamma_cols, max_deg, seed, planted, planted_rows,
                       planted_cols, planted_density)
        h = _VP()
        _check(lib().mbe_graph_generate(ctypes.byref(p), ctypes.byref(h)), "mbe_graph_generate")
        return cls(h)

    def info(self) -> dict:
        i = _GraphInfo()
        _check(lib().mbe_graph_info_get(self._h, ctypes.byref(i)), "mbe_graph_info_get")
        return {f: getattr(i, f) for f, _ in _GraphInfo._fields_}

    def csr(self):
        i = self.info()
        rp = np.zeros(i["n_rows"] + 1, np.uint64)
        ci = np.zeros(max(1, i["n_edges"]), np.uint32)
        _check(lib().mbe_graph_copy_csr(self._h, rp.ctypes.data_as(_U64P), ci.ctypes.data_as(_U32P)),
               "mbe_graph_copy_csr")
        return i["n_rows"], i["n_cols"], rp, ci[:i["n_edges"]]

    def write_bi(self, path: str):
        _check(lib().mbe_graph_write_bi(self._h, os.fsencode(path)), "mbe_graph_write_bi")

    def write_bin(self, path: str):
        """Binary graph image (checksummed normalised CSR)."""
        _check(lib().mbe_graph_write_bin(self._h, os.fsencode(path)), "mbe_graph_write_bin")

    @classmethod
    def load_bin(cls, path: str) -> "Graph":
        h = _VP()
        _check(lib().mbe_graph_load_bin(os.fsencode(path), ctypes.byref(h)), "mbe_graph_load_bin")
        return cls(h)

    @classmethod
    def load_konect(cls, path: str, skip_words: int = 0, skip_per_edge: int = 0) -> "Graph":
        """KONECT edge-pair file, numbered as data/gen_bi.cpp numbers it."""
        h = _VP()
        _check(lib().mbe_graph_load_konect(os.fsencode(path), skip_words, skip_per_edge, ctypes.byref(h)),
               "mbe_graph_load_konect")
        return cls(h)

    @classmethod
    def load_cached(cls, bi_path: str, cache_path: str) -> "Graph":
        """`.bi` file through a binary cache (reused while at least as new)."""
        h = _VP()
        _check(lib().mbe_graph_load_cached(os.fsencode(bi_path), os.fsencode(cache_path), ctypes.byref(h)),
               "mbe_graph_load_cached")
        return cls(h)


def _opts(flags=0, min_rows=0, min_cols=0, donate_min=0, blocks_per_sm=0, stack_words=0, warps_per_block=0,
          root_begin=0, root_end=0, root_stride=0, wait_timeout_ns=0) -> _Opts:
    """mbe_opts: thresholds, tuning, the root sample (positions
    [root_begin, root_end) step root_stride of the processing order) and
    the device-wait limit."""
    o = _Opts()
    o.flags = flags
    o.min_rows = min_rows
    o.min_cols = min_cols
    o.donate_min = donate_min
    o.blocks_per_sm = blocks_per_sm
    o.stack_words = stack_words
    o.warps_per_block = warps_per_block
    o.root_begin = root_begin
    o.root_end = root_end
    o.root_stride = root_stride
    o.wait_timeout_ns = wait_timeout_ns
    return o


class Engine:
    """One device context (one CUDA stream on one GPU)."""

    def __init__(self, device: int = 0):
        self._h = _VP()
        _check(lib().mbe_ctx_create(device, ctypes.byref(self._h)), "mbe_ctx_create")

    def close(self):
        if self._h and self._h.value:
            lib().mbe_ctx_destroy(self._h)
            self._h = _VP()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def upload(self, g: Graph):
        _check(lib().mbe_graph_upload(self._h, g.handle), "mbe_graph_upload")

    def release(self, g: Graph):
        _check(lib().mbe_graph_release(self._h, g.handle), "mbe_graph_release")

    def enumerate(self, g: Graph, variant: str = "cuMBE", min_rows: int = 0, min_cols: int = 0,
                  hash: bool = True, emit_cap: int = 0, emit_ids_cap: int = 0, **tuning) -> Result:
        """Counts (and hashes) the maximal bicliques of g.  emit_cap > 0 also
        returns them (MBE_OPT_EMIT) as Result.bicliques, a list of (rows,
        cols) tuples in file ids, with room for emit_cap bicliques and
        emit_ids_cap ids (default 64 per biclique); a run whose output does
        not fit raises, naming how many were written."""
        flags = OPT_TIMING | (0 if hash else OPT_NO_HASH) | (OPT_EMIT if emit_cap else 0) | \
            (OPT_L2_PIN if tuning.pop("l2_pin", False) else 0)
        o = _opts(flags=flags, min_rows=min_rows, min_cols=min_cols, **tuning)
        if emit_cap:
            ids_cap = emit_ids_cap or 64 * emit_cap
            offs = np.zeros(emit_cap + 1, dtype=np.uint32)
            nrows = np.zeros(emit_cap, dtype=np.uint32)
            ids = np.zeros(max(1, ids_cap), dtype=np.uint32)
            o.emit_offsets = offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
            o.emit_nrows = nrows.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
            o.emit_ids = ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
            o.emit_cap_bicliques = emit_cap
            o.emit_cap_ids = ids_cap
        r = _Result()
        _check(lib().mbe_enumerate(self._h, g.handle, VARIANTS[variant], ctypes.byref(o), ctypes.byref(r)),
               "mbe_enumerate")
        out = Result(r.count, r.hash, r.nodes, r.words, r.words_expand, r.ms, r.ms_prep)
        if emit_cap:
            bl = []
            for k in range(r.emitted):
                a, b = int(offs[k]), int(offs[k + 1])
                nr = int(nrows[k])
                bl.append((tuple(int(v) for v in ids[a:a + nr]), tuple(int(v) for v in ids[a + nr:b])))
            out.bicliques = bl
        return out

    def batch(self, graphs: list[Graph], variant: str = "cuMBE", min_rows: int = 0, min_cols: int = 0,
              host_chunks: bool = False, **tuning) -> tuple[list[Result], float]:
        """mbe_batch_run over `graphs`.  Its chunks launch as a captured CUDA
        graph; host_chunks=True drives them from the host instead
        (MBE_OPT_HOST_CHUNKS)."""
        n = len(graphs)
        arr = (_VP * n)(*[g.handle for g in graphs])
        res = (_Result * n)()
        tot = ctypes.c_float(0)
        o = _opts(flags=OPT_TIMING | (OPT_HOST_CHUNKS if host_chunks else 0), min_rows=min_rows, min_cols=min_cols,
                  **tuning)
        _check(lib().mbe_batch_run(self._h, arr, n, VARIANTS[variant], ctypes.byref(o), res, ctypes.byref(tot)),
               "mbe_batch_run")
        return [Result(r.count, r.hash, r.nodes, r.words, r.words_expand, r.ms, r.ms_prep) for r in res], tot.value

    def batch_tune(self, graphs: list[Graph], variant: str = "cuMBE", min_rows: int = 0,
                   min_cols: int = 0) -> list[dict]:
        """Autotunes the batched mode for the size buckets of `graphs`
        (mbe_batch_tune); later batch() calls on this device use the
        choices.  Returns one dict per bucket."""
        n = len(graphs)
        arr = (_VP * n)(*[g.handle for g in graphs])
        out = (_TuneChoice * 16)()
        k = ctypes.c_uint32()
        o = _opts(min_rows=min_rows, min_cols=min_cols)
        _check(lib().mbe_batch_tune(self._h, arr, n, VARIANTS[variant], ctypes.byref(o), out, 16, ctypes.byref(k)),
               "mbe_batch_tune")
        return [{f: getattr(out[i], f) for f, _ in _TuneChoice._fields_} for i in range(k.value)]

    def batch_tune_reset(self):
        _check(lib().mbe_batch_tune_reset(self._h), "mbe_batch_tune_reset")

    def counters(self) -> dict:
        """Cumulative kernel launches and host<->device bytes of this context."""
        l, h, d = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().mbe_ctx_counters(self._h, ctypes.byref(l), ctypes.byref(h), ctypes.byref(d)),
               "mbe_ctx_counters")
        return {"launches": l.value, "h2d": h.value, "d2h": d.value}

    def last_grid(self):
        a, b, c = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _check(lib().mbe_ctx_last_grid(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
               "mbe_ctx_last_grid")
        return a.value, b.value, c.value


def biclique_hash(rows, cols) -> int:
    r = np.ascontiguousarray(rows, dtype=np.uint32)
    c = np.ascontiguousarray(cols, dtype=np.uint32)
    r1 = r if r.size else np.zeros(1, np.uint32)
    c1 = c if c.size else np.zeros(1, np.uint32)
    return int(lib().mbe_biclique_hash(r1.ctypes.data_as(_U32P), r.size, c1.ctypes.data_as(_U32P), c.size))


class Server:
    """Continuous-batching enumeration service over device-resident graphs
    (mbe_server_*).  Requests are answered asynchronously; poll() returns
    finished ones with their timestamps on the server clock."""

    def __init__(self, device: int = 0, slots: int = 2, max_batch: int = 256, blocks_per_sm: int = 3,
                 variant: str = "cuMBE", mem_budget: int = 0, heavy_bytes: int = 0):
        cfg = _ServerConfig(slots, max_batch, blocks_per_sm, VARIANTS[variant], mem_budget, heavy_bytes)
        self._h = _VP()
        _check(lib().mbe_server_start(device, ctypes.byref(cfg), ctypes.byref(self._h)), "mbe_server_start")

    def add_graph(self, g: Graph) -> int:
        gid = ctypes.c_uint32()
        _check(lib().mbe_server_add_graph(self._h, g.handle, ctypes.byref(gid)), "mbe_server_add_graph")
        return gid.value

    def estimate(self, gid: int) -> int:
        b = ctypes.c_uint64()
        _check(lib().mbe_server_estimate(self._h, gid, ctypes.byref(b)), "mbe_server_estimate")
        return b.value

    def submit(self, gid: int, min_rows: int = 0, min_cols: int = 0) -> int:
        rid = ctypes.c_uint64()
        _check(lib().mbe_server_submit(self._h, gid, min_rows, min_cols, ctypes.byref(rid)), "mbe_server_submit")
        return rid.value

    def poll(self, cap: int = 4096) -> list[dict]:
        buf = (_RequestResult * cap)()
        n = ctypes.c_uint32()
        _check(lib().mbe_server_poll(self._h, buf, cap, ctypes.byref(n)), "mbe_server_poll")
        return [{f: getattr(buf[i], f) for f, _ in _RequestResult._fields_} for i in range(n.value)]

    def clock(self) -> float:
        return lib().mbe_server_clock(self._h)

    def warmup(self):
        """Sizes every slot's buffers for the graphs added so far (blocks
        until done)."""
        _check(lib().mbe_server_warmup(self._h), "mbe_server_warmup")

    def memory(self) -> dict:
        """Device bytes held: the slots' search buffers, the resident graphs,
        and the cap of one slot."""
        a, b, c = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().mbe_server_memory(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
               "mbe_server_memory")
        return {"search_bytes": a.value, "graph_bytes": b.value, "slot_cap": c.value}

    def stop(self):
        if self._h and self._h.value:
            _check(lib().mbe_server_stop(self._h), "mbe_server_stop")
            self._h = _VP()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass
