"""ctypes binding of the CPU oracle (oracle/mbe_oracle.c).

Test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module, as the checker or the timed CPU
baseline.  The product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC_PATH = os.path.join(HERE, "mbe_oracle.c")

VARIANTS = {"cuMBE": 0, "noRS": 1, "noES": 2, "noWS": 3}


class _Result(ctypes.Structure):
    _fields_ = [("count", ctypes.c_uint64), ("hash", ctypes.c_uint64),
                ("nodes", ctypes.c_uint64), ("scanned", ctypes.c_uint64)]


class _Gen(ctypes.Structure):
    _fields_ = [("n_rows", ctypes.c_uint32), ("n_cols", ctypes.c_uint32), ("n_edges", ctypes.c_uint64),
                ("gamma_rows", ctypes.c_double), ("gamma_cols", ctypes.c_double), ("max_deg", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("planted", ctypes.c_uint32), ("planted_rows", ctypes.c_uint32),
                ("planted_cols", ctypes.c_uint32), ("planted_density", ctypes.c_double)]


class _Emit(ctypes.Structure):
    _fields_ = [("cap_bicliques", ctypes.c_uint64), ("cap_ids", ctypes.c_uint64),
                ("n_bicliques", ctypes.c_uint64), ("n_ids", ctypes.c_uint64),
                ("offsets", ctypes.POINTER(ctypes.c_uint32)),
                ("nrows", ctypes.POINTER(ctypes.c_uint32)),
                ("ids", ctypes.POINTER(ctypes.c_uint32)),
                ("overflow", ctypes.c_int)]


@dataclass
class OracleResult:
    count: int
    hash: int
    nodes: int
    scanned: int
    bicliques: list | None = None


def build(force: bool = False) -> str:
    """Compiles liboracle.so with gcc (portable flags: x86 and Arm)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC_PATH):
        subprocess.check_call(["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-pthread",
                               "-fvisibility=hidden", SRC_PATH, "-o", LIB_PATH + ".tmp", "-lm"])
        os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        u64p = ctypes.POINTER(ctypes.c_uint64)
        u32p = ctypes.POINTER(ctypes.c_uint32)
        L.oracle_ref_enumerate.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u64p, u32p, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                                           ctypes.POINTER(_Result), ctypes.POINTER(_Emit)]
        L.oracle_ref_enumerate.restype = ctypes.c_int
        L.oracle_ref_enumerate_sampled.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u64p, u32p, ctypes.c_int,
                                                   ctypes.c_int, ctypes.c_int, ctypes.POINTER(_Result)]
        L.oracle_ref_enumerate_sampled.restype = ctypes.c_int
        L.oracle_ref_enumerate_roots.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u64p, u32p, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, ctypes.POINTER(_Result)]
        L.oracle_ref_enumerate_roots.restype = ctypes.c_int
        L.oracle_generate.argtypes = [ctypes.POINTER(_Gen), ctypes.POINTER(u64p), ctypes.POINTER(u32p),
                                      ctypes.POINTER(ctypes.c_uint64)]
        L.oracle_generate.restype = ctypes.c_int
        L.oracle_free.argtypes = [ctypes.c_void_p]
        L.oracle_free.restype = None
        L.oracle_brute.argtypes = [ctypes.c_uint32, ctypes.c_uint32, u64p, u32p, ctypes.c_uint32,
                                   ctypes.c_uint32, ctypes.POINTER(_Result), ctypes.POINTER(_Emit)]
        L.oracle_brute.restype = ctypes.c_int
        L.oracle_biclique_hash.argtypes = [u32p, ctypes.c_uint32, u32p, ctypes.c_uint32]
        L.oracle_biclique_hash.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _ptrs(row_ptr, col_idx):
    rp = np.ascontiguousarray(row_ptr, dtype=np.uint64)
    ci = np.ascontiguousarray(col_idx, dtype=np.uint32)
    if ci.size == 0:
        ci = np.zeros(1, dtype=np.uint32)
    return rp, ci, rp.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ci.ctypes.data_as(
        ctypes.POINTER(ctypes.c_uint32))


def _emit_buffers(cap_b, cap_ids):
    offs = np.zeros(cap_b + 1, dtype=np.uint32)
    nrows = np.zeros(cap_b, dtype=np.uint32)
    ids = np.zeros(cap_ids, dtype=np.uint32)
    em = _Emit(cap_b, cap_ids, 0, 0, offs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
               nrows.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
               ids.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), 0)
    return em, offs, nrows, ids


def _decode(em, offs, nrows, ids):
    out = []
    for i in range(em.n_bicliques):
        a, b = int(offs[i]), int(offs[i + 1])
        nr = int(nrows[i])
        out.append((tuple(int(v) for v in ids[a:a + nr]), tuple(int(v) for v in ids[a + nr:b])))
    return sorted(out)


def ref_enumerate(n_rows, n_cols, row_ptr, col_idx, variant="cuMBE", threads=1, min_rows=0, min_cols=0,
                  root_frac=0.0, emit_cap=0, emit_ids_cap=0) -> OracleResult:
    """Sequential (or root-parallel) restatement of the reference's search."""
    rp, ci, prp, pci = _ptrs(row_ptr, col_idx)
    res = _Result()
    em = None
    if emit_cap:
        em, offs, nrows, ids = _emit_buffers(emit_cap, emit_ids_cap or emit_cap * 64)
    rc = lib().oracle_ref_enumerate(n_rows, n_cols, prp, pci, VARIANTS[variant], threads, min_rows, min_cols,
                                    root_frac, ctypes.byref(res), ctypes.byref(em) if em else None)
    if rc != 0:
        raise RuntimeError(f"oracle_ref_enumerate failed rc={rc}")
    out = OracleResult(res.count, res.hash, res.nodes, res.scanned)
    if em:
        out.bicliques = _decode(em, offs, nrows, ids)
    return out


def ref_enumerate_sampled(n_rows, n_cols, row_ptr, col_idx, stride, variant="cuMBE", threads=1) -> OracleResult:
    """The restatement over every stride-th root only (a bounded timing sample)."""
    rp, ci, prp, pci = _ptrs(row_ptr, col_idx)
    res = _Result()
    rc = lib().oracle_ref_enumerate_sampled(n_rows, n_cols, prp, pci, VARIANTS[variant], threads, stride,
                                            ctypes.byref(res))
    if rc != 0:
        raise RuntimeError(f"oracle_ref_enumerate_sampled failed rc={rc}")
    return OracleResult(res.count, res.hash, res.nodes, res.scanned)


def ref_enumerate_roots(n_rows, n_cols, row_ptr, col_idx, root_begin=0, root_end=0, root_stride=1,
                        variant="cuMBE", threads=1, min_rows=0, min_cols=0) -> OracleResult:
    """The restatement over a root sample: processing positions p (degree
    ascending, id ascending, vertices with edges only) with root_begin <= p
    < root_end (0: no bound) and (p - root_begin) % root_stride == 0; the
    same sample mbe_opts.root_begin/root_end/root_stride selects."""
    rp, ci, prp, pci = _ptrs(row_ptr, col_idx)
    res = _Result()
    rc = lib().oracle_ref_enumerate_roots(n_rows, n_cols, prp, pci, VARIANTS[variant], threads, min_rows,
                                          min_cols, root_begin, root_end if root_end else -1, max(1, root_stride),
                                          ctypes.byref(res))
    if rc != 0:
        raise RuntimeError(f"oracle_ref_enumerate_roots failed rc={rc}")
    return OracleResult(res.count, res.hash, res.nodes, res.scanned)


def generate(n_rows, n_cols, n_edges, gamma_rows=2.1, gamma_cols=2.1, max_deg=0, seed=1, planted=0,
             planted_rows=0, planted_cols=0, planted_density=0.0):
    """The synthetic generator restated in the oracle (same graph as
    cumbe_gb300.Graph.generate): returns (n_rows, n_cols, row_ptr, col_idx)."""
    p = _Gen(n_rows, n_cols, n_edges, gamma_rows, gamma_cols, max_deg, seed, planted, planted_rows, planted_cols,
             planted_density)
    rp = ctypes.POINTER(ctypes.c_uint64)()
    ci = ctypes.POINTER(ctypes.c_uint32)()
    ne = ctypes.c_uint64()
    if lib().oracle_generate(ctypes.byref(p), ctypes.byref(rp), ctypes.byref(ci), ctypes.byref(ne)) != 0:
        raise RuntimeError("oracle_generate failed")
    try:
        row_ptr = np.ctypeslib.as_array(rp, shape=(n_rows + 1,)).copy()
        col_idx = np.ctypeslib.as_array(ci, shape=(max(1, ne.value),))[:ne.value].copy()
    finally:
        lib().oracle_free(ctypes.cast(rp, ctypes.c_void_p))
        lib().oracle_free(ctypes.cast(ci, ctypes.c_void_p))
    return n_rows, n_cols, row_ptr, col_idx


def brute(n_rows, n_cols, row_ptr, col_idx, min_rows=0, min_cols=0, emit_cap=0) -> OracleResult:
    rp, ci, prp, pci = _ptrs(row_ptr, col_idx)
    res = _Result()
    em = None
    if emit_cap:
        em, offs, nrows, ids = _emit_buffers(emit_cap, emit_cap * 96)
    rc = lib().oracle_brute(n_rows, n_cols, prp, pci, min_rows, min_cols, ctypes.byref(res),
                            ctypes.byref(em) if em else None)
    if rc != 0:
        raise RuntimeError(f"oracle_brute failed rc={rc}")
    out = OracleResult(res.count, res.hash, res.nodes, res.scanned)
    if em:
        out.bicliques = _decode(em, offs, nrows, ids)
    return out


def biclique_hash(rows, cols) -> int:
    r = np.ascontiguousarray(rows, dtype=np.uint32)
    c = np.ascontiguousarray(cols, dtype=np.uint32)
    r1 = r if r.size else np.zeros(1, np.uint32)
    c1 = c if c.size else np.zeros(1, np.uint32)
    return int(lib().oracle_biclique_hash(r1.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), r.size,
                                          c1.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), c.size))
