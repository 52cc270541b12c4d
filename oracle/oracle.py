"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module, and only as the checker or the timed CPU baseline.  The product
library never calls it.

Graphs are (offsets, col[, weight]) numpy arrays; offsets may be in the
sentinel form (n+1 entries) or the reference's n-entry form
(ptGraph/main.cu:97-121), converted by :func:`sentinel_offsets`.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libptg_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libptg_ref.so")

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)
_lib = None
_ref = None

UNREACHED = 0xFFFFFFFF


def build():
    """Compile the oracle library (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def build_ref(ref_dir=None):
    """Compile the reference-kernel harness into oracle/_ref (needs the reference sources)."""
    args = ["make", "-s", "-C", HERE, "ref"]
    if ref_dir:
        args.append("REF_DIR=" + ref_dir)
    subprocess.run(args, check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        u64, u32, f64 = ctypes.c_uint64, ctypes.c_uint32, ctypes.c_double
        sigs = {
            "orc_bfs_frontier": [u64, _u64p, _u32p, u32, u32, u32, _u32p],
            "orc_bfs_queue": [u64, _u64p, _u32p, u32, u32, u32, _u32p],
            "orc_sssp_frontier": [u64, _u64p, _u32p, _u32p, u32, u32, u32, _u32p],
            "orc_sssp_dijkstra": [u64, _u64p, _u32p, _u32p, u32, u32, u32, _u32p],
            "orc_cc_frontier": [u64, _u64p, _u32p, _u32p],
            "orc_cc_unionfind": [u64, _u64p, _u32p, _u32p],
            "orc_pagerank_f64": [u64, _u64p, _u32p, f64, u32, _f64p],
            "orc_ppr_f64": [u64, _u64p, _u32p, u32, f64, u32, _f64p],
            "orc_mt_bfs": [u64, _u64p, _u32p, u32, u32, _u32p],
            "orc_mt_sssp": [u64, _u64p, _u32p, _u32p, u32, u32, _u32p],
            "orc_mt_cc": [u64, _u64p, _u32p, u32, _u32p],
            "orc_mt_pagerank": [u64, _u64p, _u32p, f64, u32, u32, _f32p],
            "orc_sssp_certificate": [u64, _u64p, _u32p, _u32p, u32, u32, u32, _u32p, _u64p],
            "orc_mt_sssp_certificate": [u64, _u64p, _u32p, _u32p, u32, u32, u32, _u32p, u32, _u64p],
            "orc_mt_pagerank_f64": [u64, _u64p, _u32p, f64, u32, u32, _f64p],
            "orc_gen_rmat": [u32, u32, f64, f64, f64, u64, ctypes.c_int, u32, u32, u32,
                             _u64p, _u64p, ctypes.POINTER(_u64p), ctypes.POINTER(_u32p),
                             ctypes.POINTER(_u32p)],
            "orc_free": [ctypes.c_void_p],
        }
        for name, argt in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = argt
            fn.restype = ctypes.c_int if name.startswith(("orc_sssp", "orc_mt_sssp", "orc_gen")) else None
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def sentinel_offsets(offsets_n, m):
    """Reference n-entry offsets (ptGraph/main.cu:97-121) -> u64 sentinel form (n+1 entries)."""
    off = np.asarray(offsets_n, dtype=np.uint64)
    return np.ascontiguousarray(np.append(off, np.uint64(m)))


def _prep(off, col, w=None):
    """off must be the sentinel form: n+1 entries with off[n] == len(col)."""
    col = np.ascontiguousarray(col, dtype=np.uint32)
    off = np.ascontiguousarray(off, dtype=np.uint64)
    if off.size < 1 or int(off[-1]) != col.size:
        raise ValueError("offsets must have n+1 entries with offsets[n] == m")
    n = off.size - 1
    if w is not None:
        w = np.ascontiguousarray(w, dtype=np.uint32)
    if col.size == 0:
        col = np.zeros(1, dtype=np.uint32)
        if w is not None:
            w = np.zeros(1, dtype=np.uint32)
    return n, off, col, w


def bfs(off, col, src, base=1, unreached=UNREACHED, method="frontier"):
    n, off, col, _ = _prep(off, col)
    out = np.empty(n, dtype=np.uint32)
    fn = lib().orc_bfs_frontier if method == "frontier" else lib().orc_bfs_queue
    fn(n, _p(off, _u64p), _p(col, _u32p), src, base, unreached, _p(out, _u32p))
    return out


def sssp(off, col, w, src, base=1, unreached=UNREACHED, method="dijkstra"):
    n, off, col, w = _prep(off, col, w)
    out = np.empty(n, dtype=np.uint32)
    fn = lib().orc_sssp_dijkstra if method == "dijkstra" else lib().orc_sssp_frontier
    rc = fn(n, _p(off, _u64p), _p(col, _u32p), _p(w, _u32p), src, base, unreached, _p(out, _u32p))
    if rc != 0:
        raise OverflowError("SSSP distance does not fit in u32")
    return out


def sssp_certificate(off, col, w, src, dist, base=1, unreached=UNREACHED):
    """(ok, failed condition, vertex): checks dist as the exact SSSP answer
    from src in one pass over the edges (ptg_oracle.h, orc_sssp_certificate)."""
    n, off, col, w = _prep(off, col, w)
    dist = np.ascontiguousarray(dist, dtype=np.uint32)
    if dist.size != n:
        raise ValueError("dist must have n entries")
    bad = np.zeros(1, dtype=np.uint64)
    rc = lib().orc_sssp_certificate(n, _p(off, _u64p), _p(col, _u32p), _p(w, _u32p), src, base, unreached,
                                    _p(dist, _u32p), _p(bad, _u64p))
    return rc == 0, rc, int(bad[0])


def mt_sssp_certificate(off, col, w, src, dist, threads, base=1, unreached=UNREACHED):
    """sssp_certificate on `threads` host cores (same return values)."""
    n, off, col, w = _prep(off, col, w)
    dist = np.ascontiguousarray(dist, dtype=np.uint32)
    if dist.size != n:
        raise ValueError("dist must have n entries")
    bad = np.zeros(1, dtype=np.uint64)
    rc = lib().orc_mt_sssp_certificate(n, _p(off, _u64p), _p(col, _u32p), _p(w, _u32p), src, base, unreached,
                                       _p(dist, _u32p), threads, _p(bad, _u64p))
    return rc == 0, rc, int(bad[0])


def cc(off, col, method="frontier"):
    n, off, col, _ = _prep(off, col)
    out = np.empty(n, dtype=np.uint32)
    fn = lib().orc_cc_frontier if method == "frontier" else lib().orc_cc_unionfind
    fn(n, _p(off, _u64p), _p(col, _u32p), _p(out, _u32p))
    return out


def pagerank(off, col, d=0.85, iters=20):
    n, off, col, _ = _prep(off, col)
    out = np.empty(n, dtype=np.float64)
    lib().orc_pagerank_f64(n, _p(off, _u64p), _p(col, _u32p), d, iters, _p(out, _f64p))
    return out


def ppr(off, col, src, d=0.85, iters=20):
    n, off, col, _ = _prep(off, col)
    out = np.empty(n, dtype=np.float64)
    lib().orc_ppr_f64(n, _p(off, _u64p), _p(col, _u32p), src, d, iters, _p(out, _f64p))
    return out


def mt_pagerank_f64(off, col, threads, d=0.85, iters=20):
    """FP64 PageRank of a symmetric CSR on `threads` host cores (pull form of pagerank())."""
    n, off, col, _ = _prep(off, col)
    out = np.empty(n, dtype=np.float64)
    lib().orc_mt_pagerank_f64(n, _p(off, _u64p), _p(col, _u32p), d, iters, threads, _p(out, _f64p))
    return out


def gen_rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, symmetric=True, wmin=0, wmax=0,
             threads=0):
    """The benchmark's RMAT input, generated by the oracle's own restatement of
    the generator: (offsets u64 n+1, col u32, weight u32 or None)."""
    n = ctypes.c_uint64()
    m = ctypes.c_uint64()
    po, pc, pw = _u64p(), _u32p(), _u32p()
    rc = lib().orc_gen_rmat(scale, edge_factor, a, b, c, seed, 1 if symmetric else 0, wmin, wmax,
                            threads or (os.cpu_count() or 1), ctypes.byref(n), ctypes.byref(m),
                            ctypes.byref(po), ctypes.byref(pc), ctypes.byref(pw))
    if rc != 0:
        raise MemoryError("orc_gen_rmat failed (%d)" % rc) if rc == 2 else ValueError("orc_gen_rmat arguments")
    try:
        off = np.ctypeslib.as_array(po, (n.value + 1,)).copy()
        col = np.ctypeslib.as_array(pc, (max(1, m.value),))[:m.value].copy()
        w = np.ctypeslib.as_array(pw, (max(1, m.value),))[:m.value].copy() if wmax else None
    finally:
        for p in (po, pc, pw):
            if p:
                lib().orc_free(ctypes.cast(p, ctypes.c_void_p))
    return off, col, w


# --- multithreaded restatement (timed CPU baseline) ------------------------
def mt_bfs(off, col, src, threads):
    n, off, col, _ = _prep(off, col)
    out = np.empty(n, dtype=np.uint32)
    lib().orc_mt_bfs(n, _p(off, _u64p), _p(col, _u32p), src, threads, _p(out, _u32p))
    return out


def mt_sssp(off, col, w, src, threads):
    n, off, col, w = _prep(off, col, w)
    out = np.empty(n, dtype=np.uint32)
    lib().orc_mt_sssp(n, _p(off, _u64p), _p(col, _u32p), _p(w, _u32p), src, threads, _p(out, _u32p))
    return out


def mt_cc(off, col, threads):
    n, off, col, _ = _prep(off, col)
    out = np.empty(n, dtype=np.uint32)
    lib().orc_mt_cc(n, _p(off, _u64p), _p(col, _u32p), threads, _p(out, _u32p))
    return out


def mt_pagerank(off, col, threads, d=0.85, iters=20):
    n, off, col, _ = _prep(off, col)
    out = np.empty(n, dtype=np.float32)
    lib().orc_mt_pagerank(n, _p(off, _u64p), _p(col, _u32p), d, iters, threads, _p(out, _f32p))
    return out


# --- reference harness (oracle/_ref) ---------------------------------------
REF_VARIANTS = {
    "bfsCaculateInShare": 0, "bfsCaculateInOpt": 1, "bfsCaculateInAsync": 2,
    "bfsCaculateInAsyncSwap": 3, "caculateInCommon": 4, "caculateInShareOpt": 5,
    "caculateInOptChooseByDegree": 6, "ssspCaculateInShare": 10, "ssspCaculateInOpt": 11,
    "ccCaculateInShare": 20, "ccCaculateInOpt": 21,
}


def ref_available():
    return os.path.exists(REF_LIB_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        L = ctypes.CDLL(REF_LIB_PATH)
        L.ref_run.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, _u32p, _u32p, _u32p,
                              _u32p, ctypes.c_uint64, ctypes.c_uint32, _u32p, _u32p]
        L.ref_run.restype = ctypes.c_int
        _ref = L
    return _ref


def ref_run(variant, off_n, col, weight=None, src=0, budget_edges=None, fragment_size=4096):
    """Run one reference entry point's kernels (emulated on the host).

    off_n: the reference's n-entry offsets (u32).  Returns (values, iterations, src).
    """
    off_n = np.ascontiguousarray(off_n, dtype=np.uint32)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    n, m = off_n.size, col.size
    if budget_edges is None:
        budget_edges = m + 1
    w = None if weight is None else np.ascontiguousarray(weight, dtype=np.uint32)
    out = np.empty(n, dtype=np.uint32)
    iters = np.zeros(1, dtype=np.uint32)
    srcv = np.array([src], dtype=np.uint32)
    colp = col if m else np.zeros(1, dtype=np.uint32)
    rc = ref_lib().ref_run(REF_VARIANTS[variant] if isinstance(variant, str) else variant, n, m,
                           _p(off_n, _u32p), _p(colp, _u32p),
                           None if w is None else _p(w, _u32p), _p(srcv, _u32p),
                           int(budget_edges), fragment_size, _p(out, _u32p), _p(iters, _u32p))
    if rc != 0:
        raise RuntimeError("reference harness returned %d for %s" % (rc, variant))
    return out, int(iters[0]), int(srcv[0])
