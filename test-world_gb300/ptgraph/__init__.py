"""Python binding of libptgraph (ctypes over the C ABI in include/ptgraph.h).

The engine itself is C++/CUDA; this module only marshals numpy arrays into
the C ABI, the way a host program would bind it.  There is no Python or CPU
fallback: if the shared library is missing, :func:`lib` raises.

Reference mapping (ptGraph/main.cu:24-56):
  bfsCaculateIn{Opt,Async,AsyncSwap,Share}  -> Graph.bfs / compat.*
  ssspCaculateIn{Opt,Share}                 -> Graph.sssp
  ccCaculateIn{Opt,Share}                   -> Graph.cc
  prCaculateIn{Share,Opt} (a stub there)    -> Graph.pagerank
"""
import atexit
import ctypes
import weakref
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "_build", "libptgraph.so")

PTG_OK, PTG_ERR_INVALID, PTG_ERR_OOM, PTG_ERR_CUDA, PTG_ERR_TIMEOUT = 0, 1, 2, 3, 4
PTG_ERR_UNSUPPORTED, PTG_ERR_NO_DEVICE, PTG_ERR_CANCELLED, PTG_ERR_BUSY = 5, 6, 7, 8
PTG_OFFSETS_U32, PTG_OFFSETS_U64 = 0, 1
PTG_FORM_SENTINEL, PTG_FORM_REFERENCE = 0, 1
PTG_CSR_SYMMETRIC, PTG_CSR_HOST_PINNED, PTG_CSR_WIDE_OFFSETS = 1, 2, 4
PTG_RESIDENT_PREFIX, PTG_RESIDENT_NONE, PTG_RESIDENT_HOT, PTG_RESIDENT_HUBS = 0, 1, 2, 3
PTG_OUT_DEVICE, PTG_LEVEL_ZERO_BASED, PTG_UNREACHED_MINUS1 = 1, 2, 4
PTG_NO_DIRECTION_OPT, PTG_REFERENCE_SCHEDULE = 8, 16
PTG_Q_BFS, PTG_Q_SSSP, PTG_Q_PPR = 0, 1, 2
UNREACHED = 0xFFFFFFFF

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p


class PtgError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d): %s" % (_STATUS.get(status, "?"), status, msg))
        self.status = status


_STATUS = {0: "ok", 1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "timeout",
           5: "unsupported", 6: "no CUDA device", 7: "cancelled", 8: "busy"}


class Csr(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint64), ("m", ctypes.c_uint64), ("offsets", _vp),
                ("offset_type", ctypes.c_uint32), ("offset_form", ctypes.c_uint32),
                ("col", _vp), ("weight", _vp), ("edges_aos", _vp),
                ("flags", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class PartitionConfig(ctypes.Structure):
    _fields_ = [("partition_bytes", ctypes.c_uint64), ("device_budget_bytes", ctypes.c_uint64),
                ("device_frac", ctypes.c_double), ("n_staging_buffers", ctypes.c_uint32),
                ("resident_policy", ctypes.c_uint32), ("force_out_of_core", ctypes.c_uint32),
                ("hot_threshold", ctypes.c_uint32)]


class RunStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_uint32), ("bottom_up_rounds", ctypes.c_uint32),
                ("edges_relaxed", ctypes.c_uint64), ("vertices_reached", ctypes.c_uint64),
                ("edges_in_component", ctypes.c_uint64), ("link_bytes", ctypes.c_uint64),
                ("partitions_streamed", ctypes.c_uint64), ("partitions_skipped", ctypes.c_uint64),
                ("partitions_cached", ctypes.c_uint64),
                ("device_ms", ctypes.c_double), ("link_ms", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class RunOpts(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_uint32), ("delta", ctypes.c_uint32),
                ("max_iterations", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("stats", ctypes.POINTER(RunStats))]


class PrOpts(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_uint32), ("iterations", ctypes.c_uint32),
                ("damping", ctypes.c_double), ("stats", ctypes.POINTER(RunStats))]


class GraphInfo(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint64), ("m", ctypes.c_uint64), ("symmetric", ctypes.c_uint32),
                ("weighted", ctypes.c_uint32), ("out_of_core", ctypes.c_uint32),
                ("offsets_u64", ctypes.c_uint32), ("partitions", ctypes.c_uint64),
                ("resident_partitions", ctypes.c_uint64), ("partition_edges", ctypes.c_uint64),
                ("resident_edges", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64),
                ("degree_grouped", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class HostCsr(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint64), ("m", ctypes.c_uint64), ("offsets", _u64p),
                ("col", _u32p), ("weight", _u32p), ("pinned", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("lanes", ctypes.c_uint32), ("max_slots", ctypes.c_uint32), ("max_batch", ctypes.c_uint32),
                ("queue_capacity", ctypes.c_uint32), ("ppr_iterations", ctypes.c_uint32),
                ("no_calibration", ctypes.c_uint32), ("ppr_damping", ctypes.c_double),
                ("memory_budget_bytes", ctypes.c_uint64), ("schedule", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("max_batch_seen", ctypes.c_uint64),
                ("budget_bytes", ctypes.c_uint64), ("committed_bytes", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("resident_graphs", ctypes.c_uint32),
                ("streamed_graphs", ctypes.c_uint32), ("busy_ms", ctypes.c_double),
                ("fused_requests", ctypes.c_uint64 * 3), ("single_requests", ctypes.c_uint64 * 3),
                ("fused_batches", ctypes.c_uint64 * 3), ("fused_ms", ctypes.c_double * 3),
                ("single_ms", ctypes.c_double * 3)]


PTG_TUNING_VERSION = 1


class Tuning(ctypes.Structure):
    _fields_ = [("version", ctypes.c_uint32), ("bfs_alpha", ctypes.c_float), ("bfs_beta", ctypes.c_float),
                ("sssp_delta_scale", ctypes.c_float), ("expand_ctas_per_sm", ctypes.c_uint32),
                ("pr_ctas_per_sm", ctypes.c_uint32), ("pr_mid", ctypes.c_uint32), ("pr_chunk", ctypes.c_uint32),
                ("ms_pull_small", ctypes.c_uint32), ("ms_pull_chunk", ctypes.c_uint32),
                ("vertex_order", ctypes.c_uint32), ("reserved0", ctypes.c_uint32),
                ("partition_bytes", ctypes.c_uint64),
                ("reserved", ctypes.c_uint32 * 8)]

    KNOBS = ("bfs_alpha", "bfs_beta", "sssp_delta_scale", "expand_ctas_per_sm", "pr_ctas_per_sm", "pr_mid",
             "pr_chunk", "ms_pull_small", "ms_pull_chunk", "vertex_order", "partition_bytes")

    def as_dict(self):
        return {k: (round(float(getattr(self, k)), 6) if isinstance(getattr(self, k), float) else int(getattr(self, k)))
                for k in self.KNOBS}


def tuning_defaults():
    """The built-in tuning values as a dict (no GPU needed)."""
    t = Tuning()
    lib().ptg_tuning_defaults(ctypes.byref(t))
    return t.as_dict()


def _tuning_struct(values):
    t = Tuning()
    lib().ptg_tuning_defaults(ctypes.byref(t))
    for k, v in values.items():
        if k not in Tuning.KNOBS:
            raise KeyError("unknown tuning knob %r" % k)
        setattr(t, k, v)
    return t


def tuning_valid(values):
    """True if the library accepts these knob values (no GPU needed)."""
    return lib().ptg_tuning_validate(ctypes.byref(_tuning_struct(values))) == PTG_OK


# Every function the header declares, with its ctypes signature.
_SIGS = {
    "ptg_tuning_defaults": (None, [ctypes.POINTER(Tuning)]),
    "ptg_tuning_validate": (ctypes.c_int, [ctypes.POINTER(Tuning)]),
    "ptg_ctx_set_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(Tuning)]),
    "ptg_ctx_get_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(Tuning)]),
    "ptg_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "ptg_partition_config_default": (None, [ctypes.POINTER(PartitionConfig)]),
    "ptg_plan_partitions": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, _u64p, ctypes.c_uint64,
                                           ctypes.POINTER(PartitionConfig), ctypes.c_uint64, _u64p,
                                           _u64p, _u64p, _u64p]),
    "ptg_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp)]),
    "ptg_ctx_destroy": (None, [_vp]),
    "ptg_ctx_release_cache": (ctypes.c_int, [_vp]),
    "ptg_ctx_last_error": (ctypes.c_char_p, [_vp]),
    "ptg_ctx_device_info": (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_int), _u64p, _u64p]),
    "ptg_ctx_profile_enable": (ctypes.c_int, [_vp, ctypes.c_int]),
    "ptg_ctx_launch_count": (ctypes.c_uint64, [_vp]),
    "ptg_ctx_profile_entries": (ctypes.c_uint32, [_vp]),
    "ptg_ctx_profile_entry": (ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.POINTER(ctypes.c_char_p), _u64p,
                                             ctypes.POINTER(ctypes.c_double)]),
    "ptg_graph_create": (ctypes.c_int, [_vp, ctypes.POINTER(Csr), ctypes.POINTER(PartitionConfig),
                                        ctypes.POINTER(_vp)]),
    "ptg_graph_destroy": (None, [_vp]),
    "ptg_graph_info_get": (ctypes.c_int, [_vp, ctypes.POINTER(GraphInfo)]),
    "ptg_bfs": (ctypes.c_int, [_vp, ctypes.c_uint32, _vp, ctypes.POINTER(RunOpts)]),
    "ptg_sssp": (ctypes.c_int, [_vp, ctypes.c_uint32, _vp, ctypes.POINTER(RunOpts)]),
    "ptg_cc": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(RunOpts)]),
    "ptg_pagerank": (ctypes.c_int, [_vp, _vp, ctypes.POINTER(PrOpts)]),
    "ptg_ppr": (ctypes.c_int, [_vp, ctypes.c_uint32, _vp, ctypes.POINTER(PrOpts)]),
    "ptg_ppr_batch": (ctypes.c_int, [_vp, _u32p, ctypes.c_uint32, _vp, ctypes.POINTER(PrOpts)]),
    "ptg_bfs_noalloc": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp,
                                       _vp]),
    "ptg_msbfs": (ctypes.c_int, [_vp, _u32p, ctypes.c_uint32, _vp, ctypes.POINTER(RunOpts)]),
    "ptg_mssssp": (ctypes.c_int, [_vp, _u32p, ctypes.c_uint32, _vp, ctypes.POINTER(RunOpts)]),
    "ptg_cc_batch": (ctypes.c_int, [_vp, ctypes.c_uint32, _u64p, _u64p, _u32p, _u32p,
                                    ctypes.POINTER(RunOpts)]),
    "ptg_server_create": (ctypes.c_int, [_vp, ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)]),
    "ptg_server_destroy": (None, [_vp]),
    "ptg_server_add_graph": (ctypes.c_int, [_vp, _vp, _u32p]),
    "ptg_server_upload": (ctypes.c_int, [_vp, ctypes.POINTER(Csr), _u32p, _u32p]),
    "ptg_server_submit": (ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _vp,
                                         _u64p]),
    "ptg_server_wait": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_int64,
                                       ctypes.POINTER(ctypes.c_double)]),
    "ptg_server_drain": (ctypes.c_int, [_vp]),
    "ptg_server_stats_get": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    "ptg_read_csr_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(HostCsr)]),
    "ptg_write_csr_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint32, ctypes.POINTER(HostCsr)]),
    "ptg_gen_rmat": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_uint64, ctypes.c_int, ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int,
                                    ctypes.POINTER(HostCsr)]),
    "ptg_gen_er_batch": (ctypes.c_int, [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
                                        ctypes.c_double, ctypes.c_uint64, ctypes.c_uint32,
                                        ctypes.POINTER(HostCsr), ctypes.POINTER(_u64p)]),
    "ptg_host_csr_free": (None, [ctypes.POINTER(HostCsr)]),
    "ptg_free": (None, [_vp]),
    "bfsCaculateInOpt": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p, ctypes.c_uint]),
    "bfsCaculateInAsync": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p, ctypes.c_uint]),
    "bfsCaculateInAsyncSwap": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p,
                                               ctypes.c_uint]),
    "bfsCaculateInShare": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p, ctypes.c_uint]),
    "ssspCaculateInShare": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _vp, ctypes.c_uint]),
    "ssspCaculateInOpt": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _vp, ctypes.c_uint]),
    "ccCaculateInShare": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p]),
    "ccCaculateInOpt": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p]),
    "prCaculateInShare": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p]),
    "prCaculateInOpt": (ctypes.c_long, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p]),
    "caculateInCommon": (None, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p]),
    "caculateInShareOpt": (None, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p]),
    "caculateInOptChooseByDegree": (None, [ctypes.c_uint, ctypes.c_uint, _u32p, _u32p, ctypes.c_uint]),
    "ptg_compat_last_result": (ctypes.c_uint64, [_u32p, ctypes.c_uint64]),
    "ptg_compat_last_result_f32": (ctypes.c_uint64, [_f32p, ctypes.c_uint64]),
    "ptg_compat_last_error": (ctypes.c_char_p, []),
    "ptg_compat_set_partition_config": (None, [ctypes.POINTER(PartitionConfig)]),
    "ptg_compat_set_device": (None, [ctypes.c_int]),
}

_lib = None


def lib():
    """Load libptgraph.so (built by test-world_gb300/build.py); raises if absent."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError("libptgraph.so not built (run test-world_gb300/build.py): %s" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status, ctx=None):
    if status != PTG_OK:
        msg = lib().ptg_ctx_last_error(ctx).decode() if ctx else ""
        raise PtgError(status, msg)


def _ptr(a):
    """Address of a numpy array, or of a device tensor (anything with data_ptr())."""
    if hasattr(a, "data_ptr"):
        return _vp(a.data_ptr())
    return a.ctypes.data_as(_vp)


def partition_config(**kw):
    cfg = PartitionConfig()
    lib().ptg_partition_config_default(ctypes.byref(cfg))
    for k, v in kw.items():
        setattr(cfg, k, v)
    return cfg


_LIVE_CTX = weakref.WeakSet()


@atexit.register
def _close_live_contexts():
    """Close contexts still open at interpreter exit (servers, then graphs,
    then the context), while the CUDA runtime and this module are intact;
    module teardown would otherwise destroy them in arbitrary order."""
    for c in list(_LIVE_CTX):
        try:
            c.close()
        except Exception:
            pass


class Ctx:
    """A context on one CUDA device (owns streams and reusable workspace)."""

    def __init__(self, device=0):
        self.device = device
        self.h = _vp()
        self._deps = weakref.WeakSet()  # graphs and servers, closed before the context
        _check(lib().ptg_ctx_create(device, ctypes.byref(self.h)))
        _LIVE_CTX.add(self)

    def close(self):
        if self.h:
            deps = list(self._deps)
            for d in sorted(deps, key=lambda d: not isinstance(d, Server)):  # servers before graphs
                d.close()
            lib().ptg_ctx_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_info(self):
        sms = ctypes.c_int()
        hbm = ctypes.c_uint64()
        free = ctypes.c_uint64()
        _check(lib().ptg_ctx_device_info(self.h, ctypes.byref(sms), ctypes.byref(hbm),
                                         ctypes.byref(free)), self.h)
        return {"sm_count": sms.value, "hbm_bytes": hbm.value, "free_bytes": free.value}

    def release_cache(self):
        """Return the engine's cached device blocks on this device to the driver."""
        _check(lib().ptg_ctx_release_cache(self.h), self.h)

    def tuning(self):
        """The context's tuning knobs as a dict."""
        t = Tuning()
        _check(lib().ptg_ctx_get_tuning(self.h, ctypes.byref(t)), self.h)
        return t.as_dict()

    def set_tuning(self, values=None, **kw):
        """Apply tuning knobs (unnamed ones take the built-in defaults)."""
        v = dict(values or {})
        v.update(kw)
        _check(lib().ptg_ctx_set_tuning(self.h, ctypes.byref(_tuning_struct(v))), self.h)

    def load_tuning(self, path):
        """Apply the "tuning" object of an autotuner JSON file (ptgraph.tune)."""
        import json
        with open(path) as f:
            doc = json.load(f)
        self.set_tuning(doc.get("tuning", doc))
        return self.tuning()

    def profile(self, enable=True):
        """Enable/disable per-kernel CUDA-event timing (clears the totals)."""
        _check(lib().ptg_ctx_profile_enable(self.h, 1 if enable else 0), self.h)

    def launch_count(self):
        return lib().ptg_ctx_launch_count(self.h)

    def profile_entries(self):
        """{kernel name: (launches, total ms)} since profiling was enabled."""
        out = {}
        for i in range(lib().ptg_ctx_profile_entries(self.h)):
            name = ctypes.c_char_p()
            cnt = ctypes.c_uint64()
            ms = ctypes.c_double()
            _check(lib().ptg_ctx_profile_entry(self.h, i, ctypes.byref(name), ctypes.byref(cnt),
                                               ctypes.byref(ms)), self.h)
            out[name.value.decode()] = (cnt.value, ms.value)
        return out

    def graph(self, offsets, col, weight=None, symmetric=False, form=PTG_FORM_SENTINEL,
              edges_aos=None, config=None, pinned=False, wide_offsets=False):
        return Graph(self, offsets, col, weight, symmetric, form, edges_aos, config, pinned, wide_offsets)

    def cc_batch(self, vtx_begin, offsets, col, stats=None):
        vb = np.ascontiguousarray(vtx_begin, dtype=np.uint64)
        off = np.ascontiguousarray(offsets, dtype=np.uint64)
        col = np.ascontiguousarray(col, dtype=np.uint32)
        n = int(vb[-1])
        out = np.empty(n, dtype=np.uint32)
        o = RunOpts()
        st = RunStats()
        o.stats = ctypes.pointer(st)
        _check(lib().ptg_cc_batch(self.h, vb.size - 1, vb.ctypes.data_as(_u64p), off.ctypes.data_as(_u64p),
                                  col.ctypes.data_as(_u32p), out.ctypes.data_as(_u32p),
                                  ctypes.byref(o)), self.h)
        if stats is not None:
            stats.update(st.as_dict())
        return out


class Graph:
    """An uploaded CSR (resident in HBM, or resident prefix + streamed partitions)."""

    def __init__(self, ctx, offsets, col, weight=None, symmetric=False, form=PTG_FORM_SENTINEL,
                 edges_aos=None, config=None, pinned=False, wide_offsets=False):
        self.ctx = ctx
        off = np.ascontiguousarray(offsets)
        if off.dtype not in (np.uint32, np.uint64):
            off = off.astype(np.uint64)
        self._off = off
        self._col = None if col is None else np.ascontiguousarray(col, dtype=np.uint32)
        self._w = None if weight is None else np.ascontiguousarray(weight, dtype=np.uint32)
        self._aos = None if edges_aos is None else np.ascontiguousarray(edges_aos, dtype=np.uint32)
        m = self._col.size if self._col is not None else self._aos.size // 2
        n = off.size - 1 if form == PTG_FORM_SENTINEL else off.size
        c = Csr()
        c.n, c.m = n, m
        c.offsets = _ptr(off)
        c.offset_type = PTG_OFFSETS_U64 if off.dtype == np.uint64 else PTG_OFFSETS_U32
        c.offset_form = form
        c.col = _ptr(self._col) if self._col is not None and m else None
        c.weight = _ptr(self._w) if self._w is not None and m else None
        c.edges_aos = _ptr(self._aos) if self._aos is not None and m else None
        c.flags = ((PTG_CSR_SYMMETRIC if symmetric else 0) | (PTG_CSR_HOST_PINNED if pinned else 0) |
                   (PTG_CSR_WIDE_OFFSETS if wide_offsets else 0))
        if m == 0:
            # a graph without edges still needs a valid (unused) edge pointer
            self._col = np.zeros(1, dtype=np.uint32)
            c.col = _ptr(self._col)
        self.n, self.m = n, m
        self.h = _vp()
        _check(lib().ptg_graph_create(ctx.h, ctypes.byref(c), ctypes.byref(config) if config else None,
                                      ctypes.byref(self.h)), ctx.h)
        ctx._deps.add(self)

    def close(self):
        if self.h:
            lib().ptg_graph_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        gi = GraphInfo()
        _check(lib().ptg_graph_info_get(self.h, ctypes.byref(gi)))
        return {f: getattr(gi, f) for f, _ in gi._fields_}

    def _opts(self, flags, delta, stats):
        o = RunOpts()
        o.flags = flags
        o.delta = delta
        st = RunStats()
        o.stats = ctypes.pointer(st)
        return o, st

    def bfs(self, src, flags=0, stats=None, out=None):
        out = np.empty(self.n, dtype=np.uint32) if out is None else out
        o, st = self._opts(flags, 0, stats)
        _check(lib().ptg_bfs(self.h, src, _ptr(out), ctypes.byref(o)), self.ctx.h)
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def sssp(self, src, flags=0, delta=0, stats=None, out=None):
        out = np.empty(self.n, dtype=np.uint32) if out is None else out
        o, st = self._opts(flags, delta, stats)
        _check(lib().ptg_sssp(self.h, src, _ptr(out), ctypes.byref(o)), self.ctx.h)
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def cc(self, flags=0, stats=None, out=None):
        out = np.empty(self.n, dtype=np.uint32) if out is None else out
        o, st = self._opts(flags, 0, stats)
        _check(lib().ptg_cc(self.h, _ptr(out), ctypes.byref(o)), self.ctx.h)
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def pagerank(self, iterations=20, damping=0.85, stats=None, out=None, flags=0):
        out = np.empty(self.n, dtype=np.float32) if out is None else out
        o = PrOpts()
        o.flags, o.iterations, o.damping = flags, iterations, damping
        st = RunStats()
        o.stats = ctypes.pointer(st)
        _check(lib().ptg_pagerank(self.h, _ptr(out), ctypes.byref(o)), self.ctx.h)
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def ppr(self, src, iterations=20, damping=0.85, stats=None, out=None, flags=0):
        out = np.empty(self.n, dtype=np.float32) if out is None else out
        o = PrOpts()
        o.flags, o.iterations, o.damping = flags, iterations, damping
        st = RunStats()
        o.stats = ctypes.pointer(st)
        _check(lib().ptg_ppr(self.h, src, _ptr(out), ctypes.byref(o)), self.ctx.h)
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def ppr_batch(self, sources, iterations=20, damping=0.85, stats=None, out=None, flags=0):
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        out = np.empty((s.size, self.n), dtype=np.float32) if out is None else out
        o = PrOpts()
        o.flags, o.iterations, o.damping = flags, iterations, damping
        st = RunStats()
        o.stats = ctypes.pointer(st)
        _check(lib().ptg_ppr_batch(self.h, s.ctypes.data_as(_u32p), s.size, _ptr(out), ctypes.byref(o)),
               self.ctx.h)
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def msbfs(self, sources, flags=0, stats=None, out=None):
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        out = np.empty((s.size, self.n), dtype=np.uint32) if out is None else out
        o, st = self._opts(flags, 0, stats)
        _check(lib().ptg_msbfs(self.h, s.ctypes.data_as(_u32p), s.size, _ptr(out), ctypes.byref(o)),
               self.ctx.h)
        if stats is not None:
            stats.update(st.as_dict())
        return out

    def mssssp(self, sources, flags=0, stats=None, out=None):
        s = np.ascontiguousarray(sources, dtype=np.uint32)
        out = np.empty((s.size, self.n), dtype=np.uint32) if out is None else out
        o, st = self._opts(flags, 0, stats)
        _check(lib().ptg_mssssp(self.h, s.ctypes.data_as(_u32p), s.size, _ptr(out), ctypes.byref(o)),
               self.ctx.h)
        if stats is not None:
            stats.update(st.as_dict())
        return out


class Server:
    """Request server (ptg_server_*): queries on registered graphs, served by
    lanes that batch requests of the same graph and kind into fused passes."""

    def __init__(self, ctx, lanes=0, max_slots=0, max_batch=0, queue_capacity=0, ppr_iterations=0,
                 ppr_damping=0.0, memory_budget_bytes=0, calibrate=True, schedule=0):
        cfg = ServerConfig()
        cfg.no_calibration = 0 if calibrate else 1
        cfg.schedule = schedule
        cfg.lanes, cfg.max_slots, cfg.max_batch = lanes, max_slots, max_batch
        cfg.queue_capacity, cfg.ppr_iterations, cfg.ppr_damping = queue_capacity, ppr_iterations, ppr_damping
        cfg.memory_budget_bytes = memory_budget_bytes
        self.ctx = ctx
        self.h = _vp()
        _check(lib().ptg_server_create(ctx.h, ctypes.byref(cfg), ctypes.byref(self.h)), ctx.h)
        ctx._deps.add(self)
        self._keep = []      # graphs and uploaded arrays the server reads
        self._n = {}         # graph id -> vertices
        self._out = {}       # request id -> result buffer

    def add_graph(self, graph):
        gid = ctypes.c_uint32()
        _check(lib().ptg_server_add_graph(self.h, graph.h, ctypes.byref(gid)), self.ctx.h)
        self._keep.append(graph)
        self._n[gid.value] = graph.n
        return gid.value

    def upload(self, offsets, col, weight=None, symmetric=True):
        """Upload a sentinel-form CSR; returns (graph id, resident)."""
        off = np.ascontiguousarray(offsets)
        if off.dtype not in (np.uint32, np.uint64):
            off = off.astype(np.uint64)
        col = np.ascontiguousarray(col, dtype=np.uint32)
        w = None if weight is None else np.ascontiguousarray(weight, dtype=np.uint32)
        c = Csr()
        c.n, c.m = off.size - 1, col.size
        c.offsets = _ptr(off)
        c.offset_type = PTG_OFFSETS_U64 if off.dtype == np.uint64 else PTG_OFFSETS_U32
        c.offset_form = PTG_FORM_SENTINEL
        if col.size == 0:
            col = np.zeros(1, dtype=np.uint32)
        c.col = _ptr(col)
        c.weight = _ptr(w) if w is not None and c.m else None
        c.flags = PTG_CSR_SYMMETRIC if symmetric else 0
        gid = ctypes.c_uint32()
        res = ctypes.c_uint32()
        _check(lib().ptg_server_upload(self.h, ctypes.byref(c), ctypes.byref(gid), ctypes.byref(res)),
               self.ctx.h)
        self._keep.append((off, col, w))
        self._n[gid.value] = off.size - 1
        return gid.value, bool(res.value)

    def submit(self, gid, kind, src, out=None):
        """Queue a query; out (numpy array or CUDA tensor of n values) receives the result."""
        if out is None:
            out = np.empty(self._n.get(gid, 1), dtype=np.float32 if kind == PTG_Q_PPR else np.uint32)
        rid = ctypes.c_uint64()
        _check(lib().ptg_server_submit(self.h, gid, kind, src, _ptr(out), ctypes.byref(rid)), self.ctx.h)
        self._out[rid.value] = out
        return rid.value

    def wait(self, rid, timeout_ms=-1):
        """Wait for a request; returns (result, latency in microseconds)."""
        lat = ctypes.c_double()
        s = lib().ptg_server_wait(self.h, rid, timeout_ms, ctypes.byref(lat))
        if s == PTG_ERR_TIMEOUT:
            raise PtgError(s, "request not done in time")
        out = self._out.pop(rid, None)
        _check(s, self.ctx.h)
        return out, lat.value

    def drain(self):
        _check(lib().ptg_server_drain(self.h), self.ctx.h)

    def stats(self):
        st = ServerStats()
        _check(lib().ptg_server_stats_get(self.h, ctypes.byref(st)), self.ctx.h)
        return {f: (list(getattr(st, f)) if isinstance(getattr(st, f), ctypes.Array) else getattr(st, f))
                for f, _ in st._fields_}

    def close(self):
        if self.h:
            lib().ptg_server_destroy(self.h)
            self.h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def plan_partitions(offsets_n1, bytes_per_edge, device_free_bytes, config=None):
    """Host-only partition plan: (num_partitions, resident_partitions, partition_edges, first_vertex)."""
    off = np.ascontiguousarray(offsets_n1, dtype=np.uint64)
    n, m = off.size - 1, int(off[-1])
    P, R, PE = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    cfg = ctypes.byref(config) if config else None
    _check(lib().ptg_plan_partitions(n, m, off.ctypes.data_as(_u64p), bytes_per_edge, cfg,
                                     device_free_bytes, ctypes.byref(P), None, None, None))
    first = np.empty(P.value + 1, dtype=np.uint64)
    _check(lib().ptg_plan_partitions(n, m, off.ctypes.data_as(_u64p), bytes_per_edge, cfg,
                                     device_free_bytes, ctypes.byref(P), ctypes.byref(R),
                                     ctypes.byref(PE), first.ctypes.data_as(_u64p)))
    return P.value, R.value, PE.value, first


def _take(hc, weighted):
    n, m = hc.n, hc.m
    off = np.ctypeslib.as_array(hc.offsets, shape=(n + 1,)).copy()
    col = np.ctypeslib.as_array(hc.col, shape=(max(m, 1),))[:m].copy()
    w = np.ctypeslib.as_array(hc.weight, shape=(max(m, 1),))[:m].copy() if weighted else None
    lib().ptg_host_csr_free(ctypes.byref(hc))
    return off, col, w


def gen_rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, symmetric=True, wmin=0, wmax=0,
             threads=0):
    """RMAT graph as numpy arrays (offsets u64 n+1, col u32, weight u32 or None)."""
    hc = HostCsr()
    _check(lib().ptg_gen_rmat(scale, edge_factor, a, b, c, seed, 1 if symmetric else 0, wmin, wmax,
                              threads, 0, ctypes.byref(hc)))
    return _take(hc, wmax > 0)


class HostGraph:
    """A host CSR owned by the library, seen as numpy arrays without a copy
    (offsets u64 n+1, col u32, weight u32 or None); pinned when asked, so an
    out-of-core graph streams from it as it is (ctx.graph(..., pinned=True)).
    close() frees it; the arrays must not be used after."""

    def __init__(self, hc, weighted):
        self._hc = hc
        n, m = hc.n, hc.m
        self.offsets = np.ctypeslib.as_array(hc.offsets, shape=(n + 1,))
        self.col = np.ctypeslib.as_array(hc.col, shape=(max(m, 1),))[:m]
        self.weight = np.ctypeslib.as_array(hc.weight, shape=(max(m, 1),))[:m] if weighted else None
        self.pinned = bool(hc.pinned)

    def close(self):
        if self._hc is not None:
            self.offsets = self.col = self.weight = None
            lib().ptg_host_csr_free(ctypes.byref(self._hc))
            self._hc = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gen_rmat_host(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1, symmetric=True, wmin=0, wmax=0,
                  threads=0, pinned=True):
    """gen_rmat into library-owned (pinned) memory, returned as a HostGraph."""
    hc = HostCsr()
    _check(lib().ptg_gen_rmat(scale, edge_factor, a, b, c, seed, 1 if symmetric else 0, wmin, wmax,
                              threads, 1 if pinned else 0, ctypes.byref(hc)))
    return HostGraph(hc, wmax > 0)


PTG_FILE_BCSR, PTG_FILE_BWCSR, PTG_FILE_JAVA, PTG_FILE_BCSR64 = 0, 1, 2, 3


def read_csr(path, fmt):
    """Read a CSR file (PTG_FILE_*): (offsets u64 n+1, col u32, weight u32 or None)."""
    hc = HostCsr()
    _check(lib().ptg_read_csr_file(os.fsencode(path), fmt, 0, ctypes.byref(hc)))
    return _take(hc, fmt == PTG_FILE_BWCSR)


def write_csr(path, fmt, offsets, col, weight=None):
    """Write a sentinel-form CSR (offsets n+1) in one of the PTG_FILE_* formats."""
    off = np.ascontiguousarray(offsets, dtype=np.uint64)
    col = np.ascontiguousarray(col, dtype=np.uint32)
    w = None if weight is None else np.ascontiguousarray(weight, dtype=np.uint32)
    hc = HostCsr()
    hc.n, hc.m = off.size - 1, col.size
    hc.offsets = off.ctypes.data_as(_u64p)
    hc.col = col.ctypes.data_as(_u32p)
    hc.weight = w.ctypes.data_as(_u32p) if w is not None else None
    hc.pinned = 0
    _check(lib().ptg_write_csr_file(os.fsencode(path), fmt, ctypes.byref(hc)))


def gen_er_batch(num_graphs, nmin, nmax, avg_degree, seed=1, threads=0):
    """num_graphs ER graphs concatenated: (vtx_begin, offsets, col)."""
    hc = HostCsr()
    vb = _u64p()
    _check(lib().ptg_gen_er_batch(num_graphs, nmin, nmax, avg_degree, seed, threads, ctypes.byref(hc),
                                  ctypes.byref(vb)))
    vtx = np.ctypeslib.as_array(vb, shape=(num_graphs + 1,)).copy()
    lib().ptg_free(ctypes.cast(vb, _vp))
    off, col, _ = _take(hc, False)
    return vtx, off, col


class compat:
    """The reference's entry points (ptGraph/main.cu:24-56), same names and arguments."""

    @staticmethod
    def _u32(a):
        return np.ascontiguousarray(a, dtype=np.uint32)

    @staticmethod
    def _call(name, n, m, off_n, edges, *rest):
        off_n = compat._u32(off_n)
        fn = getattr(lib(), name)
        if edges.dtype != np.uint32:
            raise TypeError("edge arrays are uint32 (or (m,2) uint32 for weighted)")
        e = np.ascontiguousarray(edges)
        ep = e.ctypes.data_as(_u32p) if name.startswith(("bfs", "cc", "pr", "caculate")) else _ptr(e)
        ms = fn(n, m, off_n.ctypes.data_as(_u32p), ep, *rest)
        return ms

    @staticmethod
    def run(name, off_n, edges, src=None):
        """Call entry point `name`; returns (elapsed_ms, result array)."""
        off_n = compat._u32(off_n)
        n = off_n.size
        e = np.ascontiguousarray(edges, dtype=np.uint32)
        m = e.shape[0]
        args = [] if src is None else [src]
        ms = compat._call(name, n, m, off_n, e, *args)
        err = lib().ptg_compat_last_error().decode()
        if ms is not None and ms < 0:
            raise PtgError(PTG_ERR_INVALID, err)
        if name.startswith("pr"):
            out = np.empty(n, dtype=np.float32)
            lib().ptg_compat_last_result_f32(out.ctypes.data_as(_f32p), n)
        else:
            out = np.empty(n, dtype=np.uint32)
            lib().ptg_compat_last_result(out.ctypes.data_as(_u32p), n)
        return ms, out

    @staticmethod
    def set_partition_config(cfg):
        lib().ptg_compat_set_partition_config(ctypes.byref(cfg) if cfg is not None else None)
