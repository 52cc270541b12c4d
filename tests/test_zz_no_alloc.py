"""The allocation-free BFS entry point (ptg_bfs_noalloc) through the C ABI.

It serves callers that can pass device buffers but must not call cudaMalloc
themselves (a plugin inside a host that owns all device memory through its
own pool).  Its output must equal the regular ptg_bfs entry point's, call
after call: the scratch it works in is shared and keeps the previous call's
contents, so two calls in a row (different sources, then a repeat) check
that each call starts clean.  This file is collected last so that a run that
stops at the first failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_V = 1 << 20  # PTG_NOALLOC_MAX_VERTICES


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def test_noalloc_bfs_matches_ptg_bfs(ptg, ctx, oracle):
    torch = pytest.importorskip("torch")
    off, col, _ = ptg.gen_rmat(16, 16, seed=1, symmetric=True)
    off32 = off.astype(np.uint32)
    n, m = off32.size - 1, col.size
    G = ctx.graph(off32, col, symmetric=True)
    d_off, d_col = _dev(torch, off32), _dev(torch, col)
    out = torch.full((n,), 7, dtype=torch.int32, device="cuda")
    L = ptg.lib()
    vp = ctypes.c_void_p
    for src in (0, 4242, 0):
        rc = L.ptg_bfs_noalloc(vp(d_off.data_ptr()), vp(d_col.data_ptr()), n, m, src, vp(out.data_ptr()),
                               None)
        assert rc == ptg.PTG_OK
        torch.cuda.synchronize()
        got = out.cpu().numpy().view(np.uint32)
        assert (got == G.bfs(src)).all()
        assert (got == oracle.bfs(off, col, src, method="queue")).all()


def test_noalloc_bfs_rejects_malformed_csr(ptg, oracle):
    """A CSR that is not one of n vertices and m edges fails with
    PTG_ERR_INVALID before any edge is read through it; the next call with a
    good CSR still gives the right levels (the shared scratch starts clean)."""
    torch = pytest.importorskip("torch")
    L = ptg.lib()
    vp = ctypes.c_void_p
    n = 4
    good_off = np.array([0, 2, 3, 4, 5], np.uint32)
    good_col = np.array([1, 2, 0, 3, 2], np.uint32)
    cases = [
        (good_off, np.array([1, 7, 0, 3, 2], np.uint32)),        # a target >= n
        (np.array([0, 3, 2, 4, 5], np.uint32), good_col),        # offsets decrease
        (np.array([0, 2, 3, 4, 4], np.uint32), good_col),        # off[n] != m
        (np.array([1, 2, 3, 4, 5], np.uint32), good_col),        # off[0] != 0
        (np.array([0, 2, 3, 4, 900], np.uint32), good_col),      # would read past col
    ]
    out = torch.zeros(n, dtype=torch.int32, device="cuda")
    for off, col in cases:
        d_off, d_col = _dev(torch, off), _dev(torch, col)
        rc = L.ptg_bfs_noalloc(vp(d_off.data_ptr()), vp(d_col.data_ptr()), n, col.size, 0, vp(out.data_ptr()),
                               None)
        assert rc == ptg.PTG_ERR_INVALID, (off, col)
    d_off, d_col = _dev(torch, good_off), _dev(torch, good_col)
    assert L.ptg_bfs_noalloc(vp(d_off.data_ptr()), vp(d_col.data_ptr()), n, good_col.size, 0,
                             vp(out.data_ptr()), None) == ptg.PTG_OK
    torch.cuda.synchronize()
    assert (out.cpu().numpy().view(np.uint32) == oracle.bfs(good_off, good_col, 0, method="queue")).all()


def test_noalloc_bfs_rejects_oversized_and_bad_input(ptg):
    torch = pytest.importorskip("torch")
    L = ptg.lib()
    vp = ctypes.c_void_p
    buf = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = vp(buf.data_ptr())
    assert L.ptg_bfs_noalloc(p, p, MAX_V + 1, 4, 0, p, None) == ptg.PTG_ERR_UNSUPPORTED
    assert L.ptg_bfs_noalloc(None, p, 4, 4, 0, p, None) == ptg.PTG_ERR_INVALID
    assert L.ptg_bfs_noalloc(p, p, 4, 4, 9, p, None) == ptg.PTG_ERR_INVALID
