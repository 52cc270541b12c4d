"""The reference's on-disk CSR files (.bcsr, .bwcsr, the Java big-endian export)
and the 64-bit .bcsr variant: byte layout against an independent numpy encoder
written from the reference's readers (ptGraph/main.cu:97-121, 451-475,
2479-2573), round trips, and rejection of malformed files.  CPU only."""
import glob
import os

import numpy as np
import pytest

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def encode(fmt, off, col, w):
    """The file bytes, built field by field with numpy (no library code)."""
    n, m = off.size - 1, col.size
    if fmt == 0:  # .bcsr
        parts = [np.array([n, m], "<u4"), off[:-1].astype("<u4"), col.astype("<u4")]
    elif fmt == 1:  # .bwcsr: {toNode, weight} records
        rec = np.empty((m, 2), "<u4")
        rec[:, 0], rec[:, 1] = col, w
        parts = [np.array([n, m], "<u4"), off[:-1].astype("<u4"), rec.reshape(-1)]
    elif fmt == 2:  # Java export, big-endian
        parts = [np.array([n], ">u4"), np.array([m], ">u8"), off[:-1].astype(">u8"), col.astype(">u4")]
    else:  # .bcsr64
        parts = [np.array([n], "<u4"), np.array([m], "<u8"), off[:-1].astype("<u8"), col.astype("<u4")]
    return b"".join(p.tobytes() for p in parts)


@pytest.mark.parametrize("fmt", [0, 1, 2, 3], ids=["bcsr", "bwcsr", "java", "bcsr64"])
@pytest.mark.parametrize("path", GOLD[:6] + GOLD[-3:], ids=[os.path.basename(p)[:-4] for p in GOLD[:6] + GOLD[-3:]])
def test_layout_and_round_trip(ptg, tmp_path, fmt, path):
    z = np.load(path)
    off, col, w = z["off"].astype(np.uint64), z["col"].astype(np.uint32), z["w"].astype(np.uint32)
    f = str(tmp_path / "g.bin")
    ptg.write_csr(f, fmt, off, col, w if fmt == 1 else None)
    assert open(f, "rb").read() == encode(fmt, off, col, w)
    o2, c2, w2 = ptg.read_csr(f, fmt)
    assert np.array_equal(o2, off) and np.array_equal(c2, col)
    if fmt == 1:
        assert np.array_equal(w2, w)
    else:
        assert w2 is None


def test_generated_graph_through_bwcsr(ptg, tmp_path):
    off, col, w = ptg.gen_rmat(12, 16, seed=9, symmetric=True, wmin=1, wmax=63)
    f = str(tmp_path / "g.bwcsr")
    with open(f, "wb") as fh:
        fh.write(encode(1, off, col, w))
    o2, c2, w2 = ptg.read_csr(f, ptg.PTG_FILE_BWCSR)
    assert np.array_equal(o2, off) and np.array_equal(c2, col) and np.array_equal(w2, w)


def _expect_invalid(ptg, f, fmt):
    with pytest.raises(ptg.PtgError) as e:
        ptg.read_csr(f, fmt)
    assert e.value.status == ptg.PTG_ERR_INVALID


def test_malformed_files_are_rejected(ptg, tmp_path):
    off = np.array([0, 2, 3, 5, 5], np.uint64)
    col = np.array([1, 2, 0, 0, 1], np.uint32)
    good = encode(0, off, col, None)
    f = str(tmp_path / "g.bcsr")
    _expect_invalid(ptg, str(tmp_path / "missing.bcsr"), 0)
    for bad in (good[:-1], good + b"\0", good[:6]):  # truncated / trailing bytes / header cut
        open(f, "wb").write(bad)
        _expect_invalid(ptg, f, 0)
    open(f, "wb").write(encode(0, np.array([0, 3, 2, 5, 5], np.uint64), col, None))  # decreasing
    _expect_invalid(ptg, f, 0)
    open(f, "wb").write(encode(0, off, np.array([1, 2, 0, 4, 1], np.uint32), None))  # target >= n
    _expect_invalid(ptg, f, 0)
    open(f, "wb").write(encode(0, np.array([1, 2, 3, 5, 5], np.uint64), col, None))  # first offset != 0
    _expect_invalid(ptg, f, 0)
    open(f, "wb").write(good)
    o2, c2, _ = ptg.read_csr(f, 0)
    assert np.array_equal(o2, off) and np.array_equal(c2, col)
    with pytest.raises(ptg.PtgError):  # .bwcsr needs weights
        ptg.write_csr(f, ptg.PTG_FILE_BWCSR, off, col)
