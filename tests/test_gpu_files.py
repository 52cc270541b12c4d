"""The reference's input path on the GPU: its on-disk CSR files (.bcsr,
.bwcsr, the big-endian Java export, ptGraph/main.cu:97-121, 451-475,
2479-2573, and the 64-bit .bcsr layout), each written byte for byte by an
independent numpy encoder, read with ptg_read_csr_file, uploaded with
ptg_graph_create (resident and out of core) or handed to the drop-in entry
points, and the results compared with the reference's own (golden
fixtures)."""
import glob
import os

import numpy as np
import pytest

from test_csr_files import encode

pytestmark = pytest.mark.gpu

GOLD = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
FORMATS = [0, 1, 2, 3]
FMT_IDS = ["bcsr", "bwcsr", "java", "bcsr64"]


def load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


@pytest.mark.parametrize("fmt", FORMATS, ids=FMT_IDS)
@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(p)[:-4] for p in GOLD])
def test_file_to_gpu_matches_reference(ptg, ctx, tmp_path, fmt, path):
    g = load(path)
    sym = bool(g["symmetric"][0])
    off, col, w = g["off"].astype(np.uint64), g["col"].astype(np.uint32), g["w"].astype(np.uint32)
    f = str(tmp_path / "graph.bin")
    with open(f, "wb") as fh:
        fh.write(encode(fmt, off, col, w))
    o2, c2, w2 = ptg.read_csr(f, fmt)
    weights = w2 if fmt == 1 else w  # only .bwcsr carries weights; the others get the fixture's
    m = c2.size
    pb = max(32, (m * 8 // 8) // 8 * 8)
    cfgs = [None, ptg.partition_config(partition_bytes=pb, device_budget_bytes=2 * pb, force_out_of_core=1)]
    for cfg in cfgs:
        G = ctx.graph(o2, c2, weights, symmetric=sym, config=cfg)
        for i, s in enumerate(g["sources"]):
            assert (G.bfs(int(s)) == g["bfs"][i]).all()
            if "sssp" in g:
                assert (G.sssp(int(s)) == g["sssp"][i]).all()
        assert (G.cc() == g["cc"]).all()
        G.close()
    # the reference's own call sequence: read the file, call the entry point
    # with its n-entry offsets
    s = int(g["sources"][-1])
    _, out = ptg.compat.run("bfsCaculateInOpt", o2[:-1].astype(np.uint32), c2 if m else np.zeros(0, np.uint32), s)
    assert (out == g["bfs"][-1]).all()
    if fmt == 1 and m:
        aos = np.stack([c2, w2], axis=1).astype(np.uint32)
        _, out = ptg.compat.run("ssspCaculateInOpt", o2[:-1].astype(np.uint32), aos, s)
        assert (out == g["sssp"][-1]).all()
