"""The reference's own call sites against this library.

A C++ program that declares the entry points exactly as the reference does
(ptGraph/main.cu:30-56, with uint and EdgeWithWeight as in
ptGraph/globals.cuh:2-5) and does not include ptgraph.h is compiled with g++
and linked against libptgraph.so: it links through the C++-mangled names the
library exports beside its C ABI (csrc/compat_cxx.cpp).  Without a GPU every
call returns -1 with "no CUDA device" (CPU test); on a GPU the BFS levels,
SSSP distances and CC labels of a small graph come back as the reference
defines them (GPU test)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "test-world_gb300", "_build")

PROGRAM = r"""
#include <cstdio>
#include <cstdint>
#include <sys/types.h>

struct EdgeWithWeight {
    uint toNode;
    uint weight;
};

// ptGraph/main.cu:30-56, as the reference declares them (the 5-parameter
// caculateInOptChooseByDegree of its definition, main.cu:2196-2198)
void caculateInCommon(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList);
long bfsCaculateInShare(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList, uint sourceNode);
long bfsCaculateInOpt(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList, uint sourceNode);
long bfsCaculateInAsync(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList, uint sourceNode);
long bfsCaculateInAsyncSwap(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList, uint sourceNode);
long ssspCaculateInShare(uint testNumNodes, uint testNumEdge, uint *nodePointersI, EdgeWithWeight *edgeList,
                         uint sourceNode);
long ssspCaculateInOpt(uint testNumNodes, uint testNumEdge, uint *nodePointersI, EdgeWithWeight *edgeList,
                       uint sourceNode);
long ccCaculateInShare(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList);
long ccCaculateInOpt(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList);
long prCaculateInShare(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList);
long prCaculateInOpt(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList);
void caculateInShareOpt(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList);
void caculateInOptChooseByDegree(uint testNumNodes, uint testNumEdge, uint *nodePointersI, uint *edgeList,
                                 uint sourceNode);

// the library's result accessors (C linkage), declared by hand: the caller
// does not include ptgraph.h
extern "C" uint64_t ptg_compat_last_result(uint32_t *out, uint64_t capacity);
extern "C" const char *ptg_compat_last_error(void);

static void dump(const char *name, long ret) {
    uint32_t r[5] = {0, 0, 0, 0, 0};
    uint64_t k = ret >= 0 ? ptg_compat_last_result(r, 5) : 0;
    printf("%s %ld %llu %u %u %u %u %u | %s\n", name, ret, (unsigned long long)k, r[0], r[1], r[2], r[3], r[4],
           ret < 0 ? ptg_compat_last_error() : "");
}

int main() {
    // path 0-1-2-3 plus an isolated vertex 4, symmetric; n offsets, no sentinel (main.cu:97-121)
    uint off[5] = {0, 1, 3, 5, 6};
    uint col[6] = {1, 0, 2, 1, 3, 2};
    EdgeWithWeight ew[6] = {{1, 5}, {0, 5}, {2, 7}, {1, 7}, {3, 2}, {2, 2}};
    dump("bfsCaculateInOpt", bfsCaculateInOpt(5, 6, off, col, 0));
    dump("bfsCaculateInAsync", bfsCaculateInAsync(5, 6, off, col, 0));
    dump("bfsCaculateInAsyncSwap", bfsCaculateInAsyncSwap(5, 6, off, col, 0));
    dump("bfsCaculateInShare", bfsCaculateInShare(5, 6, off, col, 0));
    dump("ssspCaculateInOpt", ssspCaculateInOpt(5, 6, off, ew, 0));
    dump("ssspCaculateInShare", ssspCaculateInShare(5, 6, off, ew, 0));
    dump("ccCaculateInOpt", ccCaculateInOpt(5, 6, off, col));
    dump("ccCaculateInShare", ccCaculateInShare(5, 6, off, col));
    long pr = prCaculateInShare(5, 6, off, col);
    printf("prCaculateInShare %ld\n", pr);
    pr = prCaculateInOpt(5, 6, off, col);
    printf("prCaculateInOpt %ld\n", pr);
    caculateInCommon(5, 6, off, col);
    dump("caculateInCommon", 0);
    caculateInShareOpt(5, 6, off, col);
    caculateInOptChooseByDegree(5, 6, off, col, 3);
    dump("caculateInOptChooseByDegree", 0);
    return 0;
}
"""


def build_program(tmp_path):
    lib = os.path.join(BUILD, "libptgraph.so")
    if not os.path.exists(lib):
        pytest.skip("libptgraph.so not built")
    src = tmp_path / "callsite.cpp"
    src.write_text(PROGRAM)
    exe = str(tmp_path / "callsite")
    r = subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-o", exe, "-L" + BUILD, "-lptgraph",
                        "-Wl,-rpath," + BUILD], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def run_program(exe):
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return {line.split()[0]: line for line in r.stdout.splitlines()}


def test_reference_prototypes_link_without_header(tmp_path):
    exe = build_program(tmp_path)
    nm = subprocess.run(["nm", "-D", "--defined-only", os.path.join(BUILD, "libptgraph.so")],
                        capture_output=True, text=True).stdout
    for mangled in ("_Z16bfsCaculateInOptjjPjS_j", "_Z17ssspCaculateInOptjjPjP14EdgeWithWeightj",
                    "_Z15ccCaculateInOptjjPjS_", "_Z16caculateInCommonjjPjS_"):
        assert mangled in nm
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("a GPU is visible: the results are checked by the GPU test")
    out = run_program(exe)
    for name in ("bfsCaculateInOpt", "ssspCaculateInOpt", "ccCaculateInOpt"):
        fields = out[name].split()
        assert fields[1] == "-1" and "no CUDA device" in out[name]


@pytest.mark.gpu
def test_reference_call_sites_on_gpu(tmp_path):
    out = run_program(build_program(tmp_path))
    U = 0xFFFFFFFF
    for name in ("bfsCaculateInOpt", "bfsCaculateInAsync", "bfsCaculateInAsyncSwap", "bfsCaculateInShare",
                 "caculateInCommon"):
        f = out[name].split()
        assert int(f[1]) >= 0 and f[2] == "5" and [int(x) for x in f[3:8]] == [1, 2, 3, 4, U], out[name]
    f = out["ssspCaculateInOpt"].split()
    assert [int(x) for x in f[3:8]] == [1, 6, 13, 15, U]
    f = out["ssspCaculateInShare"].split()
    assert [int(x) for x in f[3:8]] == [1, 6, 13, 15, U - 1]
    for name in ("ccCaculateInOpt", "ccCaculateInShare"):
        f = out[name].split()
        assert [int(x) for x in f[3:8]] == [0, 0, 0, 0, 4]
    f = out["caculateInOptChooseByDegree"].split()
    assert [int(x) for x in f[3:8]] == [4, 3, 2, 1, U]
    assert int(out["prCaculateInShare"].split()[1]) >= 0
