"""Build libptgraph.so (the engine's C ABI) in-tree with nvcc for sm_103a.

Usage: python test-world_gb300/build.py [--debug]
Objects go to test-world_gb300/_build/; translation units compile in parallel.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libptgraph.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["devmem.cpp", "api.cu", "traverse.cu", "cc.cu", "pagerank.cu", "batch.cu", "msbfs.cu", "serve.cu", "gen.cpp",
           "noalloc.cu", "pprbatch.cu", "io.cpp", "relabel.cu", "compat_cxx.cpp"]


def _compile(src, debug, verbose):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "ptgraph.h"))
    if os.path.exists(obj) and all(os.path.getmtime(d) <= os.path.getmtime(obj) for d in deps):
        return obj, ""
    cmd = [NVCC, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-Wall", "-c", path, "-o", obj]
    if src.endswith(".cu"):
        cmd += ARCH + ["--expt-relaxed-constexpr"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    if debug:
        cmd += ["-DPTG_DEBUG"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build(debug=False, verbose=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, debug, verbose), SOURCES))
    objs = [o for o, _ in results]
    logs = "".join(l for _, l in results)
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [NVCC, "-shared", "-o", LIB] + objs + ARCH + ["-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    return LIB, logs


if __name__ == "__main__":
    lib, logs = build(debug="--debug" in sys.argv, verbose="-v" in sys.argv)
    if logs:
        print(logs)
    print(lib)
