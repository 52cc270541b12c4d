"""The ctypes mirrors of the C ABI structs (test-world_gb300/ptgraph) match
include/ptgraph.h byte for byte: a small C program compiled here prints
sizeof and offsetof of every field the mirror names."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PAIRS = [("ptg_csr", "Csr"), ("ptg_partition_config", "PartitionConfig"), ("ptg_run_stats", "RunStats"),
         ("ptg_run_opts", "RunOpts"), ("ptg_pr_opts", "PrOpts"), ("ptg_graph_info", "GraphInfo"),
         ("ptg_host_csr", "HostCsr"), ("ptg_server_config", "ServerConfig"), ("ptg_server_stats", "ServerStats"),
         ("ptg_tuning", "Tuning")]


def test_ctypes_mirrors_match_the_header(ptg, tmp_path):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if not gcc:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "ptgraph.h"', "int main(void) {"]
    expect = {}
    for cname, pyname in PAIRS:
        cls = getattr(ptg, pyname)
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        expect["%s sizeof" % cname] = __import__("ctypes").sizeof(cls)
        for f, _ in cls._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
            expect["%s %s" % (cname, f)] = getattr(cls, f).offset
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([gcc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            k, v = ln.rsplit(" ", 1)
            got[k] = int(v)
    assert got == expect
