"""Builds the engine in-tree: ascetic_gb300/_lib/libascetic_gb300.so, the
ptgraph command line and the asc-convert file converter, for sm_103a only
(nvcc, no torch extension machinery).

The translation units compile in parallel; nothing is fetched or installed.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(PKG, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "libascetic_gb300.so")
PTGRAPH_PATH = os.path.join(LIB_DIR, "ptgraph")
CONVERT_PATH = os.path.join(LIB_DIR, "asc-convert")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["engine.cu", "graph.cpp", "capi.cpp", "server.cpp"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA engine cannot be built")
    return cand


def _common_flags():
    # ASC_NVCC_EXTRA: extra nvcc flags (e.g. -DASC_EXPAND_MIN_BLOCKS=6) for tuning experiments
    extra = os.environ.get("ASC_NVCC_EXTRA", "").split()
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
            "-I" + INCLUDE, "-I" + CSRC] + extra


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(OBJ_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, "common.h"), os.path.join(INCLUDE, "ascetic.h")]
    jobs = []
    objs = []
    for src in LIB_SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OBJ_DIR, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            cmd = [nvcc] + ARCH + _common_flags() + ["-c", path, "-o", obj]
            if src.endswith(".cu"):
                cmd += ["-Xptxas", "-v"] if verbose else []
            else:
                cmd += ["-x", "c++"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("build failed:\n%s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB_PATH, objs):
        tmp = LIB_PATH + ".tmp%d" % os.getpid()
        run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, LIB_PATH)
    for exe, src in ((PTGRAPH_PATH, "ptgraph.cpp"), (CONVERT_PATH, "convert.cpp")):
        cli_src = os.path.join(CSRC, src)
        if force or _stale(exe, [cli_src, LIB_PATH] + headers):
            tmp = exe + ".tmp%d" % os.getpid()
            run(["g++", "-O2", "-std=c++17", "-Wall", "-I" + INCLUDE, cli_src, "-o", tmp, "-L" + LIB_DIR,
                 "-lascetic_gb300", "-Wl,-rpath,$ORIGIN"])
            os.replace(tmp, exe)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB_PATH)
