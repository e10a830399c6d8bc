"""Builds libmbe.so and the `mbe` CLI in-tree with nvcc for sm_103a.

Each translation unit compiles in parallel into cumbe_gb300/_build/; the
shared library and the CLI land next to this file.  Works on x86_64 and
aarch64 hosts (no host-specific flags).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmbe.so")
CLI = os.path.join(HERE, "mbe")
GEN_BI = os.path.join(HERE, "gen_bi")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["graph_host.cpp", "graph_dev.cu", "engine.cu", "capi.cu", "capi_static.cu", "server.cu"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _flags() -> list[str]:
    f = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
         "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    # MBE_PROFILE=1 compiles the per-section cycle counters of dfs_kernel in
    # (printed to stderr after each enumeration); off by default.
    if os.environ.get("MBE_PROFILE") == "1":
        f += ["-DMBE_PROFILE"]
    # MBE_COUNT_WORDS=1 compiles the DFS kernel's set-word counter in
    # (mbe_result.words); off by default, on in MBE_PROFILE=1 builds.
    # MBE_DFS_BLOCKS=N sets the resident blocks per SM the enumeration kernel
    # is compiled for (its register budget); default 7.
    if os.environ.get("MBE_DFS_BLOCKS"):
        f += ["-DMBE_DFS_MIN_BLOCKS=%d" % int(os.environ["MBE_DFS_BLOCKS"])]
    # MBE_UNROLL=E,G,P sets the scan unroll factors of the enumeration kernel
    # (expansion chunks, gather chunks, prefilter rows); default 1,1,5.
    # MBE_DFS_WARPS=N sets its warps per block; default 4.
    if os.environ.get("MBE_DFS_WARPS"):
        f += ["-DMBE_DFS_WARPS=%d" % int(os.environ["MBE_DFS_WARPS"])]
    for knob in ("MBE_KEEP_WINDOW", "MBE_POP_SLEEP_MAX", "MBE_SMEM_W", "MBE_SH_ROWS", "MBE_POLL_CYCLES", "MBE_COUNT_WORDS"):  # sweeps
        if os.environ.get(knob):
            f += ["-D%s=%d" % (knob, int(os.environ[knob]))]
    if os.environ.get("MBE_EVAL_NOINLINE") == "1":
        f += ["-DMBE_EVAL_NOINLINE"]
    if os.environ.get("MBE_UNROLL"):
        e, g, p = (int(v) for v in os.environ["MBE_UNROLL"].split(","))
        f += ["-DMBE_UNROLL_E=%d" % e, "-DMBE_UNROLL_G=%d" % g, "-DMBE_UNROLL_P=%d" % p]
    return f


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "mbe.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc()] + ARCH + _flags() + ["-c", s, "-o", o]
            if ptxas_info and src.endswith(".cu"):
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or ptxas_info or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or not os.path.exists(LIB):
        subprocess.check_call([nvcc()] + ARCH + ["-shared", "-o", LIB + ".tmp"] + objs + ["-lpthread"])
        os.replace(LIB + ".tmp", LIB)
    cli_src = os.path.join(CSRC, "mbe_cli.cpp")
    if force or _stale(CLI, [cli_src, LIB]):
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), cli_src,
                               "-o", CLI + ".tmp", "-L" + HERE, "-lmbe", "-Wl,-rpath,$ORIGIN"])
        os.replace(CLI + ".tmp", CLI)
    gen_src = os.path.join(CSRC, "gen_bi_cli.cpp")
    if force or _stale(GEN_BI, [gen_src, LIB]):
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), gen_src,
                               "-o", GEN_BI + ".tmp", "-L" + HERE, "-lmbe", "-Wl,-rpath,$ORIGIN"])
        os.replace(GEN_BI + ".tmp", GEN_BI)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
