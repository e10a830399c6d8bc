"""Builds the reference's kernels and the runner that drives them.

Test infrastructure (the oracle's pin).  Outputs go to oracle/_ref/ only
(git-ignored; carried to the GPU machine with the working tree):

  cumbe_ref.cubin  the reference's device code compiled from its own,
                   unmodified sources (src/main.cu and the headers it
                   includes) for sm_103a, with oracle/ref_shim13.h
                   force-included for the CUDA 13 cudaMemPrefetchAsync
                   signature.  Built only where the reference sources are
                   present; elsewhere a previously built cubin is used.
  ref_runner       oracle/ref_runner.cpp (host side, CUDA driver API),
                   built wherever CUDA headers are present.
  gen_bi           the reference's KONECT converter data/gen_bi.cpp,
                   compiled unmodified with g++ (reference sources only).
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# where the reference's sources are: MBE_REFERENCE_ROOT, else the read-only
# checkout this recipe was written against
REF_ROOT = os.environ.get("MBE_REFERENCE_ROOT", "/root/reference")
CUBIN = os.path.join(OUT, "cumbe_ref.cubin")
RUNNER = os.path.join(OUT, "ref_runner")
GEN_BI = os.path.join(OUT, "gen_bi")


def _cuda_home() -> str:
    nvcc = shutil.which("nvcc")
    return os.path.dirname(os.path.dirname(nvcc)) if nvcc else "/usr/local/cuda"


def build() -> dict:
    os.makedirs(OUT, exist_ok=True)
    cuda = _cuda_home()
    out = {"cubin": None, "runner": None}
    src = os.path.join(REF_ROOT, "src", "main.cu")
    if os.path.exists(src):
        if not os.path.exists(CUBIN) or os.path.getmtime(CUBIN) < os.path.getmtime(os.path.join(HERE, "ref_shim13.h")):
            subprocess.run([os.path.join(cuda, "bin", "nvcc"), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                            "-O3", "-I" + REF_ROOT, "-include", os.path.join(HERE, "ref_shim13.h"), src,
                            "-o", CUBIN], check=True, capture_output=True)
    if os.path.exists(CUBIN):
        out["cubin"] = CUBIN
    # the reference's KONECT converter, from its own unmodified source
    gen_src = os.path.join(REF_ROOT, "data", "gen_bi.cpp")
    if os.path.exists(gen_src) and not os.path.exists(GEN_BI):
        subprocess.run(["g++", "-O3", "-std=c++17", gen_src, "-o", GEN_BI], check=True, capture_output=True)
    out["gen_bi"] = GEN_BI if os.path.exists(GEN_BI) else None
    runner_src = os.path.join(HERE, "ref_runner.cpp")
    inc = os.path.join(cuda, "include")
    if os.path.exists(os.path.join(inc, "cuda.h")):
        stale = not os.path.exists(RUNNER) or os.path.getmtime(RUNNER) < os.path.getmtime(runner_src)
        if stale:
            libdirs = [os.path.join(cuda, "lib64", "stubs"), os.path.join(cuda, "lib64")]
            cmd = ["g++", "-O2", "-std=c++17", runner_src, "-I" + inc, "-o", RUNNER]
            for d in libdirs:
                cmd += ["-L" + d]
            cmd += ["-lcuda"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("ref_runner build failed:\n" + r.stderr)
        out["runner"] = RUNNER
    return out


if __name__ == "__main__":
    print(build())
