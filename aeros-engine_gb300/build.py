"""In-tree build of libaeros_gb300.so for sm_103a (no cmake, parallel nvcc).

Translation units and their floating-point contraction:
  lbm_fp32.cu  --fmad=false  drop-in form, rounds every operation as the reference
  lbm_half.cu  --fmad=true   FP16/BF16 shifted storage
  forces.cu    --fmad=false  per-cell momentum-flux terms as the reference
  voxel.cu     --fmad=false  bit-exact inside test
  capi.cu      --fmad=false  host code with -ffp-contract=off
  batch.cu     --fmad=false  host side of the many-domain batch
  post.cu      --fmad=false  world fields, vorticity / Q, samplers as the reference rounds them
  sdf.cu       --fmad=false  distance field: weights, smoothing and samplers as the reference
  surface.cu   --fmad=false  surface-pressure lift and drag: per-triangle terms as the reference
  stl.cpp      host only     STL detection and parse (-ffp-contract=off like all host code)
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "lib")
BUILD_DIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-warn-spills"]
# resident blocks per SM the step kernel's register budget targets (tuning knob)
MIN_BLOCKS = os.environ.get("AEROS_STEP_MIN_BLOCKS", "6")
FUSED_MIN_BLOCKS = os.environ.get("AEROS_FUSED_MIN_BLOCKS", "8")
BATCH_MIN_BLOCKS = os.environ.get("AEROS_BATCH_MIN_BLOCKS", "4")
FUSED_ODD_MIN_BLOCKS = os.environ.get("AEROS_FUSED_ODD_MIN_BLOCKS", FUSED_MIN_BLOCKS)
FUSED_TH_MIN_BLOCKS = os.environ.get("AEROS_FUSED_TH_MIN_BLOCKS", "6")
STEP_BLOCK = os.environ.get("AEROS_STEP_BLOCK", "128")
TAG = (f"mb{MIN_BLOCKS}f{FUSED_MIN_BLOCKS}o{FUSED_ODD_MIN_BLOCKS}t{FUSED_TH_MIN_BLOCKS}"
       f"b{BATCH_MIN_BLOCKS}" + f"k{STEP_BLOCK}")
UNITS = {
    "lbm_fp32.cu": ["--fmad=false"],
    "lbm_half.cu": ["--fmad=true"],
    "forces.cu": ["--fmad=false"],
    "voxel.cu": ["--fmad=false"],
    "capi.cu": ["--fmad=false"],
    "batch.cu": ["--fmad=false"],
    "post.cu": ["--fmad=false"],
    "sdf.cu": ["--fmad=false"],
    "surface.cu": ["--fmad=false"],
    "stl.cpp": [],
    "setup.cu": [],
}
HEADERS = ["lattice.cuh", "lbm_step.cuh", "lbm_aux.cuh", "forces.cuh", "setup.cuh", "handle.cuh"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(os.path.dirname(HERE), "include", h) for h in ("aeros_lbm.h", "aeros_batch.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(unit: str, flags: list[str], verbose: bool) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD_DIR, f"{os.path.splitext(unit)[0]}.{TAG}.o")
    if _stale(obj, src):
        cmd = [nvcc(), *ARCH, *COMMON, f"-DAEROS_STEP_MIN_BLOCKS={MIN_BLOCKS}",
               f"-DAEROS_FUSED_MIN_BLOCKS={FUSED_MIN_BLOCKS}",
               f"-DAEROS_BATCH_MIN_BLOCKS={BATCH_MIN_BLOCKS}", f"-DAEROS_FUSED_ODD_MIN_BLOCKS={FUSED_ODD_MIN_BLOCKS}",
               f"-DAEROS_FUSED_TH_MIN_BLOCKS={FUSED_TH_MIN_BLOCKS}", f"-DAEROS_STEP_BLOCK={STEP_BLOCK}",
               *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {unit}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
    return obj


FACADE = os.path.join(HERE, "facade")


def build_facade(lib: str) -> str:
    """libaeros_facade.so: the C++17 mirror of the reference solver interface
    over the C ABI (g++, linked against libaeros_gb300.so by rpath)."""
    out = os.path.join(OUT_DIR, "libaeros_facade.so")
    src = os.path.join(FACADE, "aeros_facade.cpp")
    deps = [src, os.path.join(FACADE, "aeros_facade.h"), lib]
    if os.path.exists(out) and all(os.path.getmtime(d) <= os.path.getmtime(out) for d in deps):
        return out
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-Wall", src,
           "-o", out,
           "-L" + OUT_DIR, "-laeros_gb300", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"facade build failed:\n{r.stdout}\n{r.stderr}")
    return out


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    lib = os.path.join(OUT_DIR, "libaeros_gb300.so")
    stamp = os.path.join(BUILD_DIR, "linked_with")
    last = open(stamp).read() if os.path.exists(stamp) else ""
    if (not os.path.exists(lib) or last != TAG
            or any(os.path.getmtime(o) > os.path.getmtime(lib) for o in objs)):
        cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", lib]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        with open(stamp, "w") as fh:
            fh.write(TAG)
    build_facade(lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
