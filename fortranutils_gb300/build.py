"""Build the GB300 library liblester_gpu.so in-tree with nvcc (sm_103a).

The exact FP64 translation units are compiled with ``-fmad=false`` so that
every product and sum is rounded separately, as in the reference's FP64
Fortran; the fast multigrid unit keeps FMA contraction.  Objects go to
``fortranutils_gb300/_build``; the shared library to
``fortranutils_gb300/_lib``.  Sources compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

try:
    from . import gen_f32
except ImportError:  # run as a script
    import gen_f32

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIBNAME = "liblester_gpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "-I", str(PKG.parent / "include")]
# object -> (translation unit, extra flags).  The FP64 physics units are
# built twice: exact (-fmad=false, namespace les_exact) and fast
# (-DLES_FAST_PHYS, namespace les_fast).
UNITS = {
    "lester_host": ("lester_host.cu", []),
    "k_exact": ("k_exact.cu", ["-fmad=false"]),
    "k_metric": ("k_metric.cu", ["-fmad=false"]),
    "k_sgs": ("k_sgs.cu", ["-fmad=false"]),
    "k_sgs_fast": ("k_sgs.cu", ["-DLES_FAST_PHYS"]),
    "k_fast": ("k_fast.cu", []),
    "k_phys": ("k_phys.cu", ["-fmad=false"]),
    "k_phys_fast": ("k_phys.cu", ["-DLES_FAST_PHYS"]),
    "lester_phys_host": ("lester_phys_host.cu", []),
    "k_virtbc": ("k_virtbc.cu", ["-fmad=false"]),
    "lester_step": ("lester_step.cu", []),
    "lester_noalloc": ("lester_noalloc.cu", ["-fmad=false"]),
    "k_adjoint": ("k_adjoint.cu", ["-fmad=false"]),
    "lester_adjoint": ("lester_adjoint.cu", []),
    "k_outflow": ("k_outflow.cu", ["-fmad=false"]),
    "lester_outflow": ("lester_outflow.cu", []),
    "k_graph": ("k_graph.cu", []),
    "k_dfloat": ("k_dfloat.cu", ["-fmad=false"]),
    # the tiled scalar sweep: exact FP64 (no FMA); fast FP64 and FP32
    "k_sweep": ("k_sweep.cu", ["-fmad=false", "-DLES_SWEEP_EXACT"]),
    "k_sweep_fast": ("k_sweep.cu", []),
    # the FP32-arithmetic physics build (namespace les_f32), generated from
    # k_phys.cu and k_sgs.cu by gen_f32.py into the build directory
    "k_phys_f32": ("@k_phys_f32.cu", []),
    "k_sgs_f32": ("@k_sgs_f32.cu", []),
}


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def lib_path() -> Path:
    return LIBDIR / LIBNAME


def _compile(name: str, src: str, extra: list[str], verbose: bool) -> Path:
    obj = BUILD / (name + ".o")
    # "@name": a source generated into the build directory
    path = BUILD / src[1:] if src.startswith("@") else CSRC / src
    cmd = [nvcc(), *ARCH, *COMMON, "-I", str(CSRC), *extra, "-c", str(path), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA unit for sm_103a and link the shared library."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    out = lib_path()
    gen_f32.generate(CSRC, BUILD)
    srcs = [BUILD / u[0][1:] if u[0].startswith("@") else CSRC / u[0] for u in UNITS.values()]
    srcs += list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG / "gen_f32.py"]
    srcs.append(PKG.parent / "include" / "lester_gpu.h")
    if out.exists() and not force:
        newest = max(p.stat().st_mtime for p in srcs)
        if out.stat().st_mtime >= newest:
            return out
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        futs = [ex.submit(_compile, n, s, f, verbose) for n, (s, f) in UNITS.items()]
        objs = [f.result() for f in futs]
    tmp = out.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
