"""Build recipes for the native parts: nvcc for sm_103a, gcc for host C.

Outputs (git-ignored, rebuilt on every machine -- nothing compiled on one
host architecture is reused on another):
  opencuda_gb300/_build/libhoughline_gb300.so  the product (C ABI)
  oracle/_build/libhough_oracle.so            the CPU oracle (tests only)
  oracle/_ref/houghline_ref.fatbin            reference device code (only
                                               where the reference sources
                                               are present; see oracle/)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"
LIBNAME = "libhoughline_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def nvcc() -> str:
    p = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required")
    return p


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


CU_SOURCES = ["hl_stage_a.cu", "hl_vote.cu", "hl_stage_c.cu", "hl_stage_f.cu",
              "hl_noalloc.cu", "hl_cnn.cu", "hl_synth.cu", "hl_window.cu", "hl_circle.cu"]
CXX_SOURCES = ["hl_api.cpp", "HoughLine.cpp", "HoughCircle.cpp", "Image.cpp", "hl_proposal.cpp"]
C_SOURCES = ["synth.c"]


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps if d.exists())


def build_library(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    out = BUILD / LIBNAME
    headers = list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    srcs = [CSRC / s for s in CU_SOURCES + CXX_SOURCES + C_SOURCES
            if (CSRC / s).exists()]
    if not force and _newer(out, srcs + headers + [Path(__file__)]):
        return out
    inc = ["-I", str(INCLUDE), "-I", str(CSRC)]
    jobs = []
    objs = []
    for s in CU_SOURCES:
        o = BUILD / (s + ".o")
        objs.append(o)
        jobs.append([nvcc(), "-c", *ARCH, "-O3", "-lineinfo", "-std=c++17",
                     "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills", *inc,
                     str(CSRC / s), "-o", str(o)])
    for s in CXX_SOURCES:
        if not (CSRC / s).exists():
            continue
        o = BUILD / (s + ".o")
        objs.append(o)
        jobs.append([nvcc(), "-c", "-x", "cu", *ARCH, "-O2", "-std=c++17",
                     "-Xcompiler", "-fPIC", *inc, str(CSRC / s), "-o", str(o)])
    for s in C_SOURCES:
        o = BUILD / (s + ".o")
        objs.append(o)
        jobs.append(["gcc", "-c", "-O2", "-fPIC", "-std=gnu11", *inc,
                     str(CSRC / s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    tmp = BUILD / (LIBNAME + ".tmp")
    _run([nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs),
          "-lcudart"])
    os.replace(tmp, out)
    if verbose:
        print(f"built {out}")
    return out


def build_oracle(force: bool = False) -> Path:
    outdir = ORACLE / "_build"
    outdir.mkdir(parents=True, exist_ok=True)
    out = outdir / "libhough_oracle.so"
    srcs = [ORACLE / "hough_oracle.c", ORACLE / "hough_oracle.h",
            ORACLE / "circle_oracle.c", ORACLE / "circle_oracle.h"]
    if not force and _newer(out, srcs):
        return out
    tmp = outdir / "libhough_oracle.so.tmp"
    # -ffp-contract=off: every float product and sum is rounded as written
    # (aarch64 gcc would otherwise fuse them into fmadd).
    _run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
          "-std=gnu11", str(ORACLE / "hough_oracle.c"), str(ORACLE / "circle_oracle.c"),
          "-o", str(tmp), "-lm"])
    os.replace(tmp, out)
    return out


def build_ref_runner(force: bool = False) -> Path:
    """Driver-API loader for the reference fatbin (tests only)."""
    outdir = ORACLE / "_build"
    outdir.mkdir(parents=True, exist_ok=True)
    out = outdir / "libref_runner.so"
    src = ORACLE / "ref_runner.c"
    if not force and _newer(out, [src]):
        return out
    tmp = outdir / "libref_runner.so.tmp"
    _run(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11",
          "-I", os.path.join(CUDA_HOME, "include"), str(src), "-o", str(tmp),
          "-L", os.path.join(CUDA_HOME, "lib64", "stubs"), "-lcuda"])
    os.replace(tmp, out)
    return out


def build_reference_fatbin() -> Path | None:
    """Device code of the reference's HoughLine.cu, compiled from its own
    sources for sm_103a (only where the reference tree is mounted)."""
    script = ORACLE / "build_ref.sh"
    if not script.exists():
        return None
    r = subprocess.run(["bash", str(script)], capture_output=True, text=True)
    if r.returncode == 3:      # reference sources absent on this machine
        return None
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    p = ORACLE / "_ref" / "houghline_ref.fatbin"
    return p if p.exists() else None


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_library(force=force, verbose=True))
    print(build_oracle(force=force))
    print(build_ref_runner(force=force))
    print(build_reference_fatbin())
