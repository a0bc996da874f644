"""Builds the product library in-tree: blackholerender_gb300/libbhr.so (sm_103a only).

nvcc compiles each .cu translation unit in parallel, then links one shared library with the
CUDA runtime linked statically. Host code is compiled with -ffp-contract=off so the per-view
float constants are the same on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = ROOT / "_build"
LIB = PKG / "libbhr.so"
SOURCES = ["kernels.cu", "api.cu", "noalloc.cu", "surrogate.cu", "surrogate_api.cu", "lens.cu", "shade.cu", "vol.cu",
           "bodies.cu", "bodies_vol.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libbhr.so")


# Device float code flushes denormals (as GLSL does): rsqrt and the fast divide then map to
# single SFU instructions without subnormal fix-up sequences. FP64 code is unaffected.
DEVICE_FLAGS = {"kernels.cu": ["-ftz=true"], "surrogate.cu": ["-ftz=true"], "lens.cu": ["-ftz=true"],
                # shading: IEEE +, -, *, / and sqrt without contraction, so that the noise volume
                # and every non-transcendental step round as the CPU restatement does
                "shade.cu": ["-fmad=false"], "vol.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
                "bodies.cu": ["-ftz=true"], "bodies_vol.cu": ["-ftz=true", "-prec-div=false", "-prec-sqrt=false"]}


def _flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17",
        "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
        "-I", str(ROOT / "include"), "-I", str(CSRC),
    ]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "bhr.h"]
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    jobs = []
    for src in srcs:
        obj = BUILD / (src.stem + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *_flags(), *DEVICE_FLAGS.get(src.name, []), "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(run, jobs))
    objs = [BUILD / (s.stem + ".o") for s in srcs]
    if force or jobs or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        run([nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lpthread"])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
