"""Build the sm_103a shared libraries of the fluid hot path (and the oracle).

Two flavours of the same CUDA sources are linked:
  _lib/libphx_fluid.so        production build (FMA contraction on)
  _lib/libphx_fluid_exact.so  parity build (-fmad=false, PHX_EXACT): every
                              multiply and add rounded separately, so it
                              reproduces a CPU build without contraction bit
                              for bit where the arithmetic is IEEE
                              (+, -, *, /, sqrt, fmin/fmax).
Objects are compiled in parallel with nvcc; no cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "_lib"
OBJ = PKG / "_build"
SOURCES = ["phx_api.cu", "phx_c2p.cu", "phx_flux.cu", "phx_stage.cu", "phx_geometry.cu", "phx_mlp.cu", "phx_noalloc.cu",
           "phx_fixup.cu", "phx_batch.cu", "phx_m1.cu", "phx_torus.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAVOURS = {
    "libphx_fluid.so": ["-fmad=true"],
    "libphx_fluid_exact.so": ["-fmad=false", "-DPHX_EXACT"],
}
# Sources compiled without contraction in both flavours: the FMKS geometry
# tables (built once per block) and the torus initial state equal the
# oracle's bit for bit in both.
NO_CONTRACT = {"phx_geometry.cu", "phx_torus.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_cuda(force: bool = False, verbose: bool = False, jobs: int | None = None) -> dict[str, Path]:
    """Compile every CUDA source for sm_103a and link both flavours."""
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "phx_fluid.h",
                                                                       ROOT / "include" / "phx_radiation.h"]
    tool = nvcc()
    # host code without contraction too: host-side constants (FMKS norm and
    # step, the torus' density scale) then equal the oracle's on aarch64,
    # where the host compiler would otherwise fuse multiply-adds
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
                     "--expt-relaxed-constexpr", "-I", str(ROOT / "include")]
    jobs_list = []
    for lib, extra in FLAVOURS.items():
        tag = "exact" if "exact" in lib else "fast"
        for src in SOURCES:
            s = CSRC / src
            o = OBJ / f"{s.stem}.{tag}.o"
            if force or _stale(o, [s] + headers):
                flags = ["-fmad=false" if f == "-fmad=true" and src in NO_CONTRACT else f for f in extra]
                jobs_list.append([tool, *common, *flags, "-c", str(s), "-o", str(o)])
    if jobs_list:
        n = jobs or max(1, min(len(jobs_list), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(n) as ex:
            list(ex.map(_run, jobs_list))
    out = {}
    for lib, _ in FLAVOURS.items():
        tag = "exact" if "exact" in lib else "fast"
        objs = [OBJ / f"{Path(s).stem}.{tag}.o" for s in SOURCES]
        target = LIB / lib
        if force or _stale(target, objs):
            _run([tool, *ARCH, "-shared", "-o", str(target), *map(str, objs), "-lcuda"])
        out[lib] = target
    return out


# The oracle in two builds of the same source: the parity build (contraction
# off, every operation rounded as written) that the tests compare against, and
# a timing build (-O3, contraction and unrolling on) for the CPU baseline.
# Neither uses -march=native: host code builds the same on the x86 container
# and the aarch64 GPU host (whose base ISA already has FMA and NEON).
ORACLE_BUILDS = {
    "libphx_oracle.so": ["-O2", "-ffp-contract=off"],
    "libphx_oracle_tuned.so": ["-O3", "-ffp-contract=fast", "-fno-math-errno", "-funroll-loops"],
}


def build_oracle(force: bool = False) -> Path:
    """Compile the CPU oracle (test infrastructure): the parity build and the
    timing build; returns the parity build's path."""
    src = ROOT / "oracle" / "phx_oracle.cpp"
    outdir = ROOT / "oracle" / "_build"
    outdir.mkdir(exist_ok=True)
    deps = [src, ROOT / "include" / "phx_fluid.h", ROOT / "include" / "phx_radiation.h", CSRC / "phx_math.h"]
    jobs = []
    for name, flags in ORACLE_BUILDS.items():
        target = outdir / name
        if force or _stale(target, deps):
            jobs.append(["g++", *flags, "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", str(target), str(src)])
    if jobs:
        with cf.ThreadPoolExecutor(len(jobs)) as ex:
            list(ex.map(_run, jobs))
    return outdir / "libphx_oracle.so"


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_cuda(force=force))
    print(build_oracle(force=force))
