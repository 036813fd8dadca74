"""Build libvissgb.so (and the drop-in executables) for sm_103a with nvcc.

Translation units are compiled in parallel, then linked into
viss_recon_shade_gb300/_lib/libvissgb.so.  Rebuilds only what changed.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
LIB = OUT / "libvissgb.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "--expt-relaxed-constexpr", f"-I{INCLUDE}", f"-I{CSRC}"] + os.environ.get("VISS_NVCC_FLAGS", "").split()

CU_SOURCES = ["capi.cu", "prep.cu", "vis_dft.cu", "recon.cu", "orbit.cu", "shade.cu", "probe.cu", "order.cu", "noalloc.cu", "finemap.cu"]
CPP_SOURCES = ["textio.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or Path(c).exists()):
            return c
    return "nvcc"


def _newer(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def _headers():
    return [INCLUDE / "viss_gb300.h"] + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h"))


def build(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    objs, jobs = [], []
    hdrs = _headers()
    for src in CU_SOURCES + CPP_SOURCES:
        sp = CSRC / src
        if not sp.exists():
            continue
        obj = OUT / (sp.stem + ".o")
        objs.append(obj)
        if force or _newer(obj, [sp] + hdrs):
            if src.endswith(".cu"):
                cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(sp), "-o", str(obj)]
                if ptxas_verbose:
                    cmd += ["-Xptxas", "-v"]
            else:
                cmd = [nvcc(), "-x", "c++", "-O2", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler",
                       "-fvisibility=hidden", f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(sp), "-o", str(obj)]
            jobs.append(cmd)

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for err in ex.map(run, jobs):
            if ptxas_verbose and err:
                print(err, file=sys.stderr)
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(f".{os.getpid()}.tmp.so")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
        run(cmd)
        os.replace(tmp, LIB)
    build_tools(run, force)
    return LIB


# Drop-in programs with the reference's names (one binary, dispatched on argv[0]).
TOOL_NAMES = ["vissGen10M_shade", "vissGen10M_shade_optim1", "vissGen10M_shade_optim2", "vissGen1M_shade_optim1",
              "vissGen1M_shade_optim2", "vissGen1M_shade_accurate", "vissGen1M_shade_appro", "shade1M", "shade10M", "shade30M",
              "MIncline_generate_uvw_float"]


def build_tools(run, force=False):
    src = CSRC / "dropin.cpp"
    bindir = OUT / "bin"
    bindir.mkdir(exist_ok=True)
    exe = bindir / "viss_dropin"
    if force or _newer(exe, [src, LIB, INCLUDE / "viss_gb300.h"]):
        tmp = bindir / f"viss_dropin.{os.getpid()}.tmp"
        run([nvcc(), "-x", "c++", "-O2", "-std=c++17", f"-I{INCLUDE}", str(src), "-o", str(tmp), f"-L{OUT}",
             "-lvissgb", "-lcudart", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN/.."])
        os.replace(tmp, exe)
    for name in TOOL_NAMES:
        link = bindir / name
        if not link.exists():
            link.symlink_to("viss_dropin")


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv)
    print(LIB)
