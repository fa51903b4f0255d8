"""Builds libdc_gb300.so in-tree with nvcc for sm_103a.

Each translation unit under csrc/ is compiled in parallel; the shared
library links the CUDA runtime statically so that it loads on machines
without a GPU driver (symbols can be inspected there; compute needs a
GB300).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "build"
LIB = PKG / "libdc_gb300.so"
CLI_SRC = PKG / "cli" / "dc_gb300_main.c"
CLI = PKG / "dc_gb300"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
          "-I", str(INCLUDE), "-I", str(CSRC)]
# host code that must round exactly like the reference's C: no contraction
HOST_STRICT = ["-Xcompiler", "-ffp-contract=off"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _compile(src: Path) -> Path:
    obj = BUILD / (src.name + ".o")
    deps = [src] + _headers()
    if obj.exists() and all(d.stat().st_mtime <= obj.stat().st_mtime for d in deps):
        return obj
    flags = COMMON + ARCH
    if src.suffix == ".cpp":
        flags = COMMON + HOST_STRICT
    cmd = [nvcc(), "-c", str(src), "-o", str(obj), *flags]
    if os.environ.get("DC_GB300_PTXAS_VERBOSE"):
        cmd += ["-Xptxas", "-v"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{proc.stderr}")
    if proc.stderr.strip() and os.environ.get("DC_GB300_PTXAS_VERBOSE"):
        sys.stderr.write(proc.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    # objects and library are host-architecture specific: rebuild when the
    # tree was built on another machine type
    stamp = BUILD / "ARCH"
    if not stamp.exists() or stamp.read_text().strip() != platform.machine():
        force = True
        if LIB.exists():
            LIB.unlink()
    if force:
        for o in BUILD.glob("*.o"):
            o.unlink()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    if LIB.exists() and all(o.stat().st_mtime <= LIB.stat().st_mtime for o in objs):
        build_cli()
        return LIB
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = [nvcc(), "-shared", "-o", str(tmp), *map(str, objs), *ARCH,
           "-cudart", "static", "-Xlinker", "-Bsymbolic", "-lpthread", "-ldl", "-lrt"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"link failed:\n{proc.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(platform.machine())
    if verbose:
        print(f"built {LIB}")
    build_cli(force=True)
    return LIB


def build_cli(force: bool = False) -> Path:
    """The command-line driver (cli/dc_gb300_main.c), linked against the
    library with an $ORIGIN run path."""
    deps = [CLI_SRC, LIB, INCLUDE / "dc_gb300.h"]
    if not force and CLI.exists() and all(d.stat().st_mtime <= CLI.stat().st_mtime for d in deps):
        return CLI
    tmp = CLI.with_name(f"{CLI.name}.tmp{os.getpid()}")
    cmd = ["gcc", "-O2", "-std=gnu11", "-Wall", str(CLI_SRC), "-I", str(INCLUDE),
           "-L", str(PKG), "-ldc_gb300", "-Wl,-rpath,$ORIGIN", "-lm", "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{proc.stderr}")
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
