"""Build recipe for the oracle (test infrastructure only).

* ``oracle/build/liboracle.so`` -- our C restatement (dc_oracle.c).  Built
  wherever tests run, including the GPU host, by ``build_port()``.
* ``oracle/_ref/src/`` -- the reference files this recipe compiles (the
  sources on the propagation path and the reference's ``include/``), staged
  by ``stage()`` from the reference checkout where one exists.  Git-ignored,
  never committed: it travels with the working tree to a GPU host that has
  no checkout, where the libraries below are built from it.
* ``oracle/_ref/libref.so`` -- the reference's OpenMP backend and set-up
  (``src/openmp_propagate.c``, ``src/precomp.c``, ``src/boundary.c``,
  ``src/calculate_source.c``, ``src/device_data.c``, ``src/log.c``) plus
  ``ref_driver.c``, with ``-ffp-contract=off`` so that results are
  bit-identical to an x86-64 build (the golden fixtures): the pin of the
  restatement.
* ``oracle/_ref/librefomp.so`` -- the same sources with the reference's own
  flags, ``-O3 -fopenmp`` (reference Makefile:12,34-35): the timed CPU
  baseline.  On aarch64 gcc contracts multiply-adds under these flags, as
  the reference's own build there does.
* ``oracle/_ref/librefcuda.so`` -- the reference's CUDA backend
  (``src/cuda_propagate.cu``, ``src/device_data.cu``) compiled by nvcc for
  sm_103a with the reference's CUDA flags (Makefile:16, ``-g -gencode``),
  with the host set-up sources and ``ref_driver.c`` (built with
  ``-DREF_DEVICE_BACKEND``): the reference's own GPU path, for the parity
  gate and the GPU-to-GPU comparison.

The checkout is located by the environment variable ``DC_REFERENCE_ROOT``
alone; without it the staged copy is used where one exists.  Stage once
with ``DC_REFERENCE_ROOT=<checkout> python oracle/build_oracle.py``.
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
PORT_SO = HERE / "build" / "liboracle.so"
REF_DIR = HERE / "_ref"
STAGE = REF_DIR / "src"
REF_SO = REF_DIR / "libref.so"
REF_NATIVE_SO = REF_DIR / "librefomp.so"
REF_CUDA_SO = REF_DIR / "librefcuda.so"
REF_OBJ = REF_DIR / "obj"
_ROOT_ENV = os.environ.get("DC_REFERENCE_ROOT")
REFERENCE_ROOT = Path(_ROOT_ENV) if _ROOT_ENV else None

# The reference files on the propagation path that build without MPI.
REF_SOURCES = (
    "src/openmp_propagate.c",
    "src/precomp.c",
    "src/boundary.c",
    "src/calculate_source.c",
    "src/device_data.c",
    "src/log.c",
)
# The reference's CUDA backend (Makefile:44-47) and the host set-up it
# links with.
REF_CUDA_SOURCES = ("src/cuda_propagate.cu", "src/device_data.cu")
REF_CUDA_HOST = ("src/precomp.c", "src/boundary.c", "src/calculate_source.c", "src/log.c")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{proc.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _arch_changed(so: Path) -> bool:
    stamp = so.with_name(so.name + ".arch")
    return not stamp.exists() or stamp.read_text().strip() != platform.machine()


def _stamp(so: Path) -> None:
    so.with_name(so.name + ".arch").write_text(platform.machine())


def build_port(force: bool = False) -> Path:
    src = HERE / "dc_oracle.c"
    deps = [src, HERE / "dc_oracle.h"]
    if force or _stale(PORT_SO, deps) or _arch_changed(PORT_SO):
        PORT_SO.parent.mkdir(parents=True, exist_ok=True)
        tmp = PORT_SO.with_suffix(f".so.tmp{os.getpid()}")
        _run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              "-Wl,-Bsymbolic", str(src), "-o", str(tmp), "-lm"])
        os.replace(tmp, PORT_SO)
        _stamp(PORT_SO)
    return PORT_SO


def _has_all(root: Path | None) -> bool:
    if root is None:
        return False
    files = REF_SOURCES + REF_CUDA_SOURCES
    return all((root / s).is_file() for s in files) and (root / "include").is_dir()


def stage() -> Path | None:
    """Copies the reference files this recipe compiles from the checkout into
    oracle/_ref/src (refreshing stale copies); returns the staged root, or
    None when no checkout is present (the copy already staged, if any, is
    kept)."""
    if not _has_all(REFERENCE_ROOT):
        return STAGE if _has_all(STAGE) else None
    files = list(REF_SOURCES + REF_CUDA_SOURCES)
    files += [str(p.relative_to(REFERENCE_ROOT)) for p in (REFERENCE_ROOT / "include").glob("*.h")]
    for rel in files:
        src, dst = REFERENCE_ROOT / rel, STAGE / rel
        if dst.exists() and dst.stat().st_mtime >= src.stat().st_mtime and \
                dst.stat().st_size == src.stat().st_size:
            continue
        dst.parent.mkdir(parents=True, exist_ok=True)
        if dst.exists():
            dst.chmod(0o644)
        shutil.copy2(src, dst)
        dst.chmod(0o644)
    return STAGE


def source_root() -> Path | None:
    """Where the reference sources are read from: the checkout if present,
    else the staged copy."""
    if _has_all(REFERENCE_ROOT):
        return REFERENCE_ROOT
    if _has_all(STAGE):
        return STAGE
    return None


def reference_available() -> bool:
    return source_root() is not None


def _build_ref_omp(so: Path, flags: list[str], force: bool) -> Path | None:
    root = source_root()
    if root is None:
        return None
    srcs = [root / s for s in REF_SOURCES] + [HERE / "ref_driver.c"]
    deps = srcs + [HERE / "ref_stub" / "mpi.h"]
    if force or _stale(so, deps) or _arch_changed(so):
        so.parent.mkdir(parents=True, exist_ok=True)
        tmp = so.with_suffix(f".so.tmp{os.getpid()}")
        _run(["gcc", *flags, "-fPIC", "-shared", "-Wl,-Bsymbolic", "-w",
              "-I", str(HERE / "ref_stub"), "-I", str(root / "include"),
              *map(str, srcs), "-o", str(tmp), "-lm"])
        os.replace(tmp, so)
        _stamp(so)
    return so


def build_ref(force: bool = False) -> Path | None:
    """The reference's OpenMP path, contraction off (bit-exact pin), or None
    when neither a checkout nor a staged copy exists."""
    return _build_ref_omp(REF_SO, ["-O3", "-fopenmp", "-ffp-contract=off"], force)


def build_ref_native(force: bool = False) -> Path | None:
    """The reference's OpenMP path with the reference's own flags (the timed
    CPU baseline), or None."""
    return _build_ref_omp(REF_NATIVE_SO, ["-O3", "-fopenmp"], force)


def _nvcc() -> str | None:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    return None


def build_ref_cuda(force: bool = False) -> Path | None:
    """The reference's CUDA backend for sm_103a with the one-rank driver, or
    None when the sources or nvcc are missing."""
    root = source_root()
    nvcc = _nvcc()
    if root is None or nvcc is None:
        return None
    inc = root / "include"
    cu = [root / s for s in REF_CUDA_SOURCES]
    host = [root / s for s in REF_CUDA_HOST]
    driver = HERE / "ref_driver.c"
    deps = cu + host + [driver, HERE / "ref_stub" / "mpi.h"] + list(inc.glob("*.h"))
    if not (force or _stale(REF_CUDA_SO, deps) or _arch_changed(REF_CUDA_SO)):
        return REF_CUDA_SO
    REF_OBJ.mkdir(parents=True, exist_ok=True)
    objs = []
    # reference Makefile:16 (CUDA_CFLAGS) with the GB300 architecture
    cuda_flags = ["-I", str(inc), "-g", "-gencode", "arch=compute_103a,code=sm_103a",
                  "-Xcompiler", "-fPIC"]
    for s in cu:
        o = REF_OBJ / (s.name + ".o")
        _run([nvcc, "-c", str(s), "-o", str(o), *cuda_flags])
        objs.append(o)
    for s in host + [driver]:
        o = REF_OBJ / (s.name + ".cuda.o")
        extra = ["-DREF_DEVICE_BACKEND"] if s == driver else []
        _run(["gcc", "-c", "-O3", "-fPIC", "-w", *extra, "-I", str(HERE / "ref_stub"),
              "-I", str(inc), str(s), "-o", str(o)])
        objs.append(o)
    tmp = REF_CUDA_SO.with_suffix(f".so.tmp{os.getpid()}")
    _run([nvcc, "-shared", "-o", str(tmp), *map(str, objs),
          "-gencode", "arch=compute_103a,code=sm_103a", "-cudart", "static",
          "-Xlinker", "-Bsymbolic", "-lm", "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, REF_CUDA_SO)
    _stamp(REF_CUDA_SO)
    return REF_CUDA_SO


def build_all(force: bool = False) -> dict:
    """Everything above that can be built here; the reference libraries
    only where a checkout or a staged copy exists."""
    stage()
    return {"port": build_port(force), "ref": build_ref(force),
            "ref_native": build_ref_native(force), "ref_cuda": build_ref_cuda(force)}


if __name__ == "__main__":
    for k, v in build_all(force="--force" in sys.argv).items():
        print(f"{k}: {v}")
