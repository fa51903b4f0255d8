"""Build recipe for the oracle (test infrastructure only).

* ``oracle/build/liboracle.so`` -- our C restatement (dc_oracle.c).  Built
  wherever tests run, including the GPU host, by ``build_port()``.
* ``oracle/_ref/libref.so`` -- the reference's own single-rank sources
  (OpenMP backend, medium set-up, boundary, source) compiled where they lie
  under the reference checkout, plus ``ref_driver.c``.  Built only where the
  checkout exists (``build_ref()``); never committed (``oracle/_ref/`` is
  git-ignored).  The reference's flags are ``-O3 -fopenmp``
  (reference Makefile:12,34-35); ``-ffp-contract=off`` keeps FMA contraction
  off on hosts whose default ISA has FMA, so results match an x86-64 build.
"""
from __future__ import annotations

import os
import platform
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
PORT_SO = HERE / "build" / "liboracle.so"
REF_SO = HERE / "_ref" / "libref.so"
REFERENCE_ROOT = Path(os.environ.get("DC_REFERENCE_ROOT", "/root/reference"))

# The reference files on the propagation path that build without MPI.
REF_SOURCES = (
    "src/openmp_propagate.c",
    "src/precomp.c",
    "src/boundary.c",
    "src/calculate_source.c",
    "src/device_data.c",
    "src/log.c",
)


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
    stamp = so.parent / "ARCH"
    return not stamp.exists() or stamp.read_text().strip() != platform.machine()


def _stamp(so: Path) -> None:
    (so.parent / "ARCH").write_text(platform.machine())


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


def reference_available() -> bool:
    return all((REFERENCE_ROOT / s).is_file() for s in REF_SOURCES)


def build_ref(force: bool = False) -> Path | None:
    """Compile the reference's sources into oracle/_ref/libref.so, or return
    None when the reference checkout is absent (e.g. on the GPU host)."""
    if not reference_available():
        return None
    srcs = [REFERENCE_ROOT / s for s in REF_SOURCES] + [HERE / "ref_driver.c"]
    deps = srcs + [HERE / "ref_stub" / "mpi.h"]
    if force or _stale(REF_SO, deps) or _arch_changed(REF_SO):
        REF_SO.parent.mkdir(parents=True, exist_ok=True)
        tmp = REF_SO.with_suffix(f".so.tmp{os.getpid()}")
        _run(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
              "-Wl,-Bsymbolic", "-w",
              "-I", str(HERE / "ref_stub"), "-I", str(REFERENCE_ROOT / "include"),
              *map(str, srcs), "-o", str(tmp), "-lm"])
        os.replace(tmp, REF_SO)
        _stamp(REF_SO)
    return REF_SO


if __name__ == "__main__":
    print(build_port(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
