"""The C-ABI library on the CPU: it loads without a GPU, exports every entry
point include/dc_gb300.h declares, its host-side set-up functions reproduce
the reference bit for bit, and argument errors are reported before any
device work."""
import ctypes as C
import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_library_exports_every_header_symbol(dc):
    lib = dc.lib()
    declared = dc.header_symbols()
    assert len(declared) >= 40
    missing = [n for n in declared if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes table covers every declaration
    bound = {n for n, _, _ in dc.SIGNATURES}
    assert set(declared) <= bound, set(declared) - bound


def test_exported_dynamic_symbols(dc):
    out = subprocess.run(["nm", "-D", "--defined-only", str(dc.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    names = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for n in dc.header_symbols():
        assert n in names, n


_LAYOUT_C = r"""
#include <stdio.h>
#include <stddef.h>
#include HEADER
#define O(T, f) printf("%s.%s %zu\n", #T, #f, offsetof(T, f))
int main(void) {
  O(dc_process_t, rank); O(dc_process_t, iterations); O(dc_process_t, source_index);
  O(dc_process_t, dx); O(dc_process_t, dt); O(dc_process_t, sizes);
  O(dc_process_t, anisotropy_vars); O(dc_process_t, precomp_vars); O(dc_process_t, pp);
  O(dc_process_t, qc); O(dc_process_t, hostnames); O(dc_process_t, num_workers);
  printf("dc_process_t.size %zu\n", sizeof(dc_process_t));
  O(dc_device_data, pp); O(dc_device_data, vpz); O(dc_device_data, precomp_vars);
  printf("dc_device_data.size %zu\n", sizeof(dc_device_data));
  O(dc_precomp_vars, v2pn); O(dc_anisotropy_t, delta);
  return 0;
}
"""


def _layout(tmp_path, include_dirs, header):
    src = tmp_path / "layout.c"
    src.write_text(_LAYOUT_C.replace("HEADER", f'"{header}"'))
    exe = tmp_path / "layout"
    cmd = ["gcc", "-o", str(exe), str(src)] + [f"-I{d}" for d in include_dirs]
    subprocess.run(cmd, check=True, capture_output=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict(line.split() for line in out.splitlines())


def test_struct_layouts_ctypes_match_header(dc, tmp_path):
    lay = _layout(tmp_path, [str(dc.HEADER.parent)], "dc_gb300.h")
    P, D = dc.ProcessT, dc.DeviceData
    for f in ("rank", "iterations", "source_index", "dx", "dt", "sizes", "anisotropy_vars",
              "precomp_vars", "pp", "qc", "hostnames", "num_workers"):
        assert int(lay[f"dc_process_t.{f}"]) == getattr(P, f).offset, f
    assert int(lay["dc_process_t.size"]) == C.sizeof(P)
    for f in ("pp", "vpz", "precomp_vars"):
        assert int(lay[f"dc_device_data.{f}"]) == getattr(D, f).offset, f
    assert int(lay["dc_device_data.size"]) == C.sizeof(D)
    assert int(lay["dc_precomp_vars.v2pn"]) == dc.PrecompVars.v2pn.offset
    assert int(lay["dc_anisotropy_t.delta"]) == dc.Anisotropy.delta.offset


def test_struct_layouts_match_reference_headers(dc, tmp_path, reference):
    """Our header's ABI structs against the reference's own headers
    (include/dc_process.h, include/device_data.h), compiled side by side."""
    from oracle import build_oracle
    ours = _layout(tmp_path, [str(dc.HEADER.parent)], "dc_gb300.h")
    ref_inc = build_oracle.source_root() / "include"
    stub = Path(build_oracle.__file__).resolve().parent / "ref_stub"
    theirs = _layout(tmp_path, [str(ref_inc), str(stub)], "device_data.h")
    assert ours == theirs


def test_calculate_source_bit_exact(dc):
    g = np.load(GOLDEN / "source.npz")
    for tag, dt in (("1e-3", 1e-3), ("8e-4", 8e-4), ("1e-6", 1e-6)):
        mine = np.array([dc.calculate_source(dt, i) for i in range(2001)], np.float32)
        assert np.array_equal(mine, g["dt_" + tag])


def test_parameterised_source(dc):
    assert dc.source(1e-3, 17, 40.0) == dc.calculate_source(1e-3, 17)
    # Ricker peak frequency fcut/3: the wavelet of fcut=45 peaks later than 60
    t45 = dc.source_table(1e-3, 300, 45.0)
    t60 = dc.source_table(1e-3, 300, 60.0)
    assert np.argmax(t45) > np.argmax(t60)
    assert math.isclose(t45.max(), 1.0, abs_tol=1e-2)


def test_default_anisotropy_and_boundary_bit_exact(dc):
    g = np.load(GOLDEN / "default_rvb.npz")
    sizes = tuple(int(v) for v in g["sizes"])
    n = tuple(int(v) for v in g["n"])
    a = dc.compute_anisotropy_vars(sizes)
    dc.random_velocity_boundary(sizes, sizes, (0, 0, 0), n, 4, int(g["absorb"]), a["vpz"],
                                a["vsv"], 0)
    assert np.array_equal(a["vpz"], g["vpz"])
    assert np.array_equal(a["vsv"], g["vsv"])


def test_partitioned_boundary_bit_exact(dc):
    g = np.load(GOLDEN / "rvb_partitions.npz")
    glob = tuple(int(v) for v in g["glob"])
    n = tuple(int(v) for v in g["n"])
    for k in range(int(g["parts"])):
        local = tuple(int(v) for v in g[f"p{k}_local"])
        start = tuple(int(v) for v in g[f"p{k}_start"])
        shape = (local[2], local[1], local[0])
        vpz = np.full(shape, 3000.0, np.float32)
        vsv = np.full(shape, 1296.0, np.float32)
        seed = dc.random_velocity_boundary(local, glob, start, n, 4, int(g["absorb"]), vpz, vsv)
        assert np.array_equal(vpz, g[f"p{k}_vpz"]) and np.array_equal(vsv, g[f"p{k}_vsv"])
        assert seed == int(g[f"p{k}_seed"])


def test_sponge_profile_matches_oracle(dc, port):
    for s, a, kappa in ((104, 16, 0.3), (616, 48, 0.35), (20, 0, 0.3), (30, 5, 1.0)):
        assert np.array_equal(dc.sponge_profile(s, a, kappa), port.sponge_profile(s, a, kappa))
    g = dc.sponge_profile(40, 8, 0.3)
    assert g[:4].tolist() == [1.0] * 4 and g[-4:].tolist() == [1.0] * 4
    assert np.all(g[12:28] == 1.0) and g[4] < g[11] < 1.0


def test_create_rejects_bad_arguments_before_device_work(dc):
    for sizes in ((8, 20, 20), (20, 20, 3)):
        with pytest.raises(dc.DcError) as e:
            dc.Simulation(sizes)
        assert e.value.code == dc.ERR_ARG
    with pytest.raises(dc.DcError) as e:
        dc.Simulation((20, 20, 20), dt=0.0)
    assert e.value.code == dc.ERR_ARG
    with pytest.raises(dc.DcError) as e:
        dc.Simulation((20, 20, 20), kernel=7)
    assert e.value.code == dc.ERR_ARG


def test_null_handles_are_errors(dc):
    lib = dc.lib()
    assert lib.dc_gb300_run(None, 1) == dc.ERR_ARG
    assert lib.dc_gb300_set_fields(None, None, None, None, None) == dc.ERR_ARG
    assert "null" in dc.last_error()
    assert lib.dc_gb300_steps_done(None) == 0


def test_version_string(dc):
    assert b"sm_103a" in dc.lib().dc_gb300_version()
