"""Host arrays are read and written in place by the packing kernels where
the GPU can address them (pinned memory, and pageable memory on systems
whose GPU uses the host's page tables); DC_GB300_STAGED_COPIES=1 forces the
staged copies.  Both paths must give bit-identical device state and
read-backs, for pageable and pinned arrays, through the library API and the
reference ABI."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent

SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
import __graft_entry__ as ge
dc = ge.package()
import torch
sizes = (37, 29, 23)
shape = (23, 29, 37)
rng = np.random.default_rng(5)
coef = [rng.uniform(0.1, 1.0, shape).astype(np.float32) for _ in range(6)]
coef += [rng.uniform(1e6, 2e7, shape).astype(np.float32) for _ in range(4)]
fields = [rng.standard_normal(shape).astype(np.float32) for _ in range(4)]
pinned = {pinned}
def host(a):
    if not pinned:
        return a
    t = torch.empty(a.size, dtype=torch.float32, pin_memory=True)
    v = t.numpy().reshape(a.shape)
    v[:] = a
    host.keep.append(t)
    return v
host.keep = []
coef = [host(c) for c in coef]
fields = [host(f) for f in fields]
out = {{}}
for form in (dc.MEDIUM_PRECOMP, dc.MEDIUM_PRECOMP_F16):
    with dc.Simulation(sizes, (10.0,) * 3, 1e-3, kernel=dc.KERNEL_FAST, medium=form,
                       device=0) as sim:
        sim.set_precomp(coef)
        sim.set_fields(*fields)
        back = sim.get_precomp()
        sim.run(7)
        sim.synchronize()
        f = sim.get_fields()
    out[f"coef{{form}}"] = np.stack(back)
    for k, v in f.items():
        out[f"{{k}}{{form}}"] = v
with dc.Simulation(sizes, (10.0,) * 3, 1e-3, kernel=dc.KERNEL_FAST,
                   medium=dc.MEDIUM_VPZ_VSV, device=0) as sim:
    sim.set_vpz_vsv(host(np.full(shape, 3000, np.float32)), host(np.full(shape, 1200, np.float32)))
    sim.set_fields(*fields)
    sim.run(5)
    sim.synchronize()
    for k, v in sim.get_fields().items():
        out["vv_" + k] = v
proc = dc.Process(sizes, (10.0,) * 3, 1e-3, pp=fields[0], pc=fields[1], qp=fields[2],
                  qc=fields[3], precomp=coef, source_index=-1)
data = dc.device_data_init(proc)
for it in range(3):
    dc.propagate((4, 4, 4), (33, 25, 19), sizes, data, 10.0, 10.0, 10.0, 1e-3)
    dc.device_swap_arrays(data)
dc.device_data_get_results(proc, data)
dc.device_data_free(data)
out["abi_pc"] = proc.field("pc").copy()
out["abi_qc"] = proc.field("qc").copy()
np.savez({path!r}, **out)
"""


def _run(tmp_path, staged: bool, pinned: bool):
    path = tmp_path / f"out_{int(staged)}_{int(pinned)}.npz"
    env = dict(os.environ)
    env.pop("DC_GB300_STAGED_COPIES", None)
    if staged:
        env["DC_GB300_STAGED_COPIES"] = "1"
    code = SCRIPT.format(root=str(ROOT), pinned=pinned, path=str(path))
    subprocess.run([sys.executable, "-c", code], env=env, check=True, timeout=600)
    return dict(np.load(path))


@pytest.mark.parametrize("pinned", [False, True])
def test_direct_and_staged_transfers_agree(tmp_path, pinned):
    direct = _run(tmp_path, False, pinned)
    staged = _run(tmp_path, True, pinned)
    assert direct.keys() == staged.keys()
    for k in direct:
        assert np.array_equal(direct[k], staged[k]), k
    # the read-back of the medium is the medium
    assert np.isfinite(direct["pc0"]).all() and np.abs(direct["abi_pc"]).max() > 0
