"""Argument checks of the library's newer entry points, on the CPU: every
one below is rejected with DC_GB300_ERR_ARG and a message before any device
call, so no GPU is needed."""
import ctypes as C

import pytest


@pytest.fixture(scope="module")
def lib(dc):
    return dc.lib()


def _err(lib):
    return lib.dc_gb300_last_error().decode()


def test_batch_create_rejects_bad_configs(dc, lib):
    out = C.c_void_p()
    assert lib.dc_gb300_batch_create(None, C.byref(out)) == dc.ERR_ARG
    bad = [
        dc.BatchConfig(8, 64, 64, 12.5, 12.5, 12.5, 1e-3, dc.MEDIUM_PRECOMP, 0, 10),   # too small
        dc.BatchConfig(64, 64, 64, 0.0, 12.5, 12.5, 1e-3, dc.MEDIUM_PRECOMP, 0, 10),   # dx
        dc.BatchConfig(64, 64, 64, 12.5, 12.5, 12.5, 1e-3, dc.MEDIUM_VPZ_VSV, 0, 10),  # form
        dc.BatchConfig(64, 64, 64, 12.5, 12.5, 12.5, 1e-3, dc.MEDIUM_PRECOMP, 0, 0),   # steps
    ]
    for cfg in bad:
        assert lib.dc_gb300_batch_create(C.byref(cfg), C.byref(out)) == dc.ERR_ARG
        assert _err(lib)
        assert out.value is None


def test_batch_calls_on_null_handle(dc, lib):
    shot = dc.Shot(40, 40, 40, 0, 0, 0, 20, 20, 20, 40.0, 0, 0.0)
    assert lib.dc_gb300_batch_add_shot(None, C.byref(shot), None) == dc.ERR_ARG
    assert lib.dc_gb300_batch_run(None, 1) == dc.ERR_ARG
    assert lib.dc_gb300_batch_set_tiles(None, 8, 1) == dc.ERR_ARG
    assert lib.dc_gb300_batch_set_learned_layer(None, None, 8) == dc.ERR_ARG
    assert lib.dc_gb300_batch_steps_done(None) == -1
    assert lib.dc_gb300_batch_points(None) == -1
    assert lib.dc_gb300_batch_destroy(None) == dc.OK


def test_mlp_and_learned_layer_arguments(dc, lib):
    assert lib.dc_gb300_mlp_create(0, None) == dc.ERR_ARG
    assert lib.dc_gb300_mlp_set_params(None, None) == dc.ERR_ARG
    assert lib.dc_gb300_mlp_forward(None, None, 4, None) == dc.ERR_ARG
    assert lib.dc_gb300_mlp_train(None, None, None, 10, 1, 1, 1e-3, 0, None) == dc.ERR_ARG
    assert lib.dc_gb300_mlp_device_params(None) is None
    assert lib.dc_gb300_mlp_destroy(None) == dc.OK
    assert lib.dc_gb300_set_learned_layer(None, None, 8) == dc.ERR_ARG
    n = C.c_longlong()
    off = (C.c_long * 3)(0, 0, 0)
    assert lib.dc_gb300_lb_sample(None, None, off, 8, None, None, 0, C.byref(n)) == dc.ERR_ARG
    assert lib.dc_gb300_lb_rollout(None, None, off, 4, None, None, 0, C.byref(n)) == dc.ERR_ARG


@pytest.mark.parametrize("sizes,layer", [((30, 40, 40), 8), ((64, 64, 64), 0),
                                         ((64, 64, 64), 17)])
def test_layer_cells_rejects_bad_geometry(dc, lib, sizes, layer):
    assert lib.dc_gb300_layer_cells(*sizes, layer, None, 0) == -1
    assert "layer" in _err(lib)
    with pytest.raises(dc.DcError):
        dc.layer_cells(sizes, layer)


def test_noalloc_rejects_before_touching_the_device(dc, lib):
    cfg = dc.Config(20, 20, 20, 12.5, 12.5, 12.5, 1e-3, dc.KERNEL_EXACT, dc.MEDIUM_PRECOMP, 0)
    pairs = (C.c_void_p * 2)(16, 32)
    assert lib.dc_gb300_exact_steps_noalloc(C.byref(cfg), pairs, C.c_void_p(48), 5000, None,
                                            None) == dc.ERR_ARG
    assert "4096" in _err(lib)
    fast = dc.Config(20, 20, 20, 12.5, 12.5, 12.5, 1e-3, dc.KERNEL_FAST, dc.MEDIUM_PRECOMP, 0)
    assert lib.dc_gb300_exact_steps_noalloc(C.byref(fast), pairs, C.c_void_p(48), 1, None,
                                            None) == dc.ERR_ARG
    assert lib.dc_gb300_exact_steps_noalloc(None, pairs, None, 1, None, None) == dc.ERR_ARG
