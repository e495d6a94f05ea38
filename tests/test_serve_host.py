"""Serving host logic without a GPU: the tick planner, the C struct layouts the Python
mirror relies on, and the no-device error of hsr_server_create."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_plan_tick_water_filling(product_lib):
    from hussar_gb300.serve import plan_tick
    tile = 4096
    # a short request finishes in one tick, long ones share the rest
    rem = [10 * tile + 5, 1 << 24, 1 << 22, 300]
    c = plan_tick(rem, target=1 << 20, tile=tile)
    assert c[3] == 300 and c[0] == 10 * tile + 5
    assert all(c[i] <= rem[i] for i in range(4))
    assert c[1] == c[2]  # equal shares for the two long ones
    assert c[1] % tile == 0
    assert abs(int(c.sum()) - (1 << 20)) <= 2 * tile


def test_plan_tick_properties(product_lib):
    from hussar_gb300.serve import plan_tick
    rng = np.random.default_rng(5)
    tile = 4096
    for _ in range(200):
        n = int(rng.integers(1, 40))
        rem = (2.0 ** rng.uniform(0, 25, n)).astype(np.int64)
        rem[rng.random(n) < 0.1] = 0
        target = int(2 ** rng.uniform(10, 26))
        c = plan_tick(rem, target, tile)
        assert (c >= 0).all() and (c <= rem).all()
        # every chunk that is not the request's last is a whole number of tiles
        partial = c < rem
        assert (c[partial] % tile == 0).all()
        # every request with work gets at least one tile (or finishes)
        assert ((c >= np.minimum(rem, tile)) | (rem == 0)).all()
        # the tick is not much larger than its target (or one tile per request)
        assert c.sum() <= max(target, tile * n) + tile * n


def test_plan_tick_rejects_bad_input(product_lib):
    from hussar_gb300 import HsrError
    from hussar_gb300.serve import plan_tick
    with pytest.raises(HsrError):
        plan_tick([-1], 100)
    with pytest.raises(HsrError):
        plan_tick([5], 100, tile=0)


C_LAYOUT = r"""
#include <stddef.h>
#include <stdio.h>
#include "hsr_gb300.h"
#define F(T, m) printf(#T "." #m " %zu\n", offsetof(T, m))
#define S(T) printf(#T " %zu\n", sizeof(T))
int main(void) {
    S(hsr_server_config); F(hsr_server_config, memory_bytes); F(hsr_server_config, tick_ms);
    F(hsr_server_config, phase_mode); F(hsr_server_config, flags);
    S(hsr_request); F(hsr_request, rf); F(hsr_request, tx); F(hsr_request, rx); F(hsr_request, budget);
    F(hsr_request, index_offset); F(hsr_request, out_row);
    S(hsr_request_result); F(hsr_request_result, queue_ms); F(hsr_request_result, latency_ms);
    S(hsr_server_stats); F(hsr_server_stats, device_ms); F(hsr_server_stats, max_batch);
    F(hsr_server_stats, admitted_while_busy); F(hsr_server_stats, scene_bytes);
    S(hsr_tracer_flags); S(hsr_antenna); S(hsr_rf_config);
    S(hsr_launch_config); F(hsr_launch_config, queue_threshold); F(hsr_launch_config, default_trace_ms);
    F(hsr_launch_config, field_on_hit); F(hsr_launch_config, coherent_order);
    S(hsr_ff_antenna); F(hsr_ff_antenna, polarization); F(hsr_ff_antenna, scene_center); F(hsr_ff_antenna, radius);
    return 0;
}
"""


def test_ctypes_mirrors_match_c_layout(tmp_path):
    """The ctypes structs have the C compiler's sizes and offsets."""
    from hussar_gb300 import _lib
    src = tmp_path / "layout.c"
    src.write_text(C_LAYOUT)
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    c = dict(line.rsplit(" ", 1) for line in out if line)
    mirrors = {"hsr_server_config": _lib.ServerConfigC, "hsr_request": _lib.RequestC,
               "hsr_request_result": _lib.RequestResultC, "hsr_server_stats": _lib.ServerStatsC,
               "hsr_tracer_flags": _lib.FlagsC, "hsr_antenna": _lib.AntennaC, "hsr_rf_config": _lib.RFConfigC,
               "hsr_launch_config": _lib.LaunchConfigC, "hsr_ff_antenna": _lib.FfAntennaC}
    for key, val in c.items():
        if "." in key:
            t, m = key.split(".")
            assert getattr(mirrors[t], m).offset == int(val), key
        else:
            assert ctypes.sizeof(mirrors[key]) == int(val), key


def test_server_create_without_device(product_lib):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    from hussar_gb300 import _lib
    cfg = _lib.ServerConfigC()
    product_lib.hsr_default_server_config(ctypes.byref(cfg))
    assert cfg.flags.doGuiding == 0 and cfg.flags.useGeometricalOptics == 1 and cfg.flags.maxDepth == 10
    h = ctypes.c_void_p()
    assert product_lib.hsr_server_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.HSR_ERR_NO_DEVICE
    # guided serving is supported; without geometrical optics the server refuses
    cfg.flags.doGuiding = 1
    assert product_lib.hsr_server_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.HSR_ERR_NO_DEVICE
    cfg.flags.useGeometricalOptics = 0
    assert product_lib.hsr_server_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.HSR_ERR_NOT_SUPPORTED
