"""The C ABI: the library loads without a GPU, exports every declared entry
point, its ctypes mirror matches the C layout, and configuration handling
follows the reference's ConfigParser."""
import ctypes as C
import re
import subprocess
import sys

import numpy as np
import pytest

from opensayal_gb300 import native
from opensayal_gb300.fluid import CONFIG_KEYS, default_config, load_config
from tests.conftest import ROOT

HEADER = ROOT / "include" / "opensayal_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(os_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib_built):
    lib = native.load()
    names = declared_functions()
    assert len(names) >= 14
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    bound = {n for n, _, _ in native.SIGNATURES}
    assert set(names) == bound, "ctypes signatures out of sync with the header"


def test_abi_version(lib_built):
    assert native.load().os_abi_version() == 3


def _c_layout() -> dict:
    """sizeof/offsetof of the ABI structs as the C compiler lays them out."""
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "opensayal_gb300.h"
#define F(s, m) printf(#s "." #m " %zu\n", offsetof(s, m));
int main(void) {
  printf("os_config %zu\nos_source %zu\nos_fields_view %zu\nos_batch_stats %zu\nos_diag %zu\n",
         sizeof(os_config), sizeof(os_source), sizeof(os_fields_view), sizeof(os_batch_stats),
         sizeof(os_diag));
  F(os_config, viscosity) F(os_config, storage) F(os_config, idw_mode)
  F(os_config, obstacle_radius) F(os_source, position_y) F(os_fields_view, total_s)
  F(os_batch_stats, members_in_plan) F(os_batch_stats, steps_completed)
  F(os_diag, outflow_flux) F(os_diag, active_cells)
  return 0;
}
'''
    build = ROOT / "oracle" / "build"
    build.mkdir(exist_ok=True)
    c_file = build / "layout_check.c"
    exe = build / "layout_check"
    c_file.write_text(src)
    subprocess.run(["gcc", "-std=c11", f"-I{ROOT / 'include'}", "-o", str(exe), str(c_file)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}


def test_ctypes_mirror_matches_c_layout():
    lay = _c_layout()
    assert lay["os_config"] == C.sizeof(native.OsConfig)
    assert lay["os_source"] == C.sizeof(native.OsSource)
    assert lay["os_fields_view"] == C.sizeof(native.OsFieldsView)
    assert lay["os_batch_stats"] == C.sizeof(native.OsBatchStats)
    assert lay["os_diag"] == C.sizeof(native.OsDiag)
    for key, cls in [("os_config.viscosity", native.OsConfig), ("os_config.storage", native.OsConfig),
                     ("os_config.idw_mode", native.OsConfig),
                     ("os_config.obstacle_radius", native.OsConfig),
                     ("os_source.position_y", native.OsSource),
                     ("os_fields_view.total_s", native.OsFieldsView),
                     ("os_batch_stats.members_in_plan", native.OsBatchStats),
                     ("os_batch_stats.steps_completed", native.OsBatchStats),
                     ("os_diag.outflow_flux", native.OsDiag),
                     ("os_diag.active_cells", native.OsDiag)]:
        field = key.split(".")[1]
        assert lay[key] == getattr(cls, field).offset, key


def test_defaults_follow_config_parser(lib_built):
    """src/config_parser.cpp:21-179."""
    c = default_config(1920, 1080)
    assert (c.width, c.height) == (1920, 1080)
    assert (c.block_size_x, c.block_size_y) == (64, 1)
    assert c.projection_n == 50 and abs(c.projection_o - 1.9) < 1e-7
    assert c.pipe_height == 270 and c.smoke_height == 270 and c.pipe_length == 0
    assert c.smoke_length == 1 and c.smoke_count == 1
    assert c.tunnel_speed == 0.0 and c.tunnel_smoke == 1.0 and c.g == 0.0
    assert abs(c.d_t - 0.05) < 1e-8 and c.enable_real_time == 0
    assert c.enable_drain == 1 and c.enable_pressure == 0 and c.enable_smoke == 1
    assert c.smoke_enable_decay == 0 and abs(c.smoke_decay_rate - 0.05) < 1e-8
    assert c.obstacle_enable == 1 and (c.obstacle_center_x, c.obstacle_center_y) == (960, 540)
    assert c.obstacle_radius == np.float32(1080 / 30.0)
    assert c.density == 1.0 and c.drag_coeff == 0.0
    assert c.viscosity == np.float32(0.001)
    assert c.storage == 0 and c.idw_mode == 0


@pytest.mark.parametrize("size", [(1920, 1080), (256, 128), (4096, 4096), (97, 250), (7, 3),
                                  (1000, 330), (1, 1)])
def test_python_defaults_equal_the_c_abi_defaults(lib_built, size):
    """default_config is filled in Python (no library load); it must equal
    os_config_defaults byte for byte, and so must visual_defaults."""
    from opensayal_gb300.fluid import visual_defaults
    lib = native.load()
    c = native.OsConfig()
    assert lib.os_config_defaults(size[0], size[1], C.byref(c)) == native.OS_OK
    py = default_config(*size)
    assert bytes(py) == bytes(c), (py.as_dict(), c.as_dict())
    v = native.OsVisualConfig()
    assert lib.os_visual_defaults(C.byref(v)) == native.OS_OK
    assert bytes(visual_defaults()) == bytes(v)


def test_default_config_does_not_load_the_library():
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from opensayal_gb300 import scenarios\n"
            "scenarios.default_tunnel_config(); scenarios.batched_scenarios(4)\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libopensayal_gb300' not in maps, 'library mapped'\n" % str(ROOT))
    subprocess.run([sys.executable, "-c", code], check=True)


def test_load_config_dotted_and_nested_keys(lib_built):
    """ConfigParser::get_or (inc/config_parser.hpp:131-150): a dotted key may be
    given whole at any level or as nested objects; absent keys take defaults that
    follow the parsed size."""
    cfg = load_config({"sim": {"width": 256, "height": 128, "projection.n": 7,
                               "wind_tunnel": {"speed": 2.0}},
                       "fluid.viscosity": 0.0})
    assert (cfg.width, cfg.height) == (256, 128)
    assert cfg.projection_n == 7
    assert cfg.tunnel_speed == 2.0
    assert cfg.viscosity == 0.0
    assert cfg.pipe_height == 32 and cfg.smoke_height == 32
    assert (cfg.obstacle_center_x, cfg.obstacle_center_y) == (128, 64)
    cfg2 = load_config('{"sim.width": 300, "sim": {"height": 90}}')
    assert (cfg2.width, cfg2.height) == (300, 90)
    assert cfg2.obstacle_radius == np.float32(90 / 30.0)
    # A wrong type inside a nested object yields the default (the reference's
    # catch-all around its recursion); given whole at the top level it is an error.
    assert load_config({"sim": {"enable_drain": 1}}).enable_drain == 1
    assert load_config({"sim": {"enable_drain": False, "width": "wide"}}).width == 1920
    with pytest.raises(TypeError):
        load_config({"sim.enable_drain": 1})
    assert len(CONFIG_KEYS) == 31


@pytest.mark.parametrize("bad", [
    dict(width=2), dict(height=1), dict(cell_size=0.5), dict(projection_n=-1),
    dict(storage=9), dict(smoke_count=2, pipe_height=10, smoke_height=10),
    dict(block_size_x=0), dict(projection_resident=4), dict(diffusion_block=-2),
])
def test_invalid_configs_are_rejected_before_any_device_work(lib_built, bad):
    lib = native.load()
    cfg = default_config(64, 32)
    for k, v in bad.items():
        setattr(cfg, k, v)
    h = C.c_void_p()
    rc = lib.os_create(C.byref(cfg), C.byref(h))
    assert rc == native.OS_ERR_INVALID
    assert h.value is None
    assert lib.os_last_error().decode()


def test_null_arguments_are_errors(lib_built):
    lib = native.load()
    assert lib.os_update(None, None, C.c_float(0.05)) == native.OS_ERR_INVALID
    assert lib.os_destroy(None) == native.OS_OK
    assert lib.os_config_defaults(16, 16, None) == native.OS_ERR_INVALID
    assert lib.os_fields(None, None) == native.OS_ERR_INVALID


def test_visual_defaults_follow_config_parser(lib_built):
    # src/config_parser.cpp:39-40, 120-179
    from opensayal_gb300.fluid import visual_defaults
    v = visual_defaults()
    assert (v.cell_pixel_size, v.arrow_distance, v.arrow_head_length) == (1, 20, 5)
    assert (v.trace_distance, v.trace_length) == (20, 20)
    assert abs(v.arrow_length_multiplier - 0.1) < 1e-7 and v.arrow_disable_threshold == 0.0
    assert C.sizeof(native.OsArrow) == 36 and C.sizeof(native.OsVisualConfig) == 32


def test_query_and_probe_reject_bad_arguments(lib_built):
    """Argument checks come before any device work, so they hold without a GPU."""
    lib = native.load()
    idle = C.c_int32(7)
    assert lib.os_query(None, C.byref(idle)) == native.OS_ERR_INVALID
    g = C.c_float(1.0)
    assert lib.os_probe_copy_bandwidth(0, 24, 10, C.byref(g)) == native.OS_ERR_INVALID  # not x16
    assert lib.os_probe_copy_bandwidth(0, 1 << 20, 0, C.byref(g)) == native.OS_ERR_INVALID
    assert lib.os_probe_copy_bandwidth(0, 1 << 20, 10, None) == native.OS_ERR_INVALID
    text = b'{"sim": {"width": 64, "height": 32}}'
    cfg = native.OsConfig()
    assert lib.os_config_parse(None, 0, C.byref(cfg), None) == native.OS_ERR_INVALID
    assert lib.os_config_parse(text, len(text), None, None) == native.OS_ERR_INVALID


def test_grids_beyond_int_indices_are_rejected(lib_built):
    """The reference's cell indices are int: (W + 2)(H + 2) must stay below 2^31."""
    lib = native.load()
    cfg = default_config(46340, 46340)  # (W + 2)(H + 2) > 2^31 - 1
    h = C.c_void_p()
    assert lib.os_create(C.byref(cfg), C.byref(h)) == native.OS_ERR_INVALID
    assert b"2^31" in lib.os_last_error()


def test_kernel_profile_rejects_bad_arguments(lib_built):
    lib = native.load()
    k, m = C.c_float(), C.c_float()
    assert lib.os_profile_phase_kernels(None, 3, None, C.c_float(0.05), 1, None, C.byref(k),
                                        C.byref(m), None) == native.OS_ERR_INVALID
