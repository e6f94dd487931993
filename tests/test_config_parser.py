"""The configuration loader three ways, on the same documents: the Python
`load_config`, the C ABI's `os_config_parse` and the C++ `ConfigParser` of
include/opensayal_gb300/config_parser.hpp (through tests/cpp/drop_in_main.cpp),
all following ConfigParser (inc/config_parser.hpp:118-151,
src/config_parser.cpp:11-184). CPU only: parsing touches no device."""
import ctypes as C
import json
import subprocess

import numpy as np
import pytest

from opensayal_gb300 import native
from opensayal_gb300.fluid import CONFIG_KEYS, load_config, visual_defaults
from tests.conftest import ROOT
from tests.test_cpp_dropin import build_program

# (name, document text). Every document is valid JSON.
DOCUMENTS = [
    ("empty", "{}"),
    ("nested", json.dumps({
        "sim": {"width": 320, "height": 200, "enable_drain": False, "enable_pressure": True,
                "projection": {"n": 30, "o": 1.7},
                "wind_tunnel": {"pipe_height": 44, "speed": 2.5, "smoke": 0.5,
                                "smoke_length": 3, "smoke_count": 1},
                "physics": {"g": -9.81}, "time": {"d_t": 0.02, "enable_real_time": True},
                "smoke": {"enable_decay": True, "decay_rate": 0.125},
                "obstacle": {"enable": True, "center_x": 100, "center_y": 90, "radius": 12.75}},
        "fluid": {"density": 1.25, "drag_coeff": 0.01, "viscosity": 0.0},
        "thread": {"cuda": {"block_size_x": 128, "block_size_y": 2}, "openMP": {"thread_count": 8}},
        "visual": {"arrows": {"color": {"r": 10, "g": 20, "b": 30, "a": 40}, "enable": True,
                              "distance": 16, "length_multiplier": 0.25,
                              "disable_threshold": 0.5, "head_length": 7},
                   "path_line": {"enable": True, "length": 33, "distance": 11,
                                 "color": {"r": 1, "g": 2, "b": 3, "a": 4}}}})),
    ("dotted_whole_keys", json.dumps({
        "sim.width": 300, "sim": {"height": 90, "projection.n": 7, "wind_tunnel.speed": 1.5,
                                   "obstacle": {"radius": 4}},
        "fluid.viscosity": 0.002, "visual.arrows.color.r": 99,
        "visual": {"path_line.color": {"g": 5}}})),
    # "sim.wind_tunnel" whole at the top is not seen: the lookup splits at the
    # first dot only, so it looks for "sim" and then "wind_tunnel.speed".
    ("first_dot_only", json.dumps({"sim.wind_tunnel": {"speed": 3.0}, "sim": {"width": 64}})),
    ("conversions", json.dumps({
        "sim": {"width": 200.9, "height": 100, "projection": {"n": 12.99, "o": 2},
                "wind_tunnel": {"speed": True, "pipe_height": False},
                "obstacle": {"center_x": -3.7, "radius": 10}},
        "fluid": {"density": 0.1, "viscosity": 1e-3}})),
    ("nested_wrong_types_take_defaults", json.dumps({
        "sim": {"width": "wide", "height": None, "enable_drain": 1, "enable_smoke": "yes",
                "projection": {"n": [50], "o": {"x": 1}},
                "obstacle": {"enable": 0.0}}})),
    ("non_object_members", json.dumps({"sim": [1, 2, 3], "fluid": 5, "thread": None})),
    ("duplicates_last_wins", '{"sim": {"width": 100, "width": 140, "height": 70}}'),
    ("unicode_and_escapes", '{"note": "caf\\u00e9 \\ud83d\\ude00 \\"q\\" \\n", '
                            '"sim": {"height": 96, "label": "a/b\\\\c"}, "list": [true, false, '
                            'null, -0, 1.5e-3, {"k": []}]}'),
    ("whitespace", ' \n\t{ "sim" : { "width" : 257 , "height":129 } }\r\n '),
    ("big_numbers", json.dumps({"sim": {"width": 256, "height": 128},
                                "fluid": {"density": 1e30, "viscosity": 1e-45}})),
]

# Documents the reference's loader rejects (it throws out of parse()).
INVALID = [
    ("truncated", '{"sim": {"width": 256'),
    ("trailing_comma", '{"sim": {"width": 256,}}'),
    ("bare_word", "{sim: 1}"),
    ("two_values", "{} {}"),
    ("top_level_wrong_type", json.dumps({"sim.enable_drain": 1})),
    ("top_level_wrong_number", json.dumps({"sim.width": "wide"})),
]


def c_parse(text: str):
    lib = native.load()
    cfg, vis = native.OsConfig(), native.OsVisualConfig()
    raw = text.encode()
    rc = lib.os_config_parse(raw, len(raw), C.byref(cfg), C.byref(vis))
    return rc, cfg, vis


def _get_or(obj, key, typ, default, top=True):
    """A second, independent statement of ConfigParser::get_or for the keys
    that the library's structures do not carry (colours, enables, thread count)."""
    if isinstance(obj, dict) and key in obj:
        v = obj[key]
        ok = isinstance(v, bool) if typ is bool else isinstance(v, (bool, int, float))
        if not ok:
            if top:
                raise TypeError(key)
            return default
        return int(v) if typ in (int, bool) else float(np.float32(v))
    if "." not in key:
        return default
    parent, child = key.split(".", 1)
    if not isinstance(obj, dict) or parent not in obj:
        return default
    return _get_or(obj[parent], child, typ, default, top=False)


EXTRA_KEYS = [  # (key, type, default) read only by the C++ Config
    ("thread.openMP.thread_count", int, 0),
    ("visual.arrows.color.r", int, 0), ("visual.arrows.color.g", int, 0),
    ("visual.arrows.color.b", int, 0), ("visual.arrows.color.a", int, 255),
    ("visual.arrows.enable", bool, 0), ("visual.arrows.distance", int, 20),
    ("visual.arrows.length_multiplier", float, float(np.float32(0.1))),
    ("visual.arrows.disable_threshold", float, 0.0), ("visual.arrows.head_length", int, 5),
    ("visual.path_line.enable", bool, 0), ("visual.path_line.length", int, 20),
    ("visual.path_line.color.r", int, 0), ("visual.path_line.color.g", int, 0),
    ("visual.path_line.color.b", int, 0), ("visual.path_line.color.a", int, 255),
    ("visual.path_line.distance", int, 20),
]


def expected_visual(obj) -> native.OsVisualConfig:
    v = visual_defaults()
    v.cell_pixel_size = _get_or(obj, "sim.cell_pixel_size", int, 1)
    v.arrow_distance = _get_or(obj, "visual.arrows.distance", int, 20)
    v.arrow_length_multiplier = _get_or(obj, "visual.arrows.length_multiplier", float, 0.1)
    v.arrow_disable_threshold = _get_or(obj, "visual.arrows.disable_threshold", float, 0.0)
    v.arrow_head_length = _get_or(obj, "visual.arrows.head_length", int, 5)
    v.trace_distance = _get_or(obj, "visual.path_line.distance", int, 20)
    v.trace_length = _get_or(obj, "visual.path_line.length", int, 20)
    return v


@pytest.mark.parametrize("name,text", DOCUMENTS, ids=[d[0] for d in DOCUMENTS])
def test_c_abi_parser_equals_python_loader(lib_built, name, text):
    rc, cfg, vis = c_parse(text)
    assert rc == native.OS_OK, native.load().os_last_error()
    py = load_config(text)
    assert bytes(cfg) == bytes(py), (name, cfg.as_dict(), py.as_dict())
    assert bytes(vis) == bytes(expected_visual(json.loads(text)))


@pytest.mark.parametrize("name,text", INVALID, ids=[d[0] for d in INVALID])
def test_invalid_documents_are_errors_in_both(lib_built, name, text):
    rc, _, _ = c_parse(text)
    assert rc == native.OS_ERR_INVALID
    assert native.load().os_last_error().decode().startswith("config:")
    with pytest.raises((ValueError, TypeError)):
        load_config(text)


def test_named_examples():
    first = load_config(dict(DOCUMENTS)["first_dot_only"] and json.loads(
        dict(DOCUMENTS)["first_dot_only"]))
    assert first.tunnel_speed == 0.0 and first.width == 64
    conv = load_config(json.loads(dict(DOCUMENTS)["conversions"]))
    assert (conv.width, conv.projection_n, conv.obstacle_center_x) == (200, 12, -3)
    assert conv.tunnel_speed == 1.0 and conv.pipe_height == 0 and conv.projection_o == 2.0
    wrong = load_config(json.loads(dict(DOCUMENTS)["nested_wrong_types_take_defaults"]))
    assert (wrong.width, wrong.height, wrong.enable_drain, wrong.projection_n) == (1920, 1080, 1, 50)
    assert len(CONFIG_KEYS) == 31


def cpp_config(path) -> dict:
    exe = build_program()
    out = subprocess.run([str(exe), "--config", str(path)], capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    return {k: v for k, v in (line.split() for line in out.stdout.strip().splitlines())}


@pytest.mark.parametrize("name,text", DOCUMENTS, ids=[d[0] for d in DOCUMENTS])
def test_cpp_config_parser_equals_python_loader(lib_built, tmp_path, name, text):
    path = tmp_path / "OpenSayal.conf.json"
    path.write_text(text)
    got = cpp_config(path)
    py = load_config(path)
    obj = json.loads(text)
    for key, (field, typ) in CONFIG_KEYS.items():
        want = getattr(py, field)
        if typ is float:
            assert np.float32(float(got[key])) == np.float32(want), (name, key, got[key], want)
        else:
            assert int(got[key]) == int(want), (name, key, got[key], want)
    assert int(got["sim.wind_tunnel.pipe_length"]) == 0
    for key, typ, default in EXTRA_KEYS:
        want = _get_or(obj, key, typ, default)
        if typ is float:
            assert np.float32(float(got[key])) == np.float32(want), (name, key)
        else:
            assert int(got[key]) == int(want), (name, key, got[key], want)


def test_cpp_config_parser_reports_errors(lib_built, tmp_path):
    exe = build_program()
    bad = tmp_path / "bad.json"
    bad.write_text('{"sim": ')
    out = subprocess.run([str(exe), "--config", str(bad)], capture_output=True, text=True)
    assert out.returncode == 2 and "JSON" in out.stderr
    out = subprocess.run([str(exe), "--config", str(tmp_path / "missing.json")],
                         capture_output=True, text=True)
    assert out.returncode == 2 and "cannot open" in out.stderr
    assert ROOT.exists()
