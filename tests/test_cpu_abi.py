"""The C-ABI library loads and exports every symbol include/axgb.h declares
(no device calls: this runs without a GPU)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "axgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(axgb_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_all_declared_symbols():
    import axgb
    from axgb import lib
    L = lib()
    names = _declared()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(axgb._SYMBOLS) <= set(names)


def test_version_and_config_defaults():
    import axgb
    L = axgb.lib()
    assert b"sm_103a" in L.axgb_version()
    cfg = axgb.parse_regrid_config({})
    # RegridConfig defaults (regrid_config.hpp:80-89)
    assert (cfg.method, cfg.norm_type, cfg.line_type, cfg.unmapped) == (0, 0, 1, 1)
    cfg = axgb.parse_regrid_config({"method": "conservative", "norm_type": "FracArea", "unmapped": "error"})
    assert (cfg.method, cfg.norm_type, cfg.unmapped) == (4, 1, 0)
    import pytest
    with pytest.raises(ValueError):
        axgb.parse_regrid_config({"method": "spline"})
    with pytest.raises(ValueError):
        axgb.parse_regrid_config({"norm_type": "area"})


def test_last_error_without_device():
    import axgb
    L = axgb.lib()
    h = ctypes.c_int()
    rc = L.axgb_generate_weights(12345, 67890, None, ctypes.byref(h))
    assert rc == axgb.ERR_HANDLE
    assert "unknown mesh handle" in axgb.last_error()
    assert L.axgb_destroy_matrix(999) != 0


def test_weight_cache_header_checks_without_device():
    """The blob header is validated before any device work (magic, version,
    truncation), as WeightCache::deserialize does (prop_weight_cache.cpp)."""
    import struct

    import axgb
    L = axgb.lib()
    h = ctypes.c_int()
    good = struct.pack("<IIB7xQQQ", 0x43574841, 1, 1, 2, 2, 1) + bytes(24 + 32 + 32)
    for blob, msg in ((b"XXXX" + good[4:], "magic"), (good[:4] + struct.pack("<I", 7) + good[8:], "version"),
                      (good[:30], "header"), (good[:60], "size")):
        rc = L.axgb_matrix_deserialize(ctypes.c_char_p(blob), len(blob), ctypes.byref(h))
        assert rc == axgb.ERR_INVALID, msg
        assert axgb.last_error()


def test_config_names_match_the_python_binding():
    """Every spelling parse_regrid_config of python/axis_py.cpp:144-221
    accepts maps to the RegridConfig enum value (regrid_config.hpp:24-72);
    integers pass through; an unknown name raises ValueError naming it."""
    import pytest

    import axgb
    names = {
        "method": {"bilinear": 0, "Bilinear": 0, "nearest_neighbor": 1, "NearestNeighbor": 1, "bicubic": 2,
                   "Bicubic": 2, "patch": 3, "Patch": 3, "conservative": 4, "Conservative1stOrder": 4,
                   "conservative2nd": 5, "Conservative2ndOrder": 5},
        "norm_type": {"dstarea": 0, "DstArea": 0, "fracarea": 1, "FracArea": 1},
        "unmapped": {"error": 0, "Error": 0, "ignore": 1, "Ignore": 1},
        "line_type": {"cartesian": 0, "Cartesian": 0, "great_circle": 1, "GreatCircle": 1},
    }
    for key, table in names.items():
        for text, value in table.items():
            assert getattr(axgb.parse_regrid_config({key: text}), key) == value, (key, text)
            assert getattr(axgb.parse_regrid_config({key: value}), key) == value
        with pytest.raises(ValueError, match="Unknown"):
            axgb.parse_regrid_config({key: "no_such_name"})
    assert axgb.parse_regrid_config({"use_limiter": True}).use_limiter == 1
    assert axgb.parse_regrid_config({}).extrap_method == 1  # NearestWet by default
    assert axgb.parse_regrid_config({"extrap_method": "none"}).extrap_method == 0
