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
