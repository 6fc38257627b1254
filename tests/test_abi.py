"""The C-ABI library loads and exports every symbol include/marie_vie.h declares
(no compute calls: runs without a GPU)."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    txt = (ROOT / "include" / "marie_vie.h").read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(marie_[a-zA-Z0-9_]+)\s*\(", txt)))


def test_header_declares_the_path_entry_points():
    syms = declared_symbols()
    for s in ("marie_mv_AN", "marie_mv_L", "marie_pgmres", "marie_get_operators", "marie_jvie_solve",
              "marie_plan_create", "marie_set_operator", "marie_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    import ctypes

    from marie_gb300 import _lib

    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_ctypes_signatures_cover_the_header():
    from marie_gb300 import _lib

    assert sorted(_lib.SIGNATURES) == declared_symbols()
    _lib.load()  # binds every signature; raises if a symbol is absent


def test_missing_library_fails_loudly(tmp_path):
    from marie_gb300 import _lib

    with pytest.raises(ImportError):
        _lib.load(tmp_path / "nope.so")


def test_version_and_error_string_without_gpu():
    from marie_gb300 import _lib

    lib = _lib.load()
    assert lib.marie_version() >= 1
    assert isinstance(lib.marie_last_error(), bytes)


def test_plan_settings_reject_a_null_plan_without_gpu():
    """The schedule setters and the bound-matvec entry point check their plan
    before touching the device (MARIE_EINVAL = -1 for a NULL plan)."""
    import ctypes as C

    from marie_gb300 import _lib

    lib = _lib.load()
    assert lib.marie_plan_set_batch_groups(None, 2) == _lib.MARIE_EINVAL
    assert lib.marie_plan_set_graph_refinement(None, 1) == _lib.MARIE_EINVAL
    assert lib.marie_plan_set_inner_restart(None, 20) == _lib.MARIE_EINVAL
    buf = (C.c_double * 4)()
    assert lib.marie_plan_apply_mv_AN(None, buf, buf, 1, _lib.MARIE_FP32) == _lib.MARIE_EINVAL
    assert b"NULL" in lib.marie_last_error()
