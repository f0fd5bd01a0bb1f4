"""The C-ABI library loads and exports every entry point its header declares."""
import re
from pathlib import Path

import pytest

from toucangpurt_gb300 import capi

HEADER = Path(__file__).resolve().parents[1] / "include" / "toucan_gb300.h"


def declared():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(tgs_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared()
    assert "tgs_init" in names and "tgs_batch_run" in names and len(names) > 30


def test_every_declared_symbol_is_exported(built):
    lib = capi.lib()
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built):
    names = set(declared()) - {"tgs_last_error", "tgs_version"}
    assert names <= set(capi.SIGNATURES), sorted(names - set(capi.SIGNATURES))


def test_version_and_errors(built):
    lib = capi.lib()
    assert b"sm_103a" in lib.tgs_version()
    rc = lib.tgs_validate_file(b"/nonexistent/design.bin", None, None)
    assert rc == capi.ERR_IO
    assert b"cannot open" in lib.tgs_last_error()


def test_calls_on_uninitialised_handle(built):
    import ctypes as C

    lib = capi.lib()
    h = C.c_void_p()
    assert lib.tgs_create(C.byref(h)) == 0
    stop = C.c_int()
    assert lib.tgs_eval(h, C.byref(stop)) == capi.ERR_STATE
    assert lib.tgs_eval(None, C.byref(stop)) == capi.ERR_ARG
    assert lib.tgs_destroy(h) == 0


def test_init_without_gpu_fails_cleanly(small_design):
    """Here (no GPU) init reports TGS_ERR_NO_DEVICE; on a GPU host it succeeds."""
    from toucangpurt_gb300 import sim

    dp, sp, _ = small_design
    s = sim.Simulator()
    try:
        s.init(0, dp, sp)
    except capi.TgsError as e:
        assert e.code in (capi.ERR_NO_DEVICE, capi.ERR_CUDA)
    finally:
        s.cleanup()
