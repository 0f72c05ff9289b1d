"""The C-ABI library loads and exports what include/gbattract.h declares
(no compute call: this suite also runs without a GPU)."""
import ctypes

import pytest


@pytest.fixture(scope="module")
def lib(pkg):
    from gbattract import _lib
    if not _lib.LIB_PATH.exists():
        pkg.build()
    return _lib


def test_every_declared_symbol_is_exported(lib):
    declared = lib.declared_symbols()
    assert "gba_energy_6d" in declared and "gba_create" in declared
    missing = [n for n in declared if n not in lib.exported_symbols()]
    assert not missing, f"declared but not exported: {missing}"


def test_version_and_create_error_path(lib):
    L = lib.load()
    assert b"sm_103a" in L.gba_version()
    h = ctypes.c_void_p()
    import torch
    rc = L.gba_create(0, ctypes.byref(h))
    if torch.cuda.is_available():
        assert rc == 0
        L.gba_destroy(h)
    else:
        assert rc == 6          # GBA_ERR_NO_DEVICE
        assert b"no CUDA device" in L.gba_last_error(None)


def test_null_context_rejected(lib):
    L = lib.load()
    assert L.gba_upload_protein(None, 1, None, None, None, None, 0, None, None, None) == 1
    assert L.gba_energy_6d(None, 1, 2, 3, 4, None, 0, None, None) == 1
