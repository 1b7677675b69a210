"""CPU-only checks of the C-ABI library: it loads, exports every symbol the
public header declares, keeps the reference's struct layouts, and reports
configuration errors through SR_getLastError instead of exceptions or exit()."""
import ctypes as C
import os
import re

import pytest

import cudasirecon_gb300 as sr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(sr.LIB_PATH):
        sr.build()
    return sr.load_library()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "cudasirecon.h")).read()
    return sorted(n for n in set(re.findall(r"\b(SRX?_[A-Za-z0-9_]+)\s*\(", text)) if n != "SR_PARAMS_REF")


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 12 + 5
    for n in names:
        assert hasattr(lib, n), n


def test_reference_entry_points_present(lib):
    for n in ["SR_new_from_shape", "SR_setRaw", "SR_loadAndRescaleImage", "SR_setCurTimeIdx",
              "SR_processOneVolume", "SR_getResult", "SR_getReconParams", "SR_getImageParams",
              "SR_new_from_argv", "SR_setFile", "SR_writeResult", "SR_closeFiles"]:
        assert hasattr(lib, n)


def test_struct_layouts_match_reference():
    # offsets of ReconParams / ImageParams members in the reference's
    # cudaSireconImpl.h:104-195 (LP64): bNoKz0 at 142, wiener at 144
    assert sr.ReconParamsHead.bNoKz0.offset == 142
    assert sr.ReconParamsHead.wiener.offset == 144
    assert sr.ReconParamsHead.bFilteroverlaps.offset == 92
    assert sr.ReconParamsHead.bDampenOrder0.offset == 128
    assert C.sizeof(sr.ImageParams) == 52


def test_missing_otf_file_is_an_error(lib, tmp_path):
    cfg = tmp_path / "cfg.txt"
    cfg.write_text("ndirs=3\nnphases=5\n")
    lib.SR_clearError()
    h = lib.SR_new_from_shape(64, 64, 15 * 8, str(cfg).encode())
    assert not h
    assert b"otf-file" in lib.SR_getLastError()


def test_unknown_option_is_an_error(lib, tmp_path):
    cfg = tmp_path / "cfg.txt"
    cfg.write_text("ndirs=3\nnotAnOption=1\notf-file=x.tif\n")
    lib.SR_clearError()
    h = lib.SR_new_from_shape(64, 64, 15 * 8, str(cfg).encode())
    assert not h
    assert b"notAnOption" in lib.SR_getLastError()


def test_unreadable_otf_is_an_error(lib, tmp_path):
    cfg = tmp_path / "cfg.txt"
    cfg.write_text(f"otf-file={tmp_path / 'missing.tif'}\n")
    lib.SR_clearError()
    h = lib.SR_new_from_shape(64, 64, 15 * 8, str(cfg).encode())
    assert not h
    assert b"missing.tif" in lib.SR_getLastError()


def test_null_handle_calls_do_not_crash(lib):
    lib.SR_clearError()
    lib.SR_processOneVolume(None)
    assert b"null" in lib.SR_getLastError()
    lib.SR_clearError()
