"""The C ABI library loads on a CPU-only host and exports every declared symbol."""
import os
import re

import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "gbpowspec.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gbp_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    names = _declared()
    for must in ("gbp_deposit", "gbp_power", "gbp_fft_r2c", "gbp_bins_create", "gbp_power_normalize"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from gbpowspec import _lib
    lib = _lib.load()
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(_declared()) <= bound, set(_declared()) - bound


def test_status_strings_and_version():
    from gbpowspec import _lib
    lib = _lib.load()
    assert lib.gbp_version() >= 100
    assert _lib.strerror(_lib.GBP_ERR_WORKSPACE) == "workspace too small"
    assert _lib.strerror(0) == "ok"


def test_library_path_is_in_tree():
    from gbpowspec import _lib
    assert os.path.commonpath([_lib.lib_path(), ROOT]) == ROOT
