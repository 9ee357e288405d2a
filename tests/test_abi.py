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


def test_header_is_plain_c_and_links(tmp_path):
    """A C client (cgo, a C program) can include the header as C99 and link the library."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    from gbpowspec import _lib
    lib = _lib.lib_path()
    _lib.load()                                  # builds the library when it is missing
    src = tmp_path / "client.c"
    src.write_text('#include "gbpowspec.h"\n'
                   'int main(void) {\n'
                   '  size_t b = 0;\n'
                   '  int32_t thr[3], last = 0; int reach = 0;\n'
                   '  const float e[3] = {1.0f, 2.0f, 3.0f};\n'
                   '  if (gbp_version() < 100) return 1;\n'
                   '  if (gbp_bin_thresholds(e, 3, 16, thr, &last, &reach) != GBP_OK) return 2;\n'
                   '  (void)b;\n'
                   '  return (thr[0] == 1 && thr[1] == 4 && thr[2] == 9) ? 0 : 3;\n'
                   '}\n')
    exe = tmp_path / "client"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(exe), lib,
                    "-Wl,-rpath," + os.path.dirname(lib)], check=True, capture_output=True)
    assert subprocess.run([str(exe)]).returncode == 0


def test_entry_points_reject_bad_arguments_before_any_device_work():
    """Null plans, buffers or negative sizes come back as GBP_ERR_INVALID on a host without a GPU."""
    import ctypes as C
    from gbpowspec import _lib
    lib = _lib.load()
    inv = _lib.GBP_ERR_INVALID
    null = None
    sz = C.c_size_t(0)
    assert lib.gbp_xi_workspace_size(null, null, C.byref(sz)) == inv
    assert lib.gbp_xi(null, null, null, null, null, 2, 1, null, null, null, 0, null) == inv
    assert lib.gbp_bispec_workspace_size(null, null, C.byref(sz)) == inv
    assert lib.gbp_bispec(null, null, null, null, 2, null, 3, 1000.0, null, null, null, null, null, 0, null) == inv
    assert lib.gbp_power_backward_workspace_size(null, C.byref(sz)) == inv
    assert lib.gbp_power_backward(null, null, null, 2, null, null, null, 1000.0, null, null, 0, null) == inv
    assert lib.gbp_deposit_backward(null, null, null, null, -1, 0.0, 0.0, 0.0, 1.0, 64, 2, 0, null, null, null,
                                    null, null, null) == inv
    assert lib.gbp_deposit_backward(null, null, null, null, 10, 0.0, 0.0, 0.0, 1.0, 64, 9, 0, null, null, null,
                                    null, null, null) == inv
