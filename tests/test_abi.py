"""The C ABI library builds, loads and exports what include/*.h declares.

No compute calls here (no GPU needed): symbols, struct layouts shared with
the ctypes binding, and loud failure without a device.
"""

import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT
from ennemi_gb300 import _build, _native


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        # header-only helpers are not library symbols
        text = re.sub(r"static inline[^{]*\{.*?\n\}", "", text, flags=re.S)
        for m in re.finditer(r"\b(egb_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return ctypes.CDLL(_build.LIB_PATH)


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ["egb_create", "egb_destroy", "egb_run_batch", "egb_fetch", "egb_knn_eps",
              "egb_ball_count", "egb_last_error", "egb_set_stream", "egb_timings"]:
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_string(lib):
    lib.egb_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.egb_version()


def test_struct_layouts_match_header(tmp_path):
    """sizeof / offsetof of the header's structs, compiled with gcc, equal the
    ctypes binding's."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = {"egb_column": (_native.EgbColumn, ["data", "stride"]),
              "egb_task": (_native.EgbTask, [f for f, _ in _native.EgbTask._fields_]),
              "egb_result": (_native.EgbResult, [f for f, _ in _native.EgbResult._fields_])}
    lines = []
    for st, (_, names) in fields.items():
        lines.append(f'printf("%zu\\n", sizeof({st}));')
        lines += [f'printf("%zu\\n", offsetof({st}, {f}));' for f in names]
    src = tmp_path / "lay.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "ennemi_gb.h"\n'
                   "int main(void) {\n" + "\n".join(lines) + "\nreturn 0; }\n")
    exe = tmp_path / "lay"
    subprocess.check_call([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    want = []
    for st, (cls, names) in fields.items():
        want.append(ctypes.sizeof(cls))
        want += [getattr(cls, f).offset for f in names]
    assert got == want


def test_null_arguments_rejected_without_device(lib):
    lib.egb_run_batch.restype = ctypes.c_int
    assert lib.egb_run_batch(None, None, 0, 0, None) == -1
    lib.egb_create.argtypes = [ctypes.c_int, ctypes.c_void_p]
    assert lib.egb_create(0, None) == -1
    lib.egb_set_noise.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]
    assert lib.egb_set_noise(None, None, 0) == -1


def test_library_is_built_for_sm103a():
    assert "arch=compute_103a,code=sm_103a" in " ".join(_build.NVCC_FLAGS)


def test_policy_index_matches_header(tmp_path):
    """egb_policy_index() compiled from the header equals _native.policy_index."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "pi.c"
    src.write_text(
        '#include <stdio.h>\n#include "ennemi_gb.h"\n'
        "int main(void) { long long lens[] = {1, 2, 3, 255, 256, 4095, 4096, 1000000,"
        " 1LL << 31, 1LL << 40};\n"
        "  for (int s = 0; s < 2; ++s) for (int d = 1; d <= 9; ++d) for (int K = 2; K <= 40; K += 3)"
        " for (int i = 0; i < 10; ++i) printf(\"%d\\n\", egb_policy_index(s, d, K, lens[i]));\n"
        "  return 0; }\n")
    exe = tmp_path / "pi"
    subprocess.check_call([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = [int(v) for v in subprocess.check_output([str(exe)]).split()]
    lens = [1, 2, 3, 255, 256, 4095, 4096, 1000000, 1 << 31, 1 << 40]
    want = [_native.policy_index(s, d, K, n) for s in range(2) for d in range(1, 10)
            for K in range(2, 41, 3) for n in lens]
    assert got == want
    assert max(want) < _native.POLICY_ENTRIES and min(want) >= 0
