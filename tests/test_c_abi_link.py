"""The drop-in boundary from C and C++: include/dgsw.h compiles as C11 and
C++17, a C program links libdgsw.so and calls host-only entry points, and its
results equal the Python binding's (no GPU needed)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "spectre_gb300", "_lib")


@pytest.mark.parametrize("cc,std,lang", [("gcc", "-std=c11", "c"), ("g++", "-std=c++17", "c++")])
def test_header_compiles(cc, std, lang):
    if not shutil.which(cc):
        pytest.skip(cc + " not found")
    r = subprocess.run([cc, std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", lang,
                        os.path.join(INC, "dgsw.h")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_c_program_links_and_matches_python(dgsw_lib, tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    exe = str(tmp_path / "host_calls")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", INC,
                        os.path.join(ROOT, "tests", "c_abi", "host_calls.c"), "-L", LIBDIR,
                        "-ldgsw", "-Wl,-rpath," + LIBDIR, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    lines = {ln.split()[0]: ln.split()[1:] for ln in out.stdout.splitlines()}
    assert int(lines["abi"][0]) == dgsw_lib.lib().dgsw_abi_version()
    assert int(lines["lgl"][0]) == 0
    xw = np.array(lines["lgl"][1:], dtype=float).reshape(8, 2)
    x, w = dgsw_lib.lgl_points_weights(8)
    assert np.array_equal(xw[:, 0], x) and np.array_equal(xw[:, 1], w)
    assert int(lines["amr"][0]) == 0
    assert np.array_equal(np.array(lines["amr"][1:], dtype=float).reshape(8, 4),
                          dgsw_lib.amr_matrix(4, 8, 2))
    assert lines["count"] == ["0", "8", str(8 * 5 * 216)]
    maps = dgsw_lib.index_maps([dgsw_lib.Brick((2, 2, 2), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))], 6)
    ids = np.array(lines["maps"][1:9], dtype=np.uint64)
    nbr = np.array(lines["maps"][9:], dtype=np.int32)
    assert int(lines["maps"][0]) == 0
    assert np.array_equal(ids, maps[0]) and np.array_equal(nbr, np.asarray(maps[1]).ravel())
    assert dgsw_lib.STATUS_NAMES[int(lines["error"][0])] == "DGSW_ERR_ARGUMENT"
    assert lines["error"][1] == "message"
