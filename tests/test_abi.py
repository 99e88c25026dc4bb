"""The C ABI library builds, loads without a GPU and exports every entry
point include/rsc.h declares; calls report status codes instead of exiting."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "rsc.h")) as f:
        text = f.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rsc_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ("rsc_worker_create", "rsc_worker_malloc", "rsc_set_les", "rsc_set_adm", "rsc_set_rcs",
              "rsc_upload", "rsc_download", "rsc_advance_time", "rsc_make_pulse", "rsc_download_pulse"):
        assert s in syms


def test_library_exports_every_declared_symbol(backend):
    lib = backend.load_library()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, "not exported: %s" % missing


def test_null_arguments_return_status(backend):
    lib = backend.load_library()
    assert lib.rsc_worker_create(0, None) == -1
    assert lib.rsc_device_count(None) == -1
    assert lib.rsc_make_pulse(None, None) == -1
    assert lib.rsc_advance_time(None, None, 0, None) == -1
    assert b"NULL" in lib.rsc_last_error()
    assert lib.rsc_worker_free(None) == 0


def test_product_does_not_load_the_oracle():
    """The package never imports the oracle (test infrastructure)."""
    pkg = os.path.join(ROOT, "simradar_gb300")
    for dirpath, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                with open(os.path.join(dirpath, fn)) as f:
                    src = f.read()
                assert "oracle" not in re.sub(r"(#|//|/\*|\*).*", "", src), fn


@pytest.mark.parametrize("sym", ["rsc_eval_math", "rsc_set_pulse_precision"])
def test_cdll_signature(backend, sym):
    lib = backend.load_library()
    fn = getattr(lib, sym)
    assert fn.restype is ctypes.c_int


def test_header_compiles_as_c_and_links(tmp_path, backend):
    """rs.c is C: the header must compile with a C compiler (C99, all
    warnings as errors) and a C program must link against the library and
    get status codes back without a GPU (no device here is an error code,
    not an exit)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "host.c"
    src.write_text(r'''
#include <stdio.h>
#include <string.h>
#include "rsc.h"
int main(void) {
    rsc_population pop;
    rsc_iq_params iq;
    int n = -1;
    memset(&pop, 0, sizeof(pop));
    memset(&iq, 0, sizeof(iq));
    if (sizeof(iq) != 100) return 10;
    if (rsc_worker_create(0, NULL) != RSC_ERR_ARG) return 11;
    if (rsc_make_pulse(NULL, NULL) != RSC_ERR_ARG) return 12;
    if (rsc_advance_time(NULL, &pop, 0, NULL) != RSC_ERR_ARG) return 13;
    if (rsc_batch_run(NULL, 1, NULL, NULL, NULL, 0) != RSC_ERR_ARG) return 14;
    (void)rsc_device_count(&n);
    printf("%d %s\n", n, rsc_last_error());
    return 0;
}
''')
    exe = tmp_path / "host"
    lib = backend.library_path()
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
           str(src), "-o", str(exe), lib, "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)


@pytest.mark.parametrize("std", ["c++11", "c++17", "c++20"])
def test_header_compiles_as_cpp(tmp_path, std):
    """A C++ host (any standard, C++20 keywords included) can include the
    header as it is."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "host.cpp"
    src.write_text('#include "rsc.h"\nint main() { rsc_populate_args a = {}; return (int)a.sim_concept; }\n')
    subprocess.run([gxx, "-std=" + std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I",
                    os.path.join(ROOT, "include"), str(src)], check=True)
