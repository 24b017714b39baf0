"""The C-ABI library builds, loads without a GPU and exports every declared entry point."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bib", "bib.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(bib_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from biblbm_gb300 import build

    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_the_reference_facing_entry_points():
    names = declared_functions()
    for n in ["bib_create", "bib_lattice_add_domain", "bib_lattice_send", "bib_lattice_receive",
              "bib_lattice_collide_and_stream", "bib_shape_store", "bib_particle_add", "bib_step", "bib_ibm_step"]:
        assert n in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from biblbm_gb300 import _lib

    assert set(declared_functions()) == set(_lib.exported_symbols())


def test_abi_version_without_gpu(lib):
    lib.bib_abi_version.restype = ctypes.c_int32
    assert lib.bib_abi_version() == 1
    lib.bib_status_string.restype = ctypes.c_char_p
    assert lib.bib_status_string(-1) == b"invalid argument"


def test_create_fails_cleanly_without_gpu(lib):
    """No GPU here: bib_create must return an error code, not crash or exit."""
    import torch  # only to ask whether a device exists

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from biblbm_gb300 import _lib

    L = _lib.load()
    h = ctypes.c_void_p()
    st = L.bib_create(ctypes.byref(_lib.Config(0, 0)), ctypes.byref(h))
    assert st == -3 and not h.value


def test_header_compiles_as_c99(tmp_path):
    """The drop-in boundary is a plain C header: a C99 translation unit (as a C or cgo / ctypes
    binding would compile) includes it without warnings."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "use_bib.c"
    src.write_text('#include "bib/bib.h"\nint main(void) { bib_lattice_params p; (void)p; return 0; }\n')
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                        "-c", str(src), "-o", str(tmp_path / "use_bib.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
