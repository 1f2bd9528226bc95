"""C ABI: the library builds, loads without a GPU and exports every declared symbol (CPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(bse_[a-z_0-9]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from votca_gb300 import _lib

    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(L, n), n
        assert n in _lib.SIGNATURES, f"{n} missing from the ctypes table"


def test_host_only_entry_points_without_gpu():
    from votca_gb300 import _lib

    L = _lib.load()
    assert b"sm_103a" in L.bse_version()
    # argument errors are reported as status codes, not crashes
    rc = L.bse_op_destroy(None)
    assert rc == 0
    n = ctypes.c_int64()
    rc = L.bse_op_size(None, ctypes.byref(n))
    assert rc == 1 and b"null handle" in L.bse_last_error()


def test_argument_errors_of_the_newer_entry_points_without_gpu():
    """Null inputs and bad sizes are rejected before any device work (status 1)."""
    from votca_gb300 import _lib

    L = _lib.load()
    h = ctypes.c_void_p()
    o = _lib.bse_uks_options(3, 2, 0, 0, 0, 8)
    assert L.bse_uks_op_create(None, None, None, None, None, None, 0, 0, None, 0, 0, ctypes.byref(o), 0,
                               ctypes.byref(h)) == 1
    assert L.bse_uks_op_create_dense_screening(None, None, None, None, None, None, 0, 0, None, 0, 0,
                                               ctypes.byref(o), 0, ctypes.byref(h)) == 1
    assert L.bse_mmn_fill_3c_mo(None, None, None, 4, None, 4, 4) == 1
    removed = ctypes.c_int64()
    assert L.bse_aux_pseudo_inv_sqrt(0, None, 0, 1e-7, None, 0, ctypes.byref(removed)) == 1
    assert L.bse_aux_pseudo_inv_sqrt_gwbse(3, None, 3, None, 3, 1e-7, None, 3, ctypes.byref(removed)) == 1
    assert b"bad arguments" in L.bse_last_error()


def test_python_mirror_rejects_hd_and_hd2_together():
    from votca_gb300 import bse_operator as bo
    from votca_gb300._lib import BSEError

    class Fake:
        size = 4
    with pytest.raises(BSEError):
        bo.BSE_OPERATOR(Fake(), 0, 0, 1, 1)


@pytest.mark.parametrize("compiler,std", [("gcc", "-std=c99"), ("g++", "-std=c++11")])
def test_header_is_plain_c_and_cxx(tmp_path, compiler, std):
    """include/votca_gb300_bse.h compiles as C99 and C++11 on its own (what a cgo / JNI / ctypes
    binding or a C++ adapter includes), and every declared function is callable from C."""
    import shutil
    import subprocess

    if shutil.which(compiler) is None:
        pytest.skip(f"{compiler} not available")
    names = declared_functions()
    src = tmp_path / ("use.c" if compiler == "gcc" else "use.cpp")
    body = "\n".join(f"  (void)&{n};" for n in names)
    src.write_text('#include "votca_gb300_bse.h"\nint main(void) {\n' + body + "\n  return 0;\n}\n")
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    r = subprocess.run([compiler, std, "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only", "-I", inc,
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_ctypes_table_matches_header_arity():
    """Every ctypes signature has as many arguments as the header's prototype."""
    from votca_gb300 import _lib

    src = ""
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if f.endswith(".h"):
            src += open(os.path.join(ROOT, "include", f)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = dict(re.findall(r"\b(bse_[a-z_0-9]+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S))
    assert len(protos) >= len(declared_functions())
    for name, (_, argtypes) in _lib.SIGNATURES.items():
        params = protos[name].strip()
        n = 0 if params in ("", "void") else len([p for p in params.split(",") if p.strip()])
        assert len(argtypes) == n, (name, len(argtypes), n)
