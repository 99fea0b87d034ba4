"""The C ABI: every function include/gblu.h declares is exported by
libgblu.so and bound in the Python layer (no GPU needed)."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "gblu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(gblu_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_library_builds_and_exports(pkg):
    lib_path = os.path.join(ROOT, "linearsolve.jl_gb300", "libgblu.so")
    if not os.path.exists(lib_path):
        import __graft_entry__ as ge
        ge.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (gblu_[a-z0-9_]+)", out))
    declared = declared_functions()
    assert declared, "no declarations parsed"
    missing = [d for d in declared if d not in exported]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header(pkg):
    from importlib import import_module
    lib_mod = import_module(pkg.__name__ + "._lib")
    declared = declared_functions()
    assert sorted(lib_mod.SIGNATURES) == declared


def test_julia_binding_symbols_are_declared():
    """Every symbol the Julia binding resolves with dlsym is in gblu.h."""
    src = open(os.path.join(ROOT, "linearsolve.jl_gb300", "julia", "GB300LinearSolve.jl")).read()
    used = set(re.findall(r":(gblu_[a-z0-9_]+)", src))
    assert used, "no symbols parsed"
    missing = sorted(used - set(declared_functions()))
    assert not missing, f"the Julia binding resolves undeclared symbols: {missing}"


def test_library_loads_without_gpu(pkg):
    lib = pkg.load_library()
    assert lib.gblu_version() >> 16 == 1
    import ctypes
    h = ctypes.c_void_p()
    st = lib.gblu_create(ctypes.byref(h), 0, 0)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = None
    if has_gpu is False:
        assert st != 0 and h.value is None  # ENODEVICE, never a fallback
        assert lib.gblu_last_error(None)
    elif st == 0:
        lib.gblu_destroy(h)


def test_lapack_shaped_argument_errors(pkg):
    # LAPACK's info < 0 for a bad argument, checked before any device work
    import ctypes
    lib = pkg.load_library()
    m, n, lda, info = ctypes.c_int64(-1), ctypes.c_int64(3), ctypes.c_int64(3), ctypes.c_int64(99)
    lib.gblu_dgetrf_(ctypes.byref(m), ctypes.byref(n), None, ctypes.byref(lda), None, ctypes.byref(info))
    assert info.value == -1
    m = ctypes.c_int64(4)
    lib.gblu_dgetrf_(ctypes.byref(m), ctypes.byref(n), None, ctypes.byref(lda), None, ctypes.byref(info))
    assert info.value == -4
    nn, nrhs, ldb = ctypes.c_int64(3), ctypes.c_int64(1), ctypes.c_int64(3)
    lib.gblu_dgetrs_(b"X", ctypes.byref(nn), ctypes.byref(nrhs), None, ctypes.byref(lda), None, None,
                     ctypes.byref(ldb), ctypes.byref(info), 1)
    assert info.value == -1
    m0 = ctypes.c_int64(0)
    lib.gblu_dgetrf_(ctypes.byref(m0), ctypes.byref(n), None, ctypes.byref(lda), None, ctypes.byref(info))
    assert info.value == 0  # empty matrix: nothing to do, no device touched


def _header_struct_fields(name):
    src = open(os.path.join(ROOT, "include", "gblu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\}" % name, src, flags=re.S).group(1)
    return re.findall(r"([A-Za-z_][A-Za-z0-9_]*)\s*;", body)


@pytest.mark.parametrize("c_name,py_name,jl_name", [
    ("gblu_serve_config", "ServeConfig", "ServeConfig"),
    ("gblu_request", "Request", "Request"),
    ("gblu_completion", "Completion", "Completion"),
])
def test_struct_layouts_match_header(pkg, c_name, py_name, jl_name):
    """The Python ctypes and Julia mirrors of the C structs list the header's
    fields in the header's order (a missing trailing field would let the
    library write past the caller's struct)."""
    from importlib import import_module
    lib_mod = import_module(pkg.__name__ + "._lib")
    fields = _header_struct_fields(c_name)
    assert fields
    assert [f[0] for f in getattr(lib_mod, py_name)._fields_] == fields
    src = open(os.path.join(ROOT, "linearsolve.jl_gb300", "julia", "GB300LinearSolve.jl")).read()
    body = re.search(r"struct %s\b[^\n]*\n(.*?)\nend" % jl_name, src, flags=re.S).group(1)
    assert re.findall(r"^\s*([A-Za-z0-9_]+)::", body, flags=re.M) == fields


def test_serve_config_default_fills_every_field(pkg):
    """gblu_serve_config_default writes the whole struct (no GPU needed)."""
    import ctypes
    from importlib import import_module
    lib_mod = import_module(pkg.__name__ + "._lib")
    lib = pkg.load_library()
    cfg = lib_mod.ServeConfig()
    ctypes.memset(ctypes.byref(cfg), 0x7f, ctypes.sizeof(cfg))
    assert lib.gblu_serve_config_default(ctypes.byref(cfg)) == 0
    vals = {f[0]: getattr(cfg, f[0]) for f in cfg._fields_}
    assert all(v != 0x7f7f7f7f and v != 0x7f7f7f7f7f7f7f7f for v in vals.values()), vals
    assert vals["pivoting"] == lib_mod.GBLU_PIVOT_PARTIAL and vals["max_large"] == 1


def test_constants_match_header(pkg):
    """Every GBLU_* constant the Python and Julia bindings define has the
    header's value; the Python binding defines all of the header's status,
    precision, location, mode and fallback codes."""
    from importlib import import_module
    lib_mod = import_module(pkg.__name__ + "._lib")
    src = open(os.path.join(ROOT, "include", "gblu.h")).read()
    header = {k: int(v) for k, v in re.findall(r"^#define (GBLU_[A-Z0-9_]+) (-?\d+)", src, flags=re.M)}
    assert len(header) > 25
    py = {k: getattr(lib_mod, k) for k in dir(lib_mod) if k.startswith("GBLU_") and isinstance(getattr(lib_mod, k), int)}
    missing = sorted(k for k in header if k not in py and k != "GBLU_PROFILE_KINDS")
    assert not missing, missing
    assert {k: v for k, v in py.items() if k in header} == {k: header[k] for k in py if k in header}
    jl = open(os.path.join(ROOT, "linearsolve.jl_gb300", "julia", "GB300LinearSolve.jl")).read()
    for k, v in re.findall(r"^const (GBLU_[A-Z0-9_]+) = Int32\((-?\d+)\)", jl, flags=re.M):
        assert header[k] == int(v), k
