"""The C ABI without a GPU: libikdg.so builds, loads, exports every function
declared in include/ikdg.h, the Python binding declares a signature for each,
and creating a tree with no CUDA device fails cleanly (no compute runs)."""
import ctypes as C
import importlib.util
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ikdg.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(ikdg_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    spec = importlib.util.spec_from_file_location("ikdg_build_t", os.path.join(ROOT, "ikd-tree_gb300", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    path = mod.build()
    return C.CDLL(path)


def test_header_declares_the_api():
    names = declared()
    for must in ("ikdg_create", "ikdg_build", "ikdg_add_points", "ikdg_delete_points", "ikdg_delete_boxes",
                 "ikdg_knn", "ikdg_box_search", "ikdg_radius_search", "ikdg_size", "ikdg_validnum"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_declared_symbol():
    import ikdg
    assert sorted(ikdg.SIGNATURES) == declared()


def prototypes():
    """{name: (return type, parameter count)} from include/ikdg.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for ret, name, params in re.findall(r"([A-Za-z_][\w\s\*]*?)\b(ikdg_[a-z_0-9]+)\s*\(([^)]*)\)\s*;", text,
                                        flags=re.S):
        p = params.strip()
        out[name] = (" ".join(ret.split()), 0 if p in ("", "void") else len(p.split(",")))
    return out


def test_binding_signatures_match_the_header():
    # Same parameter count and the same kind of return value for every entry
    # point: a binding out of step with the header would pass wrong arguments.
    import ikdg
    protos = prototypes()
    assert sorted(protos) == declared()
    for name, (ret, nparams) in protos.items():
        restype, argtypes = ikdg.SIGNATURES[name]
        assert len(argtypes) == nparams, f"{name}: {len(argtypes)} arguments bound, {nparams} declared"
        if ret.endswith("char*") or ret.endswith("char *"):
            assert restype is C.c_char_p, name
        else:
            assert ret.split()[-1] == "int" and restype is C.c_int, f"{name}: returns {ret}"


def test_create_without_device_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    lib.ikdg_create.restype = C.c_int
    lib.ikdg_create.argtypes = [C.c_float, C.c_float, C.c_float, C.c_int, C.POINTER(C.c_void_p)]
    st = lib.ikdg_create(0.5, 0.6, 0.2, -1, C.byref(h))
    assert st == 6 and not h.value  # IKDG_NO_DEVICE


def test_status_strings(lib):
    lib.ikdg_status_string.restype = C.c_char_p
    assert lib.ikdg_status_string(0) == b"ok"
    assert lib.ikdg_status_string(3).startswith(b"output capacity")


def test_binding_fails_loudly_without_the_library(tmp_path):
    """No CPU fallback: without libikdg.so the binding raises instead of
    answering from anywhere else."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "ikd-tree_gb300"))
    import ikdg
    saved = ikdg._lib
    ikdg._lib = None
    try:
        with pytest.raises(FileNotFoundError):
            ikdg.load(str(tmp_path / "libikdg.so"))
    finally:
        ikdg._lib = saved


def test_batch_api_without_device(lib):
    """The batch entry points are guarded like the tree ones: bad handles
    and missing devices come back as status codes, not crashes."""
    h = C.c_void_p()
    st = lib.ikdg_batch_create(0, C.byref(h))
    assert st in (0, 5, 6)  # OK, CUDA_ERR or NO_DEVICE (no GPU here)
    if st == 0:
        lib.ikdg_batch_destroy(h)
    assert lib.ikdg_batch_run(None) == 2          # BAD_ARG
    assert lib.ikdg_batch_destroy(None) == 2
