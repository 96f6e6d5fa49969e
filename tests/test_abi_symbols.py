"""The shared library loads without a GPU and exports every function declared
in include/*.h; the ctypes host mirror binds exactly those symbols."""
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fname in os.listdir(os.path.join(REPO, "include")):
        if not fname.endswith(".h"):
            continue
        text = open(os.path.join(REPO, "include", fname)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b((?:rainbow|rfmm)_\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_headers_declare_the_boundary():
    names = declared_functions()
    assert {"rainbow_api_version", "rainbow_depth_for_particles", "rfmm_create", "rfmm_step",
            "rfmm_digest", "rfmm_solve_fields"} <= names


def test_library_exports_every_declared_symbol(rfmm_mod):
    L = rfmm_mod.lib()
    missing = [n for n in sorted(declared_functions()) if not hasattr(L, n)]
    assert not missing, missing


def test_ctypes_mirror_covers_the_headers(rfmm_mod):
    assert set(rfmm_mod.SIGNATURES) == declared_functions()


def test_create_without_gpu_fails_cleanly(rfmm_mod):
    import ctypes as C
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    rc = rfmm_mod.lib().rfmm_create(1000, None, C.byref(h))
    assert rc == -6 and not h.value  # RFMM_ERR_NO_DEVICE, nothing returned


def test_status_strings(rfmm_mod):
    L = rfmm_mod.lib()
    for code, text in rfmm_mod.STATUS.items():
        assert L.rfmm_status_string(code).decode() == text
