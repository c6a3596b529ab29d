"""The C-ABI library loads and exports every entry point include/*.h declares;
without a GPU it reports errors instead of crashing (no CPU fallback)."""
import ctypes as C
import re

from conftest import ROOT


def declared_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(tsg_[a-z0-9_]+)\s*\(", text))
    return names


def test_header_declares_the_api():
    names = declared_functions()
    for must in ("tsg_create", "tsg_destroy", "tsg_load_mtx", "tsg_spgemm", "tsg_csr_free",
                 "tsg_spgemm_tiles", "tsg_csr_to_tiles", "tsg_tiles_to_csr"):
        assert must in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = C.CDLL(str(built_lib))
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header(built_lib):
    from tilespgemm_gb300 import _abi
    assert declared_functions() <= set(_abi.SIGNATURES)


def test_version_and_defaults(built_lib):
    from tilespgemm_gb300 import _abi, version
    assert "sm_103a" in version()
    o = _abi.tsg_opts()
    _abi.lib().tsg_opts_default(C.byref(o))
    assert o.validate == 1 and o.threads_numeric in (128, 256, 512)


def test_null_arguments_are_errors(built_lib):
    from tilespgemm_gb300 import _abi
    L = _abi.lib()
    assert L.tsg_create(None, 0, None) == _abi.ERR_INVALID_ARG
    assert L.tsg_spgemm(None, 1, None, None, None, None) == _abi.ERR_INVALID_ARG
    assert L.tsg_load_mtx(None, None, None) == _abi.ERR_INVALID_ARG


def test_no_gpu_means_an_error_not_a_fallback(built_lib):
    """On a machine without a GPU, creating a context fails with a status."""
    import torch
    from tilespgemm_gb300 import _abi
    if torch.cuda.is_available():
        return
    h = C.c_void_p()
    st = _abi.lib().tsg_create(C.byref(h), 0, None)
    assert st in (_abi.ERR_CUDA, _abi.ERR_INVALID_ARG, _abi.ERR_NOT_SUPPORTED)
    assert not h.value
