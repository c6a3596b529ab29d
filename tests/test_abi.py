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


def _cache_cap(env):
    """tsg_pinned_cache_cap in a fresh process (the cap is read once)."""
    import os
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, '.'); import tilespgemm_gb300 as t; "
            "print(t.pinned_cache_cap())")
    e = dict(os.environ)
    e.pop("TSG_PINNED_CACHE_BYTES", None)
    e.update(env)
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", code], cwd=root, env=e, capture_output=True, text=True, check=True)
    return int(out.stdout.strip())


def test_pinned_cache_cap(built_lib):
    """The host-output buffer cache keeps min(96 GB, 3/8 of host memory), or
    TSG_PINNED_CACHE_BYTES (at most half of host memory; malformed values
    fall back to the default)."""
    import os
    ram = os.sysconf("SC_PHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    default = min(96 << 30, ram // 8 * 3)
    assert _cache_cap({}) == default
    assert _cache_cap({"TSG_PINNED_CACHE_BYTES": "0"}) == 0
    assert _cache_cap({"TSG_PINNED_CACHE_BYTES": str(3 << 30)}) == min(3 << 30, ram // 2)
    assert _cache_cap({"TSG_PINNED_CACHE_BYTES": str(ram * 4)}) == ram // 2
    assert _cache_cap({"TSG_PINNED_CACHE_BYTES": "12GB"}) == default
    assert _cache_cap({"TSG_PINNED_CACHE_BYTES": "-5"}) == default
