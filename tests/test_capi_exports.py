"""The C-ABI library loads and exports every symbol include/*.h declares (no GPU needed)."""
import ctypes

from parry_gb300 import _build, _capi
from tests._helpers import header_symbols


def test_library_builds_and_exports_header_symbols():
    path = _build.build()
    lib = ctypes.CDLL(str(path))
    syms = header_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header():
    assert sorted(_capi.SIGNATURES) == header_symbols()


def test_create_without_gpu_reports_no_device():
    """With no visible device the library refuses loudly (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        return
    lib = _capi.lib()
    h = ctypes.c_void_p()
    st = lib.parrygpu_create(ctypes.byref(h), None)
    assert st == 8  # PARRYGPU_NO_DEVICE
