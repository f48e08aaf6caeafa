"""The C-ABI library loads and exports every function include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(bxg_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported(cuda_lib):
    lib = ctypes.CDLL(str(cuda_lib._name))
    names = declared_functions()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_host_only_calls_work_without_gpu(cuda_lib):
    lib = cuda_lib
    assert lib.bxg_version() >= 100
    assert lib.bxg_status_string(2).decode().startswith("node pool")


def test_no_device_or_bad_args_fail_cleanly(cuda_lib):
    import bonxai_gb300 as bx
    h = ctypes.c_void_p()
    # invalid geometry is rejected before any device work
    st = cuda_lib.bxg_grid_create(ctypes.byref(h), 0.1, 0, 3, 4, None)
    assert st in (1, 6)  # invalid argument (or no device in this container)
    assert not h.value
