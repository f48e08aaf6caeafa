"""Device-side forEachCell (include/bonxai/device_visit.cuh): caller code
compiled with nvcc runs a __device__ functor over every active cell."""
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
LIB_DIR = ROOT / "bonxai_gb300" / "_build"


def _build(out: Path, lib_dir: Path):
    from bonxai_gb300.build import nvcc, ARCH
    subprocess.check_call([nvcc(), "-std=c++17", "-O2", *ARCH, f"-I{ROOT / 'include'}",
                           str(ROOT / "tests" / "cpp" / "device_visit_main.cu"),
                           f"-L{lib_dir}", "-lbonxai_gb300", f"-Xlinker=-rpath,{lib_dir}",
                           "-o", str(out)])


def test_device_visit_compiles(tmp_path):
    """The header and a caller's functor compile for sm_103a (no GPU needed)."""
    if not (LIB_DIR / "libbonxai_gb300.so").exists():
        pytest.skip("library not built")
    _build(tmp_path / "device_visit", LIB_DIR)


@pytest.mark.gpu
def test_device_visit_runs(tmp_path, cuda_lib):
    exe = tmp_path / "device_visit"
    _build(exe, LIB_DIR)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("device_visit ok")
