"""The C-ABI library: builds, loads, exports every symbol include/*.h
declares, and refuses to run without a GPU (no CPU fallback)."""
import ctypes
import re
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_symbols():
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n.startswith(("gpunb", "gpupot", "irr_"))))


def test_header_declares_reference_abi():
    names = declared_symbols()
    for ref in ["gpunb_devinit_", "gpunb_open_", "gpunb_close_", "gpunb_send_", "gpunb_regf_",
                "gpunb_profile_", "gpupot_", "irr_simd_open_", "irr_simd_close_",
                "irr_simd_profile_", "irr_simd_set_jp_", "irr_simd_set_list_",
                "irr_simd_firr_vec_"]:
        assert ref in names


def test_library_exports_every_declared_symbol():
    from nbody6ppgpu_gb300 import build
    lib_path = build.build()
    lib = ctypes.CDLL(str(lib_path))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert missing == []
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (\w+)", out))
    assert set(declared_symbols()) <= exported


def test_library_is_built_for_sm_103a():
    from nbody6ppgpu_gb300 import build
    lib_path = build.build()
    out = subprocess.run(["cuobjdump", "--list-elf", str(lib_path)], capture_output=True,
                         text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


def test_fails_loudly_without_gpu():
    """On a host without a GPU the product path must raise, not fall back."""
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "import torch\n"
        "if torch.cuda.is_available(): print('HASGPU'); raise SystemExit(0)\n"
        "from nbody6ppgpu_gb300.gpunb import GpuNb, GpunbError\n"
        "try:\n"
        "    GpuNb(16)\n"
        "except GpunbError as e:\n"
        "    print('RAISED', e.code)\n"
    ) % str(ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    if "HASGPU" in r.stdout:
        pytest.skip("GPU present")
    assert "RAISED 7" in r.stdout or "RAISED 4" in r.stdout, r.stdout + r.stderr
