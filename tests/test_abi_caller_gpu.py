"""The C ABI from a plain C program (tests/abi_caller.c), the way the Fortran
integrator links libgpunb.so: no Python or torch in the process.  The
program checks its own sampled rows against a direct FP64 sum and exits 0
when lists, forces, jerks and potentials agree."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]


def test_c_caller(tmp_path):
    from nbody6ppgpu_gb300.gpunb import library_path, load
    load()                                     # builds the library if it is missing
    lib = library_path()
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = tmp_path / "abi_caller"
    subprocess.run([cc, "-O2", "-std=c99", "-ffp-contract=off", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "abi_caller.c"), "-o", str(exe), f"-L{lib.parent}",
                    "-lgpunb", f"-Wl,-rpath,{lib.parent}", "-lm"], check=True)
    r = subprocess.run([str(exe), "8192"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, (r.stdout[-3000:], r.stderr[-3000:])
