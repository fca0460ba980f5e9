"""The Fortran bind(C) interface module (include/sbm_capi.f90) compiled with
a small Fortran host program (tests/fortran/sbm_ftest.f90) and run against
the library: the way the reference program links to it.  Skipped where no
Fortran compiler exists."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_fortran_host(built, tmp_path):
    fc = shutil.which("gfortran")
    if fc is None:
        pytest.skip("no Fortran compiler")
    lib = ROOT / "elsim_gb300"
    exe = tmp_path / "sbm_ftest"
    subprocess.run([fc, "-O1", "-J", str(tmp_path), str(ROOT / "include" / "sbm_capi.f90"),
                    str(ROOT / "tests" / "fortran" / "sbm_ftest.f90"), "-L", str(lib),
                    "-lsbm_gb300", f"-Wl,-rpath,{lib}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count("fortran solve ok") == 2
    # linear table: f = 2c + 1 (the lookup's one-segment-left quirk is exact
    # for a linear table)
    vals = [float(v) for v in out.stdout.split("fortran table ok:")[1].split()]
    assert vals == pytest.approx([1.1, 2.0, 2.9], abs=1e-9)
