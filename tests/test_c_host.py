"""A C host program (tests/c/sbm_ctest.c) compiled against include/sbm_capi.h
and linked with the library: loads the shipped preconditioner weights with
sbm_net_load and solves with SBM_PC_LEARNED through the plain C-ABI."""
import shutil
import subprocess
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_c_host(built, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = ROOT / "elsim_gb300"
    exe = tmp_path / "sbm_ctest"
    subprocess.run([cc, "-O1", "-I", str(ROOT / "include"), str(ROOT / "tests" / "c" / "sbm_ctest.c"),
                    "-L", str(lib), "-lsbm_gb300", f"-Wl,-rpath,{lib}", "-lm", "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe), str(lib / "weights" / "pc_unet.bin")], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "c host ok" in out.stdout
