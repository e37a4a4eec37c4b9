"""The C++ boundary: a compiled C++ caller (tests/cpp/elphy_view_check.cpp) that includes
include/cardiomech_gb300.h and include/cardiomech_gb300_elphy.hpp, links libcmgb300.so, runs the
acCELLerate patch sketched in INTEGRATION.md and drives per-node vbElphyModel views
(ElphyModelBasis.h:184-323) against the batch path.

CPU: the caller compiles and links against the stand-in interface; where the reference tree is
present, the view also compiles against the reference's own ElphyModelBasis.h (its `override`s
then prove the signatures match). GPU: the compiled caller runs and checks itself."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
CPP = ROOT / "tests" / "cpp"
REF_SRC = Path("/root/reference/electrophysiology/src")


def _compile(cmlib, out: Path, header_dir: Path, header: str, extra=(), syntax_only=False):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    lib_dir = cmlib.LIB_PATH.parent
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", f"-I{ROOT / 'include'}", f"-I{header_dir}",
           f'-DVB_ELPHY_HEADER="{header}"', *extra, str(CPP / "elphy_view_check.cpp")]
    if syntax_only:
        cmd += ["-fsyntax-only", "-w"]
    else:
        cmd += [f"-L{lib_dir}", "-lcmgb300", f"-Wl,-rpath,{lib_dir}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def test_caller_compiles_and_links(cmlib, tmp_path):
    exe = _compile(cmlib, tmp_path / "elphy_view_check", CPP, "vb_elphy_interface.h")
    assert exe.exists() and os.access(exe, os.X_OK)


def test_view_matches_reference_interface(cmlib, tmp_path):
    if not (REF_SRC / "CellModel" / "ElphyModelBasis.h").exists():
        pytest.skip("reference tree not present")
    (tmp_path / "vb_reference.h").write_text(
        "#include <kaBasicIO.h>\nusing namespace nskaGlobal;\n#include <ElphyModelBasis.h>\n")
    inc = [f"-I{REF_SRC / d}" for d in ("CellModel", "Lattice", "MathBasics")]
    _compile(cmlib, tmp_path / "unused", tmp_path, "vb_reference.h", extra=["-DKADEBUG=0", "-DUSE_EMT", *inc],
             syntax_only=True)


@pytest.mark.gpu
def test_caller_runs(gpu, tmp_path):
    exe = _compile(gpu, tmp_path / "elphy_view_check", CPP, "vb_elphy_interface.h")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout[-2000:] + r.stderr[-4000:]
