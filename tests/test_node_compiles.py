"""The drop-in boundary at its real caller: the reference's own, unmodified
amcl3d::Node (Node.h, Node.cpp, Parameters.h) compiles against the drop-in
amcl3d::Grid3d / amcl3d::ParticleFilter headers (amcl3d_gb300/cpp), with stand-in
declarations for the ROS, tf and PCL API the node uses (tests/stand_in_node, in
front of tests/stand_in).  A syntax-only compile: it checks every call the node
makes into the filter (names, argument types and counts, constness) against the
drop-in's interface.  The node's files are copied to a temporary directory first,
because Node.h includes "ParticleFilter.h" by a quoted name, which would otherwise
find the reference's own header beside it.  Host only; skipped where the reference
tree is not present."""

import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
REF_ROOT = Path(os.environ.get("AMCL3D_REF_ROOT", str(ROOT.parent / "reference")))
REF_SRC = REF_ROOT / "amcl3d" / "src"


@pytest.mark.skipif(not (REF_SRC / "Node.cpp").exists(), reason="reference tree not present")
def test_reference_node_compiles_against_the_drop_in(tmp_path):
    for name in ("Node.h", "Node.cpp", "Parameters.h"):
        shutil.copy(REF_SRC / name, tmp_path / name)
    assert not (tmp_path / "ParticleFilter.h").exists() and not (tmp_path / "Grid3d.h").exists()
    cmd = [os.environ.get("CXX", "g++"), "-std=c++14", "-fsyntax-only", "-Wall", f"-I{tmp_path}",
           f"-I{ROOT / 'tests' / 'stand_in_node'}", f"-I{ROOT / 'tests' / 'stand_in'}",
           f"-I{ROOT / 'amcl3d_gb300' / 'cpp'}", f"-I{ROOT / 'include'}", str(tmp_path / "Node.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    # and the drop-in's headers are the ones that were used
    r = subprocess.run(cmd[:-1] + ["-H", str(tmp_path / "Node.cpp")], capture_output=True, text=True)
    used = [ln.lstrip(". ").strip() for ln in r.stderr.splitlines() if ln.startswith(".")]
    assert any(u.endswith("amcl3d_gb300/cpp/ParticleFilter.h") for u in used), used[:20]
    assert any(u.endswith("amcl3d_gb300/cpp/Grid3d.h") for u in used), used[:20]
    assert not any(str(REF_SRC) in u for u in used)
