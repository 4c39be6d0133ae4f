"""Compile the reference's point-dipole force extension into ``oracle/_ref/``.

Checker only: the built module pins ``oracle/dipole_forces_oracle.py`` (tests
and golden-vector generation in this checkout).  It compiles the single source
file ``CPU - HOOMD simulation test/dipole_forces_ext/_dipole_forces_ext.cpp``
where it lies, with g++ and the installed pybind11 headers; nothing is copied.
The reference checkout is named by the argument or the MPS_REFERENCE_ROOT
environment variable.  Skipped (returns None) when neither names an existing
reference tree, or pybind11 is absent, e.g. on a machine that only runs the
GPU tests.
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC_REL = os.path.join("CPU - HOOMD simulation test", "dipole_forces_ext", "_dipole_forces_ext.cpp")


def build(ref_root=None):
    ref_root = ref_root or os.environ.get("MPS_REFERENCE_ROOT")
    if not ref_root:
        return None
    src = os.path.join(ref_root, SRC_REL)
    if not os.path.exists(src):
        return None
    try:
        import pybind11
    except ImportError:
        return None
    os.makedirs(OUT, exist_ok=True)
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    target = os.path.join(OUT, "_dipole_forces_ext" + suffix)
    if os.path.exists(target) and os.path.getmtime(target) >= os.path.getmtime(src):
        return target
    inc = [pybind11.get_include(), sysconfig.get_paths()["include"]]
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-shared", "-fPIC", src, "-o", target]
    for i in inc:
        cmd[1:1] = ["-I", i]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference extension build failed:\n{r.stderr[-2000:]}")
    return target


def load(ref_root=None):
    path = build(ref_root)
    if path is None:
        return None
    sys.path.insert(0, OUT)
    import _dipole_forces_ext
    return _dipole_forces_ext


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None))
