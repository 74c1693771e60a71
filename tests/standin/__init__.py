"""Builds test copies of the namelist drivers against the oracle-backed
stand-in for their C-ABI calls (pg_standin.cpp); test infrastructure only."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
HERE = os.path.dirname(os.path.abspath(__file__))


def build_driver(name, outdir):
    """Compile host/<name>.cpp with the stand-in into outdir; returns the executable."""
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    inc = ["-I", os.path.join(ROOT, "oracle"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "pimd-tunneling_gb300", "host")]
    exe = os.path.join(str(outdir), name)
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    os.path.join(ROOT, "pimd-tunneling_gb300", "host", name + ".cpp"), os.path.join(HERE, "pg_standin.cpp"), "-o", exe, "-L" + os.path.join(ROOT, "oracle"),
                    "-loracle", "-Wl,-rpath," + os.path.join(ROOT, "oracle")] + inc, check=True)
    return exe


def build_library(outdir):
    """The stand-in as a shared library exporting every symbol of the header
    (the unsupported calls fail), for loading through the Python binding in a
    test subprocess; returns its path."""
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    so = os.path.join(str(outdir), "libpimdgpu_standin.so")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                    os.path.join(HERE, "pg_standin.cpp"), "-o", so,
                    "-I", os.path.join(ROOT, "oracle"), "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "pimd-tunneling_gb300", "host"), "-L" + os.path.join(ROOT, "oracle"),
                    "-loracle", "-Wl,-rpath," + os.path.join(ROOT, "oracle")], check=True)
    return so
