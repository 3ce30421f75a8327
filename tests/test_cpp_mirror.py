"""The C++ mirror of the reference interface (include/bwacuda.hpp) compiles
against the C ABI, and (on a GPU) passes the reference's own SwBackend gates."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "gates.cpp")
BIN = os.path.join(ROOT, "tests", "cpp", "gates")


def _build():
    cmd = ["g++", "-std=c++17", "-O2", "-o", BIN, SRC, "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(ROOT, "oracle"), "-L", os.path.join(ROOT, "oracle"), "-lksworacle",
           "-Wl,-rpath," + os.path.join(ROOT, "oracle"), "-L", os.path.join(ROOT, "bwa-mem4_gb300"), "-lbwacuda",
           "-Wl,-rpath," + os.path.join(ROOT, "bwa-mem4_gb300")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_mirror_compiles(built):
    _build()
    assert os.path.exists(BIN)


@pytest.mark.gpu
def test_reference_gates_through_cpp_mirror(built):
    _build()
    r = subprocess.run([BIN], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "gates ok" in r.stdout
