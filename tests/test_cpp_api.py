"""taco's C++ API (include/taco_gb300/taco.hpp) over libtacogb: tests/cpp/test_taco_api.cpp holds
taco's known-answer tests and randomized scheduling tests for the three statements, written as
a taco user writes them.  It compiles and links without a GPU; it runs on the GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "taco_gb300", "lib")
SRC = os.path.join(ROOT, "tests", "cpp", "test_taco_api.cpp")


@pytest.fixture(scope="module")
def binary(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("cpp") / "test_taco_api")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror", SRC,
                        "-I" + os.path.join(ROOT, "include"), "-L" + LIBDIR, "-ltacogb",
                        "-Wl,-rpath," + LIBDIR, "-o", out],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout
    return out


def test_cpp_api_compiles_and_links(binary):
    assert os.path.exists(binary)


@pytest.mark.gpu
def test_cpp_api_runs_taco_tests(binary):
    r = subprocess.run([binary], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=300)
    assert r.returncode == 0 and "all passed" in r.stdout, r.stdout
