"""CPU check that the drop-in C++ header compiles user code written against
the original `natural` surface."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_header_compiles(tmp_path):
    subprocess.check_call(["g++", "-std=c++20", "-fsyntax-only", "-Wall", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "natural_demo.cpp")])
