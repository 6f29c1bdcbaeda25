"""Compiles tests/struct_matrix_driver.cpp (the C++ struct-matrix class of
include/ipfem_pz.hpp, used as the reference's analysis uses its struct matrix)
with g++ against the in-tree libipfem.so; shared by the CPU and GPU tests."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build_driver(out_dir):
    import intpointsfem_gb300 as ip

    ip.lib()                                           # the library is built
    exe = os.path.join(str(out_dir), "struct_matrix_driver")
    libdir = os.path.dirname(ip.LIB_PATH)
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(HERE, "struct_matrix_driver.cpp"), "-o", exe, "-L" + libdir, "-lipfem",
                           "-Wl,-rpath," + libdir])
    return exe
