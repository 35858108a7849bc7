"""The boundary headers build as a caller would use them (no GPU needed:
the programs are compiled and linked, not run):

* a C99 program including include/pbd_c.h and taking the address of every
  entry point it declares links against libpbd_gb300.so;
* a C++17 program using the classes of include/pbd.hpp (the reference's
  class and method names) compiles and links.
"""
import os
import shutil
import subprocess

import pytest

from positionbaseddynamicsold_gb300 import build

from test_lib_exports import declared

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None or shutil.which("g++") is None,
                                reason="needs gcc and g++")


def link(tmp_path, compiler, name, src, extra):
    lib = build.build()
    f = tmp_path / name
    f.write_text(src)
    out = tmp_path / (name + ".bin")
    cmd = [compiler, *extra, "-I", INC, str(f), "-o", str(out), "-L", os.path.dirname(lib),
           "-l:" + os.path.basename(lib), "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_c_header_links_every_entry(tmp_path):
    names = declared()
    src = "#include \"pbd_c.h\"\n#include <stdio.h>\nint main(void) {\n    void *p[] = {\n"
    src += ",\n".join("        (void *)%s" % n for n in names)
    src += "\n    };\n    printf(\"%d\\n\", (int)(sizeof p / sizeof p[0]));\n    return 0;\n}\n"
    link(tmp_path, "gcc", "abi.c", src, ["-std=c99", "-Wall", "-Werror"])


def test_cpp_classes_compile_and_link(tmp_path):
    src = r'''
#include "pbd.hpp"
#include <vector>
int main(int argc, char **) {
    if (argc < 100) return 0;   // compiled and linked, never run
    pbd_object_desc d = {};
    pbd::PBDObject obj(d);
    obj.EdgeColoring(20000);
    obj.SortEdgesColors();
    obj.EvalWorksets();
    float center[3] = {0, 0, 0}, cell[3] = {0.1f, 0.1f, 0.1f};
    int size[3] = {8, 8, 8};
    pbd::SpatialHashSystem shs(obj, center, size, cell);
    shs.InitSH();
    pbd::CollisionSolver colli;
    colli.SetTarget(obj);
    colli.SetAcceStruct(shs);
    colli.SetThickness(0.03f);
    colli.SetIterations(1);
    pbd::SolverPBD solver;
    solver.SetTarget(obj);
    solver.Advect(1.0f / 60);
    solver.ProjectConstraintWithColli(PBD_GAUSSSEIDEL, 15, colli);
    solver.Integration(1.0f / 60);
    std::vector<float> p = obj.Positions();
    return (int)p.size();
}
'''
    link(tmp_path, "g++", "classes.cpp", src, ["-std=c++17", "-Wall", "-Werror"])
