"""Reference-layout views (include/picgb_view.hpp) and the C++ host program that uses them.

tests/cpp/view_plugin.cu drives the stage loop of Simulation::runOneStep through
include/picgb.h and reads E, B and both species through FieldBox and ParticlesBox the
way PIConGPU's EnergyFields and EnergyParticles plugins read the DataConnector's data
(plugins/EnergyFields.x.cpp:241-261, plugins/EnergyParticles.x.cpp:58-160).
* CPU: the header compiles as plain C++17 (g++), and the program compiles for sm_103a.
* GPU: the program, linked against libpicgb.so, matches picgb_energies (field energies
  within 1e-12, kinetic energies within 1e-6), visits every particle once through the
  frame lists and reads the periodic neighbours at guard indices.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
SRC = os.path.join(ROOT, "tests", "cpp", "view_plugin.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    pytest.skip("nvcc not found")


def test_view_header_is_plain_cxx(tmp_path):
    src = tmp_path / "use_view.cpp"
    src.write_text('#include "picgb_view.hpp"\n'
                   'int probe(picgb_sim* sim) {\n'
                   '    picgb::view::FieldBox e;\n'
                   '    picgb::view::ParticlesBox p;\n'
                   '    int r = picgb::view::makeFieldBox(sim, "E", {8, 8, 4}, &e);\n'
                   '    r |= picgb::view::makeParticlesBox(sim, "e", {8, 8, 4}, &p);\n'
                   '    return r + int(e.shift({8, 8, 4}).offset({0, 0, 0})) + int(p.frameSize);\n'
                   '}\n')
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-I", INC, str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_view_plugin_program_compiles(tmp_path):
    obj = tmp_path / "view_plugin.o"
    r = subprocess.run([_nvcc(), *ARCH, "-std=c++17", "-O2", "-I", INC, "-c", SRC, "-o", str(obj)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_view_plugin_program_matches_the_library(tmp_path):
    import picongpu_gb300 as pg

    pg.load()  # builds libpicgb.so when needed
    libdir = os.path.join(ROOT, "picongpu_gb300", "_build")
    exe = tmp_path / "view_plugin"
    r = subprocess.run([_nvcc(), *ARCH, "-std=c++17", "-O2", "-I", INC, SRC, "-o", str(exe), "-L", libdir, "-lpicgb",
                        f"-Xlinker=-rpath={libdir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(run.stdout)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "view plugin: OK" in run.stdout
