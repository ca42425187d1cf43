"""The C++ mirror of the reference's FluidSimulation / FluidSimBase
(include/sph_fluid_simulation.hpp): compiled and linked against the library
on any host; run on a GPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = ROOT / "tests" / "cpp" / "fluid_sim_host.cc"


def build_host_program(lib_path, out_dir):
    exe = out_dir / "fluid_sim_host"
    cmd = [shutil.which("g++") or "g++", "-std=c++17", "-O2",
           f"-I{ROOT / 'include'}", str(SRC), f"-L{lib_path.parent}",
           "-lsph_gb300", f"-Wl,-rpath,{lib_path.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_mirror_compiles_and_links(built_lib, tmp_path):
    exe = build_host_program(built_lib, tmp_path)
    assert exe.exists()


@pytest.mark.gpu
def test_cpp_mirror_runs(gpu_lib, built_lib, tmp_path):
    exe = build_host_program(built_lib, tmp_path)
    env = dict(os.environ, SPH_SNAPSHOT_PATH=str(tmp_path / "host.sph"))
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120, env=env)
    print(r.stdout, r.stderr)
    assert r.returncode == 0
    assert r.stdout.startswith("ok")
