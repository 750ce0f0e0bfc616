"""The reference-side drop-in (pathfinder-cpp_gb300/plugin) against the reference's own types.

Compiles SceneBuilderCuda / RendererCuda and the headless DeviceCuda / QueueCuda with the
reference's headers, links them with the reference's compiled Scene, Path2d, paint and Renderer
code (oracle/_ref), builds a scene through the reference API (with a view box that has an
origin) and checks the packed scene against the reference tiler; then runs the reference's
Renderer base class and Palette::build_paint_info on the headless device, checks its transfers,
and that RendererCuda::draw without a CUDA device logs and leaves the destination alone.  Needs
the reference tree (so it does not run where the GPU is: the reference's headers are not there);
skipped where it is absent.
"""
import glob
import os
import subprocess

import pytest

from conftest import ROOT


def test_plugin_packs_reference_scene(tmp_path, oracle_mod, pf):
    ref = oracle_mod.REF_ROOT
    if not os.path.isdir(os.path.join(ref, "pathfinder")):
        pytest.skip("reference tree not present")
    oracle_mod.build(reference=True)
    objs = sorted(glob.glob(os.path.join(ROOT, "oracle", "_ref", "obj", "**", "*.o"), recursive=True))
    exe = str(tmp_path / "plugin_driver")
    import platform
    simd = ["-msse4.1"] if platform.machine() in ("x86_64", "AMD64") else []  # Arm: sse2neon.h
    cmd = ["g++", "-std=c++17", "-O1", *simd, "-DPATHFINDER_ENABLE_SIMD", "-DPATHFINDER_ENABLE_COMPUTE",
           f"-I{ref}/pathfinder", f"-I{ref}/third_party", f"-I{ref}/third_party/umHalf",
           f"-I{ROOT}/include", f"-I{ROOT}/oracle", f"-I{ROOT}/pathfinder-cpp_gb300/plugin", "-w",
           os.path.join(ROOT, "tests", "plugin", "plugin_driver.cpp"),
           os.path.join(ROOT, "pathfinder-cpp_gb300", "plugin", "renderer_cuda.cpp"),
           os.path.join(ROOT, "pathfinder-cpp_gb300", "plugin", "device_cuda.cpp"), *objs,
           os.path.join(ROOT, "oracle", "_ref", "libpfref.so"), os.path.join(ROOT, "oracle", "_build", "libpforacle.so"),
           pf.LIB_PATH, "-lpthread", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True)
    env = dict(os.environ)
    env["LD_LIBRARY_PATH"] = ":".join([os.path.dirname(pf.LIB_PATH), os.path.join(ROOT, "oracle", "_build"),
                                       os.path.join(ROOT, "oracle", "_ref"), env.get("LD_LIBRARY_PATH", "")])
    out = subprocess.run([exe], capture_output=True, text=True, env=env)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("OK")
