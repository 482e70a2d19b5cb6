"""The C++ adapter header compiles, links against libmfg.so and drives a run."""
import os
import subprocess

import pytest

from molflow_sources_gb300.simulation import library_path, load_library

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path):
    load_library()
    lib = library_path()
    exe = str(tmp_path / "adapter_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "adapter_check.cpp"), "-o", exe,
                    "-L", os.path.dirname(lib), "-lmfg", "-Wl,-rpath," + os.path.dirname(lib)], check=True)
    return exe


def test_adapter_compiles_and_reports_no_device(tmp_path):
    exe = _build(tmp_path)
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present: covered by the gpu test")
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0 and "no-device" in out.stdout


@pytest.mark.gpu
def test_adapter_runs_on_gpu(tmp_path):
    exe = _build(tmp_path)
    for args in ([], ["fp32r"]):
        out = subprocess.run([exe] + args, capture_output=True, text=True, timeout=300)
        assert out.returncode == 0, out.stdout + out.stderr
        p = float(out.stdout.split()[1])
        # 32-gon L/R=10 tube: transmission near the Clausing value 0.19 (200k particles)
        assert abs(p - 0.19) < 0.005, out.stdout
