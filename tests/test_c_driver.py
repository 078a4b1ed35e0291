"""The C-ABI driven from plain C (tests/c_driver/olc_driver.c), compiled with
gcc against include/olcao_gpu.h and linked to libolcao_gb300.so: the host
entries run here; the GPU leg runs one primitive batch on the device."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _build(tmp_path, lib_dir):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "olc_driver")
    subprocess.run([cc, "-std=c99", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_driver", "olc_driver.c"), "-o", exe,
                    "-L", lib_dir, "-lolcao_gb300", f"-Wl,-rpath,{lib_dir}", "-lm"], check=True)
    return exe


def test_c_driver_host_entries(gpu_free_lib, tmp_path):
    lib_dir = os.path.dirname(gpu_free_lib._name)
    exe = _build(tmp_path, lib_dir)
    r = subprocess.run([exe, "host"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


@pytest.mark.gpu
def test_c_driver_gpu_primitive(gpu_lib, tmp_path):
    lib_dir = os.path.dirname(gpu_lib._name)
    exe = _build(tmp_path, lib_dir)
    r = subprocess.run([exe, "gpu"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
