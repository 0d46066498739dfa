"""The C++ DEMEngine stand-in (include/stardust_demengine.hpp) compiles
against include/stardust.h, links libstardust_gb300.so and runs a driver
written the reference's way (construct, add, prep, transfer, update in a
loop, sandbox/testDEM.cpp:60-137).  Without a GPU, transfer() must throw the
library's error; with one, the driver steps and reads the state back."""
import shutil
import subprocess

import pytest

DRIVER = r"""
#include <cstdio>
#include <stdexcept>
#include "stardust_demengine.hpp"

int main() {
    STARDUST::engineConfig cfg;
    STARDUST::DEMEngine engine(cfg, 1.0f);
    for (int i = 0; i < 8; ++i) {
        const float pos[3] = {0.2f + 0.05f * i, 0.5f, 0.3f};
        const float vel[3] = {0.0f, 0.0f, -0.1f};
        engine.add(1, 0.02f, 0.02f, 1e-3f, pos, vel);
    }
    const float cube[3] = {0.5f, 0.5f, 0.7f}, zero[3] = {0.0f, 0.0f, 0.0f};
    engine.add(2, 0.04f, 0.02f, 8e-3f, cube, zero);  // a 2 x 2 x 2 cube clump
    engine.prep();
    try {
        engine.transfer();
    } catch (const std::runtime_error& e) {
        std::printf("transfer failed: %s\n", e.what());
        return 3;
    }
    for (int s = 0; s < 100; ++s) engine.update(1e-5f);
    engine.sync();
    const sd_stats st = engine.stats();
    const std::vector<float> x = engine.positions();
    std::printf("spheres %llu steps %llu z0 %.6f\n", (unsigned long long)st.n_spheres,
                (unsigned long long)st.steps, x[2]);
    return st.n_spheres == 16 && st.steps == 100 && x[2] < 0.3f ? 0 : 1;
}
"""


def test_demengine_shim_builds_and_runs(sdlib, tmp_path):
    from stardust_gb300 import _abi
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    root = _abi.LIB_PATH.parents[1]
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "driver"
    cmd = [cxx, "-std=c++17", "-O1", f"-I{root / 'include'}", str(src), "-o", str(exe),
           f"-L{_abi.LIB_PATH.parent}", "-lstardust_gb300", f"-Wl,-rpath,{_abi.LIB_PATH.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    try:
        import torch
        gpu = torch.cuda.is_available()
    except Exception:
        gpu = False
    if gpu:
        assert r.returncode == 0, r.stdout + r.stderr
        assert "spheres 16 steps 100" in r.stdout
    else:
        # no device: the library's error reaches the caller as an exception
        assert r.returncode == 3 and "transfer failed" in r.stdout and "CUDA" in r.stdout, r.stdout + r.stderr
