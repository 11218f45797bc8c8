"""The C++ SPHSystem facade (include/sphx_system.h) keeps the reference's
semantics (src/SPHSystem.cpp:8-143): update() does nothing until
startSimulation(), then steps with dt forced to 0.003; reset() restores the
initParticles lattice and stops; `particles` mirrors the state; the
instance matrices are translate(x) * scale(h/2)."""
import os
import subprocess

import pytest

from _util import INCLUDE, PKG

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>
#include "sphx.h"
#include "sphx_system.h"

#define CHECK(c) do { if (!(c)) { std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c); return 1; } } while (0)

int main() {
    try {
        sphx::SPHSettings st(0.02f, 1000, 1, 1.04f, 0.15f, -9.8f, 0.2f);  // Tester.cpp:90
        sphx_settings a = st.args();
        sphx_derived d;
        CHECK(sphx_derive(&a, &d) == SPHX_OK);
        CHECK(st.poly6 == d.poly6 && st.spikyGrad == d.spiky_grad && st.selfDens == d.self_dens);
        CHECK(st.sphereScale[0] == 0.075f && st.sphereScale[15] == 1.f);

        sphx::SPHSystem sys(6, st, false);
        const size_t n = sys.particleCount;
        CHECK(n == 216);
        std::vector<float> init(3 * n);
        sphx_reference_scene(6, 0.15f, init.data());
        for (size_t i = 0; i < n; ++i)
            CHECK(std::memcmp(sys.particles[i].position, &init[3 * i], 12) == 0);

        sys.update(0.016f);  // not started: nothing happens
        for (size_t i = 0; i < n; ++i)
            CHECK(std::memcmp(sys.particles[i].position, &init[3 * i], 12) == 0);

        sys.startSimulation();
        sys.update(0.016f);  // forced to 0.003
        sphx_handle *h = nullptr;
        sphx_box box;
        sphx_box_reference(&box);
        CHECK(sphx_create(&a, &box, nullptr, n, init.data(), nullptr, &h) == SPHX_OK);
        CHECK(sphx_step(h, 0.003f, 1) == SPHX_OK);
        std::vector<float> pos(3 * n), vel(3 * n), rho(n);
        CHECK(sphx_read_state(h, pos.data(), vel.data(), rho.data(), nullptr, nullptr) == SPHX_OK);
        for (size_t i = 0; i < n; ++i) {
            CHECK(std::memcmp(sys.particles[i].position, &pos[3 * i], 12) == 0);
            CHECK(std::memcmp(sys.particles[i].velocity, &vel[3 * i], 12) == 0);
            CHECK(sys.particles[i].density == rho[i]);
        }
        const float *m = sys.transforms();
        for (size_t i = 0; i < n; ++i) {
            CHECK(m[16 * i + 0] == 0.075f && m[16 * i + 5] == 0.075f && m[16 * i + 10] == 0.075f);
            CHECK(m[16 * i + 12] == pos[3 * i] && m[16 * i + 13] == pos[3 * i + 1]);
            CHECK(m[16 * i + 15] == 1.f && m[16 * i + 1] == 0.f);
        }
        sphx_destroy(h);

        sys.reset();  // lattice back, stopped
        CHECK(!sys.started());
        for (size_t i = 0; i < n; ++i)
            CHECK(std::memcmp(sys.particles[i].position, &init[3 * i], 12) == 0);
        sys.update(0.016f);
        for (size_t i = 0; i < n; ++i)
            CHECK(std::memcmp(sys.particles[i].position, &init[3 * i], 12) == 0);
        std::printf("OK\n");
        return 0;
    } catch (const std::exception &e) {
        std::printf("error: %s\n", e.what());
        return 2;
    }
}
"""


def build(tmp_path):
    src = tmp_path / "facade.cpp"
    src.write_text(PROGRAM)
    exe = str(tmp_path / "facade")
    libdir = os.path.join(PKG, "lib")
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", INCLUDE, str(src), "-L", libdir, "-lsphx",
                    "-Wl,-rpath," + libdir, "-o", exe], check=True, capture_output=True, text=True)
    return exe


def test_facade_compiles_and_fails_loudly_without_gpu(sphx_lib, tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = subprocess.run([build(tmp_path)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "error:" in r.stdout


@pytest.mark.gpu
def test_facade_semantics_on_gpu(sphx_lib, tmp_path):
    r = subprocess.run([build(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip().endswith("OK"), r.stdout + r.stderr
