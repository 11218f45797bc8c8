"""The reference-side binding (include/integration/sphGPU_sphx.cpp, a
replacement for the reference's sphGPU.cu) links against the unmodified
reference sources and libsphx.so, and the reference's own
updateParticles(..., onGPU=true) dispatch reaches sphx.

Needs the reference checkout (skipped elsewhere).  Without a GPU the call
must fail loudly inside sphx (no CPU fallback); with one it must succeed."""
import os
import subprocess

import pytest

from _util import INCLUDE, ORACLE, PKG

MAIN = r"""
#include <cstdio>
#include <vector>
#include "SPHSystem.h"
#include "sph.h"
#include "sphx.h"

// SPHSettings' constructor lives in the reference's SPHSystem.cpp next to
// graphics code; the constants come from sphx_derive here.
SPHSettings::SPHSettings(float mass, float restDensity, float gasConst, float viscosity,
                         float h, float g, float tension)
    : mass(mass), restDensity(restDensity), gasConstant(gasConst), viscosity(viscosity), h(h),
      g(g), tension(tension) {
    sphx_settings a = {mass, restDensity, gasConst, viscosity, h, g, tension};
    sphx_derived d;
    sphx_derive(&a, &d);
    poly6 = d.poly6; spikyGrad = d.spiky_grad; spikyLap = d.spiky_lap; h2 = d.h2;
    selfDens = d.self_dens; massPoly6Product = d.mass_poly6_product;
}

int main() {
    SPHSettings s(0.02f, 1000, 1, 1.04f, 0.15f, -9.8f, 0.2f);
    std::vector<Particle> p(512);
    std::vector<float> pos(3 * 512);
    sphx_reference_scene(8, 0.15f, pos.data());
    for (int i = 0; i < 512; ++i) {
        p[i] = Particle();
        p[i].position = glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    }
    std::vector<glm::mat4> t(512);
    updateParticles(p.data(), t.data(), p.size(), s, 0.003f, true);
    std::printf("stepped %f %f\n", p[0].position.y, p[0].density);
    return 0;
}
"""


STUB = os.path.join(INCLUDE, "integration", "sphGPU_sphx.cpp")


def test_reference_links_against_sphx_and_dispatches(sphx_lib, tmp_path):
    import build_oracle
    src = os.path.join(build_oracle.reference_dir(), "src")
    if not os.path.isfile(os.path.join(src, "sph.cpp")):
        pytest.skip("reference checkout not present")
    (tmp_path / "main.cpp").write_text(MAIN)
    libdir = os.path.join(PKG, "lib")
    exe = str(tmp_path / "ref_with_sphx")
    cmd = ["g++", "-O1", "-std=c++17", "-w", "-pthread", "-I", os.path.join(ORACLE, "shim"), "-I", src,
           "-I", INCLUDE, STUB, str(tmp_path / "main.cpp"),
           os.path.join(src, "sph.cpp"), os.path.join(src, "neighborTable.cpp"),
           os.path.join(src, "timer.cpp"), "-L", libdir, "-lsphx", "-Wl,-rpath," + libdir, "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    import torch
    if torch.cuda.is_available():
        assert r.returncode == 0, r.stderr
        assert "stepped" in r.stdout
    else:
        assert r.returncode != 0
        assert "sphx:" in r.stderr  # failed loudly inside sphx, no CPU fallback
