// Reference-side binding for lijenicol/SPH-Fluid-Simulator: a replacement for
// src/kernels/sphGPU.cu that implements the reference's GPU backend symbol
//   void updateParticlesGPU(Particle*, glm::mat4*, size_t, const SPHSettings&, float)
// (src/kernels/sphGPU.h:8-11) on top of libsphx.  Drop it into the reference
// build in place of sphGPU.cu and link with -lsphx; sph.cpp, SPHSystem.cpp and
// Tester.cpp compile unchanged, and updateParticles(..., onGPU = true)
// (src/sph.cpp:277-290) then steps on the GB300.
#include <cstdio>
#include <cstdlib>

#include <kernels/sphGPU.h>
#include "sphx.h"

static_assert(sizeof(Particle) == 60, "Particle.h layout");

void updateParticlesGPU(Particle *particles, glm::mat4 *particleTransforms,
                        const size_t particleCount, const SPHSettings &settings,
                        float deltaTime) {
    const sphx_settings s = {settings.mass, settings.restDensity, settings.gasConstant,
                             settings.viscosity, settings.h, settings.g, settings.tension};
    const int rc = sphx_update_particles(particles, &particleTransforms[0][0][0], particleCount,
                                         &s, /*box: the CPU path's walls*/ nullptr, deltaTime);
    if (rc != SPHX_OK) {
        std::fprintf(stderr, "sphx: %s\n", sphx_last_error());
        std::abort();
    }
}
