// sphx::SPHSystem — the reference's SPHSystem interface (src/SPHSystem.h,
// src/SPHSystem.cpp) over the resident GPU step.
#include "sphx_system.h"

#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

namespace sphx {

namespace {

void check(int rc, const char *what) {
    if (rc != SPHX_OK)
        throw std::runtime_error(std::string(what) + ": " + sphx_last_error());
}

}  // namespace

// SPHSystem.cpp:8-26 (through sphx_derive, bit-identical constants).
SPHSettings::SPHSettings(float mass_, float restDensity_, float gasConst, float viscosity_,
                         float h_, float g_, float tension_) {
    const sphx_settings a{mass_, restDensity_, gasConst, viscosity_, h_, g_, tension_};
    sphx_derived d;
    check(sphx_derive(&a, &d), "SPHSettings");
    std::memcpy(sphereScale, d.sphere_scale, sizeof sphereScale);
    poly6 = d.poly6;
    spikyGrad = d.spiky_grad;
    spikyLap = d.spiky_lap;
    gasConstant = d.gas_constant;
    mass = d.mass;
    h2 = d.h2;
    selfDens = d.self_dens;
    restDensity = d.rest_density;
    viscosity = d.viscosity;
    h = d.h;
    g = d.g;
    tension = d.tension;
    massPoly6Product = d.mass_poly6_product;
}

sphx_settings SPHSettings::args() const {
    return sphx_settings{mass, restDensity, gasConstant, viscosity, h, g, tension};
}

// SPHSystem.cpp:28-69 minus the graphics buffers.
SPHSystem::SPHSystem(size_t cubeWidth, const SPHSettings &s, const bool & /*runOnGPU*/)
    : settings(s), particleCubeWidth(cubeWidth) {
    particleCount = cubeWidth * cubeWidth * cubeWidth;
    particles = static_cast<Particle *>(std::calloc(particleCount ? particleCount : 1, sizeof(Particle)));
    if (!particles) throw std::runtime_error("SPHSystem: host allocation failed");
    std::vector<float> pos3;
    initParticles(pos3);
    const sphx_settings a = settings.args();
    sphx_box box;
    sphx_box_reference(&box);
    const int rc = sphx_create(&a, &box, nullptr, particleCount, pos3.data(), nullptr, &h);
    if (rc != SPHX_OK) {
        std::free(particles);
        check(rc, "SPHSystem");
    }
    for (size_t i = 0; i < particleCount; ++i)
        std::memcpy(particles[i].position, &pos3[3 * i], 12);
    isStarted = false;
}

SPHSystem::~SPHSystem() {
    sphx_destroy(h);
    std::free(particles);
}

void SPHSystem::initParticles(std::vector<float> &pos3) const {
    pos3.assign(3 * particleCount, 0.f);
    check(sphx_reference_scene(particleCubeWidth, settings.h, pos3.data()), "initParticles");
}

// SPHSystem.cpp:110-117.
void SPHSystem::update(float deltaTime) {
    if (!isStarted) return;
    if (fixedTimestep) deltaTime = 0.003f;
    check(sphx_step(h, deltaTime, 1), "update");
    if (hostMirror) refreshParticles();
}

// SPHSystem.cpp:136-139.
void SPHSystem::reset() {
    std::vector<float> pos3;
    initParticles(pos3);
    check(sphx_set_state(h, pos3.data(), nullptr), "reset");
    std::memset(particles, 0, particleCount * sizeof(Particle));
    for (size_t i = 0; i < particleCount; ++i)
        std::memcpy(particles[i].position, &pos3[3 * i], 12);
    isStarted = false;
}

// SPHSystem.cpp:141-143.
void SPHSystem::startSimulation() { isStarted = true; }

void SPHSystem::refreshParticles() {
    const size_t n = particleCount;
    std::vector<float> pos(3 * n), vel(3 * n), force(3 * n), rho(n), prs(n);
    std::vector<uint16_t> hash(n);
    check(sphx_read_state(h, pos.data(), vel.data(), rho.data(), prs.data(), force.data()),
          "read state");
    check(sphx_read_cells(h, nullptr, hash.data()), "read cells");
    for (size_t i = 0; i < n; ++i) {
        Particle &p = particles[i];
        std::memcpy(p.position, &pos[3 * i], 12);
        std::memcpy(p.velocity, &vel[3 * i], 12);
        std::memcpy(p.force, &force[3 * i], 12);
        p.density = rho[i];
        p.pressure = prs[i];
        p.hash = hash[i];
    }
}

const float *SPHSystem::transforms() {
    transformBuf.resize(16 * particleCount);
    check(sphx_read_transforms(h, transformBuf.data()), "transforms");
    return transformBuf.data();
}

}  // namespace sphx
