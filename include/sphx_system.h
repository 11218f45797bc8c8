// C++ facade with the reference's simulation interface
// (lijenicol/SPH-Fluid-Simulator src/SPHSystem.h:13-58), running every step on
// the GPU through the sphx C-ABI (include/sphx.h).
//
//   sphx::SPHSettings  — SPHSystem.h:13-22: same constructor, same derived
//                        fields in the same order (sphereScale first, as a
//                        column-major float[16] in place of glm::mat4), values
//                        bit-identical to SPHSystem.cpp:8-26.
//   sphx::Particle     — Particle.h:4-10: the same 60-byte record.
//   sphx::SPHSystem    — SPHSystem.h:24-58: constructor(cubeWidth, settings,
//                        runOnGPU), update(dt), reset(), startSimulation(),
//                        public `particles` / `particleCount`.
//
// Behaviour kept from the reference: update() is a no-op until
// startSimulation(); it then forces dt = 0.003 (SPHSystem.cpp:110-117,
// switchable with setFixedTimestep); reset() restores the initParticles
// lattice (srand(1024), SPHSystem.cpp:76-108) and stops; walls are the CPU
// path's (x, z in [-8, 8], floor y = 0, no ceiling).
//
// Differences: runOnGPU is accepted and ignored (this library is the GPU
// path; there is no CPU fallback); `particles` is a host mirror refreshed
// after each update (setHostMirror(false) skips the copy) and kept in the
// constructor's order rather than re-sorted by hash every step; draw() is
// not provided (no graphics API) — transforms() returns the per-particle
// translate(x) * scale(h/2) matrices the instanced renderer consumes, and
// handle() gives device-resident state for zero-copy consumers.  Errors
// throw std::runtime_error where the reference has no error channel.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "sphx.h"

namespace sphx {

struct SPHSettings {
    SPHSettings(float mass, float restDensity, float gasConst, float viscosity, float h, float g,
                float tension);

    float sphereScale[16];
    float poly6, spikyGrad, spikyLap, gasConstant, mass, h2, selfDens, restDensity, viscosity, h,
        g, tension, massPoly6Product;

    sphx_settings args() const;  // the constructor arguments
};

struct Particle {
    float position[3], velocity[3], acceleration[3], force[3];
    float density;
    float pressure;
    uint16_t hash;
};
static_assert(sizeof(Particle) == 60, "Particle must match the reference layout");

class SPHSystem {
public:
    SPHSystem(size_t particleCubeWidth, const SPHSettings &settings, const bool &runOnGPU);
    ~SPHSystem();
    SPHSystem(const SPHSystem &) = delete;
    SPHSystem &operator=(const SPHSystem &) = delete;

    Particle *particles;
    size_t particleCount;

    // One step when started (dt forced to 0.003 unless setFixedTimestep(false)).
    void update(float deltaTime);
    void reset();
    void startSimulation();

    // Beyond the reference.
    void setFixedTimestep(bool on) { fixedTimestep = on; }
    void setHostMirror(bool on) { hostMirror = on; }
    void refreshParticles();              // copies device state into `particles`
    const float *transforms();            // n column-major mat4, refreshed on call
    sphx_handle *handle() const { return h; }
    bool started() const { return isStarted; }

private:
    void initParticles(std::vector<float> &pos3) const;

    SPHSettings settings;
    size_t particleCubeWidth;
    bool isStarted = false;
    bool fixedTimestep = true;
    bool hostMirror = true;
    sphx_handle *h = nullptr;
    std::vector<float> transformBuf;
};

}  // namespace sphx
