// Test infrastructure only — never part of the product path.
//
// C-ABI wrapper around the reference's own CPU hot path, compiled unmodified
// from src/sph.cpp, src/neighborTable.cpp and src/timer.cpp of
// lijenicol/SPH-Fluid-Simulator against the project-written GLM shim in
// oracle/shim.  The result is oracle/_ref/libsphref.so, used by the tests (and
// by tests/golden/make_golden.py) to pin the oracle restatement
// (oracle/sph_oracle.cpp) against the real reference code.
//
// Two pieces of the reference are not compiled because their translation
// unit (src/SPHSystem.cpp) also creates graphics buffers: the SPHSettings
// constructor (SPHSystem.cpp:8-26) is restated below with the same
// expression types, and the particle identity that the reference lacks is
// carried through its in-place sort in the never-written `acceleration`
// field (Particle.h:6; sph.cpp never reads or writes it).
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <thread>
#include <vector>

#include <glm/gtx/norm.hpp>

#include "Particle.h"
#include "SPHSystem.h"
#include "neighborTable.h"
#include "sph.h"

#define PI 3.14159265f

// SPHSystem.cpp:8-26 — same operand types: pow() runs in double and the
// result is rounded to float on assignment.
SPHSettings::SPHSettings(float mass, float restDensity, float gasConst,
                         float viscosity, float h, float g, float tension)
    : mass(mass), restDensity(restDensity), gasConstant(gasConst),
      viscosity(viscosity), h(h), g(g), tension(tension) {
    poly6 = 315.0f / (64.0f * PI * pow(h, 9));
    spikyGrad = -45.0f / (PI * pow(h, 6));
    spikyLap = 45.0f / (PI * pow(h, 6));
    h2 = h * h;
    selfDens = mass * poly6 * pow(h, 6);
    massPoly6Product = mass * poly6;
    sphereScale = glm::scale(glm::vec3(h / 2.f));
}

// Reference functions that sph.h does not declare (sph.cpp:28,80,195).
void parallelDensityAndPressures(Particle *, const size_t, const size_t,
                                 const size_t, const uint32_t *,
                                 const SPHSettings &);
void parallelForces(Particle *, const size_t, const size_t, const size_t,
                    const uint32_t *, const SPHSettings &);
void updateParticlesCPU(Particle *, glm::mat4 *, const size_t,
                        const SPHSettings &, float);

// The reference links its GPU backend here (sph.cpp:282-284); the oracle
// never selects it.
static int g_gpu_called = 0;
void updateParticlesGPU(Particle *, glm::mat4 *, const size_t,
                        const SPHSettings &, float) {
    g_gpu_called = 1;
}

namespace {

struct CerrSilencer {  // the reference's Timer prints to stderr (timer.cpp:23)
    std::stringstream sink;
    std::streambuf *old;
    CerrSilencer() : old(std::cerr.rdbuf(sink.rdbuf())) {}
    ~CerrSilencer() { std::cerr.rdbuf(old); }
};

SPHSettings make_settings(const float *a) {
    return SPHSettings(a[0], a[1], a[2], a[3], a[4], a[5], a[6]);
}

void load(Particle *p, size_t n, const float *pos, const float *vel) {
    for (size_t i = 0; i < n; ++i) {
        std::memset(&p[i], 0, sizeof(Particle));
        p[i].position = glm::vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        p[i].velocity = vel ? glm::vec3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2])
                            : glm::vec3(0.f);
        uint32_t id = (uint32_t)i;
        std::memcpy(&p[i].acceleration.x, &id, 4);
    }
}

uint32_t id_of(const Particle &p) {
    uint32_t id;
    std::memcpy(&id, &p.acceleration.x, 4);
    return id;
}

uint64_t mix64(uint64_t z) {  // SplitMix64 finaliser, a multiset fingerprint
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

extern "C" {

int ref_sizeof_particle(void) { return (int)sizeof(Particle); }

uint32_t ref_get_hash(int x, int y, int z) { return getHash(glm::ivec3(x, y, z)); }

void ref_get_cell(float x, float y, float z, float h, int *out) {
    Particle p;
    std::memset(&p, 0, sizeof p);
    p.position = glm::vec3(x, y, z);
    glm::ivec3 c = getCell(&p, h);
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
}

// out[0..12] = poly6, spikyGrad, spikyLap, gasConstant, mass, h2, selfDens,
// restDensity, viscosity, h, g, tension, massPoly6Product; out[13..28] =
// sphereScale (column-major).
void ref_settings(const float *args, float *out) {
    SPHSettings s = make_settings(args);
    const float v[13] = {s.poly6, s.spikyGrad, s.spikyLap, s.gasConstant,
                         s.mass, s.h2, s.selfDens, s.restDensity, s.viscosity,
                         s.h, s.g, s.tension, s.massPoly6Product};
    std::memcpy(out, v, sizeof v);
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[13 + 4 * c + r] = s.sphereScale[c][r];
}

// One call of the reference's updateParticlesCPU (sph.cpp:195-275) on n
// particles.  Outputs are in the reference's post-step (hash-sorted) order;
// ids[k] is the input index of output particle k.  density/pressure/force
// are the values the step used to integrate; hash is the stored uint16 key;
// transforms holds 16 floats per particle (column-major).
int ref_update_cpu(size_t n, const float *pos, const float *vel,
                   const float *args, float dt, uint32_t *ids, float *pos_out,
                   float *vel_out, float *rho, float *prs, float *force,
                   uint16_t *hash, float *transforms) {
    SPHSettings s = make_settings(args);
    std::vector<Particle> p(n);
    std::vector<glm::mat4> t(n);
    load(p.data(), n, pos, vel);
    {
        CerrSilencer quiet;
        updateParticlesCPU(p.data(), t.data(), n, s, dt);
    }
    for (size_t k = 0; k < n; ++k) {
        const Particle &q = p[k];
        if (ids) ids[k] = id_of(q);
        if (pos_out) { pos_out[3 * k] = q.position.x; pos_out[3 * k + 1] = q.position.y; pos_out[3 * k + 2] = q.position.z; }
        if (vel_out) { vel_out[3 * k] = q.velocity.x; vel_out[3 * k + 1] = q.velocity.y; vel_out[3 * k + 2] = q.velocity.z; }
        if (rho) rho[k] = q.density;
        if (prs) prs[k] = q.pressure;
        if (force) { force[3 * k] = q.force.x; force[3 * k + 1] = q.force.y; force[3 * k + 2] = q.force.z; }
        if (hash) hash[k] = q.hash;
        if (transforms)
            for (int c = 0; c < 4; ++c)
                for (int r = 0; r < 4; ++r) transforms[16 * k + 4 * c + r] = t[k][c][r];
    }
    return g_gpu_called ? -1 : 0;
}

// Candidate walk of the reference (sph.cpp:35-66) driven by the reference's
// own getCell / getHash / sortParticles / createNeighborTable: for each input
// particle, the number of accepted (r^2 < h^2) visits and the wrapping sum of
// mix64(id) over them — a fingerprint of the accepted neighbour multiset,
// counting a particle as often as the walk visits it.
int ref_neighbor_digest(size_t n, const float *pos, float h, uint32_t *count,
                        uint64_t *digest) {
    float args[7] = {1.f, 1.f, 1.f, 1.f, h, 0.f, 0.f};
    SPHSettings s = make_settings(args);
    std::vector<Particle> p(n);
    load(p.data(), n, pos, nullptr);
    parallelCalculateHashes(p.data(), 0, n, s);
    sortParticles(p.data(), n);
    uint32_t *table = createNeighborTable(p.data(), n);
    for (size_t pi = 0; pi < n; ++pi) {
        glm::ivec3 cell = getCell(&p[pi], s.h);
        uint32_t cnt = 0;
        uint64_t dig = 0;
        for (int x = -1; x <= 1; x++)
            for (int y = -1; y <= 1; y++)
                for (int z = -1; z <= 1; z++) {
                    uint16_t ch = getHash(cell + glm::ivec3(x, y, z));
                    uint32_t pj = table[ch];
                    if (pj == NO_PARTICLE) continue;
                    while (pj < n) {
                        if (pj == pi) { pj++; continue; }
                        if (p[pj].hash != ch) break;
                        float d2 = glm::length2(p[pj].position - p[pi].position);
                        if (d2 < s.h2) { cnt++; dig += mix64(id_of(p[pj])); }
                        pj++;
                    }
                }
        const uint32_t id = id_of(p[pi]);
        count[id] = cnt;
        digest[id] = dig;
    }
    free(table);
    return 0;
}

}  // extern "C"
