// Stateless host utilities of the C-ABI (include/sphx.h): error reporting,
// the reference's settings constants, hash and cell functions, the
// bucket-collision test, lattice generators and presets.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>

#include "sphx_internal.h"

namespace {

thread_local std::string g_err;

uint64_t mix64(uint64_t z) {  // SplitMix64 output function of state z - gamma
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

}  // namespace

namespace sphx {

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

Derived derive_constants(float mass, float restDensity, float gasConst, float viscosity, float h,
                         float g, float tension) {
    const float PI = 3.14159265f;  // SPHSystem.cpp:6
    Derived d;
    d.mass = mass;
    d.restDensity = restDensity;
    d.gasConstant = gasConst;
    d.viscosity = viscosity;
    d.h = h;
    d.g = g;
    d.tension = tension;
    d.poly6 = (float)(315.0f / ((double)(64.0f * PI) * std::pow((double)h, 9.0)));
    d.spikyGrad = (float)(-45.0f / ((double)PI * std::pow((double)h, 6.0)));
    d.spikyLap = (float)(45.0f / ((double)PI * std::pow((double)h, 6.0)));
    d.h2 = h * h;
    d.selfDens = (float)((double)(mass * d.poly6) * std::pow((double)h, 6.0));
    d.massPoly6Product = mass * d.poly6;
    return d;
}

}  // namespace sphx

using sphx::fail;

extern "C" {

const char *sphx_version(void) { return "sphx 0.1 (sm_103a)"; }
const char *sphx_last_error(void) { return g_err.c_str(); }

void sphx_settings_reference(sphx_settings *s) {
    if (s) *s = sphx_settings{0.02f, 1000.f, 1.f, 1.04f, 0.15f, -9.8f, 0.2f};
}

void sphx_box_reference(sphx_box *b) {
    if (b) *b = sphx_box{-8.f, 8.f, 0.f, 0.f, -8.f, 8.f, 0.5f, 0.0001f, 0};
}

void sphx_options_default(sphx_options *o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->reorder_interval = 1;
    o->use_graph = 1;
    o->device = 0;
    o->stream = nullptr;
    o->grid_ymax = 0.f;
    o->max_cell_occupancy = 16384;
    o->density_threads = 128;
    o->force_threads = 128;
    o->neighbor_slots = 256;
}

int sphx_derive(const sphx_settings *s, sphx_derived *out) {
    if (!s || !out) return fail(SPHX_ERR_INVALID, "null argument");
    const sphx::Derived d = sphx::derive_constants(s->mass, s->rest_density, s->gas_const,
                                                   s->viscosity, s->h, s->g, s->tension);
    static_assert(sizeof(sphx::Derived) == 13 * sizeof(float), "layout");
    std::memcpy(out, &d, sizeof d);
    const float sc = s->h / 2.f;  // glm::scale(vec3(h / 2)), SPHSystem.cpp:25
    for (int k = 0; k < 16; ++k) out->sphere_scale[k] = 0.f;
    out->sphere_scale[0] = sc;
    out->sphere_scale[5] = sc;
    out->sphere_scale[10] = sc;
    out->sphere_scale[15] = 1.f;
    return SPHX_OK;
}

uint32_t sphx_hash(int32_t cx, int32_t cy, int32_t cz) { return sphx::hash18(cx, cy, cz); }

void sphx_cell(float x, float y, float z, float h, int32_t out[3]) {
    out[0] = sphx::trunc_to_int(sphx::cell_quotient(x, h));
    out[1] = sphx::trunc_to_int(sphx::cell_quotient(y, h));
    out[2] = sphx::trunc_to_int(sphx::cell_quotient(z, h));
}

uint32_t sphx_collision_flags(int32_t cx, int32_t cy, int32_t cz, uint32_t face_mask) {
    return sphx::collision_flags(cx, cy, cz, face_mask);
}

int sphx_lattice(const sphx_lattice_desc *d, float *pos3) {
    if (!d || !pos3) return fail(SPHX_ERR_INVALID, "null argument");
    const float scale = 5.9604644775390625e-08f;  // 2^-24
    size_t idx = 0;
    for (uint32_t k = 0; k < d->nz; ++k)
        for (uint32_t j = 0; j < d->ny; ++j)
            for (uint32_t i = 0; i < d->nx; ++i, ++idx) {
                const uint32_t ijk[3] = {i, j, k};
                for (int a = 0; a < 3; ++a) {
                    const uint64_t r = mix64(d->seed + (3ull * idx + (uint64_t)a) * 0x9E3779B97F4A7C15ull);
                    const float u = (float)(r >> 40) * scale;
                    const float jit = (u * 2.0f - 1.0f) * d->jitter;
                    const float base = d->origin[a] + (float)ijk[a] * d->spacing;
                    pos3[3 * idx + a] = base + jit;
                }
            }
    return SPHX_OK;
}

int sphx_reference_scene(size_t W, float h, float *pos3) {
    if (!pos3) return fail(SPHX_ERR_INVALID, "null argument");
    std::srand(1024);  // SPHSystem.cpp:78
    const float sep = h + 0.01f;
    for (int i = 0; i < (int)W; i++)
        for (int j = 0; j < (int)W; j++)
            for (int k = 0; k < (int)W; k++) {
                const float rx = (float(std::rand()) / float(RAND_MAX) * 0.5f - 1) * h / 10;
                const float ry = (float(std::rand()) / float(RAND_MAX) * 0.5f - 1) * h / 10;
                const float rz = (float(std::rand()) / float(RAND_MAX) * 0.5f - 1) * h / 10;
                const size_t p = i + (j + W * k) * W;
                pos3[3 * p] = i * sep + rx - 1.5f;
                pos3[3 * p + 1] = j * sep + ry + h + 0.1f;
                pos3[3 * p + 2] = k * sep + rz - 1.5f;
            }
    return SPHX_OK;
}

}  // extern "C"
