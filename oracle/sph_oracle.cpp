// Test infrastructure only — the ORACLE.  Never linked into, loaded by or
// called from the product path; only tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline / reference arm use it, as the checker.
//
// A CPU restatement of lijenicol/SPH-Fluid-Simulator's per-step hot path
// (SPHSystem::update -> updateParticles -> updateParticlesCPU), written for
// this project without GLM.  Every function cites the reference file:line it
// follows.  Parity of this restatement is pinned against the reference's own
// code compiled headless (oracle/_ref/libsphref.so, see oracle/build_oracle.py)
// and against the committed fixtures in tests/golden/.
//
// Arithmetic follows the reference operand by operand (build with
// -ffp-contract=off so that no multiply-add is fused):
//   * glm::length2(d) = (dx*dx + dy*dy) + dz*dz                  (sph.cpp:57)
//   * density term: float += float * std::pow(double, 3)  -> double add,
//     then rounded to float                                       (sph.cpp:59-60)
//   * glm::normalize(d) = d * (1 / sqrt(dot(d, d)))              (sph.cpp:111)
//   * vec3 *= std::pow(float, 2): the double factor is rounded to float
//     before the multiply                                         (sph.cpp:115)
//   * cells truncate toward zero; hashes wrap in 32 bits and are stored in a
//     uint16_t                                  (neighborTable.cpp:5-17, Particle.h:9)
// The neighbour walk visits the 27 hash buckets around a particle's cell and
// accepts every bucket member with r^2 < h^2, so a bucket reached through two
// offsets is walked twice (sph.cpp:40-66); std::sort is unstable
// (sph.cpp:184-192), so within-bucket order is whatever libstdc++ produces —
// sorting (hash, index) pairs with the same comparator yields the same
// permutation as sorting the reference's 60-byte records.
//
// Extensions over the reference, each defaulting to the reference behaviour:
// per-axis box bounds, wall damping and offset (reference: x,z in [-8, 8],
// floor y = 0, no ceiling, damping 0.5, offset 1e-4; sph.cpp:139-176), an
// optional ceiling, a stable-sort switch (to measure the reference's own
// sort-order noise floor) and an FP64 evaluation of the same accepted
// neighbour sets.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr uint32_t kTableSize = 262144;    // neighborTable.h:9
constexpr uint32_t kNoParticle = 0xFFFFFFFFu;  // neighborTable.h:10
constexpr float kPi = 3.14159265f;          // SPHSystem.cpp:6

struct V3 {
    float x, y, z;
};

// Layout-identical to the reference's Particle (Particle.h:4-10): 60 bytes.
// `acc` is never used by the physics; it carries the particle id through the
// sort exactly as the reference would carry an unused field.
struct P {
    V3 pos, vel, acc, force;
    float density, pressure;
    uint16_t hash;
};
static_assert(sizeof(P) == 60, "Particle layout");

struct Settings {  // SPHSystem.h:13-22
    float poly6, spikyGrad, spikyLap, gasConstant, mass, h2, selfDens,
        restDensity, viscosity, h, g, tension, massPoly6Product;
};

struct Box {
    float xmin, xmax, ymin, ymax, zmin, zmax, damping, offset;
    int has_ceiling;
};

// SPHSystem.cpp:8-26.  pow(h, n) runs in double (float promoted), and each
// result is rounded to float on assignment.
Settings derive(const float *a) {
    Settings s;
    s.mass = a[0];
    s.restDensity = a[1];
    s.gasConstant = a[2];
    s.viscosity = a[3];
    s.h = a[4];
    s.g = a[5];
    s.tension = a[6];
    const float h = s.h;
    s.poly6 = (float)(315.0f / ((double)(64.0f * kPi) * std::pow((double)h, 9.0)));
    s.spikyGrad = (float)(-45.0f / ((double)kPi * std::pow((double)h, 6.0)));
    s.spikyLap = (float)(45.0f / ((double)kPi * std::pow((double)h, 6.0)));
    s.h2 = h * h;
    s.selfDens = (float)((double)(s.mass * s.poly6) * std::pow((double)h, 6.0));
    s.massPoly6Product = s.mass * s.poly6;
    return s;
}

// neighborTable.cpp:5-12: (uint)(c*P) products wrap modulo 2^32; the result
// modulo TABLE_SIZE is stored in a uint16_t (Particle.h:9, sph.cpp:22,43).
inline uint32_t hash18(int x, int y, int z) {
    return (((uint32_t)x * 73856093u) ^ ((uint32_t)y * 19349663u) ^
            ((uint32_t)z * 83492791u)) % kTableSize;
}
inline uint16_t hash16(int x, int y, int z) { return (uint16_t)hash18(x, y, z); }

// neighborTable.cpp:14-17: ivec3(p / h) truncates toward zero.
inline void cell_of(const V3 &p, float h, int *c) {
    c[0] = (int)(p.x / h);
    c[1] = (int)(p.y / h);
    c[2] = (int)(p.z / h);
}

inline float len2(float dx, float dy, float dz) { return dx * dx + dy * dy + dz * dz; }

uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint32_t id_of(const P &p) {
    uint32_t id;
    std::memcpy(&id, &p.acc.x, 4);
    return id;
}

// sph.cpp:17-24
void calc_hashes(P *p, size_t b, size_t e, float h) {
    for (size_t i = b; i < e; ++i) {
        int c[3];
        cell_of(p[i].pos, h, c);
        p[i].hash = hash16(c[0], c[1], c[2]);
    }
}

// sph.cpp:184-192 (std::sort, unstable).  Sorting (hash, index) pairs with
// the same comparator yields the same permutation the reference's sort of
// 60-byte records does; the records are then moved once.
void sort_particles(std::vector<P> &p, bool stable) {
    const size_t n = p.size();
    std::vector<std::pair<uint16_t, uint32_t>> k(n);
    for (size_t i = 0; i < n; ++i) k[i] = {p[i].hash, (uint32_t)i};
    auto cmp = [](const std::pair<uint16_t, uint32_t> &a,
                  const std::pair<uint16_t, uint32_t> &b) { return a.first < b.first; };
    if (stable) std::stable_sort(k.begin(), k.end(), cmp);
    else std::sort(k.begin(), k.end(), cmp);
    std::vector<P> q(n);
    for (size_t i = 0; i < n; ++i) q[i] = p[k[i].second];
    p.swap(q);
}

// neighborTable.cpp:19-37
std::vector<uint32_t> make_table(const std::vector<P> &p) {
    std::vector<uint32_t> t(kTableSize, kNoParticle);
    uint32_t prev = kNoParticle;
    for (size_t i = 0; i < p.size(); ++i) {
        const uint32_t cur = p[i].hash;
        if (cur != prev) {
            t[cur] = (uint32_t)i;
            prev = cur;
        }
    }
    return t;
}

// The 27-bucket walk of sph.cpp:40-66 / 90-127: calls f(j) for every visit of
// a bucket member j != i with r^2 < h^2 (float test, identical to the
// reference), in the reference's visiting order.
template <class F>
inline void walk(const P *p, size_t n, size_t i, const uint32_t *table,
                 const Settings &s, F &&f) {
    int c[3];
    cell_of(p[i].pos, s.h, c);
    for (int x = -1; x <= 1; x++)
        for (int y = -1; y <= 1; y++)
            for (int z = -1; z <= 1; z++) {
                const uint16_t ch = hash16(c[0] + x, c[1] + y, c[2] + z);
                uint32_t j = table[ch];
                if (j == kNoParticle) continue;
                while (j < n) {
                    if (j == i) { j++; continue; }
                    if (p[j].hash != ch) break;
                    const float d2 = len2(p[j].pos.x - p[i].pos.x,
                                          p[j].pos.y - p[i].pos.y,
                                          p[j].pos.z - p[i].pos.z);
                    if (d2 < s.h2) f(j, d2);
                    j++;
                }
            }
}

// sph.cpp:28-76
void density_pressure(P *p, size_t n, size_t b, size_t e, const uint32_t *t,
                      const Settings &s) {
    const float mp6 = s.mass * s.poly6;
    for (size_t i = b; i < e; ++i) {
        float dens = 0.f;
        walk(p, n, i, t, s, [&](uint32_t, float d2) {
            dens = (float)((double)dens +
                           (double)mp6 * std::pow((double)(s.h2 - d2), 3.0));
        });
        p[i].density = dens + s.selfDens;
        p[i].pressure = s.gasConstant * (p[i].density - s.restDensity);
    }
}

// sph.cpp:80-129
void forces(P *p, size_t n, size_t b, size_t e, const uint32_t *t,
            const Settings &s) {
    for (size_t i = b; i < e; ++i) {
        V3 F = {0.f, 0.f, 0.f};
        const P &pi = p[i];
        walk(p, n, i, t, s, [&](uint32_t j, float d2) {
            const P &pj = p[j];
            const float dist = std::sqrt(d2);
            const float dx = pj.pos.x - pi.pos.x, dy = pj.pos.y - pi.pos.y,
                        dz = pj.pos.z - pi.pos.z;
            const float inv = 1.f / std::sqrt(len2(dx, dy, dz));
            const float nx = dx * inv, ny = dy * inv, nz = dz * inv;
            const float psum = pi.pressure + pj.pressure;
            const float twoRho = 2.f * pj.density;
            float px = (((-nx) * s.mass) * psum) / twoRho * s.spikyGrad;
            float py = (((-ny) * s.mass) * psum) / twoRho * s.spikyGrad;
            float pz = (((-nz) * s.mass) * psum) / twoRho * s.spikyGrad;
            const float sq = (float)std::pow((double)(s.h - dist), 2.0);
            px = px * sq; py = py * sq; pz = pz * sq;
            F.x = F.x + px; F.y = F.y + py; F.z = F.z + pz;
            const float mm = s.viscosity * s.mass;
            const float hd = s.h - dist;
            const float vx = ((mm * ((pj.vel.x - pi.vel.x) / pj.density)) * s.spikyLap) * hd;
            const float vy = ((mm * ((pj.vel.y - pi.vel.y) / pj.density)) * s.spikyLap) * hd;
            const float vz = ((mm * ((pj.vel.z - pi.vel.z) / pj.density)) * s.spikyLap) * hd;
            F.x = F.x + vx; F.y = F.y + vy; F.z = F.z + vz;
        });
        p[i].force = F;
    }
}

// sph.cpp:133-181, generalised to per-axis bounds.  At the reference preset
// (xmin = zmin = -8, xmax = zmax = 8, ymin = 0, no ceiling) every bound
// expression evaluates to the same float as the reference's:
// h - 8 == h + (-8) and -(h - 8) == 8 - h exactly.
void integrate(P *p, size_t b, size_t e, float *tr, const Settings &s,
               const Box &bx, float dt) {
    const float sc = s.h / 2.f;
    const float ylo = bx.ymin + s.h, xlo = s.h + bx.xmin, xhi = bx.xmax - s.h;
    const float zlo = s.h + bx.zmin, zhi = bx.zmax - s.h, yhi = bx.ymax - s.h;
    for (size_t i = b; i < e; ++i) {
        P &q = p[i];
        const float ax = q.force.x / q.density + 0.f;
        const float ay = q.force.y / q.density + s.g;
        const float az = q.force.z / q.density + 0.f;
        q.vel.x = q.vel.x + ax * dt;
        q.vel.y = q.vel.y + ay * dt;
        q.vel.z = q.vel.z + az * dt;
        q.pos.x = q.pos.x + q.vel.x * dt;
        q.pos.y = q.pos.y + q.vel.y * dt;
        q.pos.z = q.pos.z + q.vel.z * dt;
        if (q.pos.y < ylo) {
            q.pos.y = -q.pos.y + 2 * ylo + bx.offset;
            q.vel.y = -q.vel.y * bx.damping;
        }
        if (bx.has_ceiling && q.pos.y > yhi) {
            q.pos.y = -q.pos.y + 2 * yhi - bx.offset;
            q.vel.y = -q.vel.y * bx.damping;
        }
        if (q.pos.x < xlo) {
            q.pos.x = -q.pos.x + 2 * xlo + bx.offset;
            q.vel.x = -q.vel.x * bx.damping;
        }
        if (q.pos.x > xhi) {
            q.pos.x = -q.pos.x + 2 * xhi - bx.offset;
            q.vel.x = -q.vel.x * bx.damping;
        }
        if (q.pos.z < zlo) {
            q.pos.z = -q.pos.z + 2 * zlo + bx.offset;
            q.vel.z = -q.vel.z * bx.damping;
        }
        if (q.pos.z > zhi) {
            q.pos.z = -q.pos.z + 2 * zhi - bx.offset;
            q.vel.z = -q.vel.z * bx.damping;
        }
        if (tr) {  // translate(position) * scale(h/2), column-major
            float *m = tr + 16 * i;
            for (int k = 0; k < 16; ++k) m[k] = 0.f;
            m[0] = sc; m[5] = sc; m[10] = sc;
            m[12] = q.pos.x + 0.f; m[13] = q.pos.y + 0.f; m[14] = q.pos.z + 0.f;
            m[15] = 1.f;
        }
    }
}

template <class Fn>
void parallel(size_t n, int threads, Fn &&fn) {
    // sph.cpp:200-209: equal blocks, the last one takes the remainder.
    if (threads <= 1) { fn(0, n); return; }
    std::vector<size_t> bnd(threads + 1);
    const size_t bs = n / threads;
    for (int i = 0; i < threads; ++i) bnd[i] = i * bs;
    bnd[threads] = n;
    std::vector<std::thread> th;
    th.reserve(threads);
    for (int i = 0; i < threads; ++i) th.emplace_back(fn, bnd[i], bnd[i + 1]);
    for (auto &t : th) t.join();
}

int resolve_threads(int t) {
    if (t > 0) return t;
    const unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

Box box_from(const float *b) {
    Box bx;
    if (!b) {  // the reference's hard-coded box (sph.cpp:139-140)
        bx = {-8.f, 8.f, 0.f, 0.f, -8.f, 8.f, 0.5f, 0.0001f, 0};
        return bx;
    }
    bx = {b[0], b[1], b[2], b[3], b[4], b[5], b[6], b[7], b[8] != 0.f};
    return bx;
}

// One reference step (sph.cpp:195-275) on a persistent AoS array.
void step(std::vector<P> &p, const Settings &s, const Box &bx, float dt,
          int threads, bool stable, float *tr) {
    const size_t n = p.size();
    P *d = p.data();
    parallel(n, threads, [&](size_t b, size_t e) { calc_hashes(d, b, e, s.h); });
    sort_particles(p, stable);
    d = p.data();
    std::vector<uint32_t> t = make_table(p);
    parallel(n, threads, [&](size_t b, size_t e) { density_pressure(d, n, b, e, t.data(), s); });
    parallel(n, threads, [&](size_t b, size_t e) { forces(d, n, b, e, t.data(), s); });
    parallel(n, threads, [&](size_t b, size_t e) { integrate(d, b, e, tr, s, bx, dt); });
}

void load(std::vector<P> &p, size_t n, const float *pos, const float *vel) {
    p.assign(n, P{});
    for (size_t i = 0; i < n; ++i) {
        std::memset(&p[i], 0, sizeof(P));
        p[i].pos = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
        if (vel) p[i].vel = {vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]};
        const uint32_t id = (uint32_t)i;
        std::memcpy(&p[i].acc.x, &id, 4);
    }
}

}  // namespace

extern "C" {

int orc_sizeof_particle(void) { return (int)sizeof(P); }
int orc_hw_threads(void) { return resolve_threads(0); }
uint32_t orc_hash18(int x, int y, int z) { return hash18(x, y, z); }
uint32_t orc_hash16(int x, int y, int z) { return hash16(x, y, z); }

void orc_cell(float x, float y, float z, float h, int *out) {
    V3 p = {x, y, z};
    cell_of(p, h, out);
}

// Same output layout as ref_settings (13 constants + 16 of sphereScale).
void orc_settings(const float *args, float *out) {
    Settings s = derive(args);
    std::memcpy(out, &s, 13 * sizeof(float));
    for (int k = 0; k < 16; ++k) out[13 + k] = 0.f;
    const float sc = s.h / 2.f;
    out[13] = sc; out[18] = sc; out[23] = sc; out[28] = 1.f;
}

// Reference scene of SPHSystem::initParticles (SPHSystem.cpp:76-108):
// srand(1024), lattice spacing h + 0.01, one-sided jitter, index
// i + (j + W*k)*W.  Writes 3*W^3 floats.
void orc_reference_scene(size_t W, float h, float *pos) {
    std::srand(1024);
    const float sep = h + 0.01f;
    for (int i = 0; i < (int)W; i++)
        for (int j = 0; j < (int)W; j++)
            for (int k = 0; k < (int)W; k++) {
                const float rx = (float(std::rand()) / float(RAND_MAX) * 0.5f - 1) * h / 10;
                const float ry = (float(std::rand()) / float(RAND_MAX) * 0.5f - 1) * h / 10;
                const float rz = (float(std::rand()) / float(RAND_MAX) * 0.5f - 1) * h / 10;
                const size_t idx = i + (j + W * k) * W;
                pos[3 * idx] = i * sep + rx - 1.5f;
                pos[3 * idx + 1] = j * sep + ry + h + 0.1f;
                pos[3 * idx + 2] = k * sep + rz - 1.5f;
            }
}

// One step, same outputs as ref_update_cpu.  box: 9 floats
// (xmin, xmax, ymin, ymax, zmin, zmax, damping, offset, has_ceiling) or NULL
// for the reference box.  stable != 0 swaps std::sort for std::stable_sort.
int orc_step(size_t n, const float *pos, const float *vel, const float *args,
             const float *box, float dt, int threads, int stable, uint32_t *ids,
             float *pos_out, float *vel_out, float *rho, float *prs,
             float *force, uint16_t *hash, float *transforms) {
    std::vector<P> p;
    load(p, n, pos, vel);
    const Settings s = derive(args);
    step(p, s, box_from(box), dt, resolve_threads(threads), stable != 0, transforms);
    for (size_t k = 0; k < n; ++k) {
        const P &q = p[k];
        if (ids) ids[k] = id_of(q);
        if (pos_out) { pos_out[3 * k] = q.pos.x; pos_out[3 * k + 1] = q.pos.y; pos_out[3 * k + 2] = q.pos.z; }
        if (vel_out) { vel_out[3 * k] = q.vel.x; vel_out[3 * k + 1] = q.vel.y; vel_out[3 * k + 2] = q.vel.z; }
        if (rho) rho[k] = q.density;
        if (prs) prs[k] = q.pressure;
        if (force) { force[3 * k] = q.force.x; force[3 * k + 1] = q.force.y; force[3 * k + 2] = q.force.z; }
        if (hash) hash[k] = q.hash;
    }
    return 0;
}

// nsteps reference steps on a persistent state; outputs are written in id
// order (input index), so that rollouts can be compared by identity.
int orc_run(size_t n, const float *pos, const float *vel, const float *args,
            const float *box, float dt, int nsteps, int threads, float *pos_out,
            float *vel_out, float *rho, float *prs) {
    std::vector<P> p;
    load(p, n, pos, vel);
    const Settings s = derive(args);
    const Box bx = box_from(box);
    const int th = resolve_threads(threads);
    for (int k = 0; k < nsteps; ++k) step(p, s, bx, dt, th, false, nullptr);
    for (size_t k = 0; k < n; ++k) {
        const P &q = p[k];
        const uint32_t id = id_of(q);
        if (pos_out) { pos_out[3 * id] = q.pos.x; pos_out[3 * id + 1] = q.pos.y; pos_out[3 * id + 2] = q.pos.z; }
        if (vel_out) { vel_out[3 * id] = q.vel.x; vel_out[3 * id + 1] = q.vel.y; vel_out[3 * id + 2] = q.vel.z; }
        if (rho) rho[id] = q.density;
        if (prs) prs[id] = q.pressure;
    }
    return 0;
}

// Accepted-neighbour fingerprint per input particle (see ref_neighbor_digest
// in oracle/ref_harness.cpp): visit count and wrapping sum of mix64(id).
int orc_neighbor_digest(size_t n, const float *pos, float h, uint32_t *count,
                        uint64_t *digest) {
    std::vector<P> p;
    load(p, n, pos, nullptr);
    float args[7] = {1.f, 1.f, 1.f, 1.f, h, 0.f, 0.f};
    const Settings s = derive(args);
    calc_hashes(p.data(), 0, n, h);
    sort_particles(p, false);
    std::vector<uint32_t> t = make_table(p);
    for (size_t i = 0; i < n; ++i) {
        uint32_t c = 0;
        uint64_t d = 0;
        walk(p.data(), n, i, t.data(), s, [&](uint32_t j, float) {
            c++;
            d += mix64(id_of(p[j]));
        });
        const uint32_t id = id_of(p[i]);
        count[id] = c;
        digest[id] = d;
    }
    return 0;
}

// FP64 evaluation of density, pressure and force over exactly the accepted
// neighbour visits of the FP32 reference walk (same cells, hashes, float
// r^2 < h^2 test), with positions, velocities and constants widened to
// double.  Outputs by input index.
int orc_fields_f64(size_t n, const float *pos, const float *vel,
                   const float *args, double *rho, double *prs, double *force) {
    std::vector<P> p;
    load(p, n, pos, vel);
    const Settings s = derive(args);
    calc_hashes(p.data(), 0, n, s.h);
    sort_particles(p, false);
    std::vector<uint32_t> t = make_table(p);
    std::vector<double> R(n), Pr(n);
    const double mp6 = (double)s.mass * (double)s.poly6, h = s.h, h2 = (double)s.h * (double)s.h;
    const int th = resolve_threads(0);
    parallel(n, th, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            double d = 0.0;
            walk(p.data(), n, i, t.data(), s, [&](uint32_t j, float) {
                const double dx = (double)p[j].pos.x - p[i].pos.x;
                const double dy = (double)p[j].pos.y - p[i].pos.y;
                const double dz = (double)p[j].pos.z - p[i].pos.z;
                const double u = h2 - (dx * dx + dy * dy + dz * dz);
                d += mp6 * u * u * u;
            });
            R[i] = d + (double)s.mass * (double)s.poly6 * std::pow(h, 6.0);
            Pr[i] = (double)s.gasConstant * (R[i] - (double)s.restDensity);
        }
    });
    parallel(n, th, [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            double F[3] = {0, 0, 0};
            walk(p.data(), n, i, t.data(), s, [&](uint32_t j, float) {
                const double d[3] = {(double)p[j].pos.x - p[i].pos.x,
                                     (double)p[j].pos.y - p[i].pos.y,
                                     (double)p[j].pos.z - p[i].pos.z};
                const double r = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
                const double vi[3] = {p[i].vel.x, p[i].vel.y, p[i].vel.z};
                const double vj[3] = {p[j].vel.x, p[j].vel.y, p[j].vel.z};
                const double pf = -(double)s.mass * (Pr[i] + Pr[j]) / (2.0 * R[j]) *
                                  (double)s.spikyGrad * (h - r) * (h - r) / r;
                const double vf = (double)s.viscosity * (double)s.mass *
                                  (double)s.spikyLap * (h - r) / R[j];
                for (int a = 0; a < 3; ++a) F[a] += pf * d[a] + vf * (vj[a] - vi[a]);
            });
            const uint32_t id = id_of(p[i]);
            force[3 * id] = F[0]; force[3 * id + 1] = F[1]; force[3 * id + 2] = F[2];
        }
    });
    for (size_t i = 0; i < n; ++i) {
        const uint32_t id = id_of(p[i]);
        rho[id] = R[i];
        prs[id] = Pr[i];
    }
    return 0;
}

}  // extern "C"
