// Shared host/device definitions of the SPH step: the reference's integer
// cell hash, the cell function, the settings-derived constants, and the
// GF(2) test that decides when the fast cell walk is exact.
//
// Reference semantics being reproduced (lijenicol/SPH-Fluid-Simulator):
//   * getCell = ivec3(p / h), truncation toward zero     neighborTable.cpp:14-17
//   * getHash = ((uint)(x*73856093) ^ (uint)(y*19349663) ^ (uint)(z*83492791))
//               % 262144, stored in a uint16_t            neighborTable.cpp:5-12,
//                                                          Particle.h:9, sph.cpp:43
//   * a particle's neighbour candidates are all members of the 27 buckets
//     hash16(cell + o), o in {-1,0,1}^3, visited once per offset, accepted
//     when |pj - pi|^2 < h^2 in float                     sph.cpp:40-66, 90-127
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define SPHX_HD __host__ __device__ __forceinline__
#else
#define SPHX_HD inline
#endif

namespace sphx {

constexpr uint32_t kTableSize = 262144u;  // neighborTable.h:9
constexpr uint32_t kHashP1 = 73856093u;   // neighborTable.cpp:8-10
constexpr uint32_t kHashP2 = 19349663u;
constexpr uint32_t kHashP3 = 83492791u;

// Flag bits of a particle's cell (see collision_flags).
constexpr uint32_t kFlagDup = 1u;          // two of the 27 neighbour cells share a bucket
constexpr uint32_t kFlagFaceShift = 1u;    // bits 1..6: face (-x,+x,-y,+y,-z,+z)
constexpr uint32_t kFlagNearShift = 8u;    // bits 8..13: particle within slack of that face

// The hash the reference stores per particle: the low 16 bits of the xor of
// three wrapped 32-bit products (% 262144 then uint16 truncation keeps the
// low 16 bits).
SPHX_HD uint32_t hash18(int x, int y, int z) {
    return (((uint32_t)x * kHashP1) ^ ((uint32_t)y * kHashP2) ^ ((uint32_t)z * kHashP3)) &
           (kTableSize - 1u);
}
SPHX_HD uint32_t hash16(int x, int y, int z) { return hash18(x, y, z) & 0xFFFFu; }

// ivec3(p / h): IEEE division, then truncation toward zero.
SPHX_HD float cell_quotient(float x, float h) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(x, h);
#else
    return x / h;
#endif
}
SPHX_HD int trunc_to_int(float q) {
#if defined(__CUDA_ARCH__)
    return __float2int_rz(q);
#else
    return (int)q;
#endif
}

#if defined(__CUDA_ARCH__)
#define SPHX_UNROLL _Pragma("unroll")
#else
#define SPHX_UNROLL
#endif

// xor-basis insertion ("x = min(x, x ^ b)" over the basis in insertion order
// keeps every element reduced at the leading bits of the earlier ones).  The
// basis has a fixed slot per inserted vector, 0 for one that reduced to 0:
// x ^ 0 = x, so such a slot changes no later reduction, and with constant
// indexes the basis stays in registers.
template <int kN>
SPHX_HD uint32_t reduce_basis(uint32_t x, const uint32_t *b) {
    SPHX_UNROLL
    for (int k = 0; k < kN; ++k) {
        const uint32_t y = x ^ b[k];
        x = y < x ? y : x;
    }
    return x;
}

// Whether one of the nine cells two steps across face `face` (-x, +x, -y,
// +y, -z, +z) has the bucket of one of the 27 cells around the centre; A, B,
// C hold the low 16 bits of the axis products at offsets -2..2.  In the
// face's frame (u across it, v and w along it, as the slow walk steps them)
// a bucket is the xor of three axis terms.
SPHX_HD bool face_collides(const uint32_t *A, const uint32_t *B, const uint32_t *C, int face) {
    const int axis = face >> 1, far = (face & 1) ? 4 : 0;
    const uint32_t *P[3] = {A, B, C};
    const uint32_t *U = P[axis], *V = P[(axis + 1) % 3], *W = P[(axis + 2) % 3];
    for (int v = 1; v <= 3; ++v)
        for (int w = 1; w <= 3; ++w) {
            const uint32_t hf = U[far] ^ V[v] ^ W[w];
            for (int u = 1; u <= 3; ++u)
                for (int v2 = 1; v2 <= 3; ++v2)
                    for (int w2 = 1; w2 <= 3; ++w2)
                        if ((U[u] ^ V[v2] ^ W[w2]) == hf) return true;
        }
    return false;
}

// Bucket-collision structure of the 27 cells around (cx, cy, cz).
//
// With A[k] = low16((cx+k)*P1), B[k], C[k] likewise, hash16(cell+o) =
// A[ox] ^ B[oy] ^ C[oz].  Two distinct offsets share a bucket iff a non-zero
// combination of a1 = A[-1]^A[0], a2 = A[0]^A[1], b1, b2, c1, c2 xors to zero,
// i.e. iff those six 16-bit vectors are linearly dependent over GF(2); then
// kFlagDup is set and the reference visits some bucket twice.
//
// A cell two steps away across the +x face, (cx+2, cy+dy, cz+dz), can share
// a bucket with one of the 27 only if A[1]^A[2] lies in the span of the six
// vectors (necessary, not sufficient); likewise for the other five faces.
// Only then are the nine cells of that face compared with the 27 buckets,
// and the face bit is set iff one of them matches: exact, like kFlagDup.
SPHX_HD uint32_t collision_flags(int cx, int cy, int cz, uint32_t face_mask) {
    uint32_t A[5], B[5], C[5];
    for (int k = 0; k < 5; ++k) {
        A[k] = ((uint32_t)(cx + k - 2) * kHashP1) & 0xFFFFu;
        B[k] = ((uint32_t)(cy + k - 2) * kHashP2) & 0xFFFFu;
        C[k] = ((uint32_t)(cz + k - 2) * kHashP3) & 0xFFFFu;
    }
    const uint32_t v[6] = {A[1] ^ A[2], A[2] ^ A[3], B[1] ^ B[2],
                           B[2] ^ B[3], C[1] ^ C[2], C[2] ^ C[3]};
    uint32_t basis[6];
    basis[0] = v[0];
    basis[1] = reduce_basis<1>(v[1], basis);
    basis[2] = reduce_basis<2>(v[2], basis);
    basis[3] = reduce_basis<3>(v[3], basis);
    basis[4] = reduce_basis<4>(v[4], basis);
    basis[5] = reduce_basis<5>(v[5], basis);
    uint32_t flags = (basis[0] && basis[1] && basis[2] && basis[3] && basis[4] && basis[5]) ? 0u : kFlagDup;
    const uint32_t f[6] = {A[0] ^ A[1], A[3] ^ A[4], B[0] ^ B[1],
                           B[3] ^ B[4], C[0] ^ C[1], C[3] ^ C[4]};
    // the span test first: it rules out almost every face at once
    SPHX_UNROLL
    for (int i = 0; i < 6; ++i)
        if ((face_mask >> i) & 1u)
            if (reduce_basis<6>(f[i], basis) == 0u && face_collides(A, B, C, i))
                flags |= 1u << (kFlagFaceShift + i);
    return flags;
}

// Whether a particle at quotient q (= x / h) in cell c = trunc(q) could be
// within h, allowing for float rounding, of a particle in cell c - 2 (bit 0)
// or c + 2 (bit 1).  Cell m covers [m, m+1) for m > 0, (m-1, m] for m < 0 and
// (-1, 1) for m = 0 (truncation toward zero).  A particle of cell c+2 has a
// quotient above (c+2 > 0 ? c+2 : c+1), so it can only be within one cell
// width of q when q > (c+2 > 0 ? c+1 : c); symmetrically for c-2.  eps is
// about 16x the worst-case rounding slack of the division and r^2 test.
SPHX_HD uint32_t near_faces_1d(float q, int c) {
    const float aq = q < 0.f ? -q : q;
    const float eps = (aq + 8.0f) * 9.5367431640625e-07f;  // 2^-20
    const float up = (float)((c + 2 > 0) ? c + 1 : c);
    const float lo = (float)((c - 2 >= 0) ? c : c - 1);
    return (q < lo + eps ? 1u : 0u) | (q > up - eps ? 2u : 0u);
}

// Constants of SPHSettings (SPHSystem.h:19-21), in the reference's order.
struct Derived {
    float poly6, spikyGrad, spikyLap, gasConstant, mass, h2, selfDens,
        restDensity, viscosity, h, g, tension, massPoly6Product;
};

// SPHSystem.cpp:8-26.  pow(h, n) of a float runs in double; each result is
// rounded to float on assignment; PI is the float literal 3.14159265f.
Derived derive_constants(float mass, float restDensity, float gasConst,
                         float viscosity, float h, float g, float tension);

// Uniform cell grid that particle keys are taken modulo.  Cell (cx, cy, cz)
// maps to slot ((cz-oz) mod gz, (cy-oy) mod gy, (cx-ox) mod gx); cells that
// share a slot are at least gx-1 (gy-1, gz-1) cells apart, so with every
// dimension >= 5 no particle of an aliased cell can pass the r^2 < h^2 test:
// aliasing costs time, never exactness.
struct Grid {
    int ox, oy, oz;
    int gx, gy, gz;
};

SPHX_HD int wrap_mod(int a, int m) {
    int r = a % m;
    return r < 0 ? r + m : r;
}

// Everything one step's kernels read, passed by value.
struct StepParams {
    // physics (SPHSettings)
    float h, h2, mp6, selfDens, gasConstant, restDensity, mass, viscosity;
    float spikyGrad, spikyLap, g, halfH;
    float forceKp;  // mass * spikyGrad / 2
    float forceKv;  // viscosity * mass * spikyLap
    // walls (sph.cpp:153-176 generalised): reflect below ylo / above yhi ...
    float ylo, yhi, xlo, xhi, zlo, zhi, damping, offset;
    int hasCeiling;
    float dt;
    float h2w;  // h^2 (1 + 2^-18): squared half-width bound of the walk's row windows
    Grid grid;
    uint32_t n;
};

// Device-side description of the scenes one launch covers: scene s owns
// particles [pofs[s], pofs[s+1]) and cell-grid slots [sofs[s], sofs[s+1]) of
// the concatenated buffers, with constants params[s].  A single scene is a
// table of one.  Particles stay inside their scene's range through every
// sort, because the scenes' slot ranges are disjoint and ordered.
struct SceneTable {
    const StepParams *params;
    const uint32_t *pofs;
    const uint32_t *sofs;
    uint32_t nscenes;
    uint32_t n;  // total particles
    // nscenes + 1 offsets of each scene's first cell row (gy * gz rows of gx
    // slots each); NULL where rows are not used
    const uint32_t *rofs = nullptr;
    uint32_t rows = 0;  // cell rows of all scenes
};

}  // namespace sphx
