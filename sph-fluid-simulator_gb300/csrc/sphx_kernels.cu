// sm_103a kernels of the SPH step (hand-written CUDA, FP32 physics, exact
// integer cell/hash work).  One step is:
//
//   k_keys        cell of every particle -> slot key in a modular cell grid,
//                 per-slot counts (atomics) and each particle's arrival rank
//   k_scan_*      exclusive prefix sum of the counts -> cellStart[slot]
//   k_scatter     order[cellStart[key] + rank] = particle
//   k_cellsort    within each cell run, ascending particle index, so that the
//                 order (and hence every float sum) is deterministic
//   k_gather      every R steps: permute pos/vel/id into cell order
//   k_density     poly6 density and pressure            (sph.cpp:28-76)
//   k_force       spiky pressure + viscosity force, then integration and
//                 damped wall reflection                 (sph.cpp:80-181)
//
// The neighbour walk visits the 27 cells around a particle's cell through the
// grid (x-adjacent cells are adjacent slots, so each of the 9 (dy, dz) rows is
// one contiguous run of cell-sorted particles).  The reference walks hash
// buckets instead (sph.cpp:40-66); its accepted multiset equals this one
// except where buckets collide, which collision_flags detects exactly and the
// slow path reproduces (bucket visited twice -> neighbours counted twice; a
// cell two away that shares a visited bucket -> its particles tested too).
#include <cuda_runtime.h>
#include <stdint.h>

#include "sphx_common.h"
#include "sphx_kernels.h"

namespace sphx {
namespace {

__device__ __forceinline__ uint32_t slot_of(const Grid &g, int cx, int cy, int cz, int &mx,
                                            int &my, int &mz) {
    mx = wrap_mod(cx - g.ox, g.gx);
    my = wrap_mod(cy - g.oy, g.gy);
    mz = wrap_mod(cz - g.oz, g.gz);
    return ((uint32_t)mz * (uint32_t)g.gy + (uint32_t)my) * (uint32_t)g.gx + (uint32_t)mx;
}

struct CellPos {
    float qx, qy, qz;
    int cx, cy, cz;
};

__device__ __forceinline__ CellPos cell_pos(float4 p, float h) {
    CellPos c;
    c.qx = cell_quotient(p.x, h);
    c.qy = cell_quotient(p.y, h);
    c.qz = cell_quotient(p.z, h);
    c.cx = trunc_to_int(c.qx);
    c.cy = trunc_to_int(c.qy);
    c.cz = trunc_to_int(c.qz);
    return c;
}

__device__ __forceinline__ bool in_domain(float q) { return fabsf(q) < 1073741824.0f; }

// ---------------------------------------------------------------- keys / sort

__global__ void k_keys(StepParams P, const float4 *__restrict__ pos, uint32_t *__restrict__ key,
                       uint32_t *__restrict__ rank, uint32_t *__restrict__ count,
                       uint32_t *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const CellPos c = cell_pos(pos[i], P.h);
    uint32_t k = 0;
    if (in_domain(c.qx) && in_domain(c.qy) && in_domain(c.qz)) {
        int mx, my, mz;
        k = slot_of(P.grid, c.cx, c.cy, c.cz, mx, my, mz);
    } else {
        atomicOr(status, kStatusDomainBit);
    }
    key[i] = k;
    rank[i] = atomicAdd(&count[k], 1u);
}

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr uint32_t kScanTile = kScanThreads * kScanItems;

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t &excl) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t block_tot;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, d);
        if (lane >= d) inc += t;
    }
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t w = lane < nw ? warp_tot[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += t;
        }
        if (lane < nw) warp_tot[lane] = wi - w;  // exclusive warp offsets
        if (lane == nw - 1) block_tot = wi;
    }
    __syncthreads();
    excl = warp_tot[warp] + inc - v;
    const uint32_t total = block_tot;
    __syncthreads();
    return total;
}

__global__ void k_scan_tiles(const uint32_t *__restrict__ count, uint32_t m,
                             uint32_t *__restrict__ tile_sum, uint32_t max_cell,
                             uint32_t *__restrict__ status) {
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t s = 0, mx = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint32_t v = base + k < m ? count[base + k] : 0u;
        s += v;
        mx = max(mx, v);
    }
    if (mx > max_cell) atomicOr(status, kStatusOverflowBit);
    uint32_t excl;
    const uint32_t tot = block_exclusive_scan(s, excl);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

// Single block: exclusive scan of the tile sums in place.
__global__ void k_scan_tile_sums(uint32_t *__restrict__ tile_sum, uint32_t ntiles) {
    uint32_t carry = 0;
    for (uint32_t base = 0; base < ntiles; base += kScanTile) {
        uint32_t v[kScanItems];
        uint32_t s = 0;
        const uint32_t b = base + threadIdx.x * kScanItems;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            v[k] = b + k < ntiles ? tile_sum[b + k] : 0u;
            s += v[k];
        }
        uint32_t excl;
        const uint32_t tot = block_exclusive_scan(s, excl);
        uint32_t run = carry + excl;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            if (b + k < ntiles) tile_sum[b + k] = run;
            run += v[k];
        }
        carry += tot;
    }
}

// cellStart[i] = exclusive prefix of count[i]; count is cleared for the next
// step in the same pass.
__global__ void k_scan_apply(uint32_t *__restrict__ count, uint32_t m,
                             const uint32_t *__restrict__ tile_prefix,
                             uint32_t *__restrict__ start) {
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < m ? count[base + k] : 0u;
        s += v[k];
    }
    uint32_t excl;
    block_exclusive_scan(s, excl);
    uint32_t run = tile_prefix[blockIdx.x] + excl;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < m) {
            start[base + k] = run;
            count[base + k] = 0u;
        }
        run += v[k];
    }
}

__global__ void k_scatter(uint32_t n, const uint32_t *__restrict__ key,
                          const uint32_t *__restrict__ rank, const uint32_t *__restrict__ start,
                          uint32_t *__restrict__ order, const uint32_t *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (*status & kStatusOverflowBit)) return;
    order[start[key[i]] + rank[i]] = i;
}

// The particle that arrived first in a cell sorts the cell's run ascending.
__global__ void k_cellsort(uint32_t n, const uint32_t *__restrict__ key,
                           const uint32_t *__restrict__ rank, const uint32_t *__restrict__ start,
                           uint32_t *__restrict__ order, const uint32_t *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || rank[i] != 0u || (*status & kStatusOverflowBit)) return;
    const uint32_t k = key[i];
    const uint32_t a = start[k], b = start[k + 1];
    for (uint32_t x = a + 1; x < b; ++x) {
        const uint32_t v = order[x];
        uint32_t y = x;
        while (y > a && order[y - 1] > v) {
            order[y] = order[y - 1];
            --y;
        }
        order[y] = v;
    }
}

__global__ void k_gather(uint32_t n, const uint32_t *__restrict__ order,
                         const float4 *__restrict__ pos_in, const float4 *__restrict__ vel_in,
                         const uint32_t *__restrict__ id_in, float4 *__restrict__ pos_out,
                         float4 *__restrict__ vel_out, uint32_t *__restrict__ id_out,
                         const uint32_t *__restrict__ status) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n || (*status & kStatusOverflowBit)) return;
    const uint32_t s = order[t];
    pos_out[t] = pos_in[s];
    vel_out[t] = vel_in[s];
    id_out[t] = id_in[s];
}

// ---------------------------------------------------------------- walks

struct WalkCtx {
    const float4 *__restrict__ pos;
    const uint32_t *__restrict__ order;
    const uint32_t *__restrict__ start;
    Grid grid;
    float h2;
};

// One run of cell-sorted slots [a, b): every particle j != self with
// |pj - pi|^2 < h^2 (reference's float r^2, sph.cpp:57: (dx*dx + dy*dy) + dz*dz,
// no fused multiply-add) is passed to the visitor `w` times.
template <bool kInd, class V>
__device__ __forceinline__ void scan_run(const WalkCtx &W, uint32_t a, uint32_t b, uint32_t self,
                                         float4 pi, uint32_t w, V &vis) {
    for (uint32_t t = a; t < b; ++t) {
        const uint32_t j = kInd ? W.order[t] : t;
        if (j == self) continue;
        const float4 pj = W.pos[j];
        const float dx = __fsub_rn(pj.x, pi.x);
        const float dy = __fsub_rn(pj.y, pi.y);
        const float dz = __fsub_rn(pj.z, pi.z);
        const float d2 =
            __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
        if (d2 < W.h2)
            for (uint32_t r = 0; r < w; ++r) vis(j, dx, dy, dz, d2);
    }
}

__device__ __forceinline__ int wrap1(int v, int m) {
    v = v < 0 ? v + m : v;
    return v >= m ? v - m : v;
}

// Fast path: the 27 cells around (mx, my, mz), each visited once.
template <bool kInd, class V>
__device__ __forceinline__ void walk_rows(const WalkCtx &W, int mx, int my, int mz, uint32_t self,
                                          float4 pi, V &vis) {
    const Grid &g = W.grid;
    const bool contiguous = mx >= 1 && mx + 1 < g.gx;
#pragma unroll 1
    for (int dz = -1; dz <= 1; ++dz) {
        const int z = wrap1(mz + dz, g.gz);
#pragma unroll 1
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = wrap1(my + dy, g.gy);
            const uint32_t base = ((uint32_t)z * (uint32_t)g.gy + (uint32_t)y) * (uint32_t)g.gx;
            if (contiguous) {
                scan_run<kInd>(W, W.start[base + mx - 1], W.start[base + mx + 2], self, pi, 1u,
                               vis);
            } else {
                for (int dx = -1; dx <= 1; ++dx) {
                    const uint32_t k = base + (uint32_t)wrap1(mx + dx, g.gx);
                    scan_run<kInd>(W, W.start[k], W.start[k + 1], self, pi, 1u, vis);
                }
            }
        }
    }
}

template <bool kInd, class V>
__device__ __forceinline__ void walk_cell(const WalkCtx &W, int cx, int cy, int cz, uint32_t self,
                                          float4 pi, uint32_t w, V &vis) {
    int mx, my, mz;
    const uint32_t k = slot_of(W.grid, cx, cy, cz, mx, my, mz);
    scan_run<kInd>(W, W.start[k], W.start[k + 1], self, pi, w, vis);
}

// Slow path, taken when `flags` reports a bucket collision: every neighbour
// cell is walked with weight = number of the 27 offsets whose bucket equals
// its bucket (the reference walks a bucket once per offset that hashes to it,
// sph.cpp:40-63), and, for each flagged face, the nine cells two steps away
// whose bucket is among the 27 are walked with that same weight.
template <bool kInd, class V>
__device__ __noinline__ void walk_slow(const WalkCtx &W, int cx, int cy, int cz, uint32_t flags,
                                       uint32_t self, float4 pi, V &vis) {
    uint32_t H[27];
    int o = 0;
    for (int x = -1; x <= 1; ++x)
        for (int y = -1; y <= 1; ++y)
            for (int z = -1; z <= 1; ++z) H[o++] = hash16(cx + x, cy + y, cz + z);
    o = 0;
    for (int x = -1; x <= 1; ++x)
        for (int y = -1; y <= 1; ++y)
            for (int z = -1; z <= 1; ++z) {
                uint32_t w = 0;
                for (int k = 0; k < 27; ++k) w += H[k] == H[o] ? 1u : 0u;
                walk_cell<kInd>(W, cx + x, cy + y, cz + z, self, pi, w, vis);
                ++o;
            }
    for (int f = 0; f < 6; ++f) {
        if (!((flags >> (kFlagFaceShift + f)) & 1u)) continue;
        const int axis = f >> 1, step = (f & 1) ? 2 : -2;
        for (int a = -1; a <= 1; ++a)
            for (int b = -1; b <= 1; ++b) {
                int c[3] = {cx, cy, cz};
                c[axis] += step;
                c[(axis + 1) % 3] += a;
                c[(axis + 2) % 3] += b;
                const uint32_t hf = hash16(c[0], c[1], c[2]);
                uint32_t w = 0;
                for (int k = 0; k < 27; ++k) w += H[k] == hf ? 1u : 0u;
                if (w) walk_cell<kInd>(W, c[0], c[1], c[2], self, pi, w, vis);
            }
    }
}

// Cell, slot and collision flags of a particle; returns true when the fast
// 27-cell walk is exact for it.
struct WalkStart {
    CellPos c;
    int mx, my, mz;
    uint32_t flags;
};

__device__ __forceinline__ bool walk_start(const StepParams &P, float4 pi, WalkStart &s) {
    s.c = cell_pos(pi, P.h);
    slot_of(P.grid, s.c.cx, s.c.cy, s.c.cz, s.mx, s.my, s.mz);
    const uint32_t near = near_faces_1d(s.c.qx, s.c.cx) | (near_faces_1d(s.c.qy, s.c.cy) << 2) |
                          (near_faces_1d(s.c.qz, s.c.cz) << 4);
    s.flags = collision_flags(s.c.cx, s.c.cy, s.c.cz, near);
    return s.flags == 0u;
}

template <bool kInd, class V>
__device__ __forceinline__ void walk(const WalkCtx &W, const WalkStart &s, uint32_t self, float4 pi,
                                     V &vis) {
    if (s.flags == 0u)
        walk_rows<kInd>(W, s.mx, s.my, s.mz, self, pi, vis);
    else
        walk_slow<kInd>(W, s.c.cx, s.c.cy, s.c.cz, s.flags, self, pi, vis);
}

// ---------------------------------------------------------------- physics

// Compensated (Kahan) accumulation: the GPU sums the same terms as the
// reference in a different order, so both are kept close to the exact sum
// and the remaining difference is the reference's own float rounding.
__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

struct DensityVisitor {
    float h2;
    float acc, comp;  // compensated sum of (h^2 - r^2)^3
    __device__ __forceinline__ void operator()(uint32_t, float, float, float, float d2) {
        const float u = __fsub_rn(h2, d2);
        kahan_add(acc, comp, __fmul_rn(__fmul_rn(u, u), u));
    }
};

// sph.cpp:28-76.  The reference accumulates m*poly6*(h^2-r^2)^3 term by term;
// here the cubes are summed and scaled once (the two differ by float
// rounding only).
template <bool kInd>
__global__ void __launch_bounds__(256) k_density(StepParams P, WalkCtx W, float2 *__restrict__ rp,
                                                 const uint32_t *__restrict__ status) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.n || *status) return;
    const uint32_t i = kInd ? W.order[t] : t;
    const float4 pi = W.pos[i];
    WalkStart s;
    walk_start(P, pi, s);
    DensityVisitor v{P.h2, 0.f, 0.f};
    walk<kInd>(W, s, i, pi, v);
    const float rho = __fadd_rn(__fmul_rn(P.mp6, v.acc), P.selfDens);
    const float prs = __fmul_rn(P.gasConstant, __fsub_rn(rho, P.restDensity));
    rp[i] = make_float2(rho, prs);
}

// One accepted pair of sph.cpp:107-121, operation for operation in FP32
// without fused multiply-adds.
struct ForceVisitor {
    const float4 *__restrict__ vel;
    const float2 *__restrict__ rp;
    float4 vi;
    float presI, h, mass, mm, spikyGrad, spikyLap;
    float fx, fy, fz;
    float cx, cy, cz;  // Kahan compensations
    __device__ __forceinline__ void operator()(uint32_t j, float dx, float dy, float dz, float d2) {
        const float4 vj = vel[j];
        const float2 q = rp[j];
        const float dist = __fsqrt_rn(d2);
        const float inv = __fdiv_rn(1.f, dist);  // normalize: d * (1 / sqrt(dot(d, d)))
        const float nx = __fmul_rn(dx, inv), ny = __fmul_rn(dy, inv), nz = __fmul_rn(dz, inv);
        const float psum = __fadd_rn(presI, q.y);
        const float twoRho = __fmul_rn(2.f, q.x);
        const float hd = __fsub_rn(h, dist);
        const float sq = __fmul_rn(hd, hd);  // (float)pow(double(h - dist), 2)
        const float px = __fmul_rn(
            __fmul_rn(__fdiv_rn(__fmul_rn(__fmul_rn(-nx, mass), psum), twoRho), spikyGrad), sq);
        const float py = __fmul_rn(
            __fmul_rn(__fdiv_rn(__fmul_rn(__fmul_rn(-ny, mass), psum), twoRho), spikyGrad), sq);
        const float pz = __fmul_rn(
            __fmul_rn(__fdiv_rn(__fmul_rn(__fmul_rn(-nz, mass), psum), twoRho), spikyGrad), sq);
        kahan_add(fx, cx, px);
        kahan_add(fy, cy, py);
        kahan_add(fz, cz, pz);
        const float vx =
            __fmul_rn(__fmul_rn(__fmul_rn(mm, __fdiv_rn(__fsub_rn(vj.x, vi.x), q.x)), spikyLap), hd);
        const float vy =
            __fmul_rn(__fmul_rn(__fmul_rn(mm, __fdiv_rn(__fsub_rn(vj.y, vi.y), q.x)), spikyLap), hd);
        const float vz =
            __fmul_rn(__fmul_rn(__fmul_rn(mm, __fdiv_rn(__fsub_rn(vj.z, vi.z), q.x)), spikyLap), hd);
        kahan_add(fx, cx, vx);
        kahan_add(fy, cy, vy);
        kahan_add(fz, cz, vz);
    }
};

// sph.cpp:133-181 with per-axis bounds: a = F/rho + (0, g, 0); v += a dt;
// x += v dt; damped reflection in the reference's order (floor, [ceiling],
// x low, x high, z low, z high).
__device__ __forceinline__ void integrate(const StepParams &P, float4 &x, float4 &v, float fx,
                                          float fy, float fz, float rho) {
    const float ax = __fadd_rn(__fdiv_rn(fx, rho), 0.f);
    const float ay = __fadd_rn(__fdiv_rn(fy, rho), P.g);
    const float az = __fadd_rn(__fdiv_rn(fz, rho), 0.f);
    v.x = __fadd_rn(v.x, __fmul_rn(ax, P.dt));
    v.y = __fadd_rn(v.y, __fmul_rn(ay, P.dt));
    v.z = __fadd_rn(v.z, __fmul_rn(az, P.dt));
    x.x = __fadd_rn(x.x, __fmul_rn(v.x, P.dt));
    x.y = __fadd_rn(x.y, __fmul_rn(v.y, P.dt));
    x.z = __fadd_rn(x.z, __fmul_rn(v.z, P.dt));
    if (x.y < P.ylo) {
        x.y = __fadd_rn(__fadd_rn(-x.y, __fmul_rn(2.f, P.ylo)), P.offset);
        v.y = __fmul_rn(-v.y, P.damping);
    }
    if (P.hasCeiling && x.y > P.yhi) {
        x.y = __fsub_rn(__fadd_rn(-x.y, __fmul_rn(2.f, P.yhi)), P.offset);
        v.y = __fmul_rn(-v.y, P.damping);
    }
    if (x.x < P.xlo) {
        x.x = __fadd_rn(__fadd_rn(-x.x, __fmul_rn(2.f, P.xlo)), P.offset);
        v.x = __fmul_rn(-v.x, P.damping);
    }
    if (x.x > P.xhi) {
        x.x = __fsub_rn(__fadd_rn(-x.x, __fmul_rn(2.f, P.xhi)), P.offset);
        v.x = __fmul_rn(-v.x, P.damping);
    }
    if (x.z < P.zlo) {
        x.z = __fadd_rn(__fadd_rn(-x.z, __fmul_rn(2.f, P.zlo)), P.offset);
        v.z = __fmul_rn(-v.z, P.damping);
    }
    if (x.z > P.zhi) {
        x.z = __fsub_rn(__fadd_rn(-x.z, __fmul_rn(2.f, P.zhi)), P.offset);
        v.z = __fmul_rn(-v.z, P.damping);
    }
}

template <bool kInd>
__global__ void __launch_bounds__(256)
    k_force(StepParams P, WalkCtx W, const float4 *__restrict__ vel, const float2 *__restrict__ rp,
            float4 *__restrict__ pos_out, float4 *__restrict__ vel_out,
            float4 *__restrict__ force_out, const uint32_t *__restrict__ status) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.n || *status) return;
    const uint32_t i = kInd ? W.order[t] : t;
    float4 pi = W.pos[i];
    float4 vi = vel[i];
    const float2 q = rp[i];
    WalkStart s;
    walk_start(P, pi, s);
    ForceVisitor v{vel,    rp,      vi, q.y, P.h, P.mass, __fmul_rn(P.viscosity, P.mass),
                   P.spikyGrad, P.spikyLap, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    walk<kInd>(W, s, i, pi, v);
    force_out[i] = make_float4(v.fx, v.fy, v.fz, 0.f);
    integrate(P, pi, vi, v.fx, v.fy, v.fz, q.x);
    pos_out[i] = pi;
    vel_out[i] = vi;
}

// ---------------------------------------------------------------- readouts

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct DigestVisitor {
    const uint32_t *__restrict__ id;
    uint32_t count;
    uint64_t sum;
    __device__ __forceinline__ void operator()(uint32_t j, float, float, float, float) {
        ++count;
        sum += mix64(id[j]);
    }
};

template <bool kInd>
__global__ void k_digest(StepParams P, WalkCtx W, const uint32_t *__restrict__ id,
                         uint32_t *__restrict__ count_out, uint64_t *__restrict__ digest_out,
                         const uint32_t *__restrict__ status) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P.n || *status) return;
    const uint32_t i = kInd ? W.order[t] : t;
    const float4 pi = W.pos[i];
    WalkStart s;
    walk_start(P, pi, s);
    DigestVisitor v{id, 0u, 0ull};
    walk<kInd>(W, s, i, pi, v);
    count_out[id[i]] = v.count;
    digest_out[id[i]] = v.sum;
}

__global__ void k_upload(uint32_t n, const float *__restrict__ pos3, const float *__restrict__ vel3,
                         float4 *__restrict__ pos, float4 *__restrict__ vel,
                         uint32_t *__restrict__ id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    pos[i] = make_float4(pos3[3 * i], pos3[3 * i + 1], pos3[3 * i + 2], 0.f);
    vel[i] = vel3 ? make_float4(vel3[3 * i], vel3[3 * i + 1], vel3[3 * i + 2], 0.f)
                  : make_float4(0.f, 0.f, 0.f, 0.f);
    id[i] = i;
}

// Field readout in id order: 3 floats per particle for vec fields, 1 for
// scalars.  field: 0 pos, 1 vel, 2 force, 3 rho, 4 prs.
__global__ void k_read_field(uint32_t n, int field, const uint32_t *__restrict__ id,
                             const float4 *__restrict__ v4, const float2 *__restrict__ rp,
                             float *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t d = id[i];
    if (field <= 2) {
        const float4 v = v4[i];
        out[3 * d] = v.x;
        out[3 * d + 1] = v.y;
        out[3 * d + 2] = v.z;
    } else {
        const float2 q = rp[i];
        out[d] = field == 3 ? q.x : q.y;
    }
}

// translate(position) * scale(h/2) (sph.cpp:178-179), column-major, id order.
// GLM's product leaves exact zeros off the diagonal and adds +0 to the
// translation (so -0 reads back as +0).
__global__ void k_transforms(uint32_t n, float half_h, const uint32_t *__restrict__ id,
                             const float4 *__restrict__ pos, float4 *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    float4 *m = out + 4 * (size_t)id[i];
    m[0] = make_float4(half_h, 0.f, 0.f, 0.f);
    m[1] = make_float4(0.f, half_h, 0.f, 0.f);
    m[2] = make_float4(0.f, 0.f, half_h, 0.f);
    m[3] = make_float4(__fadd_rn(p.x, 0.f), __fadd_rn(p.y, 0.f), __fadd_rn(p.z, 0.f), 1.f);
}

// Cell (truncated quotient) and stored uint16 hash per particle, id order.
__global__ void k_cells(uint32_t n, float h, const uint32_t *__restrict__ id,
                        const float4 *__restrict__ pos, int *__restrict__ cells,
                        uint16_t *__restrict__ hash) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const CellPos c = cell_pos(pos[i], h);
    const uint32_t d = id[i];
    if (cells) {
        cells[3 * d] = c.cx;
        cells[3 * d + 1] = c.cy;
        cells[3 * d + 2] = c.cz;
    }
    if (hash) hash[d] = (uint16_t)hash16(c.cx, c.cy, c.cz);
}

inline unsigned blocks(uint32_t n, unsigned bs) { return (n + bs - 1) / bs; }

}  // namespace

// ---------------------------------------------------------------- launchers

cudaError_t launch_sort(const StepParams &P, const SortBuffers &B, const float4 *pos,
                        cudaStream_t st) {
    const unsigned bs = 256;
    const uint32_t n = P.n;
    const uint32_t m = B.slots + 1;  // count[slots] stays 0 -> start[slots] = n
    const uint32_t ntiles = (m + kScanTile - 1) / kScanTile;
    if (n) k_keys<<<blocks(n, bs), bs, 0, st>>>(P, pos, B.key, B.rank, B.count, B.status);
    k_scan_tiles<<<ntiles, kScanThreads, 0, st>>>(B.count, m, B.tile_sum, B.max_cell, B.status);
    k_scan_tile_sums<<<1, kScanThreads, 0, st>>>(B.tile_sum, ntiles);
    k_scan_apply<<<ntiles, kScanThreads, 0, st>>>(B.count, m, B.tile_sum, B.start);
    if (n) {
        k_scatter<<<blocks(n, bs), bs, 0, st>>>(n, B.key, B.rank, B.start, B.order, B.status);
        k_cellsort<<<blocks(n, bs), bs, 0, st>>>(n, B.key, B.rank, B.start, B.order, B.status);
    }
    return cudaGetLastError();
}

cudaError_t launch_gather(uint32_t n, const SortBuffers &B, const float4 *pos_in,
                          const float4 *vel_in, const uint32_t *id_in, float4 *pos_out,
                          float4 *vel_out, uint32_t *id_out, cudaStream_t st) {
    if (n) k_gather<<<blocks(n, 256), 256, 0, st>>>(n, B.order, pos_in, vel_in, id_in, pos_out,
                                                    vel_out, id_out, B.status);
    return cudaGetLastError();
}

static WalkCtx make_ctx(const StepParams &P, const SortBuffers &B, const float4 *pos) {
    WalkCtx W;
    W.pos = pos;
    W.order = B.order;
    W.start = B.start;
    W.grid = P.grid;
    W.h2 = P.h2;
    return W;
}

cudaError_t launch_density(const StepParams &P, const SortBuffers &B, const float4 *pos,
                           float2 *rp, bool indirect, cudaStream_t st) {
    const WalkCtx W = make_ctx(P, B, pos);
    if (P.n) {
        if (indirect) k_density<true><<<blocks(P.n, 256), 256, 0, st>>>(P, W, rp, B.status);
        else k_density<false><<<blocks(P.n, 256), 256, 0, st>>>(P, W, rp, B.status);
    }
    return cudaGetLastError();
}

cudaError_t launch_force(const StepParams &P, const SortBuffers &B, const float4 *pos,
                         const float4 *vel, const float2 *rp, float4 *pos_out, float4 *vel_out,
                         float4 *force_out, bool indirect, cudaStream_t st) {
    const WalkCtx W = make_ctx(P, B, pos);
    if (P.n) {
        if (indirect)
            k_force<true><<<blocks(P.n, 256), 256, 0, st>>>(P, W, vel, rp, pos_out, vel_out,
                                                            force_out, B.status);
        else
            k_force<false><<<blocks(P.n, 256), 256, 0, st>>>(P, W, vel, rp, pos_out, vel_out,
                                                             force_out, B.status);
    }
    return cudaGetLastError();
}

cudaError_t launch_digest(const StepParams &P, const SortBuffers &B, const float4 *pos,
                          const uint32_t *id, uint32_t *count, uint64_t *digest, bool indirect,
                          cudaStream_t st) {
    const WalkCtx W = make_ctx(P, B, pos);
    if (P.n) {
        if (indirect)
            k_digest<true><<<blocks(P.n, 256), 256, 0, st>>>(P, W, id, count, digest, B.status);
        else
            k_digest<false><<<blocks(P.n, 256), 256, 0, st>>>(P, W, id, count, digest, B.status);
    }
    return cudaGetLastError();
}

cudaError_t launch_upload(uint32_t n, const float *pos3, const float *vel3, float4 *pos,
                          float4 *vel, uint32_t *id, cudaStream_t st) {
    if (n) k_upload<<<blocks(n, 256), 256, 0, st>>>(n, pos3, vel3, pos, vel, id);
    return cudaGetLastError();
}

cudaError_t launch_read_field(uint32_t n, int field, const uint32_t *id, const float4 *v4,
                              const float2 *rp, float *out, cudaStream_t st) {
    if (n) k_read_field<<<blocks(n, 256), 256, 0, st>>>(n, field, id, v4, rp, out);
    return cudaGetLastError();
}

cudaError_t launch_transforms(uint32_t n, float half_h, const uint32_t *id, const float4 *pos,
                              float *out16, cudaStream_t st) {
    if (n)
        k_transforms<<<blocks(n, 256), 256, 0, st>>>(n, half_h, id, pos,
                                                     reinterpret_cast<float4 *>(out16));
    return cudaGetLastError();
}

cudaError_t launch_cells(uint32_t n, float h, const uint32_t *id, const float4 *pos, int *cells,
                         uint16_t *hash, cudaStream_t st) {
    if (n) k_cells<<<blocks(n, 256), 256, 0, st>>>(n, h, id, pos, cells, hash);
    return cudaGetLastError();
}

}  // namespace sphx
