// sm_103a kernels of the SPH step (hand-written CUDA, FP32 physics, exact
// integer cell/hash work).  One step is:
//
//   k_keys        cell of every particle -> slot key in a modular cell grid,
//                 per-slot counts (atomics) and each particle's arrival rank
//   k_scan_*      exclusive prefix sum of the counts -> cellStart[slot]
//   k_scatter     (particle, x) into its cell's run, in arrival order
//   k_cellsort    each particle's place in its cell's run by (x, index), so
//                 that rows of cells are x-sorted and the order (and hence
//                 every float sum) is deterministic (k_cellsort_large: cells
//                 of more than 64 particles)
//   k_gather      every R steps: permute pos/vel/id into cell order
//   k_row_warps   the density pass's warps, one cell row each
//   k_density     poly6 density and pressure            (sph.cpp:28-76),
//                 the neighbour lists and records for the force pass
//                 (k_density_deferred: particles with a bucket collision)
//   k_force       spiky pressure + viscosity force over the lists, then
//                 integration and damped wall reflection (sph.cpp:80-181)
//                 (k_force_walk: particles past their list; k_force_deferred:
//                 those of them off the cooperative walk)
//
// Once per grid, k_cell_flags tabulates every slot's collision flags.
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

#include <algorithm>

#include "sphx_common.h"
#include "sphx_kernels.h"

// Resident threads per SM the walk kernels are compiled for (register cap
// 65536 / threads); the block size is a template parameter chosen per launch
// (128 or 256, see Tuning).
constexpr int kDensityThreadsPerSM = 1024;
constexpr int kForceListThreadsPerSM = 1024;
constexpr int kForceThreadsPerSM = 1024;

namespace sphx {
namespace {

__device__ __forceinline__ uint32_t slot_of(const Grid &g, int cx, int cy, int cz, int &mx,
                                            int &my, int &mz) {
    // inside the grid's extent (almost always) the modulo is the identity
    const int dx = cx - g.ox, dy = cy - g.oy, dz = cz - g.oz;
    mx = (unsigned)dx < (unsigned)g.gx ? dx : wrap_mod(dx, g.gx);
    my = (unsigned)dy < (unsigned)g.gy ? dy : wrap_mod(dy, g.gy);
    mz = (unsigned)dz < (unsigned)g.gz ? dz : wrap_mod(dz, g.gz);
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

// Scene of particle (storage index) i: the last s with pofs[s] <= i.
__device__ __forceinline__ uint32_t scene_of(const SceneTable &T, uint32_t i) {
    if (T.nscenes == 1) return 0;
    uint32_t lo = 0, hi = T.nscenes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (T.pofs[mid] <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// ---------------------------------------------------------------- keys / sort

__global__ void k_keys(SceneTable T, const float4 *__restrict__ pos, uint32_t *__restrict__ key,
                       uint32_t *__restrict__ rank, uint32_t *__restrict__ count,
                       uint32_t *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T.n) return;
    const uint32_t sc = scene_of(T, i);
    const StepParams &P = T.params[sc];
    const CellPos c = cell_pos(pos[i], P.h);
    uint32_t k = T.sofs[sc];
    if (in_domain(c.qx) && in_domain(c.qy) && in_domain(c.qz)) {
        int mx, my, mz;
        k += slot_of(P.grid, c.cx, c.cy, c.cz, mx, my, mz);
        // a cell outside the grid's x extent shares its slot with a cell gx
        // away: rows are then no longer sorted by x across their cells
        if ((unsigned)(c.cx - P.grid.ox) >= (unsigned)P.grid.gx) status[1] = 1u;
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

// Single block: exclusive scan of the tile sums in place (grids of more
// than kSelfPrefixTiles tiles).
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
// step in the same pass.  The tile's offset: with kSelfPrefix the sum of the
// earlier tiles' totals, added up by one warp (up to kSelfPrefixTiles tiles,
// which saves the pass over the tile sums), else tile_sum already holds it.
constexpr uint32_t kSelfPrefixTiles = 1024;
template <bool kSelfPrefix>
__global__ void k_scan_apply(uint32_t *__restrict__ count, uint32_t m,
                             const uint32_t *__restrict__ tile_sum,
                             uint32_t *__restrict__ start) {
    __shared__ uint32_t s_prefix;
    if (threadIdx.x < 32) {
        uint32_t p = 0;
        if (kSelfPrefix) {
            for (uint32_t b = threadIdx.x; b < blockIdx.x; b += 32) p += tile_sum[b];
#pragma unroll
            for (int d = 16; d; d >>= 1) p += __shfl_xor_sync(0xffffffffu, p, d);
        } else {
            p = tile_sum[blockIdx.x];
        }
        if (threadIdx.x == 0) s_prefix = p;
    }
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < m ? count[base + k] : 0u;
        s += v[k];
    }
    uint32_t excl;
    block_exclusive_scan(s, excl);  // its barriers also publish s_prefix
    uint32_t run = s_prefix + excl;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < m) {
            start[base + k] = run;
            count[base + k] = 0u;
        }
        run += v[k];
    }
}

// Each cell's run in arrival order: (particle, x bits) pairs.
__global__ void k_scatter(uint32_t n, const float4 *__restrict__ pos,
                          uint32_t *__restrict__ key, uint32_t *__restrict__ rank,
                          const uint32_t *__restrict__ start, uint2 *__restrict__ scat,
                          const uint32_t *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (*status & kStatusOverflowBit)) return;
    const uint32_t k = key[i], a = start[k], c = start[k + 1] - a, r = rank[i];
    scat[a + r] = make_uint2(i, __float_as_uint(pos[i].x));
    // for the cell sort: the cell's run and the place in it (c <= max_cell
    // <= kLargeCell < 2^16 without an overflow)
    key[i] = a;
    rank[i] = r | (c << 16);
}

// Each particle's place in its cell's run sorted by (x, particle index): the
// number of run members before it in that order (a strict total order on
// finite x, so the places form a permutation).  Sorting by x makes every run
// of x-consecutive cells sorted by x, which the walk's x window relies on,
// and the index makes the order, and hence every float sum, deterministic.
// Runs longer than kSmallCell (clumped fluid) are queued, by the particle
// that arrived first, for k_cellsort_large instead.
constexpr uint32_t kSmallCell = 64;

__global__ void k_cellsort(uint32_t n, const uint32_t *__restrict__ key,
                           const uint32_t *__restrict__ rank, const uint2 *__restrict__ scat,
                           uint32_t *__restrict__ order, uint32_t *__restrict__ status,
                           uint2 *__restrict__ large, uint32_t large_cap) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (status[0] & kStatusErrorMask)) return;
    // k_scatter left the cell's run start in key and (place | count << 16) in rank
    const uint32_t a = key[i], rc = rank[i], c = rc >> 16, place = rc & 0xFFFFu;
    if (c > kSmallCell) {
        if (place == 0u) {
            const uint32_t slot = atomicAdd(&status[2], 1u);
            if (slot < large_cap) large[slot] = make_uint2(a, c);
        }
        return;
    }
    const float xi = __uint_as_float(scat[a + place].y);  // k_scatter's copy of x
    uint32_t r = 0;
#pragma unroll 4
    for (uint32_t t = a; t < a + c; ++t) {
        const uint2 e = scat[t];
        const float xj = __uint_as_float(e.y);
        r += (xj < xi || (xj == xi && e.x < i)) ? 1u : 0u;
    }
    order[a + r] = i;
}

// Total order of floats as unsigned integers (finite values).
__device__ __forceinline__ uint32_t float_order(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// One CTA per queued large cell: bitonic sort of (x, particle index) keys in
// shared memory (up to kLargeCell entries), written back to the cell's run.
__global__ void __launch_bounds__(512) k_cellsort_large(const uint2 *__restrict__ scat,
                                                        uint32_t *__restrict__ order,
                                                        const uint32_t *__restrict__ status,
                                                        const uint2 *__restrict__ large,
                                                        uint32_t large_cap) {
    extern __shared__ unsigned long long skeys[];
    if (status[0] & kStatusErrorMask) return;
    const uint32_t count = min(status[2], large_cap);
    for (uint32_t c = blockIdx.x; c < count; c += gridDim.x) {
        const uint2 cell = large[c];  // (start, length), length <= kLargeCell
        uint32_t m = 2;
        while (m < cell.y) m <<= 1;
        for (uint32_t t = threadIdx.x; t < m; t += blockDim.x) {
            unsigned long long v = ~0ull;
            if (t < cell.y) {
                const uint2 e = scat[cell.x + t];
                v = ((unsigned long long)float_order(__uint_as_float(e.y)) << 32) | e.x;
            }
            skeys[t] = v;
        }
        __syncthreads();
        for (uint32_t k = 2; k <= m; k <<= 1)
            for (uint32_t jj = k >> 1; jj > 0; jj >>= 1) {
                for (uint32_t t = threadIdx.x; t < m; t += blockDim.x) {
                    const uint32_t u = t ^ jj;
                    if (u > t) {
                        const unsigned long long x = skeys[t], y = skeys[u];
                        const bool up = (t & k) == 0;
                        if ((x > y) == up) {
                            skeys[t] = y;
                            skeys[u] = x;
                        }
                    }
                }
                __syncthreads();
            }
        for (uint32_t t = threadIdx.x; t < cell.y; t += blockDim.x)
            order[cell.x + t] = (uint32_t)skeys[t];
        __syncthreads();
    }
}

__global__ void k_gather(uint32_t n, const uint32_t *__restrict__ order,
                         const float4 *__restrict__ pos_in, const float4 *__restrict__ vel_in,
                         const uint32_t *__restrict__ id_in, float4 *__restrict__ pos_out,
                         float4 *__restrict__ vel_out, uint32_t *__restrict__ id_out,
                         const uint32_t *__restrict__ status) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n || (*status & kStatusErrorMask)) return;
    const uint32_t s = order[t];
    pos_out[t] = pos_in[s];
    vel_out[t] = vel_in[s];
    id_out[t] = id_in[s];
}

// ---------------------------------------------------------------- walks

struct WalkCtx {
    const float4 *__restrict__ pos;
    const uint32_t *__restrict__ order;
    const uint32_t *__restrict__ start;  // this scene's first slot
    Grid grid;
    float h2;
    float h;
    float h2w;  // h^2 (1 + 2^-18): squared half-width bound of the row windows
    bool xmono;  // every particle inside the grid's x extent this step
    const uint8_t *__restrict__ cflags;  // this scene's cell flags (k_cell_flags), or NULL
};

// One run of cell-sorted slots [a, b): every particle j != self with
// |pj - pi|^2 < h^2 (reference's float r^2, sph.cpp:57: (dx*dx + dy*dy) + dz*dz,
// no fused multiply-add) is passed to the visitor `w` times.
template <class V>
__device__ __forceinline__ void test_pair(const WalkCtx &W, uint32_t j, float4 pj, uint32_t self,
                                          float4 pi, uint32_t w, V &vis) {
    vis.on_test();
    const float dx = __fsub_rn(pj.x, pi.x);
    const float dy = __fsub_rn(pj.y, pi.y);
    const float dz = __fsub_rn(pj.z, pi.z);
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    if (d2 < W.h2 && j != self)
        for (uint32_t r = 0; r < w; ++r) vis(j, dx, dy, dz, d2);
}

// Two candidates are loaded per iteration so that their loads overlap.
template <bool kInd, class V>
__device__ __forceinline__ void scan_run(const WalkCtx &W, uint32_t a, uint32_t b, uint32_t self,
                                         float4 pi, uint32_t w, V &vis) {
    uint32_t t = a;
    for (; t + 1 < b; t += 2) {
        const uint32_t j0 = kInd ? W.order[t] : t;
        const uint32_t j1 = kInd ? W.order[t + 1] : t + 1;
        const float4 p0 = W.pos[j0];
        const float4 p1 = W.pos[j1];
        test_pair(W, j0, p0, self, pi, w, vis);
        test_pair(W, j1, p1, self, pi, w, vis);
    }
    if (t < b) {
        const uint32_t j = kInd ? W.order[t] : t;
        test_pair(W, j, W.pos[j], self, pi, w, vis);
    }
}

// As scan_run, over a run sorted by x, visiting only candidates whose x lies
// in [xlo, xhi]: the run is entered at its first x >= xlo and left at the
// first x > xhi.  Any j with float r^2 < h^2 has |xj - xi| < h (1 + 2^-22),
// so a window of half-width h (1 + 2^-20) plus rounding slack loses none.
// When some particle lies outside the grid's x extent (xmono false) the run
// is not monotone in x and candidates past xhi are skipped, not the rest of
// the run.

template <bool kInd, class V>
__device__ __forceinline__ void scan_run_x(const WalkCtx &W, uint32_t a, uint32_t b, uint32_t self,
                                           float4 pi, float xlo, float xhi, bool xmono, V &vis) {
    uint32_t t = a;
    if (xmono) {  // the run is x-sorted: binary search for the first x >= xlo
        uint32_t lo = a, hi = b;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            const float x = W.pos[kInd ? W.order[mid] : mid].x;
            if (x < xlo) lo = mid + 1;
            else hi = mid;
        }
        t = lo;
    }
    for (; t + 1 < b; t += 2) {
        const uint32_t j0 = kInd ? W.order[t] : t;
        const uint32_t j1 = kInd ? W.order[t + 1] : t + 1;
        const float4 p0 = W.pos[j0];
        const float4 p1 = W.pos[j1];
        if (xmono && p0.x > xhi) return;
        if (p0.x >= xlo && p0.x <= xhi) test_pair(W, j0, p0, self, pi, 1u, vis);
        if (xmono && p1.x > xhi) return;
        if (p1.x >= xlo && p1.x <= xhi) test_pair(W, j1, p1, self, pi, 1u, vis);
    }
    if (t < b) {
        const uint32_t j = kInd ? W.order[t] : t;
        const float4 p = W.pos[j];
        if (p.x >= xlo && p.x <= xhi) test_pair(W, j, p, self, pi, 1u, vis);
    }
}

__device__ __forceinline__ int wrap1(int v, int m) {
    v = v < 0 ? v + m : v;
    return v >= m ? v - m : v;
}

// The nine (dy, dz) neighbour rows of a cell, in the order every walk
// visits them (and the neighbour lists record them): the dz = 0 layer, then
// dz = +1, then dz = -1, each as dy = 0, -1, +1.  The particle's own row and
// layer come first: their neighbours are the ones the neighbouring lanes of
// a force warp gather too.
__device__ __forceinline__ int row_dz(int r) { return r < 3 ? 0 : (r < 6 ? 1 : -1); }
__device__ __forceinline__ int row_dy(int r) {
    const int q = r % 3;
    return q == 0 ? 0 : (q == 1 ? -1 : 1);
}

// Fast path: the 27 cells around (mx, my, mz), each visited once.
__device__ __forceinline__ uint32_t row_base(const Grid &g, int my, int mz, int r) {
    const int z = wrap1(mz + row_dz(r), g.gz);
    const int y = wrap1(my + row_dy(r), g.gy);
    return ((uint32_t)z * (uint32_t)g.gy + (uint32_t)y) * (uint32_t)g.gx;
}

// Squared half-width budget of row r's x window: h^2 (widened) less the
// squared gaps to the row in y and z (ey2m, ey2p, ez2m, ez2p: below and
// above); the row holds no accepted neighbour unless it is positive.
__device__ __forceinline__ float row_w2(float h2w, float ey2m, float ey2p, float ez2m, float ez2p,
                                        int r) {
    const int dy = row_dy(r), dz = row_dz(r);
    const float ey = dy < 0 ? ey2m : (dy > 0 ? ey2p : 0.f);
    const float ez = dz < 0 ? ez2m : (dz > 0 ? ez2p : 0.f);
    return h2w - ey - ez;
}

// Lower bound on the distance from coordinate y (quotient cell c) to any
// particle of cell c + d, d = +1 or -1.  Cell m covers quotients [m, m+1) for
// m > 0, (m-1, m] for m < 0 and (-1, 1) for m = 0.  A particle can sit in
// cell m while a few ulps past m*h (the division rounds), so the bound is
// lowered by (|y| + |bound| + h) 2^-20 and clamped at 0.
__device__ __forceinline__ float gap_to_cell(float y, int c, int d, float h) {
    float bound, gap;
    if (d > 0) {
        const int m = c + 1;
        bound = (float)(m > 0 ? m : m - 1) * h;
        gap = bound - y;
    } else {
        const int m = c - 1;
        bound = (float)(m >= 0 ? m + 1 : m) * h;
        gap = y - bound;
    }
    const float slack = (fabsf(y) + fabsf(bound) + h) * 9.5367431640625e-07f;
    return fmaxf(gap - slack, 0.f);
}

// Fast path: the 27 cells around (mx, my, mz), each visited once.  With the
// particle's slot away from the grid's x seam, each (dy, dz) row of three
// cells is one contiguous, x-sorted run.  A row whose cells are at least
// (ey, ez) away in y and z can only hold accepted particles with
// dx^2 < h^2 - ey^2 - ez^2, so it is scanned inside that narrower x window
// and skipped when the window is empty; the bounds of the next row to scan
// are loaded before the current one is scanned.
template <bool kInd, class V>
__device__ __forceinline__ void walk_rows(const WalkCtx &W, const CellPos &c, int mx, int my,
                                          int mz, uint32_t self, float4 pi, V &vis) {
    const Grid &g = W.grid;
    if (mx >= 1 && mx + 1 < g.gx) {
        const float h = W.h;
        const float eym = gap_to_cell(pi.y, c.cy, -1, h), eyp = gap_to_cell(pi.y, c.cy, 1, h);
        const float ezm = gap_to_cell(pi.z, c.cz, -1, h), ezp = gap_to_cell(pi.z, c.cz, 1, h);
        const float ey2[3] = {eym * eym, 0.f, eyp * eyp};
        const float ez2[3] = {ezm * ezm, 0.f, ezp * ezp};
        uint32_t rows = 0;
#pragma unroll
        for (int r = 0; r < 9; ++r)
            if (W.h2w - ey2[row_dy(r) + 1] - ez2[row_dz(r) + 1] > 0.f) rows |= 1u << r;
        const float xpad = fabsf(pi.x) * 2.384185791015625e-07f;  // |x| 2^-22
        int r = __ffs(rows) - 1;
        rows &= rows - 1;
        uint32_t base = row_base(g, my, mz, r);
        uint32_t a = W.start[base + mx - 1], b = W.start[base + mx + 2];
#pragma unroll 1
        while (r >= 0) {
            const uint32_t ca = a, cb = b;
            const int cr = r;
            r = rows ? __ffs(rows) - 1 : -1;
            rows &= rows - 1;
            if (r >= 0) {
                base = row_base(g, my, mz, r);
                a = W.start[base + mx - 1];
                b = W.start[base + mx + 2];
            }
            const int iy = row_dy(cr) + 1, iz = row_dz(cr) + 1;
            const float eyy = iy == 0 ? ey2[0] : (iy == 2 ? ey2[2] : 0.f);
            const float ezz = iz == 0 ? ez2[0] : (iz == 2 ? ez2[2] : 0.f);
            const float hx = fmaf(sqrtf(W.h2w - eyy - ezz), 1.0000009536743164f, xpad);
            scan_run_x<kInd>(W, ca, cb, self, pi, pi.x - hx, pi.x + hx, W.xmono, vis);
        }
    } else {
#pragma unroll 1
        for (int r = 0; r < 9; ++r) {
            const uint32_t base = row_base(g, my, mz, r);
            for (int dx = -1; dx <= 1; ++dx) {
                const uint32_t k = base + (uint32_t)wrap1(mx + dx, g.gx);
                scan_run<kInd>(W, W.start[k], W.start[k + 1], self, pi, 1u, vis);
            }
        }
    }
}

// Slow path, taken when `flags` reports a bucket collision: every neighbour
// cell is walked with weight = number of the 27 offsets whose bucket equals
// its bucket (the reference walks a bucket once per offset that hashes to it,
// sph.cpp:40-63), and, for each flagged face, the nine cells two steps away
// whose bucket is among the 27 are walked with that same weight.
// slow_cells calls f(slot, weight) for those cells, in walk order.
template <class F>
__device__ __forceinline__ void slow_cells(const Grid &g, int cx, int cy, int cz, uint32_t flags,
                                           F &&f) {
    uint32_t H[27];
    int o = 0;
    for (int x = -1; x <= 1; ++x)
        for (int y = -1; y <= 1; ++y)
            for (int z = -1; z <= 1; ++z) H[o++] = hash16(cx + x, cy + y, cz + z);
    int mx, my, mz;
    o = 0;
    for (int x = -1; x <= 1; ++x)
        for (int y = -1; y <= 1; ++y)
            for (int z = -1; z <= 1; ++z) {
                uint32_t w = 0;
                for (int k = 0; k < 27; ++k) w += H[k] == H[o] ? 1u : 0u;
                f(slot_of(g, cx + x, cy + y, cz + z, mx, my, mz), w);
                ++o;
            }
    for (int fc = 0; fc < 6; ++fc) {
        if (!((flags >> (kFlagFaceShift + fc)) & 1u)) continue;
        const int axis = fc >> 1, step = (fc & 1) ? 2 : -2;
        for (int a = -1; a <= 1; ++a)
            for (int b = -1; b <= 1; ++b) {
                int c[3] = {cx, cy, cz};
                c[axis] += step;
                c[(axis + 1) % 3] += a;
                c[(axis + 2) % 3] += b;
                const uint32_t hf = hash16(c[0], c[1], c[2]);
                uint32_t w = 0;
                for (int k = 0; k < 27; ++k) w += H[k] == hf ? 1u : 0u;
                if (w) f(slot_of(g, c[0], c[1], c[2], mx, my, mz), w);
            }
    }
}

template <bool kInd, class V>
__device__ __noinline__ void walk_slow(const WalkCtx &W, int cx, int cy, int cz, uint32_t flags,
                                       uint32_t self, float4 pi, V &vis) {
    slow_cells(W.grid, cx, cy, cz, flags, [&](uint32_t k, uint32_t w) {
        scan_run<kInd>(W, W.start[k], W.start[k + 1], self, pi, w, vis);
    });
}

// Cell, slot and collision flags of a particle; returns true when the fast
// 27-cell walk is exact for it.
struct WalkStart {
    CellPos c;
    int mx, my, mz;
    uint32_t flags;
};

// The flags come from the scene's cell-flag table when the particle's cell
// is the one its slot was computed for (the grid's own extent), else they
// are computed here.
__device__ __forceinline__ bool walk_start(const WalkCtx &W, const StepParams &P, float4 pi,
                                           WalkStart &s) {
    s.c = cell_pos(pi, P.h);
    const uint32_t k = slot_of(P.grid, s.c.cx, s.c.cy, s.c.cz, s.mx, s.my, s.mz);
    const uint32_t near = near_faces_1d(s.c.qx, s.c.cx) | (near_faces_1d(s.c.qy, s.c.cy) << 2) |
                          (near_faces_1d(s.c.qz, s.c.cz) << 4);
    const bool own = (uint32_t)s.c.cx - (uint32_t)P.grid.ox == (uint32_t)s.mx &&
                     (uint32_t)s.c.cy - (uint32_t)P.grid.oy == (uint32_t)s.my &&
                     (uint32_t)s.c.cz - (uint32_t)P.grid.oz == (uint32_t)s.mz;
    if (W.cflags && own)
        s.flags = W.cflags[k] & (kFlagDup | (near << kFlagFaceShift));
    else
        s.flags = collision_flags(s.c.cx, s.c.cy, s.c.cz, near);
    return s.flags == 0u;
}

// Collision flags of every slot's own cell (all six faces), once per grid.
__global__ void k_cell_flags(SceneTable T, uint32_t slots, uint8_t *__restrict__ cflags) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= slots) return;
    uint32_t lo = 0, hi = T.nscenes;  // scene: the last s with sofs[s] <= k
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (T.sofs[mid] <= k) lo = mid;
        else hi = mid;
    }
    const Grid &g = T.params[lo].grid;
    const uint32_t l = k - T.sofs[lo], gx = (uint32_t)g.gx, gy = (uint32_t)g.gy;
    const int mx = (int)(l % gx), my = (int)((l / gx) % gy), mz = (int)(l / (gx * gy));
    cflags[k] = (uint8_t)collision_flags(mx + g.ox, my + g.oy, mz + g.oz, 0x3Fu);
}

template <bool kInd, class V>
__device__ __forceinline__ void walk(const WalkCtx &W, const WalkStart &s, uint32_t self, float4 pi,
                                     V &vis) {
    if (s.flags == 0u)
        walk_rows<kInd>(W, s.c, s.mx, s.my, s.mz, self, pi, vis);
    else
        walk_slow<kInd>(W, s.c.cx, s.c.cy, s.c.cz, s.flags, self, pi, vis);
}

// Warp-cooperative form of the fast path.  Consecutive threads hold
// consecutive cell-sorted particles, so most of a warp sits in one (y, z) row
// of cells and shares its nine neighbour rows.  Lanes with the same scene and
// row form a group; for each neighbour row the group copies the union of its
// lanes' three-cell runs into this warp's shared-memory chunk (coalesced,
// kCoopChunk particles at a time), then every lane scans its own run inside
// the chunk with the same x window and early exit as scan_run_x.  The set of
// pairs tested is exactly walk_rows'; only the loads are shared and the lanes
// stay in step.  Lanes off the fast path (bucket collisions, the grid's x
// seam) walk alone afterwards.
//
// What the chunk holds and how a lane scans its part of it is the scanner's
// (PosScan: positions, for density and the digest; RecordScan: the force
// kernel's 32-byte neighbour records).
// 256 positions (4 KB a warp): fewer chunk rounds per row once cells fill
// up; 2 % faster than 128 positions from step 40 of the 2,097,152-particle
// dam-break block on, measured with CUDA events on a GB300.
constexpr int kScanUnroll = 4;
constexpr uint32_t kCoopChunk = 256;

struct CoopLane {
    bool valid;  // holds a particle that walks
    bool fast;   // takes the cooperative path
    uint64_t key;
};

__device__ __forceinline__ CoopLane coop_lane(bool valid, uint32_t sc, const WalkCtx &W,
                                              const WalkStart &s) {
    CoopLane c;
    c.valid = valid;
    c.fast = valid && s.flags == 0u && s.mx >= 1 && s.mx + 1 < W.grid.gx;
    c.key = c.fast ? (((uint64_t)sc << 32) | ((uint32_t)s.mz * (uint32_t)W.grid.gy + (uint32_t)s.my))
                   : ~0ull;
    return c;
}

// One group's walk by its members alone (gmask): they load the chunks
// between them and scan them.  For warps that are one group or a few large
// ones (the common case: consecutive particles share a cell row).
template <bool kInd, class S>
__device__ __forceinline__ void coop_rows_group(const WalkCtx &W, const WalkStart &s, uint32_t self,
                                                float4 pi, uint32_t gmask, uint32_t lane, S &scan) {
    const float h = W.h;
    const float eym = gap_to_cell(pi.y, s.c.cy, -1, h), eyp = gap_to_cell(pi.y, s.c.cy, 1, h);
    const float ezm = gap_to_cell(pi.z, s.c.cz, -1, h), ezp = gap_to_cell(pi.z, s.c.cz, 1, h);
    const float ey2[3] = {eym * eym, 0.f, eyp * eyp};
    const float ez2[3] = {ezm * ezm, 0.f, ezp * ezp};
    uint32_t rows = 0;
#pragma unroll
    for (int r = 0; r < 9; ++r)
        if (W.h2w - ey2[row_dy(r) + 1] - ez2[row_dz(r) + 1] > 0.f) rows |= 1u << r;
    const float xpad = fabsf(pi.x) * 2.384185791015625e-07f;  // |x| 2^-22
    uint32_t todo = __reduce_or_sync(gmask, rows);
    const uint32_t mxlo = __reduce_min_sync(gmask, (uint32_t)s.mx);
    const uint32_t mxhi = __reduce_max_sync(gmask, (uint32_t)s.mx);
    const uint32_t rank = __popc(gmask & ((1u << lane) - 1u)), gsize = __popc(gmask);
#pragma unroll 1
    while (todo) {
        const int r = __ffs(todo) - 1;
        todo &= todo - 1;
        const uint32_t base = row_base(W.grid, s.my, s.mz, r);
        const uint32_t A = W.start[base + mxlo - 1], B = W.start[base + mxhi + 2];
        const uint32_t a = W.start[base + s.mx - 1], b = W.start[base + s.mx + 2];
        const int iy = row_dy(r) + 1, iz = row_dz(r) + 1;
        const float eyy = iy == 0 ? ey2[0] : (iy == 2 ? ey2[2] : 0.f);
        const float ezz = iz == 0 ? ez2[0] : (iz == 2 ? ez2[2] : 0.f);
        bool done = !((rows >> r) & 1u) || a == b;
        const float hx = done ? 0.f : fmaf(sqrtf(W.h2w - eyy - ezz), 1.0000009536743164f, xpad);
        const float xlo = pi.x - hx, xhi = pi.x + hx;
#pragma unroll 1
        for (uint32_t c0 = A; c0 < B; c0 += S::kChunk) {
            const uint32_t m = min(S::kChunk, B - c0);
            for (uint32_t k = rank; k < m; k += gsize) scan.load(W, k, kInd ? W.order[c0 + k] : c0 + k);
            __syncwarp(gmask);
            if (!done && b > c0 && a < c0 + m)
                done = scan.scan(W, c0, a > c0 ? a - c0 : 0u, min(b - c0, m), xlo, xhi, self, pi);
            __syncwarp(gmask);
        }
    }
}

// One group's walk, every lane of the warp taking part: all of them load
// the chunks, the members scan them.  For groups that are a few lanes of a
// warp (particles of a clumped region among others).
template <bool kInd, class S>
__device__ __forceinline__ void coop_rows_warp(const WalkCtx &W, const WalkStart &s, uint32_t self,
                                          float4 pi, bool member, uint32_t leader, uint32_t lane,
                                          S &scan) {
    float ey2[3] = {0.f, 0.f, 0.f}, ez2[3] = {0.f, 0.f, 0.f};
    uint32_t rows = 0;
    if (member) {
        const float h = W.h;
        const float eym = gap_to_cell(pi.y, s.c.cy, -1, h), eyp = gap_to_cell(pi.y, s.c.cy, 1, h);
        const float ezm = gap_to_cell(pi.z, s.c.cz, -1, h), ezp = gap_to_cell(pi.z, s.c.cz, 1, h);
        ey2[0] = eym * eym;
        ey2[2] = eyp * eyp;
        ez2[0] = ezm * ezm;
        ez2[2] = ezp * ezp;
#pragma unroll
        for (int r = 0; r < 9; ++r)
            if (W.h2w - ey2[row_dy(r) + 1] - ez2[row_dz(r) + 1] > 0.f) rows |= 1u << r;
    }
    const float xpad = fabsf(pi.x) * 2.384185791015625e-07f;  // |x| 2^-22
    uint32_t todo = __reduce_or_sync(0xffffffffu, rows);
    const uint32_t mxlo = __reduce_min_sync(0xffffffffu, member ? (uint32_t)s.mx : 0xffffffffu);
    const uint32_t mxhi = __reduce_max_sync(0xffffffffu, member ? (uint32_t)s.mx : 0u);
#pragma unroll 1
    while (todo) {
        const int r = __ffs(todo) - 1;
        todo &= todo - 1;
        uint32_t A = 0, B = 0, a = 0, b = 0;
        if (member) {
            const uint32_t base = row_base(W.grid, s.my, s.mz, r);
            A = W.start[base + mxlo - 1];
            B = W.start[base + mxhi + 2];
            a = W.start[base + s.mx - 1];
            b = W.start[base + s.mx + 2];
        }
        A = __shfl_sync(0xffffffffu, A, leader);
        B = __shfl_sync(0xffffffffu, B, leader);
        const int iy = row_dy(r) + 1, iz = row_dz(r) + 1;
        const float eyy = iy == 0 ? ey2[0] : (iy == 2 ? ey2[2] : 0.f);
        const float ezz = iz == 0 ? ez2[0] : (iz == 2 ? ez2[2] : 0.f);
        bool done = !member || !((rows >> r) & 1u) || a == b;
        const float hx = done ? 0.f : fmaf(sqrtf(W.h2w - eyy - ezz), 1.0000009536743164f, xpad);
        const float xlo = pi.x - hx, xhi = pi.x + hx;
#pragma unroll 1
        for (uint32_t c0 = A; c0 < B; c0 += S::kChunk) {
            const uint32_t m = min(S::kChunk, B - c0);
            for (uint32_t k = lane; k < m; k += 32u) scan.load(W, k, kInd ? W.order[c0 + k] : c0 + k);
            __syncwarp();
            if (!done && b > c0 && a < c0 + m)
                done = scan.scan(W, c0, a > c0 ? a - c0 : 0u, min(b - c0, m), xlo, xhi, self, pi);
            __syncwarp();
        }
    }
}

// What coop_walk does with the valid lanes off the cooperative path: walk
// them alone with `vis` (kTailAll) or leave them to the caller (kTailNone,
// which lists them for a later kernel).  Keeping the slow walk, a call, out
// of a kernel frees its register allocation.
enum CoopTail { kTailNone, kTailAll };

// Runs the scanner over every fast lane's neighbours, one group after
// another (kWarpLoad: coop_rows_warp, else coop_rows_group), then the tail.
// Every lane of the warp calls it (lanes without a walk pass valid = false).
template <bool kInd, bool kWarpLoad, int kTail, class S, class V>
__device__ __forceinline__ void coop_walk(const WalkCtx &W, const WalkStart &s, const CoopLane &cl,
                                          uint32_t self, float4 pi, S &scan, V &vis) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gm = __match_any_sync(0xffffffffu, cl.key);
    uint32_t pending = __ballot_sync(0xffffffffu, cl.fast);
#pragma unroll 1
    while (pending) {
        const uint32_t leader = __ffs(pending) - 1;
        if (kWarpLoad) {
            const uint32_t gmask = __shfl_sync(0xffffffffu, gm, leader);
            coop_rows_warp<kInd>(W, s, self, pi, cl.fast && ((gmask >> lane) & 1u), leader, lane,
                                 scan);
            pending &= ~gmask;
        } else {
            if (cl.fast && ((gm >> leader) & 1u)) coop_rows_group<kInd>(W, s, self, pi, gm, lane, scan);
            pending &= ~__shfl_sync(0xffffffffu, gm, leader);
        }
    }
    if (kTail == kTailAll && cl.valid && !cl.fast) walk<kInd>(W, s, self, pi, vis);
}

// Appends the warp's lanes with `defer` set to a deferred list (*counter
// counts it), one atomic per warp.  Every lane of the warp calls it.
__device__ __forceinline__ void defer_lanes(bool defer, uint32_t t, uint32_t *__restrict__ deferred,
                                            uint32_t *__restrict__ counter) {
    const uint32_t m = __ballot_sync(0xffffffffu, defer);
    if (!m) return;
    const uint32_t lane = threadIdx.x & 31u, leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (defer) deferred[base + __popc(m & ((1u << lane) - 1u))] = t;
}

// Chunk of candidate positions; the lane's visitor sees each candidate of its
// run inside the x window (scan_run_x's test, same order).
// Chunk of candidate positions; the lane's visitor sees each candidate of
// its run inside the x window (scan_run_x's test, same order).
template <bool kInd>
struct PosSmem {
    float4 pos[kCoopChunk];
    __device__ __forceinline__ float px(uint32_t k) const { return pos[k].x; }
    __device__ __forceinline__ float4 p(uint32_t k) const { return pos[k]; }
    __device__ __forceinline__ void put(uint32_t k, float4 v) { pos[k] = v; }
    uint32_t idx[kInd ? kCoopChunk : 1];
};

template <bool kInd, class V>
struct PosScan {
    static constexpr uint32_t kChunk = kCoopChunk;
    PosSmem<kInd> &sm;
    V &vis;
    __device__ __forceinline__ void load(const WalkCtx &W, uint32_t k, uint32_t j) {
        sm.put(k, W.pos[j]);
        if (kInd) sm.idx[k] = j;
    }
    __device__ __forceinline__ void test(const WalkCtx &W, uint32_t c0, uint32_t k, uint32_t self,
                                         float4 pi) {
        test_pair(W, kInd ? sm.idx[k] : c0 + k, sm.p(k), self, pi, 1u, vis);
    }
    // Every candidate of chunk slots [0, m), with weight w, for a whole warp
    // walking one particle: lane l tests slot l (the reference's float r^2),
    // then lane 0 hands the accepted ones to its visitor in slot order, w
    // times each: scan_run's visits, in its order, with its values.
    __device__ __forceinline__ void test_all_warp(const WalkCtx &W, uint32_t c0, uint32_t m,
                                                  uint32_t self, float4 pi, uint32_t w) {
        const uint32_t lane = threadIdx.x & 31u;
        bool acc = false;
        float d2 = 0.f;
        uint32_t j = 0u;
        if (lane < m) {
            const float4 p = sm.p(lane);
            j = kInd ? sm.idx[lane] : c0 + lane;
            const float dx = __fsub_rn(p.x, pi.x);
            const float dy = __fsub_rn(p.y, pi.y);
            const float dz = __fsub_rn(p.z, pi.z);
            d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            acc = d2 < W.h2 && j != self;
        }
        uint32_t mask = __ballot_sync(0xffffffffu, acc);
        while (mask) {  // warp-uniform
            const int l = __ffs(mask) - 1;
            mask &= mask - 1u;
            const float dl = __shfl_sync(0xffffffffu, d2, l);
            const uint32_t jl = __shfl_sync(0xffffffffu, j, l);
            if (lane == 0)
                for (uint32_t r = 0; r < w; ++r) vis(jl, 0.f, 0.f, 0.f, dl);
        }
    }
    // Chunk slots [lo, hi), the chunk starting at cell-sorted slot c0; true
    // once past the window's end.
    __device__ __forceinline__ bool scan(const WalkCtx &W, uint32_t c0, uint32_t lo, uint32_t hi,
                                         float xlo, float xhi, uint32_t self, float4 pi) {
        if (!W.xmono) {  // runs not x-sorted this step: test the window bounds one by one
            for (uint32_t k = lo; k < hi; ++k) {
                const float4 p = sm.p(k);
                if (p.x >= xlo && p.x <= xhi)
                    test_pair(W, kInd ? sm.idx[k] : c0 + k, p, self, pi, 1u, vis);
            }
            return false;
        }
        {  // x-sorted: start at the first x >= xlo
            uint32_t l = lo, u = hi;
            while (l < u) {
                const uint32_t mid = (l + u) >> 1;
                if (sm.px(mid) < xlo) l = mid + 1;
                else u = mid;
            }
            lo = l;
        }
        // every candidate from the searched start on has x >= xlo
#pragma unroll kScanUnroll
        for (uint32_t k = lo; k < hi; ++k) {
            const float4 p = sm.p(k);
            if (p.x > xhi) return true;
            test_pair(W, kInd ? sm.idx[k] : c0 + k, p, self, pi, 1u, vis);
        }
        return false;
    }
};

// One particle's walk by a whole warp, for the particles the walk kernels
// defer.  The lanes copy each cell's run into the scanner's chunk, 32
// candidates at a time, test one candidate each, and lane 0 visits the
// accepted ones in order: the same cells, order and weights as walk() (the
// slow path's cells where buckets collide, else the 27 cells row by row,
// which is walk_rows' order), so the sums are walk()'s bit for bit, while
// the loads and the r^2 tests of a candidate run go out together instead of
// one after another.
template <bool kInd, class S>
__device__ __forceinline__ void warp_walk_cell(const WalkCtx &W, uint32_t k, uint32_t w,
                                               uint32_t self, float4 pi, S &scan) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t a = W.start[k], b = W.start[k + 1];
#pragma unroll 1
    for (uint32_t c0 = a; c0 < b; c0 += 32u) {
        const uint32_t m = min(32u, b - c0);
        if (lane < m) scan.load(W, lane, kInd ? W.order[c0 + lane] : c0 + lane);
        __syncwarp();
        scan.test_all_warp(W, c0, m, self, pi, w);
        __syncwarp();
    }
}

template <bool kInd, class S>
__device__ __forceinline__ void warp_walk(const WalkCtx &W, const WalkStart &s, uint32_t self,
                                          float4 pi, S &scan) {
    auto cell = [&](uint32_t k, uint32_t w) { warp_walk_cell<kInd>(W, k, w, self, pi, scan); };
    if (s.flags != 0u) {
        slow_cells(W.grid, s.c.cx, s.c.cy, s.c.cz, s.flags, cell);
        return;
    }
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        const uint32_t base = row_base(W.grid, s.my, s.mz, r);
        for (int dx = -1; dx <= 1; ++dx) cell(base + (uint32_t)wrap1(s.mx + dx, W.grid.gx), 1u);
    }
}

// ---------------------------------------------------------------- row warps

// The cooperative walk shares a warp's loads among lanes of the same cell
// row; a warp whose particles straddle two rows walks them as two groups,
// one after the other, with half its lanes idle each time.  So the density
// pass gives every warp the particles of one row only: row R's particles
// [start[first], start[first + gx]) go to ceil(count / 32) warps, numbered
// from wofs[R], an exclusive scan of those counts over all rows (entry rows
// is the total).  Lanes past a row's end idle.

// Scene of global cell row R: the last s with rofs[s] <= R.
__device__ __forceinline__ uint32_t scene_of_row(const SceneTable &T, uint32_t R) {
    if (T.nscenes == 1) return 0;
    uint32_t lo = 0, hi = T.nscenes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (T.rofs[mid] <= R) lo = mid;
        else hi = mid;
    }
    return lo;
}

// First slot of row R (of scene sc).
__device__ __forceinline__ uint32_t row_first_slot(const SceneTable &T, uint32_t sc, uint32_t R) {
    return T.sofs[sc] + (R - T.rofs[sc]) * (uint32_t)T.params[sc].grid.gx;
}

// Row of warp w (< wofs[rows]): the last R < rows with wofs[R] <= w, which
// has warps, since a row after it with the same offset has none.  A 32-way
// search, the whole warp calling with the same w: each round every lane
// tests one point of [lo, hi) and the range shrinks to the gap after the
// last point that passed; wofs[lo] <= w throughout.
__device__ __forceinline__ uint32_t row_of_warp(const uint32_t *__restrict__ wofs, uint32_t rows,
                                                uint32_t w) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t lo = 0, hi = rows;
    while (hi - lo > 1) {
        const uint32_t stride = (hi - lo + 31u) >> 5;
        const uint32_t x = lo + lane * stride;
        const unsigned b = __ballot_sync(0xffffffffu, x < hi && __ldg(wofs + x) <= w);
        lo += (uint32_t)(31 - __clz(b)) * stride;  // lane 0 always passes
        hi = min(lo + stride, hi);
    }
    return lo;
}

// Threads a density launch needs: at most n / 32 + rows warps (each row's
// last warp is partial).
__host__ __forceinline__ uint32_t launch_threads(const SceneTable &T) {
    return (T.n / 32u + T.rows + 1u) * 32u;
}

// Kernel 1, kScanTile rows per block: every row's warp count, scanned within
// the block into wofs, and the block's total into tile_sum.  After an error
// no row has warps.
__global__ void k_row_warps(SceneTable T, const uint32_t *__restrict__ start,
                            uint32_t *__restrict__ wofs, uint32_t *__restrict__ tile_sum,
                            const uint32_t *__restrict__ status) {
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    const bool err = status[0] & kStatusErrorMask;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const uint32_t R = base + k;
        v[k] = 0u;
        if (R < T.rows && !err) {
            const uint32_t sc = scene_of_row(T, R);
            const uint32_t f = row_first_slot(T, sc, R);
            v[k] = (start[f + (uint32_t)T.params[sc].grid.gx] - start[f] + 31u) >> 5;
        }
        s += v[k];
    }
    uint32_t excl;
    const uint32_t tot = block_exclusive_scan(s, excl);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k <= T.rows) wofs[base + k] = excl;
        excl += v[k];
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

// Kernel 2 (more than one block of rows): adds the earlier blocks' totals.
__global__ void k_row_offsets(uint32_t rows, uint32_t *__restrict__ wofs,
                              const uint32_t *__restrict__ tile_sum) {
    __shared__ uint32_t s_prefix;
    if (threadIdx.x < 32) {
        uint32_t p = 0;
        for (uint32_t b = threadIdx.x; b < blockIdx.x; b += 32) p += tile_sum[b];
#pragma unroll
        for (int d = 16; d; d >>= 1) p += __shfl_xor_sync(0xffffffffu, p, d);
        if (threadIdx.x == 0) s_prefix = p;
    }
    __syncthreads();
    const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k)
        if (base + k <= rows) wofs[base + k] += s_prefix;
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

// kahan_add of u^3, the cube's last product fused into the compensation
// step: u^3 - c is rounded once instead of twice.  As accurate as the plain
// form (checked on the CPU against an FP64 sum over the dam-break block) and
// one instruction shorter.
__device__ __forceinline__ void kahan_add_cube(float &s, float &c, float u) {
    const float u2 = __fmul_rn(u, u);
    const float y = __fmaf_rn(u2, u, -c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

// Neighbour lists in tiles of 32 cell-sorted slots (a force warp's
// particles), four entries per slot side by side: entry k of slot t is
// nbr[(t / 32) * slots * 32 + (k / 4) * 128 + (t % 32) * 4 + k % 4], so that
// a force warp's 16-byte load of entries k..k+3 of its 32 slots reads 512
// contiguous bytes instead of 32 rows' lines.  list_base(L, t) is the address
// of entry 0 of slot t, list_offset(k) the offset of entry k from it.
__device__ __forceinline__ uint32_t *list_base(const NbrList &L, uint32_t t) {
    return L.nbr + (size_t)(t >> 5) * L.slots * 32u + (t & 31u) * 4u;
}
__device__ __forceinline__ uint32_t list_offset(uint32_t k) { return k + (k & ~3u) * 31u; }

// Accepted neighbours of a particle, in walk order, are also recorded for
// the force kernel (list_base: k < slots, written by one lane front to
// back); a particle with more (clumped fluid), or of a crowded cell, stores
// its count only and the force kernel walks for it instead.
struct DensityVisitor {
    __device__ __forceinline__ void on_test() {}
    float h2;
    float acc, comp;  // compensated sum of (h^2 - r^2)^3
    uint32_t *row;    // list_base of the particle's slot, or NULL: nothing recorded
    uint32_t slots;
    uint32_t cnt;
    __device__ __forceinline__ void operator()(uint32_t j, float, float, float, float d2) {
        kahan_add_cube(acc, comp, __fsub_rn(h2, d2));
        // streaming store: the force pass reads the row once, after every
        // other row has been written
        if (row && cnt < slots) __stcs(row + list_offset(cnt), j);
        ++cnt;
    }
};

// Per-thread walk context of scene sc.
__device__ __forceinline__ WalkCtx walk_ctx(const SceneTable &T, const WalkCtx &G, uint32_t sc,
                                            const StepParams &P, const uint32_t *status) {
    WalkCtx W = G;
    W.start = G.start + T.sofs[sc];
    if (G.cflags) W.cflags = G.cflags + T.sofs[sc];
    W.grid = P.grid;
    W.h2 = P.h2;
    W.h = P.h;
    W.h2w = P.h2w;
    W.xmono = status[1] == 0u;
    return W;
}

// Threads and blocks of the kernels that take the deferred particles: few
// in fluid (none in the dam-break block), at most n.
constexpr int kDeferredThreads = 128;
// Eight blocks per SM: a batch of small scenes near the origin (where
// buckets collide) defers thousands of particles, and a deferred walk is a
// chain of dependent loads that wants other warps beside it (the 512-scene
// step took 3.43 ms against 3.54 with two blocks per SM).
constexpr unsigned kDeferredBlocks = 8 * 152;
// No list is recorded for a particle whose cell holds more than
// slots / kListSkipFactor particles; its count then carries kNoList.
constexpr uint32_t kListSkipFactor = 4;
constexpr uint32_t kNoList = 0x80000000u;

// A particle's list row, or NULL when its own cell holds so many particles
// (clumped fluid) that it has more neighbours than the row holds and the
// force pass walks for it: recording them would only cost writes.  Either
// way the force is the same.
__device__ __forceinline__ uint32_t *density_row(const WalkCtx &W, const WalkStart &s,
                                                 const NbrList &L, uint32_t t) {
    if (!L.nbr) return nullptr;
    const uint32_t k = ((uint32_t)s.mz * (uint32_t)W.grid.gy + (uint32_t)s.my) *
                           (uint32_t)W.grid.gx + (uint32_t)s.mx;
    const uint32_t occ = W.start[k + 1] - W.start[k];
    return occ * kListSkipFactor <= L.slots ? list_base(L, t) : nullptr;
}

// Density, pressure, the list count and the neighbour record of particle i
// from its compensated sum of cubes `acc` and its accepted count (`listed`:
// whether a list row was recorded).
__device__ __forceinline__ void density_finish(const StepParams &P, float acc, uint32_t cnt,
                                               bool listed, uint32_t i, float4 pi,
                                               const float4 *__restrict__ vel,
                                               float4 *__restrict__ rp, float4 *__restrict__ fr,
                                               const NbrList &L) {
    const float rho = __fadd_rn(__fmul_rn(P.mp6, acc), P.selfDens);
    const float prs = __fmul_rn(P.gasConstant, __fsub_rn(rho, P.restDensity));
    const float inv = __frcp_rn(rho);
    rp[i] = make_float4(rho, prs, inv, 0.f);
    if (L.nbr) L.count[i] = listed ? cnt : (cnt | kNoList);
    if (fr) {
        // what the force kernel reads of a neighbour, in one 32-byte record
        const float4 vi = vel[i];
        fr[2 * (size_t)i] = make_float4(pi.x, pi.y, pi.z, prs);
        fr[2 * (size_t)i + 1] = make_float4(vi.x, vi.y, vi.z, inv);
    }
}

// The density pass's chunk of a neighbour row: cell-sorted positions c0,
// c0 + 1, ... as three coordinate arrays (so that two neighbouring
// candidates' coordinates load as one 8-byte pair), and with kInd their
// particle indices.
template <bool kInd>
struct DensityChunk {
    __align__(16) float x[kCoopChunk];
    __align__(16) float y[kCoopChunk];
    __align__(16) float z[kCoopChunk];
    uint32_t idx[kInd ? kCoopChunk : 1];
};

// Two FP32 values in one 64-bit register pair, and the packed
// round-to-nearest arithmetic on them (each half rounded on its own, as
// __fsub_rn / __fmul_rn / __fadd_rn round it).
__device__ __forceinline__ uint64_t f32x2_dup(float v) {
    const uint64_t b = __float_as_uint(v);
    return b | (b << 32);
}
__device__ __forceinline__ float f32x2_lo(uint64_t v) { return __uint_as_float((uint32_t)v); }
__device__ __forceinline__ float f32x2_hi(uint64_t v) { return __uint_as_float((uint32_t)(v >> 32)); }
__device__ __forceinline__ uint64_t f32x2_sub(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f32x2_mul(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t f32x2_add(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// One lane's scan of chunk slots [lo, hi) of a neighbour row (the chunk
// holds cell-sorted positions c0, c0 + 1, ...): every candidate inside the
// lane's x window is tested with the reference's float r^2 (sph.cpp:57: (dx*dx
// + dy*dy) + dz*dz, no fused multiply-add; two candidates at a time in
// packed pairs, each rounded as alone); an accepted one adds (h^2 - r^2)^3
// to the row's sum rs (one fused multiply-add) and its index to the list row
// (while it has room).  x-sorted runs (xmono): start at the first x >= xlo
// (binary search), stop at the first x > xhi; returns true once past the
// window.  Otherwise every slot is checked against the window.  kSelf: the
// particle's own row, the only one that holds the particle itself (skipped
// by its cell-sorted position self).
template <bool kInd, bool kSelf>
__device__ __forceinline__ bool density_scan(const DensityChunk<kInd> &sm, uint32_t c0, uint32_t lo,
                                             uint32_t hi, float xlo, float xhi, bool xmono,
                                             float4 pi, float h2, uint32_t self, float &rs,
                                             uint32_t &cnt, uint32_t *lrow, uint32_t lcap) {
    auto accept = [&](uint32_t k, float d2) {
        if (d2 < h2 && (!kSelf || c0 + k != self)) {
            const float u = __fsub_rn(h2, d2);
            rs = __fmaf_rn(__fmul_rn(u, u), u, rs);
            // streaming store: the force pass reads the row once, after
            // every other row has been written
            if (cnt < lcap) __stcs(lrow + list_offset(cnt), kInd ? sm.idx[k] : c0 + k);
            ++cnt;
        }
    };
    auto one = [&](uint32_t k, float px) {
        const float dx = __fsub_rn(px, pi.x);
        const float dy = __fsub_rn(sm.y[k], pi.y);
        const float dz = __fsub_rn(sm.z[k], pi.z);
        accept(k, __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
    };
    if (!xmono) {
        for (uint32_t k = lo; k < hi; ++k) {
            const float px = sm.x[k];
            if (px >= xlo && px <= xhi) one(k, px);
        }
        return false;
    }
    uint32_t k = lo, u = hi;
    while (k < u) {
        const uint32_t mid = (k + u) >> 1;
        if (sm.x[mid] < xlo) k = mid + 1;
        else u = mid;
    }
    if ((k & 1u) && k < hi) {  // pairs start at even slots
        const float px = sm.x[k];
        if (px > xhi) return true;
        one(k, px);
        ++k;
    }
    const uint64_t PX = f32x2_dup(pi.x), PY = f32x2_dup(pi.y), PZ = f32x2_dup(pi.z);
#pragma unroll 4
    for (; k + 1u < hi; k += 2u) {
        const uint64_t X = *reinterpret_cast<const uint64_t *>(sm.x + k);
        if (f32x2_lo(X) > xhi) return true;
        const uint64_t Y = *reinterpret_cast<const uint64_t *>(sm.y + k);
        const uint64_t Z = *reinterpret_cast<const uint64_t *>(sm.z + k);
        const uint64_t dX = f32x2_sub(X, PX), dY = f32x2_sub(Y, PY), dZ = f32x2_sub(Z, PZ);
        const uint64_t D2 =
            f32x2_add(f32x2_add(f32x2_mul(dX, dX), f32x2_mul(dY, dY)), f32x2_mul(dZ, dZ));
        accept(k, f32x2_lo(D2));
        if (f32x2_hi(X) > xhi) return true;
        accept(k + 1u, f32x2_hi(D2));
    }
    if (k < hi) {
        const float px = sm.x[k];
        if (px > xhi) return true;
        one(k, px);
    }
    return false;
}

// Density and pressure, sph.cpp:28-76, one warp per cell-row segment (the
// warps k_row_warps counted).  The reference accumulates m*poly6*(h^2-r^2)^3
// term by term; here the cubes of each neighbour row are summed with fused
// multiply-adds, the nine row sums are added with compensation (Kahan) and
// the total is scaled once: the two differ by float rounding only.  (A row's
// sum costs one dependent operation per term instead of a four-operation
// compensated step, which matters where clumped rows hold hundreds of terms;
// the compensation across rows keeps the total's error at the level of one
// row's.)
//
// A warp's particles are up to 32 consecutive cell-sorted particles of one
// row of slots (my, mz), hence x-sorted, and share its nine neighbour rows.
// Row, scene and grid are warp-uniform.  For each neighbour row, in walk
// order (row_base), the warp copies the union of its lanes' three-cell runs
// into its shared-memory chunk (coalesced, kCoopChunk positions at a time)
// and every lane scans its own x window of its own run there
// (density_scan); a row the narrowing rules out for every lane is skipped.
// The pairs and their order are walk_rows': the neighbour lists, recorded
// in that order, are what the force pass and its walkers sum over.  Lanes
// off this path (a bucket collision, or a slot at the grid's x seam, whose
// three x-adjacent cells are not one run) are listed for
// k_density_deferred.
template <bool kInd, int kThreads>
__global__ void __launch_bounds__(kThreads, kDensityThreadsPerSM / kThreads)
    k_density(SceneTable T, WalkCtx G, const float4 *__restrict__ vel, float4 *__restrict__ rp,
              float4 *__restrict__ fr, NbrList L, RowWarps RW, uint32_t *__restrict__ deferred,
              uint32_t *__restrict__ status) {
    __shared__ DensityChunk<kInd> s_chunk[kThreads / 32];
    if (status[0] & kStatusErrorMask) return;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= RW.wofs[T.rows]) return;  // whole warps leave together
    // the warp's row of slots and its scene (warp-uniform)
    const uint32_t R = row_of_warp(RW.wofs, T.rows, w);
    const uint32_t sc = scene_of_row(T, R);
    const StepParams &P = T.params[sc];
    const WalkCtx W = walk_ctx(T, G, sc, P, status);
    const Grid &g = W.grid;
    const uint32_t gx = (uint32_t)g.gx, gy = (uint32_t)g.gy;
    const uint32_t Rl = R - T.rofs[sc];  // my + gy * mz
    const int my = (int)(Rl % gy), mz = (int)(Rl / gy);
    const uint32_t f = Rl * gx;
    const uint32_t t = W.start[f] + ((w - RW.wofs[R]) << 5) + lane;
    const bool valid = t < W.start[f + gx];
    const uint32_t i = valid ? (kInd ? G.order[t] : t) : 0u;
    const float4 pi = G.pos[i];
    WalkStart s;
    walk_start(W, P, pi, s);
    const bool fast = valid && s.flags == 0u && s.mx >= 1 && s.mx + 1 < g.gx;
    defer_lanes(valid && !fast, t, deferred, &status[kStatusDeferred]);
    if (!__any_sync(0xffffffffu, fast)) return;
    const uint32_t mxlo = __reduce_min_sync(0xffffffffu, fast ? (uint32_t)s.mx : 0xffffffffu);
    const uint32_t mxhi = __reduce_max_sync(0xffffffffu, fast ? (uint32_t)s.mx : 0u);
    // narrowing: lower bounds on the distance to the rows above and below
    const float h = P.h;
    float ey2m = gap_to_cell(pi.y, s.c.cy, -1, h), ey2p = gap_to_cell(pi.y, s.c.cy, 1, h);
    float ez2m = gap_to_cell(pi.z, s.c.cz, -1, h), ez2p = gap_to_cell(pi.z, s.c.cz, 1, h);
    ey2m *= ey2m;
    ey2p *= ey2p;
    ez2m *= ez2m;
    ez2p *= ez2p;
    const float xpad = fabsf(pi.x) * 2.384185791015625e-07f;  // |x| 2^-22
    uint32_t *lrow = fast ? density_row(W, s, L, t) : nullptr;
    const uint32_t lcap = lrow ? L.slots : 0u;
    float ks = 0.f, kc = 0.f;
    uint32_t cnt = 0u;
    DensityChunk<kInd> &sm = s_chunk[threadIdx.x >> 5];
#pragma unroll 1
    for (int r = 0; r < 9; ++r) {
        const float w2 = row_w2(W.h2w, ey2m, ey2p, ez2m, ez2p, r);
        const bool need = fast && w2 > 0.f;
        if (!__any_sync(0xffffffffu, need)) continue;
        const uint32_t base = row_base(g, my, mz, r);
        const uint32_t A = W.start[base + mxlo - 1], B = W.start[base + mxhi + 2];
        uint32_t a = 0u, b = 0u;
        if (need) {
            a = W.start[base + s.mx - 1];
            b = W.start[base + s.mx + 2];
        }
        const float hx = need ? fmaf(sqrtf(w2), 1.0000009536743164f, xpad) : 0.f;
        const float xlo = pi.x - hx, xhi = pi.x + hx;
        bool done = !need || a == b;
        float rs = 0.f;
#pragma unroll 1
        for (uint32_t c0 = A; c0 < B; c0 += kCoopChunk) {
            const uint32_t m = min(kCoopChunk, B - c0);
            for (uint32_t k = lane; k < m; k += 32u) {
                const uint32_t j = kInd ? G.order[c0 + k] : c0 + k;
                const float4 p = G.pos[j];
                sm.x[k] = p.x;
                sm.y[k] = p.y;
                sm.z[k] = p.z;
                if (kInd) sm.idx[k] = j;
            }
            __syncwarp();
            if (!done && b > c0 && a < c0 + m) {
                if (r == 0)
                    done = density_scan<kInd, true>(sm, c0, a > c0 ? a - c0 : 0u, min(b - c0, m), xlo,
                                                    xhi, W.xmono, pi, W.h2, t, rs, cnt, lrow, lcap);
                else
                    done = density_scan<kInd, false>(sm, c0, a > c0 ? a - c0 : 0u, min(b - c0, m), xlo,
                                                     xhi, W.xmono, pi, W.h2, t, rs, cnt, lrow, lcap);
            }
            __syncwarp();
        }
        kahan_add(ks, kc, rs);
    }
    if (fast) density_finish(P, ks, cnt, lrow != nullptr, i, pi, vel, rp, fr, L);
}

// The particles k_density deferred, one warp each (warp_walk).
template <bool kInd>
__global__ void __launch_bounds__(kDeferredThreads)
    k_density_deferred(SceneTable T, WalkCtx G, const float4 *__restrict__ vel,
                       float4 *__restrict__ rp, float4 *__restrict__ fr, NbrList L,
                       const uint32_t *__restrict__ deferred, const uint32_t *__restrict__ status) {
    if (status[0] & kStatusErrorMask) return;
    __shared__ PosSmem<kInd> s_chunk[kDeferredThreads / 32];
    const uint32_t m = status[kStatusDeferred];
    const uint32_t lane = threadIdx.x & 31u, nw = gridDim.x * (kDeferredThreads / 32);
#pragma unroll 1
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < m; q += nw) {
        const uint32_t t = deferred[q];
        const uint32_t i = kInd ? G.order[t] : t;
        const uint32_t sc = scene_of(T, i);
        const StepParams &P = T.params[sc];
        const WalkCtx W = walk_ctx(T, G, sc, P, status);
        const float4 pi = W.pos[i];
        WalkStart s;
        walk_start(W, P, pi, s);
        DensityVisitor v{P.h2, 0.f, 0.f, lane == 0 ? density_row(W, s, L, t) : nullptr, L.slots, 0u};
        PosScan<kInd, DensityVisitor> scan{s_chunk[threadIdx.x >> 5], v};
        warp_walk<kInd>(W, s, i, pi, scan);
        if (lane == 0) density_finish(P, v.acc, v.cnt, v.row != nullptr, i, pi, vel, rp, fr, L);
    }
}

// One accepted pair of sph.cpp:107-121.  With d = pj - pi, r = |d| and
// hd = h - r, the reference's two terms are
//   pressure   -(d / r) * m * (pi + pj) / (2 rho_j) * spikyGrad * hd^2
//   viscosity  mu * m * (vj - vi) / rho_j * spikyLap * hd
// evaluated here as -cp * d + cv * (vj - vi) with cp = kp (pi + pj) hd^2 / (rho_j r),
// kp = m spikyGrad / 2, and cv = kv hd / rho_j, kv = mu m spikyLap: the same
// products without divisions (1/rho_j comes precomputed with the density).
// Per term this moves the result by a few float ulps; summed forces stay
// within about 1e-6 of the reference's (rms-floored relative metric).
struct ForcePair {
    float4 vi;
    float presI, h, kp, kv;
    float fx, fy, fz;
    float cx, cy, cz;  // Kahan compensations
    // pj_w = neighbour pressure, vj = (velocity, 1/density)
    __device__ __forceinline__ void add(float dx, float dy, float dz, float d2, float pj_w,
                                        float4 vj) {
        const float invr = rsqrtf(d2);
        const float r = d2 * invr;
        const float hd = h - r;
        const float cp = kp * (presI + pj_w) * vj.w * (hd * hd) * invr;
        const float cv = kv * hd * vj.w;
        // compensated add of cv (vj - vi) - cp d: the term minus the running
        // compensation in two fused multiply-adds (one rounding each)
        kahan_add_term(fx, cx, fmaf(cv, vj.x - vi.x, fmaf(-cp, dx, -cx)));
        kahan_add_term(fy, cy, fmaf(cv, vj.y - vi.y, fmaf(-cp, dy, -cy)));
        kahan_add_term(fz, cz, fmaf(cv, vj.z - vi.z, fmaf(-cp, dz, -cz)));
    }
    // The rest of kahan_add given y = term - c.
    __device__ __forceinline__ static void kahan_add_term(float &s, float &c, float y) {
        const float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
};

// r^2 of the reference (sph.cpp:57) from a neighbour's record, then the pair.
__device__ __forceinline__ void pair_add_record(ForcePair &pair, float4 a, float4 b, float4 pi) {
    const float dx = __fsub_rn(a.x, pi.x);
    const float dy = __fsub_rn(a.y, pi.y);
    const float dz = __fsub_rn(a.z, pi.z);
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    pair.add(dx, dy, dz, d2, a.w, b);
}

// A neighbour's 32-byte record (32-byte aligned: fr is), read-only during
// the force pass: one 256-bit load (four 64-bit lanes).
__device__ __forceinline__ void load_record(const float4 *__restrict__ fr, uint32_t j, float4 &a,
                                            float4 &b) {
    const float4 *p = fr + 2 * (size_t)j;
    unsigned long long q0, q1, q2, q3;
    asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];" : "=l"(q0), "=l"(q1), "=l"(q2), "=l"(q3) : "l"(p));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(q0));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.z), "=f"(a.w) : "l"(q1));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(b.x), "=f"(b.y) : "l"(q2));
    asm("mov.b64 {%0, %1}, %2;" : "=f"(b.z), "=f"(b.w) : "l"(q3));
}

__device__ __forceinline__ void pair_from_record(ForcePair &pair, const float4 *__restrict__ fr,
                                                 uint32_t j, float4 pi) {
    float4 a, b;
    load_record(fr, j, a, b);
    pair_add_record(pair, a, b, pi);
}

// Force walk over a chunk of neighbour records (RecordScan): a lane first
// tests up to 32 candidates of its run and marks the accepted ones in a bit
// mask, then adds the marked pairs; the pair math thus runs with the lanes in
// step instead of under the acceptance branch (about one candidate in four
// passes), and every operand comes from shared memory.
constexpr uint32_t kForceChunk = 64;

template <bool kInd>
struct RecordSmem {
    float4 a[kForceChunk];  // x, y, z, pressure
    float4 b[kForceChunk];  // vx, vy, vz, 1/density
    uint32_t idx[kInd ? kForceChunk : 1];
};

template <bool kInd>
struct RecordScan {
    static constexpr uint32_t kChunk = kForceChunk;
    RecordSmem<kInd> &sm;
    const float4 *__restrict__ fr;
    ForcePair &pair;
    __device__ __forceinline__ void load(const WalkCtx &, uint32_t k, uint32_t j) {
        sm.a[k] = fr[2 * (size_t)j];
        sm.b[k] = fr[2 * (size_t)j + 1];
        if (kInd) sm.idx[k] = j;
    }
    // Every candidate of chunk slots [0, m), with weight w, for a whole warp
    // walking one particle: lane l tests slot l, then lane 0 adds the
    // accepted pairs from the chunk's records in slot order, w times each:
    // ForceVisitor's pairs under scan_run, in its order.
    __device__ __forceinline__ void test_all_warp(const WalkCtx &W, uint32_t c0, uint32_t m,
                                                  uint32_t self, float4 pi, uint32_t w) {
        const uint32_t lane = threadIdx.x & 31u;
        bool acc = false;
        if (lane < m) {
            const float4 p = sm.a[lane];
            const float dx = __fsub_rn(p.x, pi.x);
            const float dy = __fsub_rn(p.y, pi.y);
            const float dz = __fsub_rn(p.z, pi.z);
            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
            const uint32_t j = kInd ? sm.idx[lane] : c0 + lane;
            acc = d2 < W.h2 && j != self;
        }
        uint32_t mask = __ballot_sync(0xffffffffu, acc);
        if (lane == 0)
            while (mask) {
                const uint32_t k = __ffs(mask) - 1;
                mask &= mask - 1u;
                for (uint32_t r = 0; r < w; ++r) pair_add_record(pair, sm.a[k], sm.b[k], pi);
            }
    }
    __device__ __forceinline__ bool scan(const WalkCtx &W, uint32_t c0, uint32_t lo, uint32_t hi,
                                         float xlo, float xhi, uint32_t self, float4 pi) {
        bool done = false;
#pragma unroll 1
        for (uint32_t k0 = lo; k0 < hi && !done; k0 += 32) {
            const uint32_t k1 = min(hi, k0 + 32);
            uint32_t acc = 0;
            for (uint32_t k = k0; k < k1; ++k) {
                const float4 p = sm.a[k];
                if (p.x > xhi) {
                    if (W.xmono) { done = true; break; }
                    continue;
                }
                if (p.x < xlo) continue;
                const float dx = __fsub_rn(p.x, pi.x);
                const float dy = __fsub_rn(p.y, pi.y);
                const float dz = __fsub_rn(p.z, pi.z);
                const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                const uint32_t j = kInd ? sm.idx[k] : c0 + k;
                if (d2 < W.h2 && j != self) acc |= 1u << (k - k0);
            }
#pragma unroll 1
            while (acc) {
                const uint32_t k = k0 + __ffs(acc) - 1;
                acc &= acc - 1;
                pair_add_record(pair, sm.a[k], sm.b[k], pi);
            }
        }
        return done;
    }
};

// Lanes off the fast path add each accepted pair as the walk finds it.
struct ForceVisitor {
    __device__ __forceinline__ void on_test() {}
    ForcePair &pair;
    const float4 *__restrict__ fr;
    float4 pi;
    __device__ __forceinline__ void operator()(uint32_t j, float, float, float, float) {
        pair_from_record(pair, fr, j, pi);
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

// Force, then integration and walls, of particle i (density rho).
__device__ __forceinline__ void force_finish(const StepParams &P, const ForcePair &pair, uint32_t i,
                                             float4 pi, float4 vi, float rho,
                                             float4 *__restrict__ pos_out,
                                             float4 *__restrict__ vel_out,
                                             float4 *__restrict__ force_out) {
    const float fx = pair.fx, fy = pair.fy, fz = pair.fz;
    force_out[i] = make_float4(fx, fy, fz, 0.f);
    float4 x = pi, v = vi;
    integrate(P, x, v, fx, fy, fz, rho);
    pos_out[i] = x;
    vel_out[i] = v;
}

// Force of every particle whose neighbours fit its list (same neighbours,
// same order as the density walk), then integration and walls.  The others
// are k_force_walk's, which this kernel tells which warps (32 cell-sorted
// particles) hold one: keeping the walk out of this kernel leaves it 48
// registers instead of 64 with spills (0.257 against 0.276 ms at 2.1M).
template <bool kInd, int kThreads>
__global__ void __launch_bounds__(kThreads, kForceListThreadsPerSM / kThreads)
    k_force(SceneTable T, WalkCtx G, const float4 *__restrict__ vel, const float4 *__restrict__ rp,
            const float4 *__restrict__ fr, NbrList L, float4 *__restrict__ pos_out,
            float4 *__restrict__ vel_out, float4 *__restrict__ force_out,
            uint32_t *__restrict__ walk_warps, uint32_t *__restrict__ status) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (status[0] & kStatusErrorMask) return;
    const bool valid = t < T.n;  // the grid is whole blocks: every lane gets here
    const uint32_t i = valid ? (kInd ? G.order[t] : t) : 0u;
    const uint32_t cnt = valid ? L.count[i] : 0u;
    const uint32_t wm = __ballot_sync(0xffffffffu, valid && cnt > L.slots);
    if (wm && (threadIdx.x & 31u) == (uint32_t)(__ffs(wm) - 1))
        walk_warps[atomicAdd(&status[kStatusWalkWarps], 1u)] = t >> 5;
    if (!valid || cnt > L.slots) return;
    const uint32_t sc = scene_of(T, i);
    const StepParams &P = T.params[sc];
    const float4 pi = G.pos[i];
    const float4 vi = vel[i];
    const float4 q = rp[i];
    ForcePair pair{vi, q.y, P.h, P.forceKp, P.forceKv, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    // four entries per 16-byte load, the warp's 32 slots side by side
    // (list_base): one load of the warp reads 512 contiguous bytes; entries
    // past cnt in the last load are never used
    const uint4 *row = reinterpret_cast<const uint4 *>(list_base(L, t));
#pragma unroll 1
    for (uint32_t k = 0; k < cnt; k += 4) {
        const uint4 e = row[(k >> 2) * 32u];
        const uint32_t left = cnt - k;
        {  // two records in flight, then summed in list order
            const uint32_t j1 = left > 1 ? e.y : e.x;
            float4 a0, b0, a1, b1;
            load_record(fr, e.x, a0, b0);
            load_record(fr, j1, a1, b1);
            pair_add_record(pair, a0, b0, pi);
            if (left > 1) pair_add_record(pair, a1, b1, pi);
        }
        if (left > 2) {
            const uint32_t j3 = left > 3 ? e.w : e.z;
            float4 a2, b2, a3, b3;
            load_record(fr, e.z, a2, b2);
            load_record(fr, j3, a3, b3);
            pair_add_record(pair, a2, b2, pi);
            if (left > 3) pair_add_record(pair, a3, b3, pi);
        }
    }
    force_finish(P, pair, i, pi, vi, q.x, pos_out, vel_out, force_out);
}

// Force of the particles past their list (clumped fluid), over the warps
// k_force listed: a warp-cooperative walk over the neighbour records in the
// density walk's order, the whole warp loading for its walking lanes.
// Walkers off the cooperative path (bucket collision, grid seam) are listed
// in `deferred` for k_force_deferred.
template <bool kInd, int kThreads>
__global__ void __launch_bounds__(kThreads, kForceThreadsPerSM / kThreads)
    k_force_walk(SceneTable T, WalkCtx G, const float4 *__restrict__ vel,
                 const float4 *__restrict__ rp, const float4 *__restrict__ fr, NbrList L,
                 float4 *__restrict__ pos_out, float4 *__restrict__ vel_out,
                 float4 *__restrict__ force_out, const uint32_t *__restrict__ walk_warps,
                 uint32_t *__restrict__ deferred, uint32_t *__restrict__ status) {
    __shared__ RecordSmem<kInd> s_coop[kThreads / 32];
    if (status[0] & kStatusErrorMask) return;
    // each warp takes the next listed warp until none is left: clumps make
    // some walks far longer than others, so the work is handed out as it
    // goes; warps past the list's length have nothing to take
    const uint32_t m = status[kStatusWalkWarps], lane = threadIdx.x & 31u;
    if (((blockIdx.x * blockDim.x + threadIdx.x) >> 5) >= m) return;
#pragma unroll 1
    for (;;) {
        uint32_t q = 0;
        if (lane == 0) q = atomicAdd(&status[kStatusWalkNext], 1u);
        q = __shfl_sync(0xffffffffu, q, 0);
        if (q >= m) break;
        const uint32_t t = walk_warps[q] * 32u + lane;
        const bool valid = t < T.n;
        const uint32_t i = valid ? (kInd ? G.order[t] : t) : 0u;
        const bool walker = valid && L.count[i] > L.slots;
        const uint32_t sc = valid ? scene_of(T, i) : 0u;
        const StepParams &P = T.params[sc];
        const float4 pi = G.pos[i];
        const float4 vi = vel[i];
        const float4 r = rp[i];
        ForcePair pair{vi, r.y, P.h, P.forceKp, P.forceKv, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const WalkCtx W = walk_ctx(T, G, sc, P, status);
        WalkStart s;
        walk_start(W, P, pi, s);
        RecordScan<kInd> scan{s_coop[threadIdx.x >> 5], fr, pair};
        ForceVisitor v{pair, fr, pi};
        const CoopLane cl = coop_lane(walker, sc, W, s);
        defer_lanes(walker && !cl.fast, t, deferred, &status[kStatusDeferredForce]);
        coop_walk<kInd, true, kTailNone>(W, s, cl, i, pi, scan, v);
        if (cl.fast) force_finish(P, pair, i, pi, vi, r.x, pos_out, vel_out, force_out);
    }
}

// The particles k_force deferred, one warp each (warp_walk over the
// neighbour records).
template <bool kInd>
__global__ void __launch_bounds__(kDeferredThreads)
    k_force_deferred(SceneTable T, WalkCtx G, const float4 *__restrict__ vel,
                     const float4 *__restrict__ rp, const float4 *__restrict__ fr, NbrList L,
                     float4 *__restrict__ pos_out, float4 *__restrict__ vel_out,
                     float4 *__restrict__ force_out, const uint32_t *__restrict__ deferred,
                     const uint32_t *__restrict__ status) {
    if (status[0] & kStatusErrorMask) return;
    __shared__ RecordSmem<kInd> s_chunk[kDeferredThreads / 32];
    const uint32_t m = status[kStatusDeferredForce];
    const uint32_t lane = threadIdx.x & 31u, nw = gridDim.x * (kDeferredThreads / 32);
#pragma unroll 1
    for (uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; q < m; q += nw) {
        const uint32_t t = deferred[q];
        const uint32_t i = kInd ? G.order[t] : t;
        const uint32_t sc = scene_of(T, i);
        const StepParams &P = T.params[sc];
        const WalkCtx W = walk_ctx(T, G, sc, P, status);
        const float4 pi = W.pos[i];
        const float4 vi = vel[i];
        const float4 r = rp[i];
        ForcePair pair{vi, r.y, P.h, P.forceKp, P.forceKv, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        WalkStart s;
        walk_start(W, P, pi, s);
        RecordScan<kInd> scan{s_chunk[threadIdx.x >> 5], fr, pair};
        warp_walk<kInd>(W, s, i, pi, scan);
        if (lane == 0) force_finish(P, pair, i, pi, vi, r.x, pos_out, vel_out, force_out);
    }
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
    uint32_t tests;  // candidates whose r^2 the walk evaluated
    __device__ __forceinline__ void on_test() { ++tests; }
    __device__ __forceinline__ void operator()(uint32_t j, float, float, float, float) {
        ++count;
        sum += mix64(id[j]);
    }
};

constexpr int kDigestThreads = 256;

template <bool kInd>
__global__ void k_digest(SceneTable T, WalkCtx G, const uint32_t *__restrict__ id,
                         uint32_t *__restrict__ count_out, uint64_t *__restrict__ digest_out,
                         uint32_t *__restrict__ tests_out, const uint32_t *__restrict__ status) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if ((t & ~31u) >= T.n || (status[0] & kStatusErrorMask)) return;
    const bool valid = t < T.n;
    const uint32_t i = valid ? (kInd ? G.order[t] : t) : 0u;
    const uint32_t sc = valid ? scene_of(T, i) : 0u;
    const StepParams &P = T.params[sc];
    const WalkCtx W = walk_ctx(T, G, sc, P, status);
    const float4 pi = W.pos[i];
    WalkStart s;
    walk_start(W, P, pi, s);
    DigestVisitor v{id, 0u, 0ull, 0u};
    // the same walk as k_density's
    __shared__ PosSmem<kInd> s_coop[kDigestThreads / 32];
    PosScan<kInd, DigestVisitor> scan{s_coop[threadIdx.x >> 5], v};
    coop_walk<kInd, false, kTailAll>(W, s, coop_lane(valid, sc, W, s), i, pi, scan, v);
    if (!valid) return;
    const uint32_t d = T.pofs[sc] + id[i];
    count_out[d] = v.count;
    digest_out[d] = v.sum;
    if (tests_out) tests_out[d] = v.tests;
}

// Rows [first, first + n) from host-ordered staging arrays (vel3 all zero
// or uploaded).  Without keep_order, row first + i takes particle i and its
// id becomes i (scene-local).  With keep_order, every row keeps its particle
// (id[row]) and takes that particle's values: the storage stays in the cell
// order of the last step, so the next step's sort and gather find it sorted.
// keep_order holds only while no step stopped on an error since the last
// upload (status word 0 clear): such a step leaves the ids behind the data.
// With `bad` set, a position that is non-finite or whose cell quotient x / h
// is 2^30 or more in magnitude (the host check of a new scene, done here for
// state replacements) lowers *bad to first + its particle index.
__global__ void k_upload_rows(uint32_t first, uint32_t n, const float *__restrict__ pos3,
                              const float *__restrict__ vel3, float4 *__restrict__ pos,
                              float4 *__restrict__ vel, uint32_t *__restrict__ id, float h,
                              uint32_t *__restrict__ bad, bool keep_order,
                              const uint32_t *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keep_order = keep_order && !(status[0] & kStatusErrorMask);
    const uint32_t r = first + i;
    // the particle (index into the staging arrays); an id outside the scene
    // (never, while the ids are a permutation) falls back to the row's index
    uint32_t d = i;
    if (keep_order) {
        const uint32_t k = id[r];
        d = k < n ? k : i;
    }
    const float x = pos3[3 * d], y = pos3[3 * d + 1], z = pos3[3 * d + 2];
    if (bad) {
        const bool ok = in_domain(__fdiv_rn(x, h)) && in_domain(__fdiv_rn(y, h)) &&
                        in_domain(__fdiv_rn(z, h));  // NaN and inf fail the bound too
        if (!ok) atomicMin(bad, first + d);
    }
    pos[r] = make_float4(x, y, z, 0.f);
    vel[r] = make_float4(vel3[3 * d], vel3[3 * d + 1], vel3[3 * d + 2], 0.f);
    if (!keep_order) id[r] = i;
}

// The dam-break lattice of sphx_lattice (host, sphx_host.cpp) generated in
// place: same SplitMix64 counters and the same float operations in the same
// order, so rows are bit-identical to the host generator's.  Velocity 0.
__global__ void k_lattice_rows(uint32_t first, LatticeGen L, float4 *__restrict__ pos,
                               float4 *__restrict__ vel, uint32_t *__restrict__ id) {
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = L.nx * L.ny * L.nz;
    if (idx >= n) return;
    const uint32_t k = idx / (L.nx * L.ny), rem = idx - k * L.nx * L.ny;
    const uint32_t j = rem / L.nx, i = rem - j * L.nx;
    const uint32_t ijk[3] = {i, j, k};
    float out[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        uint64_t z = L.seed + (3ull * idx + (uint64_t)a) * 0x9E3779B97F4A7C15ull + 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        const float u = __fmul_rn(__ull2float_rn(z >> 40), 5.9604644775390625e-08f);  // 2^-24
        const float jit = __fmul_rn(__fsub_rn(__fmul_rn(u, 2.0f), 1.0f), L.jitter);
        const float base = __fadd_rn(L.origin[a], __fmul_rn(__uint2float_rn(ijk[a]), L.spacing));
        out[a] = __fadd_rn(base, jit);
    }
    const uint32_t r = first + idx;
    pos[r] = make_float4(out[0], out[1], out[2], 0.f);
    vel[r] = make_float4(0.f, 0.f, 0.f, 0.f);
    id[r] = idx;
}

// One scene's rows [first, first + n) to staging in scene-local id order.
// field: 0 pos, 1 vel, 2 force, 3 rho, 4 prs.
__global__ void k_read_rows(uint32_t first, uint32_t n, int field, const uint32_t *__restrict__ id,
                            const float4 *__restrict__ v4, const float4 *__restrict__ rp,
                            float *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t r = first + i;
    const uint32_t d = id[r];
    if (field <= 2) {
        const float4 v = v4[r];
        out[3 * d] = v.x;
        out[3 * d + 1] = v.y;
        out[3 * d + 2] = v.z;
    } else {
        const float4 q = rp[r];
        out[d] = field == 3 ? q.x : q.y;
    }
}

// Field readout in id order: 3 floats per particle for vec fields, 1 for
// scalars.  field: 0 pos, 1 vel, 2 force, 3 rho, 4 prs.
__global__ void k_read_field(SceneTable T, int field, const uint32_t *__restrict__ id,
                             const float4 *__restrict__ v4, const float4 *__restrict__ rp,
                             float *__restrict__ out, const uint32_t *__restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // after a failed step the ids need not be a permutation: write nothing
    if (i >= T.n || (status[0] & kStatusErrorMask)) return;
    const uint32_t sc = scene_of(T, i);
    const uint32_t first = T.pofs[sc], local = id[i];
    if (local >= T.pofs[sc + 1] - first) return;
    const uint32_t d = first + local;
    if (field <= 2) {
        const float4 v = v4[i];
        out[3 * d] = v.x;
        out[3 * d + 1] = v.y;
        out[3 * d + 2] = v.z;
    } else {
        const float4 q = rp[i];
        out[d] = field == 3 ? q.x : q.y;
    }
}

// translate(position) * scale(h/2) (sph.cpp:178-179), column-major, id order.
// GLM's product leaves exact zeros off the diagonal and adds +0 to the
// translation (so -0 reads back as +0).
__global__ void k_transforms(SceneTable T, const uint32_t *__restrict__ id,
                             const float4 *__restrict__ pos, float4 *__restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T.n) return;
    const uint32_t sc = scene_of(T, i);
    const float half_h = T.params[sc].halfH;
    const float4 p = pos[i];
    float4 *m = out + 4 * ((size_t)T.pofs[sc] + id[i]);
    m[0] = make_float4(half_h, 0.f, 0.f, 0.f);
    m[1] = make_float4(0.f, half_h, 0.f, 0.f);
    m[2] = make_float4(0.f, 0.f, half_h, 0.f);
    m[3] = make_float4(__fadd_rn(p.x, 0.f), __fadd_rn(p.y, 0.f), __fadd_rn(p.z, 0.f), 1.f);
}

// Cell (truncated quotient) and stored uint16 hash per particle, id order.
__global__ void k_cells(SceneTable T, const uint32_t *__restrict__ id,
                        const float4 *__restrict__ pos, int *__restrict__ cells,
                        uint16_t *__restrict__ hash) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= T.n) return;
    const uint32_t sc = scene_of(T, i);
    const CellPos c = cell_pos(pos[i], T.params[sc].h);
    const uint32_t d = T.pofs[sc] + id[i];
    if (cells) {
        cells[3 * d] = c.cx;
        cells[3 * d + 1] = c.cy;
        cells[3 * d + 2] = c.cz;
    }
    if (hash) hash[d] = (uint16_t)hash16(c.cx, c.cy, c.cz);
}

// The reference's 60-byte Particle record (Particle.h:4-10): four vec3, two
// floats and the uint16 hash (plus 2 bytes of tail padding).
struct ParticleRec {
    float pos[3], vel[3], acc[3], force[3];
    float density, pressure;
    uint16_t hash;
    uint16_t pad;
};
static_assert(sizeof(ParticleRec) == 60, "Particle layout");

// AoS -> resident SoA (id = record index).  hash_pre keeps hash16 of each
// record's pre-step cell, which the reference's GPU path leaves in the
// record (sphGPU.cu:31-40 runs before the positions move).
__global__ void k_aos_unpack(uint32_t n, float h, const ParticleRec *__restrict__ rec,
                             float4 *__restrict__ pos, float4 *__restrict__ vel,
                             uint32_t *__restrict__ id, uint16_t *__restrict__ hash_pre) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const ParticleRec &r = rec[i];
    const float4 p = make_float4(r.pos[0], r.pos[1], r.pos[2], 0.f);
    pos[i] = p;
    vel[i] = make_float4(r.vel[0], r.vel[1], r.vel[2], 0.f);
    id[i] = i;
    const CellPos c = cell_pos(p, h);
    hash_pre[i] = (uint16_t)hash16(c.cx, c.cy, c.cz);
}

// Resident SoA -> AoS records in the caller's order, plus the instanced
// renderer's transforms; `acceleration` (never written by the reference) is
// left as the caller passed it.
__global__ void k_aos_pack(uint32_t n, float half_h, ParticleRec *__restrict__ rec,
                           const uint32_t *__restrict__ id, const float4 *__restrict__ pos,
                           const float4 *__restrict__ vel, const float4 *__restrict__ force,
                           const float4 *__restrict__ rp, const uint16_t *__restrict__ hash_pre,
                           float4 *__restrict__ transforms) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t d = id[i];
    ParticleRec &r = rec[d];
    const float4 p = pos[i], v = vel[i], f = force[i];
    const float4 q = rp[i];
    r.pos[0] = p.x; r.pos[1] = p.y; r.pos[2] = p.z;
    r.vel[0] = v.x; r.vel[1] = v.y; r.vel[2] = v.z;
    r.force[0] = f.x; r.force[1] = f.y; r.force[2] = f.z;
    r.density = q.x;
    r.pressure = q.y;
    r.hash = hash_pre[d];
    if (transforms) {
        float4 *m = transforms + 4 * (size_t)d;
        m[0] = make_float4(half_h, 0.f, 0.f, 0.f);
        m[1] = make_float4(0.f, half_h, 0.f, 0.f);
        m[2] = make_float4(0.f, 0.f, half_h, 0.f);
        m[3] = make_float4(__fadd_rn(p.x, 0.f), __fadd_rn(p.y, 0.f), __fadd_rn(p.z, 0.f), 1.f);
    }
}

inline unsigned blocks(uint32_t n, unsigned bs) { return (n + bs - 1) / bs; }

}  // namespace

// ---------------------------------------------------------------- launchers

cudaError_t launch_sort(const SceneTable &T, const SortBuffers &B, const float4 *pos,
                        cudaStream_t st) {
    const unsigned bs = 256;
    const uint32_t n = T.n;
    const uint32_t m = B.slots + 1;  // count[slots] stays 0 -> start[slots] = n
    const uint32_t ntiles = (m + kScanTile - 1) / kScanTile;
    cudaMemsetAsync(B.status + 1, 0, 8, st);  // x-wrap flag, large-cell count
    if (n) k_keys<<<blocks(n, bs), bs, 0, st>>>(T, pos, B.key, B.rank, B.count, B.status);
    k_scan_tiles<<<ntiles, kScanThreads, 0, st>>>(B.count, m, B.tile_sum, B.max_cell, B.status);
    if (ntiles <= kSelfPrefixTiles) {
        k_scan_apply<true><<<ntiles, kScanThreads, 0, st>>>(B.count, m, B.tile_sum, B.start);
    } else {
        k_scan_tile_sums<<<1, kScanThreads, 0, st>>>(B.tile_sum, ntiles);
        k_scan_apply<false><<<ntiles, kScanThreads, 0, st>>>(B.count, m, B.tile_sum, B.start);
    }
    if (n) {
        k_scatter<<<blocks(n, bs), bs, 0, st>>>(n, pos, B.key, B.rank, B.start, B.scat, B.status);
        k_cellsort<<<blocks(n, bs), bs, 0, st>>>(n, B.key, B.rank, B.scat, B.order,
                                                 B.status, B.large, B.large_cap);
        k_cellsort_large<<<kLargeBlocks, 512, 8 * kLargeCell, st>>>(B.scat, B.order, B.status,
                                                                    B.large, B.large_cap);
    }
    return cudaGetLastError();
}

cudaError_t launch_cell_flags(const SceneTable &T, uint32_t slots, uint8_t *cflags,
                              cudaStream_t st) {
    if (slots) k_cell_flags<<<blocks(slots, 256), 256, 0, st>>>(T, slots, cflags);
    return cudaGetLastError();
}

// The force list kernel uses no shared memory and is bound by L1 throughput
// on the neighbour records: all of the SM's L1 as cache (carveout 0) took it
// from 0.268 to 0.261 ms at 2.1M particles.  The density kernel gained
// nothing either way (it keeps the driver's choice).
constexpr int kForceCarveout = 0;

// Preferred shared-memory share of an SM's L1 for a kernel (percent of the
// maximum; -1 leaves the driver's choice).
template <class K>
static cudaError_t carveout(K *kernel, int percent) {
    return percent < 0 ? cudaSuccess
                       : cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                              percent);
}

cudaError_t prepare_device() {
    cudaError_t e = cudaFuncSetAttribute(k_cellsort_large, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         8 * kLargeCell);
    if (e == cudaSuccess) e = carveout(k_force<false, 128>, kForceCarveout);
    if (e == cudaSuccess) e = carveout(k_force<true, 128>, kForceCarveout);
    if (e == cudaSuccess) e = carveout(k_force<false, 256>, kForceCarveout);
    if (e == cudaSuccess) e = carveout(k_force<true, 256>, kForceCarveout);
    return e;
}

cudaError_t launch_gather(uint32_t n, const SortBuffers &B, const float4 *pos_in,
                          const float4 *vel_in, const uint32_t *id_in, float4 *pos_out,
                          float4 *vel_out, uint32_t *id_out, cudaStream_t st) {
    if (n) k_gather<<<blocks(n, 256), 256, 0, st>>>(n, B.order, pos_in, vel_in, id_in, pos_out,
                                                    vel_out, id_out, B.status);
    return cudaGetLastError();
}

static WalkCtx global_ctx(const SortBuffers &B, const float4 *pos) {
    WalkCtx W{};
    W.pos = pos;
    W.order = B.order;
    W.start = B.start;
    W.xmono = true;
    W.cflags = B.cflags;
    return W;
}

template <int kThreads>
static void density_launch(const SceneTable &T, const WalkCtx &G, const float4 *vel, float4 *rp,
                           float4 *fr, const NbrList &L, const RowWarps &RW, bool indirect,
                           uint32_t *deferred, uint32_t *status, cudaStream_t st) {
    const uint32_t threads = launch_threads(T);
    if (indirect) {
        k_density<true, kThreads><<<blocks(threads, kThreads), kThreads, 0, st>>>(
            T, G, vel, rp, fr, L, RW, deferred, status);
        k_density_deferred<true><<<kDeferredBlocks, kDeferredThreads, 0, st>>>(T, G, vel, rp, fr, L,
                                                                             deferred, status);
    } else {
        k_density<false, kThreads><<<blocks(threads, kThreads), kThreads, 0, st>>>(
            T, G, vel, rp, fr, L, RW, deferred, status);
        k_density_deferred<false><<<kDeferredBlocks, kDeferredThreads, 0, st>>>(T, G, vel, rp, fr, L,
                                                                              deferred, status);
    }
}

cudaError_t launch_density(const SceneTable &T, const SortBuffers &B, const float4 *pos,
                           const float4 *vel, float4 *rp, float4 *fr, const NbrList &L,
                           bool indirect, cudaStream_t st, int threads, const RowWarps &RW) {
    if (!T.rofs || !T.rows || !RW.wofs) return cudaErrorInvalidValue;
    const WalkCtx G = global_ctx(B, pos);
    if (T.n) {
        // rows + 1 scan entries; the sort's tile sums are free again
        const uint32_t ntiles = (T.rows + 1 + kScanTile - 1) / kScanTile;
        k_row_warps<<<ntiles, kScanThreads, 0, st>>>(T, B.start, RW.wofs, B.tile_sum, B.status);
        if (ntiles > 1) k_row_offsets<<<ntiles, kScanThreads, 0, st>>>(T.rows, RW.wofs, B.tile_sum);
        // both deferred counts, the walker warps' count and their next one
        cudaMemsetAsync(B.status + kStatusDeferred, 0, 16, st);
        if (threads == 128) density_launch<128>(T, G, vel, rp, fr, L, RW, indirect, B.deferred, B.status, st);
        else density_launch<256>(T, G, vel, rp, fr, L, RW, indirect, B.deferred, B.status, st);
    }
    return cudaGetLastError();
}

template <int kThreads>
static void force_launch(const SceneTable &T, const WalkCtx &G, const float4 *vel,
                         const float4 *rp, const float4 *fr, const NbrList &L, float4 *pos_out,
                         float4 *vel_out, float4 *force_out, bool indirect,
                         uint32_t *deferred, uint32_t *walk_warps, uint32_t *status,
                         cudaStream_t st) {
    // the walkers' kernel: as many warps as the GPU holds at once (or fewer)
    const unsigned walk_blocks =
        std::min<unsigned>(blocks(T.n, kThreads), 152u * (kForceThreadsPerSM / kThreads));
    if (indirect) {
        k_force<true, kThreads><<<blocks(T.n, kThreads), kThreads, 0, st>>>(
            T, G, vel, rp, fr, L, pos_out, vel_out, force_out, walk_warps, status);
        k_force_walk<true, kThreads><<<walk_blocks, kThreads, 0, st>>>(
            T, G, vel, rp, fr, L, pos_out, vel_out, force_out, walk_warps, deferred, status);
        k_force_deferred<true><<<kDeferredBlocks, kDeferredThreads, 0, st>>>(
            T, G, vel, rp, fr, L, pos_out, vel_out, force_out, deferred, status);
    } else {
        k_force<false, kThreads><<<blocks(T.n, kThreads), kThreads, 0, st>>>(
            T, G, vel, rp, fr, L, pos_out, vel_out, force_out, walk_warps, status);
        k_force_walk<false, kThreads><<<walk_blocks, kThreads, 0, st>>>(
            T, G, vel, rp, fr, L, pos_out, vel_out, force_out, walk_warps, deferred, status);
        k_force_deferred<false><<<kDeferredBlocks, kDeferredThreads, 0, st>>>(
            T, G, vel, rp, fr, L, pos_out, vel_out, force_out, deferred, status);
    }
}

cudaError_t launch_force(const SceneTable &T, const SortBuffers &B, const float4 *pos,
                         const float4 *vel, const float4 *rp, const float4 *fr, const NbrList &L,
                         float4 *pos_out, float4 *vel_out, float4 *force_out, bool indirect,
                         cudaStream_t st, int threads) {
    const WalkCtx G = global_ctx(B, pos);
    if (T.n) {
        if (threads == 128)
            force_launch<128>(T, G, vel, rp, fr, L, pos_out, vel_out, force_out, indirect,
                              B.deferred + T.n, B.deferred + 2 * (size_t)T.n, B.status, st);
        else
            force_launch<256>(T, G, vel, rp, fr, L, pos_out, vel_out, force_out, indirect,
                              B.deferred + T.n, B.deferred + 2 * (size_t)T.n, B.status, st);
    }
    return cudaGetLastError();
}

cudaError_t launch_digest(const SceneTable &T, const SortBuffers &B, const float4 *pos,
                          const uint32_t *id, uint32_t *count, uint64_t *digest, uint32_t *tests,
                          bool indirect, cudaStream_t st) {
    const WalkCtx G = global_ctx(B, pos);
    if (T.n) {
        if (indirect)
            k_digest<true><<<blocks(T.n, kDigestThreads), kDigestThreads, 0, st>>>(
                T, G, id, count, digest, tests, B.status);
        else
            k_digest<false><<<blocks(T.n, kDigestThreads), kDigestThreads, 0, st>>>(
                T, G, id, count, digest, tests, B.status);
    }
    return cudaGetLastError();
}

cudaError_t launch_upload_rows(uint32_t first, uint32_t n, const float *pos3, const float *vel3,
                               float4 *pos, float4 *vel, uint32_t *id, float h, uint32_t *bad,
                               bool keep_order, const uint32_t *status, cudaStream_t st) {
    if (n)
        k_upload_rows<<<blocks(n, 256), 256, 0, st>>>(first, n, pos3, vel3, pos, vel, id, h, bad,
                                                      keep_order && status, status);
    return cudaGetLastError();
}

cudaError_t launch_lattice_rows(uint32_t first, const LatticeGen &L, float4 *pos, float4 *vel,
                                uint32_t *id, cudaStream_t st) {
    const uint32_t n = L.nx * L.ny * L.nz;
    if (n) k_lattice_rows<<<blocks(n, 256), 256, 0, st>>>(first, L, pos, vel, id);
    return cudaGetLastError();
}

cudaError_t launch_read_rows(uint32_t first, uint32_t n, int field, const uint32_t *id,
                             const float4 *v4, const float4 *rp, float *out, cudaStream_t st) {
    if (n) k_read_rows<<<blocks(n, 256), 256, 0, st>>>(first, n, field, id, v4, rp, out);
    return cudaGetLastError();
}

cudaError_t launch_read_field(const SceneTable &T, int field, const uint32_t *id, const float4 *v4,
                              const float4 *rp, float *out, const uint32_t *status,
                              cudaStream_t st) {
    if (T.n) k_read_field<<<blocks(T.n, 256), 256, 0, st>>>(T, field, id, v4, rp, out, status);
    return cudaGetLastError();
}

cudaError_t launch_transforms(const SceneTable &T, const uint32_t *id, const float4 *pos,
                              float *out16, cudaStream_t st) {
    if (T.n)
        k_transforms<<<blocks(T.n, 256), 256, 0, st>>>(T, id, pos, reinterpret_cast<float4 *>(out16));
    return cudaGetLastError();
}

cudaError_t launch_cells(const SceneTable &T, const uint32_t *id, const float4 *pos, int *cells,
                         uint16_t *hash, cudaStream_t st) {
    if (T.n) k_cells<<<blocks(T.n, 256), 256, 0, st>>>(T, id, pos, cells, hash);
    return cudaGetLastError();
}

cudaError_t launch_aos_unpack(uint32_t n, float h, const void *rec, float4 *pos, float4 *vel,
                              uint32_t *id, uint16_t *hash_pre, cudaStream_t st) {
    if (n)
        k_aos_unpack<<<blocks(n, 256), 256, 0, st>>>(n, h, static_cast<const ParticleRec *>(rec),
                                                     pos, vel, id, hash_pre);
    return cudaGetLastError();
}

cudaError_t launch_aos_pack(uint32_t n, float half_h, void *rec, const uint32_t *id,
                            const float4 *pos, const float4 *vel, const float4 *force,
                            const float4 *rp, const uint16_t *hash_pre, float *transforms16,
                            cudaStream_t st) {
    if (n)
        k_aos_pack<<<blocks(n, 256), 256, 0, st>>>(n, half_h, static_cast<ParticleRec *>(rec), id,
                                                   pos, vel, force, rp, hash_pre,
                                                   reinterpret_cast<float4 *>(transforms16));
    return cudaGetLastError();
}

}  // namespace sphx
