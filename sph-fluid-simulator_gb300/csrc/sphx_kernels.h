// Launchers of the SPH step kernels (sphx_kernels.cu).  Host code only sees
// these plain functions; every launch goes to the caller's stream and
// returns cudaGetLastError().
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sphx_common.h"

namespace sphx {

// Device scratch of the counting sort.  count has slots + 1 entries and is
// all-zero between steps (the scan clears it); start has slots + 1 entries.
struct SortBuffers {
    uint32_t *key;       // n: slot of each particle
    uint32_t *rank;      // n: arrival rank within its slot
    uint32_t *order;     // n: particle (data index) at each cell-sorted slot
    uint2 *scat;         // n: (particle, x bits) of each slot in arrival order
    uint32_t *count;     // slots + 1
    uint32_t *start;     // slots + 1
    uint32_t *tile_sum;  // ceil((slots + 1) / 4096)
    uint32_t *status;    // 2 words: error bits, x-wrap flag (see below)
    uint2 *large;        // cells longer than 64 queued for the block sort
    const uint8_t *cflags;  // slots: collision flags of each slot's own cell, or NULL
    uint32_t *deferred;  // 2n + n / 32 + 1: cell-sorted positions of the particles the
                         // density pass (first n) and the force pass (next n) defer,
                         // then the warps of the force pass that hold a walker
    uint32_t large_cap;  // entries of `large` (n / 64 + 2 suffices)
    uint32_t slots;      // gx * gy * gz
    uint32_t max_cell;   // occupancy above which a step refuses to walk (<= kLargeCell)
};

// Largest cell the step sorts (shared-memory bitonic sort of 8-byte keys) and
// the CTAs that share the queued large cells.
constexpr uint32_t kLargeCell = 16384;
constexpr unsigned kLargeBlocks = 152;
inline uint32_t large_list_cap(uint32_t n) { return n / 64 + 2; }

// status[0]: sticky error bits; status[1]: set during a step's sort when a
// particle lies outside the grid's x extent; status[2]: number of large
// cells queued (both cleared at each sort).
constexpr uint32_t kStatusDomainBit = 1u;    // non-finite or |x/h| >= 2^30
constexpr uint32_t kStatusOverflowBit = 2u;  // a cell above max_cell
constexpr uint32_t kStatusErrorMask = 3u;
// status[3]: first rejected row of an upload; status[4], status[5]:
// particles the density and force passes deferred to their per-particle
// companions; status[6]: warps of the force pass that hold a walker;
// status[7]: the next of those the walkers' kernel hands out (all four
// cleared before the density pass).
constexpr uint32_t kStatusDeferred = 4u;
constexpr uint32_t kStatusDeferredForce = 5u;
constexpr uint32_t kStatusWalkWarps = 6u;
constexpr uint32_t kStatusWalkNext = 7u;

cudaError_t launch_sort(const SceneTable &T, const SortBuffers &B, const float4 *pos,
                        cudaStream_t st);
// The collision flags (dup bit, six exact face bits) of every slot's own
// cell, for the walks' lookup; once per change of the scenes' grids.
cudaError_t launch_cell_flags(const SceneTable &T, uint32_t slots, uint8_t *cflags,
                              cudaStream_t st);
// Once per device before the first launch_sort (outside any stream capture):
// allows the large-cell sort its shared memory.
cudaError_t prepare_device();
cudaError_t launch_gather(uint32_t n, const SortBuffers &B, const float4 *pos_in,
                          const float4 *vel_in, const uint32_t *id_in, float4 *pos_out,
                          float4 *vel_out, uint32_t *id_out, cudaStream_t st);
// Accepted-neighbour lists the density kernel records for the force kernel,
// in tiles of 32 cell-sorted slots: entry k < min(count[i], slots) of the
// particle at slot t is nbr[(t / 32) * slots * 32 + (k / 4) * 128 +
// (t % 32) * 4 + k % 4] (nbr holds slots entries for every slot, n rounded
// up to 32), slots a multiple of 4; a count above `slots` means the force
// kernel walks for that particle.  nbr NULL: nothing is recorded (the
// density pass alone).
struct NbrList {
    uint32_t *nbr;
    uint32_t *count;
    uint32_t slots;
};
constexpr uint32_t kNbrSlotsDefault = 256, kNbrSlotsMax = 1024;

// The density pass's warps, each inside one cell row (see k_row_warps):
// wofs[R] = first warp of cell row R, rows + 1 entries.
struct RowWarps {
    uint32_t *wofs;
};

// fr: 2 float4 per particle, (x, y, z, p) and (vx, vy, vz, 1/rho), written
// by the density kernel when fr is set (vel then required).  Each warp of
// the pass takes particles of one cell row: T.rofs / T.rows describe the
// rows and rw.wofs receives their warp offsets (rows + 1 entries).
cudaError_t launch_density(const SceneTable &T, const SortBuffers &B, const float4 *pos,
                           const float4 *vel, float4 *rp, float4 *fr, const NbrList &L,
                           bool indirect, cudaStream_t st, int threads, const RowWarps &rw);
cudaError_t launch_force(const SceneTable &T, const SortBuffers &B, const float4 *pos,
                         const float4 *vel, const float4 *rp, const float4 *fr, const NbrList &L,
                         float4 *pos_out, float4 *vel_out, float4 *force_out, bool indirect,
                         cudaStream_t st, int threads = 256);
// Per particle (scene offset + id): accepted neighbour visits, their id
// fingerprint and, if tests is set, the candidates whose r^2 was evaluated.
cudaError_t launch_digest(const SceneTable &T, const SortBuffers &B, const float4 *pos,
                          const uint32_t *id, uint32_t *count, uint64_t *digest, uint32_t *tests,
                          bool indirect, cudaStream_t st);
// Rows [first, first + n) from host-ordered staging (scene-local ids), and
// back: one scene's rows to staging in its id order (field: 0 pos, 1 vel,
// 2 force, 3 rho, 4 prs).
// bad: NULL, or a device word lowered to first + the index of the first
// particle whose position is outside the walk's domain for cell size h.
// keep_order: rows keep their particles (id unchanged) unless the sticky
// error bits of status (word 0) are set, see k_upload_rows.
cudaError_t launch_upload_rows(uint32_t first, uint32_t n, const float *pos3, const float *vel3,
                               float4 *pos, float4 *vel, uint32_t *id, float h, uint32_t *bad,
                               bool keep_order, const uint32_t *status, cudaStream_t st);
// Dam-break lattice generated on the device into rows [first, first + n).
struct LatticeGen {
    uint32_t nx, ny, nz;
    float origin[3];
    float spacing, jitter;
    uint64_t seed;
};
cudaError_t launch_lattice_rows(uint32_t first, const LatticeGen &L, float4 *pos, float4 *vel,
                                uint32_t *id, cudaStream_t st);
cudaError_t launch_read_rows(uint32_t first, uint32_t n, int field, const uint32_t *id,
                             const float4 *v4, const float4 *rp, float *out, cudaStream_t st);
// All scenes' rows to staging in id order; writes nothing when the sticky
// error bits of status (word 0) are set, and skips a row whose id is out of
// its scene's range.
cudaError_t launch_read_field(const SceneTable &T, int field, const uint32_t *id, const float4 *v4,
                              const float4 *rp, float *out, const uint32_t *status,
                              cudaStream_t st);
cudaError_t launch_transforms(const SceneTable &T, const uint32_t *id, const float4 *pos,
                              float *out16, cudaStream_t st);
cudaError_t launch_cells(const SceneTable &T, const uint32_t *id, const float4 *pos, int *cells,
                         uint16_t *hash, cudaStream_t st);

// The reference's 60-byte Particle records (Particle.h:4-10) <-> resident state.
cudaError_t launch_aos_unpack(uint32_t n, float h, const void *rec, float4 *pos, float4 *vel,
                              uint32_t *id, uint16_t *hash_pre, cudaStream_t st);
cudaError_t launch_aos_pack(uint32_t n, float half_h, void *rec, const uint32_t *id,
                            const float4 *pos, const float4 *vel, const float4 *force,
                            const float4 *rp, const uint16_t *hash_pre, float *transforms16,
                            cudaStream_t st);

}  // namespace sphx
