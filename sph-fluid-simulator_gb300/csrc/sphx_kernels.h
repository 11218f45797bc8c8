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
    uint32_t *count;     // slots + 1
    uint32_t *start;     // slots + 1
    uint32_t *tile_sum;  // ceil((slots + 1) / 4096)
    uint32_t *status;    // 2 words: error bits, x-wrap flag (see below)
    uint32_t slots;      // gx * gy * gz
    uint32_t max_cell;   // occupancy above which a step refuses to walk
};

// status[0]: sticky error bits; status[1]: set during a step's sort when a
// particle lies outside the grid's x extent (cleared at each sort).
constexpr uint32_t kStatusDomainBit = 1u;    // non-finite or |x/h| >= 2^30
constexpr uint32_t kStatusOverflowBit = 2u;  // a cell above max_cell
constexpr uint32_t kStatusErrorMask = 3u;

cudaError_t launch_sort(const StepParams &P, const SortBuffers &B, const float4 *pos,
                        cudaStream_t st);
cudaError_t launch_gather(uint32_t n, const SortBuffers &B, const float4 *pos_in,
                          const float4 *vel_in, const uint32_t *id_in, float4 *pos_out,
                          float4 *vel_out, uint32_t *id_out, cudaStream_t st);
cudaError_t launch_density(const StepParams &P, const SortBuffers &B, const float4 *pos,
                           float4 *rp, bool indirect, cudaStream_t st);
cudaError_t launch_force(const StepParams &P, const SortBuffers &B, const float4 *pos,
                         const float4 *vel, const float4 *rp, float4 *pos_out, float4 *vel_out,
                         float4 *force_out, bool indirect, cudaStream_t st);
cudaError_t launch_digest(const StepParams &P, const SortBuffers &B, const float4 *pos,
                          const uint32_t *id, uint32_t *count, uint64_t *digest, bool indirect,
                          cudaStream_t st);
cudaError_t launch_upload(uint32_t n, const float *pos3, const float *vel3, float4 *pos,
                          float4 *vel, uint32_t *id, cudaStream_t st);
cudaError_t launch_read_field(uint32_t n, int field, const uint32_t *id, const float4 *v4,
                              const float4 *rp, float *out, cudaStream_t st);
cudaError_t launch_transforms(uint32_t n, float half_h, const uint32_t *id, const float4 *pos,
                              float *out16, cudaStream_t st);
cudaError_t launch_cells(uint32_t n, float h, const uint32_t *id, const float4 *pos, int *cells,
                         uint16_t *hash, cudaStream_t st);

// The reference's 60-byte Particle records (Particle.h:4-10) <-> resident state.
cudaError_t launch_aos_unpack(uint32_t n, float h, const void *rec, float4 *pos, float4 *vel,
                              uint32_t *id, uint16_t *hash_pre, cudaStream_t st);
cudaError_t launch_aos_pack(uint32_t n, float half_h, void *rec, const uint32_t *id,
                            const float4 *pos, const float4 *vel, const float4 *force,
                            const float4 *rp, const uint16_t *hash_pre, float *transforms16,
                            cudaStream_t st);

}  // namespace sphx
