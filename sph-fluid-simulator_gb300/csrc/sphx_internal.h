// Internals shared by the host translation units of libsphx: the handle (one
// or many resident scenes), error reporting and the step sequence.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "sphx.h"
#include "sphx_common.h"
#include "sphx_kernels.h"

namespace sphx {

// Records msg as the calling thread's last error and returns code.
int fail(int code, const std::string &msg);

#define SPHX_CUDA(call)                                                                         \
    do {                                                                                        \
        const cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess)                                                                  \
            return ::sphx::fail(SPHX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

Derived derive_constants(float mass, float restDensity, float gasConst, float viscosity, float h,
                         float g, float tension);

// Block sizes of the two walk kernels and the reorder interval.
struct Tuning {
    int density_threads = 128;
    int force_threads = 128;
    int reorder_interval = 1;
};

struct GraphEntry {
    bool reorder;
    int pv, idc;
    Tuning tune;
    cudaGraphExec_t exec;
};

// One scene of a handle: particles [first, first + n) and grid slots
// [slot0, slot0 + slots) of the concatenated buffers.
struct Scene {
    sphx_settings s;
    Derived d;
    sphx_box box;
    Grid grid;
    uint32_t n, first, slots, slot0;
};

}  // namespace sphx

struct sphx_handle {
    sphx_options opt{};
    std::vector<sphx::Scene> scenes;
    uint32_t n = 0;      // particles of all scenes
    uint32_t slots = 0;  // grid slots of all scenes
    uint32_t cap_n = 0, cap_slots = 0, cap_scenes = 0;  // arena capacities
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // host <-> device copies of sphx_set_state / sphx_read_state, beside the
    // kernels on `stream`; both streams are idle when either call returns
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_kernels = nullptr, ev_copies = nullptr;
    char *arena = nullptr;
    float4 *pos[2] = {nullptr, nullptr};
    float4 *vel[2] = {nullptr, nullptr};
    uint32_t *id[2] = {nullptr, nullptr};  // scene-local particle ids
    float4 *rp = nullptr;                  // density, pressure, 1/density, 0
    float4 *force = nullptr;
    float4 *fr = nullptr;         // 32-byte neighbour records (density -> force)
    uint32_t *nbr = nullptr;      // accepted-neighbour lists (tiles of 32 slots, see sphx_kernels.h)
    uint32_t *ncount = nullptr;   // accepted-neighbour count per particle
    float *staging = nullptr;     // 6 floats per particle of capacity
    float *transforms = nullptr;  // 16 floats per particle, allocated on first use
    size_t transforms_cap = 0;
    sphx::SortBuffers sb{};
    sphx::StepParams *d_params = nullptr;  // one entry per scene
    uint32_t *d_pofs = nullptr;            // scenes + 1 particle offsets
    uint32_t *d_sofs = nullptr;            // scenes + 1 slot offsets
    uint32_t *d_rofs = nullptr;            // scenes + 1 cell-row offsets
    uint32_t rows = 0;                     // cell rows of all scenes
    sphx::RowWarps row_warps{};            // density warps aligned to cell rows
    std::vector<sphx::StepParams> params;  // last uploaded table
    float params_dt = 0.f;
    bool params_valid = false;
    sphx::Tuning tune;
    uint32_t *h_status = nullptr;  // pinned
    int pv = 0, idc = 0;
    uint64_t step_count = 0;
    int error = 0;
    bool profiling = false;
    std::vector<cudaEvent_t> events;  // 4 per profiled step
    std::vector<uint32_t> launches_per_step;
    size_t events_used = 0;
    sphx_kernel_times acc{};
    std::vector<sphx::GraphEntry> graphs;
};

namespace sphx {

inline SceneTable table_of(const sphx_handle *h) {
    return SceneTable{h->d_params, h->d_pofs,  h->d_sofs, (uint32_t)h->scenes.size(), h->n,
                      h->d_rofs,   h->rows};
}

// A scene to place in a handle: host state (pos3/vel3, vel3 may be NULL),
// or a scene already resident in `src` (kept through a relayout).
struct SceneInit {
    sphx_settings s;
    sphx_box box;
    uint32_t n;
    const float *pos3;
    const float *vel3;
    int keep;  // >= 0: index of a scene of the current layout to keep
    // keep >= 0 and resettle: keep the particles, replace settings, box and grid
    bool resettle;
    Grid grid;
    // keep < 0 and lattice set: generate the positions on the device
    const sphx_lattice_desc *lattice;
};

// Validates and creates a handle for the given scenes.
int create_handle(const SceneInit *scenes, size_t nscenes, const sphx_options *opt,
                  sphx_handle **out);
// Replaces the handle's scene list: kept scenes move (device to device) to
// their new ranges, new scenes are uploaded; capacity grows as needed.
int relayout(sphx_handle *h, const std::vector<SceneInit> &scenes);
// Copies scene `sc`'s state to host arrays (scene-local id order; any NULL).
int read_scene(sphx_handle *h, size_t sc, float *pos3, float *vel3, float *rho, float *prs,
               float *force3);
int ensure_params(sphx_handle *h, float dt);
int run_steps(sphx_handle *h, float dt, int nsteps);
int read_status(sphx_handle *h);
void destroy_graphs(sphx_handle *h);

}  // namespace sphx
