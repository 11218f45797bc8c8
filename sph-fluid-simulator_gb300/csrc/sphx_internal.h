// Internals shared by the host translation units of libsphx: the scene
// handle, error reporting and the step sequence.
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

#define SPHX_CUDA(call)                                                                  \
    do {                                                                                 \
        const cudaError_t e_ = (call);                                                   \
        if (e_ != cudaSuccess)                                                           \
            return ::sphx::fail(SPHX_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

Derived derive_constants(float mass, float restDensity, float gasConst, float viscosity, float h,
                         float g, float tension);

struct GraphEntry {
    bool reorder;
    int pv, idc;
    uint32_t dt_bits;
    cudaGraphExec_t exec;
};

}  // namespace sphx

struct sphx_handle {
    sphx_settings s;
    sphx::Derived d;
    sphx_box box;
    sphx_options opt;
    uint32_t n = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    sphx::Grid grid{};
    char *arena = nullptr;
    float4 *pos[2] = {nullptr, nullptr};
    float4 *vel[2] = {nullptr, nullptr};
    uint32_t *id[2] = {nullptr, nullptr};
    float4 *rp = nullptr;  // density, pressure, 1/density, 0
    float4 *force = nullptr;
    float *staging = nullptr;     // 6n floats
    float *transforms = nullptr;  // 16n floats, allocated on first use
    sphx::SortBuffers sb{};
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

// Enqueues nsteps steps (graph, profiled or plain launches).
int run_steps(sphx_handle *h, float dt, int nsteps);
// Synchronises and converts kernel-raised status bits into an error.
int read_status(sphx_handle *h);

}  // namespace sphx
