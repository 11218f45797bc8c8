// sphx_density_static: density and pressure of caller-owned device positions
// without allocating anything.
//
// Some callers of this library cannot allocate device memory when they need
// a result: a render or game-engine plugin that runs inside a frame with a
// fixed GPU memory budget, or a host that hands the library device buffers
// but does not let it call cudaMalloc (or any allocating routine) on its
// behalf.  For them this entry point keeps every scratch buffer the density
// pass needs (sort keys, ranks, cell order, the cell-grid counts and starts,
// scan tile sums, the status word, the per-row warp offsets and the
// per-particle (rho, p, 1/rho) record) in one file-scope __device__ array of
// fixed size.  The caller
// passes the inputs (positions) and outputs (density, pressure) as device
// pointers; nothing is allocated or freed, by this code or by a library it
// calls.
//
// Limits and sharing:
//   * at most kMaxParticles (131,072) particles per call; more is rejected
//     with SPHX_ERR_INVALID;
//   * the array (about 7 MiB) lives in every GPU that loads the library
//     until the process exits;
//   * every call on a device uses the same array, which keeps the previous
//     call's contents: the counts and status words are cleared at the start
//     of each call, and two calls whose work overlaps on the GPU race on the
//     array (serialise them, e.g. on one stream);
//   * a call synchronises its stream and reads a status word back, so it
//     cannot be made while that stream is being captured into a CUDA graph;
//   * the array's device address is looked up (cudaGetSymbolAddress) with
//     the device current, the first time a call runs in a given CUDA context
//     of that device, and cached with that context: a call made in another
//     context of the same device (after cudaDeviceReset, or a context a
//     driver-API host made current) looks it up again.
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <mutex>
#include <string>

#include "sphx_internal.h"

namespace {

constexpr uint32_t kMaxParticles = 1u << 17;
constexpr int kGridDim = 64;  // modular 64^3 cell grid: exact for any extent (aliasing only slows)
constexpr int kGridOrigin = -32;  // cells -32..31 on each axis map without wrapping
constexpr uint32_t kSlots = (uint32_t)kGridDim * kGridDim * kGridDim;
constexpr uint32_t kTiles = (kSlots + 1 + 4095) / 4096;
constexpr int kMaxDevices = 64;

// Byte offsets of the scratch buffers inside the array (all 256-aligned).
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kOffKey = 0;
constexpr size_t kOffRank = kOffKey + align256(4ull * kMaxParticles);
constexpr size_t kOffOrder = kOffRank + align256(4ull * kMaxParticles);
constexpr size_t kOffCount = kOffOrder + align256(4ull * kMaxParticles);
constexpr size_t kOffStart = kOffCount + align256(4ull * (kSlots + 1));
constexpr size_t kOffTiles = kOffStart + align256(4ull * (kSlots + 1));
constexpr size_t kOffStatus = kOffTiles + align256(4ull * kTiles);
constexpr size_t kOffTable = kOffStatus + 256;  // StepParams + particle / slot offsets
constexpr size_t kOffRp = kOffTable + 1024;
constexpr size_t kOffLarge = kOffRp + 16ull * kMaxParticles;  // queued large cells
constexpr size_t kOffScat = kOffLarge + align256(8ull * (kMaxParticles / 64 + 2));
constexpr size_t kOffDeferred = kOffScat + 8ull * kMaxParticles;
constexpr uint32_t kRows = (uint32_t)kGridDim * kGridDim;  // cell rows of the grid
constexpr size_t kOffRowWarps = kOffDeferred + align256(4ull * kMaxParticles);
constexpr size_t kScratchBytes = kOffRowWarps + align256(4ull * (kRows + 1));
static_assert(sizeof(sphx::StepParams) + 24 <= 1024, "scene table fits its scratch slot");

static __device__ __align__(256) uint4 g_scratch[kScratchBytes / sizeof(uint4)];

std::mutex g_mu;
// Per device: the context the cached address belongs to, and the address.
void *g_ctx[kMaxDevices] = {};
char *g_addr[kMaxDevices] = {};

// The calling thread's current CUDA context (the driver's cuCtxGetCurrent,
// reached through the runtime so that the library does not link the driver
// library itself), or NULL when it cannot be determined.
void *current_context() {
    using GetCurrent = int (*)(void **);
    static GetCurrent fn = [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            f = nullptr;
        }
        return reinterpret_cast<GetCurrent>(f);
    }();
    void *ctx = nullptr;
    if (!fn || fn(&ctx) != 0) return nullptr;
    return ctx;
}

// Device address of g_scratch in the current context of the current device.
// It is looked up (and the device's kernels prepared) once per context, and
// cached only once both succeeded.
int scratch_address(char **out) {
    int dev = 0;
    SPHX_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return sphx::fail(SPHX_ERR_CUDA, "device ordinal out of range");
    void *ctx = current_context();  // NULL before the runtime made one current
    std::lock_guard<std::mutex> lock(g_mu);
    if (ctx && g_ctx[dev] == ctx && g_addr[dev]) {
        *out = g_addr[dev];
        return SPHX_OK;
    }
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess)
        return sphx::fail(SPHX_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    const cudaError_t e2 = sphx::prepare_device();
    if (e2 != cudaSuccess)
        return sphx::fail(SPHX_ERR_CUDA, std::string("prepare_device: ") + cudaGetErrorString(e2));
    // the lookup made the device's primary context current if none was;
    // without a context handle nothing is cached and the next call looks up
    ctx = current_context();
    g_ctx[dev] = ctx;
    g_addr[dev] = ctx ? static_cast<char *>(p) : nullptr;
    *out = static_cast<char *>(p);
    return SPHX_OK;
}

__global__ void k_split_rho_prs(uint32_t n, const float4 *__restrict__ rp, float *__restrict__ rho,
                                float *__restrict__ prs) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 q = rp[i];
    rho[i] = q.x;
    prs[i] = q.y;
}

}  // namespace

extern "C" int sphx_density_static(const sphx_settings *s, const void *d_pos4, size_t n,
                                   float *d_rho, float *d_prs, void *stream) {
    using sphx::fail;
    if (!s || !d_pos4 || !d_rho || !d_prs) return fail(SPHX_ERR_INVALID, "null argument");
    if (n == 0 || n > kMaxParticles)
        return fail(SPHX_ERR_INVALID, "sphx_density_static: particle count " + std::to_string(n) +
                                          " outside [1, " + std::to_string(kMaxParticles) +
                                          "], the size of its static scratch");
    if (!(s->h > 0.f) || !std::isfinite(s->h)) return fail(SPHX_ERR_INVALID, "h must be finite and > 0");
    char *base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    const sphx::Derived d = sphx::derive_constants(s->mass, s->rest_density, s->gas_const,
                                                   s->viscosity, s->h, s->g, s->tension);
    sphx::StepParams P{};
    P.h = d.h;
    P.h2 = d.h2;
    P.mp6 = d.massPoly6Product;
    P.selfDens = d.selfDens;
    P.gasConstant = d.gasConstant;
    P.restDensity = d.restDensity;
    P.mass = d.mass;
    P.halfH = d.h / 2.f;
    P.h2w = d.h * d.h * (1.0f + 3.814697265625e-06f);
    P.grid = sphx::Grid{kGridOrigin, kGridOrigin, kGridOrigin, kGridDim, kGridDim, kGridDim};
    P.n = (uint32_t)n;
    // the one-scene table lives in the static array too: params, pofs {0, n},
    // sofs {0, slots}, rofs {0, rows}
    struct {
        sphx::StepParams p;
        uint32_t pofs[2];
        uint32_t sofs[2];
        uint32_t rofs[2];
    } tbl = {P, {0u, (uint32_t)n}, {0u, kSlots}, {0u, kRows}};
    char *dtbl = base + kOffTable;
    sphx::SceneTable T{reinterpret_cast<const sphx::StepParams *>(dtbl),
                       reinterpret_cast<const uint32_t *>(dtbl + offsetof(decltype(tbl), pofs)),
                       reinterpret_cast<const uint32_t *>(dtbl + offsetof(decltype(tbl), sofs)),
                       1u, (uint32_t)n};
    T.rofs = reinterpret_cast<const uint32_t *>(dtbl + offsetof(decltype(tbl), rofs));
    T.rows = kRows;
    const sphx::RowWarps RW{reinterpret_cast<uint32_t *>(base + kOffRowWarps)};

    sphx::SortBuffers B;
    B.key = reinterpret_cast<uint32_t *>(base + kOffKey);
    B.rank = reinterpret_cast<uint32_t *>(base + kOffRank);
    B.order = reinterpret_cast<uint32_t *>(base + kOffOrder);
    B.scat = reinterpret_cast<uint2 *>(base + kOffScat);
    B.count = reinterpret_cast<uint32_t *>(base + kOffCount);
    B.start = reinterpret_cast<uint32_t *>(base + kOffStart);
    B.tile_sum = reinterpret_cast<uint32_t *>(base + kOffTiles);
    B.status = reinterpret_cast<uint32_t *>(base + kOffStatus);
    B.large = reinterpret_cast<uint2 *>(base + kOffLarge);
    B.deferred = reinterpret_cast<uint32_t *>(base + kOffDeferred);
    B.cflags = nullptr;  // the walks compute the flags
    B.large_cap = kMaxParticles / 64 + 2;
    B.slots = kSlots;
    B.max_cell = sphx::kLargeCell;
    float4 *rp = reinterpret_cast<float4 *>(base + kOffRp);
    const float4 *pos = static_cast<const float4 *>(d_pos4);

    // The previous call's contents stay in the array: counts and status
    // must start from zero.
    SPHX_CUDA(cudaMemsetAsync(B.count, 0, 4ull * (kSlots + 1), st));
    SPHX_CUDA(cudaMemsetAsync(B.status, 0, 16, st));
    SPHX_CUDA(cudaMemcpyAsync(dtbl, &tbl, sizeof tbl, cudaMemcpyHostToDevice, st));
    SPHX_CUDA(sphx::launch_sort(T, B, pos, st));
    SPHX_CUDA(sphx::launch_density(T, B, pos, nullptr, rp, nullptr, sphx::NbrList{nullptr, nullptr, 0},
                                   /*indirect=*/true, st, 128, RW));
    k_split_rho_prs<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(P.n, rp, d_rho, d_prs);
    SPHX_CUDA(cudaGetLastError());

    uint32_t status = 0;
    SPHX_CUDA(cudaMemcpyAsync(&status, B.status, 4, cudaMemcpyDeviceToHost, st));
    SPHX_CUDA(cudaStreamSynchronize(st));
    if (status & sphx::kStatusDomainBit)
        return fail(SPHX_ERR_DOMAIN, "a position is non-finite or |x/h| >= 2^30");
    if (status & sphx::kStatusOverflowBit)
        return fail(SPHX_ERR_OVERFLOW, "a cell holds more than 16384 particles");
    return SPHX_OK;
}
