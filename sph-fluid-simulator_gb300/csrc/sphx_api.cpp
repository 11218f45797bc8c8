// C-ABI of the resident SPH step (include/sphx.h): handle lifetime, device
// memory layout, step orchestration (streams, CUDA graphs), readouts and
// host-side reference utilities.
//
// Replaces, behind the same call sequence, the reference's per-step path
// SPHSystem::update -> updateParticles -> updateParticlesCPU/GPU
// (src/SPHSystem.cpp:110-117, src/sph.cpp:195-290, src/kernels/sphGPU.cu:244-309).
// Where the reference copies the whole particle array to the device and back
// and cudaMallocs every step, a handle keeps its state in one device arena
// for its lifetime and a step is a fixed sequence of launches on one stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sphx_internal.h"

namespace {

thread_local std::string g_err;

uint64_t mix64(uint64_t z) {  // SplitMix64 output function of state z - gamma
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

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

namespace {

bool finite_args(const sphx_settings &s) {
    const float v[7] = {s.mass, s.rest_density, s.gas_const, s.viscosity, s.h, s.g, s.tension};
    for (float x : v)
        if (!std::isfinite(x)) return false;
    return s.h > 0.f;
}

int check_positions(const float *pos3, size_t n, float h) {
    for (size_t i = 0; i < 3 * n; ++i) {
        const float q = pos3[i] / h;
        if (!std::isfinite(pos3[i]) || !(std::fabs(q) < 1073741824.0f))
            return fail(SPHX_ERR_DOMAIN, "position " + std::to_string(i / 3) +
                                             " is non-finite or too far from the origin");
    }
    return SPHX_OK;
}

// Cell grid covering the walls and the initial particles, padded by two
// cells; dimensions are automatic unless the options fix them.
sphx::Grid choose_grid(const sphx_box &b, const sphx_options &o, float h, const float *pos3,
                       size_t n) {
    float lo[3] = {b.xmin, b.ymin, b.zmin}, hi[3] = {b.xmax, b.ymin, b.zmax};
    float plo[3] = {INFINITY, INFINITY, INFINITY}, phi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            plo[a] = std::min(plo[a], pos3[3 * i + a]);
            phi[a] = std::max(phi[a], pos3[3 * i + a]);
        }
    for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], plo[a]);
        hi[a] = std::max(hi[a], phi[a]);
    }
    if (b.has_ceiling) hi[1] = std::max(hi[1], b.ymax);
    else if (o.grid_ymax > b.ymin) hi[1] = std::max(hi[1], o.grid_ymax);
    else hi[1] = std::max(hi[1], phi[1] + 0.25f * (phi[1] - lo[1]) + 4.f * h);
    sphx::Grid g;
    int org[3], dim[3];
    for (int a = 0; a < 3; ++a) {
        const double c0 = std::floor((double)lo[a] / h) - 2.0, c1 = std::floor((double)hi[a] / h) + 2.0;
        org[a] = (int)c0;
        dim[a] = std::max(5, (int)(c1 - c0) + 1);
    }
    // Bound the slot count: past it, slots are shared modulo the grid (exact,
    // only slower where the occupied region wraps).
    const double cap = std::max(16.0 * (double)n, (double)(1 << 22));
    while ((double)dim[0] * dim[1] * dim[2] > cap) {
        int a = 0;
        if (dim[1] > dim[a]) a = 1;
        if (dim[2] > dim[a]) a = 2;
        if (dim[a] <= 5) break;
        dim[a] = std::max(5, dim[a] / 2);
    }
    if (o.grid_dims[0] > 0 && o.grid_dims[1] > 0 && o.grid_dims[2] > 0) {
        for (int a = 0; a < 3; ++a) {
            dim[a] = std::max(5, o.grid_dims[a]);
            org[a] = o.grid_origin[a];
        }
    }
    g.ox = org[0];
    g.oy = org[1];
    g.oz = org[2];
    g.gx = dim[0];
    g.gy = dim[1];
    g.gz = dim[2];
    return g;
}

sphx::StepParams make_params(const sphx_handle *h, float dt) {
    sphx::StepParams P;
    const sphx::Derived &d = h->d;
    P.h = d.h;
    P.h2 = d.h2;
    P.mp6 = d.massPoly6Product;
    P.selfDens = d.selfDens;
    P.gasConstant = d.gasConstant;
    P.restDensity = d.restDensity;
    P.mass = d.mass;
    P.viscosity = d.viscosity;
    P.spikyGrad = d.spikyGrad;
    P.spikyLap = d.spikyLap;
    P.g = d.g;
    P.halfH = d.h / 2.f;
    P.forceKp = 0.5f * d.mass * d.spikyGrad;
    P.forceKv = d.viscosity * d.mass * d.spikyLap;
    // sph.cpp:153-176: y < h, x < h - 8, x > -h + 8, z likewise.
    P.ylo = h->box.ymin + d.h;
    P.yhi = h->box.ymax - d.h;
    P.xlo = d.h + h->box.xmin;
    P.xhi = h->box.xmax - d.h;
    P.zlo = d.h + h->box.zmin;
    P.zhi = h->box.zmax - d.h;
    P.damping = h->box.damping;
    P.offset = h->box.offset;
    P.hasCeiling = h->box.has_ceiling;
    P.dt = dt;
    P.grid = h->grid;
    P.n = h->n;
    return P;
}

int upload(sphx_handle *h, const float *pos3, const float *vel3) {
    const size_t n = h->n;
    SPHX_CUDA(cudaMemcpyAsync(h->staging, pos3, 12 * n, cudaMemcpyHostToDevice, h->stream));
    if (vel3)
        SPHX_CUDA(cudaMemcpyAsync(h->staging + 3 * n, vel3, 12 * n, cudaMemcpyHostToDevice,
                                  h->stream));
    SPHX_CUDA(sphx::launch_upload(h->n, h->staging, vel3 ? h->staging + 3 * n : nullptr,
                                  h->pos[h->pv], h->vel[h->pv], h->id[h->idc], h->stream));
    SPHX_CUDA(cudaMemsetAsync(h->sb.status, 0, 8, h->stream));
    SPHX_CUDA(cudaMemsetAsync(h->rp, 0, 16 * n, h->stream));
    SPHX_CUDA(cudaMemsetAsync(h->force, 0, 16 * n, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    h->error = 0;
    return SPHX_OK;
}

// Enqueues one step starting from buffer parities (pv, idc); returns the
// parities after it.  Pure with respect to the handle, so that it can be
// captured into a graph.
cudaError_t enqueue_step(sphx_handle *h, const sphx::StepParams &P, bool reorder, int &pv,
                         int &idc, cudaEvent_t *ev) {
    cudaStream_t st = h->stream;
    cudaError_t e;
    if (ev) cudaEventRecord(ev[0], st);
    if ((e = sphx::launch_sort(P, h->sb, h->pos[pv], st)) != cudaSuccess) return e;
    if (reorder) {
        if ((e = sphx::launch_gather(P.n, h->sb, h->pos[pv], h->vel[pv], h->id[idc],
                                     h->pos[pv ^ 1], h->vel[pv ^ 1], h->id[idc ^ 1], st)) !=
            cudaSuccess)
            return e;
        pv ^= 1;
        idc ^= 1;
    }
    if (ev) cudaEventRecord(ev[1], st);
    if ((e = sphx::launch_density(P, h->sb, h->pos[pv], h->rp, !reorder, st)) != cudaSuccess)
        return e;
    if (ev) cudaEventRecord(ev[2], st);
    if ((e = sphx::launch_force(P, h->sb, h->pos[pv], h->vel[pv], h->rp, h->pos[pv ^ 1],
                                h->vel[pv ^ 1], h->force, !reorder, st)) != cudaSuccess)
        return e;
    if (ev) cudaEventRecord(ev[3], st);
    pv ^= 1;
    return cudaSuccess;
}

int read_status_impl(sphx_handle *h) {
    SPHX_CUDA(cudaMemcpyAsync(h->h_status, h->sb.status, 4, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    const uint32_t st = *h->h_status;
    if (st & sphx::kStatusDomainBit) {
        h->error = SPHX_ERR_DOMAIN;
        return fail(SPHX_ERR_DOMAIN, "a particle left the representable domain (non-finite or "
                                     "|x/h| >= 2^30); state is invalid until sphx_set_state");
    }
    if (st & sphx::kStatusOverflowBit) {
        h->error = SPHX_ERR_OVERFLOW;
        return fail(SPHX_ERR_OVERFLOW, "a cell exceeded max_cell_occupancy; state is invalid "
                                       "until sphx_set_state");
    }
    return SPHX_OK;
}

void destroy_graphs(sphx_handle *h) {
    for (auto &g : h->graphs) cudaGraphExecDestroy(g.exec);
    h->graphs.clear();
}

int run_graph_step(sphx_handle *h, const sphx::StepParams &P, bool reorder) {
    uint32_t dt_bits;
    std::memcpy(&dt_bits, &P.dt, 4);
    sphx::GraphEntry *hit = nullptr;
    for (auto &g : h->graphs)
        if (g.reorder == reorder && g.pv == h->pv && g.idc == h->idc && g.dt_bits == dt_bits)
            hit = &g;
    if (!hit) {
        if (h->graphs.size() >= 16) destroy_graphs(h);
        int pv = h->pv, idc = h->idc;
        cudaGraph_t graph;
        SPHX_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const cudaError_t e = enqueue_step(h, P, reorder, pv, idc, nullptr);
        const cudaError_t e2 = cudaStreamEndCapture(h->stream, &graph);
        if (e != cudaSuccess) return fail(SPHX_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
        if (e2 != cudaSuccess) return fail(SPHX_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e2));
        sphx::GraphEntry g{reorder, h->pv, h->idc, dt_bits, nullptr};
        const cudaError_t e3 = cudaGraphInstantiate(&g.exec, graph, 0ULL);
        cudaGraphDestroy(graph);
        if (e3 != cudaSuccess) return fail(SPHX_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e3));
        h->graphs.push_back(g);
        hit = &h->graphs.back();
    }
    SPHX_CUDA(cudaGraphLaunch(hit->exec, h->stream));
    if (reorder) h->idc ^= 1;
    // reorder flips pv twice (gather, force), otherwise once
    if (!reorder) h->pv ^= 1;
    return SPHX_OK;
}

}  // namespace

int sphx::read_status(sphx_handle *h) { return read_status_impl(h); }

namespace {

#define HANDLE_CHECK(h)                                                 \
    do {                                                                \
        if (!(h)) return fail(SPHX_ERR_INVALID, "null handle");          \
        SPHX_CUDA(cudaSetDevice((h)->opt.device));                       \
    } while (0)

}  // namespace

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
    o->max_cell_occupancy = 1024;
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

int sphx_create(const sphx_settings *s, const sphx_box *box, const sphx_options *opt, size_t n,
                const float *pos3, const float *vel3, sphx_handle **out) {
    if (!s || !pos3 || !out) return fail(SPHX_ERR_INVALID, "null argument");
    *out = nullptr;
    if (n == 0 || n >= (size_t)1 << 31) return fail(SPHX_ERR_INVALID, "particle count must be in [1, 2^31)");
    if (!finite_args(*s)) return fail(SPHX_ERR_INVALID, "settings must be finite with h > 0");
    sphx_options o;
    if (opt) o = *opt;
    else sphx_options_default(&o);
    if (o.reorder_interval < 1) return fail(SPHX_ERR_INVALID, "reorder_interval must be >= 1");
    if (o.max_cell_occupancy == 0) o.max_cell_occupancy = 1024;
    sphx_box b;
    if (box) b = *box;
    else sphx_box_reference(&b);
    if (!(b.xmin < b.xmax) || !(b.zmin < b.zmax) || !std::isfinite(b.ymin) || !std::isfinite(b.damping) ||
        !std::isfinite(b.offset) || (b.has_ceiling && !(b.ymin < b.ymax)))
        return fail(SPHX_ERR_INVALID, "box bounds must be ordered and finite");
    int rc = check_positions(pos3, n, s->h);
    if (rc) return rc;
    if (vel3)
        for (size_t i = 0; i < 3 * n; ++i)
            if (!std::isfinite(vel3[i])) return fail(SPHX_ERR_DOMAIN, "non-finite velocity");

    int ndev = 0;
    SPHX_CUDA(cudaGetDeviceCount(&ndev));
    if (o.device < 0 || o.device >= ndev) return fail(SPHX_ERR_CUDA, "no such CUDA device");
    SPHX_CUDA(cudaSetDevice(o.device));

    sphx_handle *h = new sphx_handle();
    h->s = *s;
    h->d = sphx::derive_constants(s->mass, s->rest_density, s->gas_const, s->viscosity, s->h, s->g,
                                  s->tension);
    h->box = b;
    h->opt = o;
    h->n = (uint32_t)n;
    h->grid = choose_grid(b, o, s->h, pos3, n);
    const uint64_t slots = (uint64_t)h->grid.gx * h->grid.gy * h->grid.gz;
    if (slots >= (1ull << 31)) {
        delete h;
        return fail(SPHX_ERR_INVALID, "cell grid too large");
    }
    h->sb.slots = (uint32_t)slots;
    h->sb.max_cell = o.max_cell_occupancy;

    // One arena, 256-byte aligned sub-buffers.
    const size_t ntiles = (slots + 1 + 4095) / 4096;
    const size_t sizes[] = {16 * n, 16 * n, 16 * n, 16 * n,  // pos[2], vel[2]
                            4 * n,  4 * n,                    // id[2]
                            16 * n, 16 * n,                   // rp, force
                            4 * n,  4 * n,  4 * n,            // key, rank, order
                            4 * (slots + 1), 4 * (slots + 1), // count, start
                            4 * ntiles, 256,                  // tile_sum, status
                            24 * n};                          // staging
    size_t total = 0;
    for (size_t z : sizes) total += align_up(z, 256);
    if (cudaMalloc(&h->arena, total) != cudaSuccess) {
        delete h;
        cudaGetLastError();
        return fail(SPHX_ERR_NOMEM, "device allocation of " + std::to_string(total) + " bytes failed");
    }
    char *p = h->arena;
    void *ptrs[16];
    for (int k = 0; k < 16; ++k) {
        ptrs[k] = p;
        p += align_up(sizes[k], 256);
    }
    h->pos[0] = (float4 *)ptrs[0];
    h->pos[1] = (float4 *)ptrs[1];
    h->vel[0] = (float4 *)ptrs[2];
    h->vel[1] = (float4 *)ptrs[3];
    h->id[0] = (uint32_t *)ptrs[4];
    h->id[1] = (uint32_t *)ptrs[5];
    h->rp = (float4 *)ptrs[6];
    h->force = (float4 *)ptrs[7];
    h->sb.key = (uint32_t *)ptrs[8];
    h->sb.rank = (uint32_t *)ptrs[9];
    h->sb.order = (uint32_t *)ptrs[10];
    h->sb.count = (uint32_t *)ptrs[11];
    h->sb.start = (uint32_t *)ptrs[12];
    h->sb.tile_sum = (uint32_t *)ptrs[13];
    h->sb.status = (uint32_t *)ptrs[14];
    h->staging = (float *)ptrs[15];

    if (o.stream) {
        h->stream = (cudaStream_t)o.stream;
    } else {
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaFree(h->arena);
            delete h;
            return fail(SPHX_ERR_CUDA, "stream creation failed");
        }
        h->own_stream = true;
    }
    if (cudaMallocHost(&h->h_status, 4) != cudaSuccess) {
        sphx_destroy(h);
        return fail(SPHX_ERR_NOMEM, "pinned allocation failed");
    }
    if (cudaMemsetAsync(h->sb.count, 0, 4 * (slots + 1), h->stream) != cudaSuccess) {
        sphx_destroy(h);
        return fail(SPHX_ERR_CUDA, "memset failed");
    }
    rc = upload(h, pos3, vel3);
    if (rc) {
        const std::string msg = g_err;
        sphx_destroy(h);
        return fail(rc, msg);
    }
    *out = h;
    return SPHX_OK;
}

int sphx_destroy(sphx_handle *h) {
    if (!h) return SPHX_OK;
    cudaSetDevice(h->opt.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    destroy_graphs(h);
    for (cudaEvent_t e : h->events) cudaEventDestroy(e);
    if (h->transforms) cudaFree(h->transforms);
    if (h->arena) cudaFree(h->arena);
    if (h->h_status) cudaFreeHost(h->h_status);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return SPHX_OK;
}

size_t sphx_count(const sphx_handle *h) { return h ? h->n : 0; }

int sphx_set_state(sphx_handle *h, const float *pos3, const float *vel3) {
    HANDLE_CHECK(h);
    if (!pos3) return fail(SPHX_ERR_INVALID, "null positions");
    int rc = check_positions(pos3, h->n, h->s.h);
    if (rc) return rc;
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    return upload(h, pos3, vel3);
}

int sphx_step(sphx_handle *h, float dt, int nsteps) {
    HANDLE_CHECK(h);
    if (h->error) return fail(SPHX_ERR_STATE, "handle is in an error state; call sphx_set_state");
    if (nsteps < 0 || !std::isfinite(dt)) return fail(SPHX_ERR_INVALID, "bad dt or step count");
    return sphx::run_steps(h, dt, nsteps);
}

}  // extern "C"

int sphx::run_steps(sphx_handle *h, float dt, int nsteps) {
    const sphx::StepParams P = make_params(h, dt);
    for (int k = 0; k < nsteps; ++k) {
        const bool reorder = (h->step_count % (uint64_t)h->opt.reorder_interval) == 0;
        if (h->profiling) {
            if (h->events_used + 4 > h->events.size()) {
                for (int e = 0; e < 4 * 64; ++e) {
                    cudaEvent_t ev;
                    SPHX_CUDA(cudaEventCreate(&ev));
                    h->events.push_back(ev);
                }
            }
            cudaEvent_t *ev = &h->events[h->events_used];
            h->launches_per_step.resize(h->events.size() / 4);
            h->launches_per_step[h->events_used / 4] = reorder ? 9u : 8u;
            h->events_used += 4;
            int pv = h->pv, idc = h->idc;
            SPHX_CUDA(enqueue_step(h, P, reorder, pv, idc, ev));
            h->pv = pv;
            h->idc = idc;
        } else if (h->opt.use_graph) {
            const int rc = run_graph_step(h, P, reorder);
            if (rc) return rc;
        } else {
            int pv = h->pv, idc = h->idc;
            SPHX_CUDA(enqueue_step(h, P, reorder, pv, idc, nullptr));
            h->pv = pv;
            h->idc = idc;
        }
        ++h->step_count;
    }
    return SPHX_OK;
}

extern "C" {

int sphx_synchronize(sphx_handle *h) {
    HANDLE_CHECK(h);
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    if (h->error) return fail(h->error, "handle is in an error state; call sphx_set_state");
    return sphx::read_status(h);
}

int sphx_read_state(sphx_handle *h, float *pos3, float *vel3, float *rho, float *prs,
                    float *force3) {
    const int rc = sphx_synchronize(h);
    if (rc) return rc;
    const size_t n = h->n;
    struct F {
        float *dst;
        int field;
        const float4 *src;
        size_t floats;
    } fields[] = {{pos3, 0, h->pos[h->pv], 3 * n},
                  {vel3, 1, h->vel[h->pv], 3 * n},
                  {force3, 2, h->force, 3 * n},
                  {rho, 3, nullptr, n},
                  {prs, 4, nullptr, n}};
    for (const F &f : fields) {
        if (!f.dst) continue;
        SPHX_CUDA(sphx::launch_read_field(h->n, f.field, h->id[h->idc], f.src, h->rp, h->staging,
                                          h->stream));
        SPHX_CUDA(cudaMemcpyAsync(f.dst, h->staging, 4 * f.floats, cudaMemcpyDeviceToHost,
                                  h->stream));
        SPHX_CUDA(cudaStreamSynchronize(h->stream));
    }
    return SPHX_OK;
}

int sphx_read_transforms(sphx_handle *h, float *mat16) {
    const int rc = sphx_synchronize(h);
    if (rc) return rc;
    if (!mat16) return fail(SPHX_ERR_INVALID, "null output");
    if (!h->transforms && cudaMalloc(&h->transforms, 64 * (size_t)h->n) != cudaSuccess) {
        h->transforms = nullptr;
        cudaGetLastError();
        return fail(SPHX_ERR_NOMEM, "transform buffer allocation failed");
    }
    SPHX_CUDA(sphx::launch_transforms(h->n, h->d.h / 2.f, h->id[h->idc], h->pos[h->pv],
                                      h->transforms, h->stream));
    SPHX_CUDA(cudaMemcpyAsync(mat16, h->transforms, 64 * (size_t)h->n, cudaMemcpyDeviceToHost,
                              h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    return SPHX_OK;
}

int sphx_read_cells(sphx_handle *h, int32_t *cells3, uint16_t *hash16) {
    const int rc = sphx_synchronize(h);
    if (rc) return rc;
    const size_t n = h->n;
    int *dc = reinterpret_cast<int *>(h->staging);
    uint16_t *dh = reinterpret_cast<uint16_t *>(h->staging + 3 * n);
    SPHX_CUDA(sphx::launch_cells(h->n, h->d.h, h->id[h->idc], h->pos[h->pv], dc, dh, h->stream));
    if (cells3)
        SPHX_CUDA(cudaMemcpyAsync(cells3, dc, 12 * n, cudaMemcpyDeviceToHost, h->stream));
    if (hash16)
        SPHX_CUDA(cudaMemcpyAsync(hash16, dh, 2 * n, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    return SPHX_OK;
}

int sphx_neighbor_digest(sphx_handle *h, uint32_t *count, uint64_t *digest) {
    int rc = sphx_synchronize(h);
    if (rc) return rc;
    if (!count || !digest) return fail(SPHX_ERR_INVALID, "null output");
    const size_t n = h->n;
    const sphx::StepParams P = make_params(h, 0.f);
    uint32_t *dcount = reinterpret_cast<uint32_t *>(h->staging);
    uint64_t *ddig = reinterpret_cast<uint64_t *>(h->staging + 2 * n);  // 8-byte aligned
    SPHX_CUDA(sphx::launch_sort(P, h->sb, h->pos[h->pv], h->stream));
    SPHX_CUDA(sphx::launch_digest(P, h->sb, h->pos[h->pv], h->id[h->idc], dcount, ddig, true,
                                  h->stream));
    rc = sphx::read_status(h);
    if (rc) return rc;
    SPHX_CUDA(cudaMemcpyAsync(count, dcount, 4 * n, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaMemcpyAsync(digest, ddig, 8 * n, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    return SPHX_OK;
}

int sphx_device_state(sphx_handle *h, sphx_device_view *out) {
    HANDLE_CHECK(h);
    if (!out) return fail(SPHX_ERR_INVALID, "null output");
    out->pos = h->pos[h->pv];
    out->vel = h->vel[h->pv];
    out->force = h->force;
    out->rho_prs = h->rp;
    out->id = h->id[h->idc];
    out->n = h->n;
    out->stream = h->stream;
    return SPHX_OK;
}

int sphx_set_profiling(sphx_handle *h, int enable) {
    HANDLE_CHECK(h);
    h->profiling = enable != 0;
    return SPHX_OK;
}

int sphx_get_kernel_times(sphx_handle *h, sphx_kernel_times *out) {
    HANDLE_CHECK(h);
    if (!out) return fail(SPHX_ERR_INVALID, "null output");
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    for (size_t k = 0; k + 4 <= h->events_used; k += 4) {
        float a = 0.f, b = 0.f, c = 0.f;
        SPHX_CUDA(cudaEventElapsedTime(&a, h->events[k], h->events[k + 1]));
        SPHX_CUDA(cudaEventElapsedTime(&b, h->events[k + 1], h->events[k + 2]));
        SPHX_CUDA(cudaEventElapsedTime(&c, h->events[k + 2], h->events[k + 3]));
        h->acc.sort_ms += a;
        h->acc.density_ms += b;
        h->acc.force_ms += c;
        h->acc.steps += 1;
        h->acc.launches += h->launches_per_step[k / 4];
    }
    h->events_used = 0;
    *out = h->acc;
    h->acc = sphx_kernel_times{};
    return SPHX_OK;
}

}  // extern "C"
