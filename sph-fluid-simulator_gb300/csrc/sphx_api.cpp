// Resident scenes behind the C-ABI (include/sphx.h): handle lifetime, the
// device memory layout, the step sequence (one stream, CUDA graphs), the
// batched form, readouts and the autotuner.
//
// Replaces, behind the same call sequence, the reference's per-step path
// SPHSystem::update -> updateParticles -> updateParticlesCPU/GPU
// (src/SPHSystem.cpp:110-117, src/sph.cpp:195-290, src/kernels/sphGPU.cu:244-309).
// Where the reference copies the whole particle array to the device and back
// and cudaMallocs every step, a handle keeps its state in one device arena
// for its lifetime and a step is a fixed sequence of launches on one stream.
// A handle holds one scene (sphx_create) or many (sphx_create_batch); every
// launch covers all of them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "sphx_internal.h"

using sphx::fail;

namespace {

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

bool finite_args(const sphx_settings &s) {
    const float v[7] = {s.mass, s.rest_density, s.gas_const, s.viscosity, s.h, s.g, s.tension};
    for (float x : v)
        if (!std::isfinite(x)) return false;
    return s.h > 0.f;
}

bool box_ok(const sphx_box &b) {
    return b.xmin < b.xmax && b.zmin < b.zmax && std::isfinite(b.ymin) &&
           std::isfinite(b.damping) && std::isfinite(b.offset) &&
           (!b.has_ceiling || b.ymin < b.ymax);
}

// Every coordinate's cell quotient x / h must be below 2^30 in magnitude,
// which non-finite values fail too.  One branch-free pass (it vectorises),
// a second only to name the first offender.
int check_positions(const float *pos3, size_t n, float h) {
    const size_t m = 3 * n;
    unsigned bad = 0;
    for (size_t i = 0; i < m; ++i) bad |= !(std::fabs(pos3[i] / h) < 1073741824.0f);
    if (!bad) return SPHX_OK;
    size_t i = 0;
    while (i < m && std::fabs(pos3[i] / h) < 1073741824.0f) ++i;
    return fail(SPHX_ERR_DOMAIN, "position " + std::to_string(i / 3) +
                                     " is non-finite or too far from the origin");
}

// Cell grid covering the walls and the initial particles, padded by two
// cells; dimensions are automatic unless the options fix them.
sphx::Grid choose_grid(const sphx_box &b, const sphx_options &o, float h, const float *pos3,
                       size_t n) {
    float lo[3] = {b.xmin, b.ymin, b.zmin}, hi[3] = {b.xmax, b.ymin, b.zmax};
    float plo[3] = {INFINITY, INFINITY, INFINITY}, phi[3] = {-INFINITY, -INFINITY, -INFINITY};
    // four particles (12 floats) per iteration, one accumulator per float:
    // the inner loop vectorises; accumulator k holds component k % 3
    float blo[12], bhi[12];
    for (int k = 0; k < 12; ++k) {
        blo[k] = INFINITY;
        bhi[k] = -INFINITY;
    }
    const size_t m = 3 * n, m12 = m - m % 12;
    for (size_t i = 0; i < m12; i += 12)
        for (int k = 0; k < 12; ++k) {
            blo[k] = std::min(blo[k], pos3[i + k]);
            bhi[k] = std::max(bhi[k], pos3[i + k]);
        }
    for (int k = 0; k < 12; ++k) {
        plo[k % 3] = std::min(plo[k % 3], blo[k]);
        phi[k % 3] = std::max(phi[k % 3], bhi[k]);
    }
    for (size_t i = m12; i < m; ++i) {
        plo[i % 3] = std::min(plo[i % 3], pos3[i]);
        phi[i % 3] = std::max(phi[i % 3], pos3[i]);
    }
    for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(lo[a], plo[a]);
        hi[a] = std::max(hi[a], phi[a]);
    }
    if (b.has_ceiling) hi[1] = std::max(hi[1], b.ymax);
    else if (o.grid_ymax > b.ymin) hi[1] = std::max(hi[1], o.grid_ymax);
    else hi[1] = std::max(hi[1], phi[1] + 0.25f * (phi[1] - lo[1]) + 4.f * h);
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
    return sphx::Grid{org[0], org[1], org[2], dim[0], dim[1], dim[2]};
}

sphx::StepParams make_params(const sphx::Scene &sc, float dt) {
    sphx::StepParams P;
    std::memset(&P, 0, sizeof P);
    const sphx::Derived &d = sc.d;
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
    P.ylo = sc.box.ymin + d.h;
    P.yhi = sc.box.ymax - d.h;
    P.xlo = d.h + sc.box.xmin;
    P.xhi = sc.box.xmax - d.h;
    P.zlo = d.h + sc.box.zmin;
    P.zhi = sc.box.zmax - d.h;
    P.damping = sc.box.damping;
    P.offset = sc.box.offset;
    P.hasCeiling = sc.box.has_ceiling;
    P.dt = dt;
    P.h2w = d.h * d.h * (1.0f + 3.814697265625e-06f);
    P.grid = sc.grid;
    P.n = sc.n;
    return P;
}

// Sub-buffers of a handle's arena for the given capacities, 256-byte aligned.
struct Layout {
    enum {
        kPos0, kPos1, kVel0, kVel1, kId0, kId1, kRp, kForce, kKey, kRank, kOrder, kCount,
        kStart, kTiles, kStatus, kStaging, kParams, kPofs, kSofs, kLarge, kFr, kNbr, kNcount,
        kScat, kRofs, kRowOfs, kDeferred, kCflags, kNum
    };
    size_t off[kNum];
    size_t total;
};

Layout layout_for(size_t cn, size_t cs, size_t csc, size_t slots) {
    const size_t ntiles = (cs + 1 + 4095) / 4096;
    const size_t sizes[Layout::kNum] = {16 * cn, 16 * cn, 16 * cn, 16 * cn, 4 * cn, 4 * cn,
                                        16 * cn, 16 * cn, 4 * cn, 4 * cn, 4 * cn,
                                        4 * (cs + 1), 4 * (cs + 1), 4 * ntiles, 256, 24 * cn,
                                        sizeof(sphx::StepParams) * csc, 4 * (csc + 1),
                                        4 * (csc + 1), 8ull * sphx::large_list_cap((uint32_t)cn),
                                        32 * cn, 4ull * slots * ((cn + 31) / 32 * 32), 4 * cn, 8 * cn,
                                        4 * (csc + 1), 4 * (cs + 1), 8 * cn + 4 * (cn / 32 + 1),
                                        cs + 1};
    Layout L;
    size_t o = 0;
    for (int k = 0; k < Layout::kNum; ++k) {
        L.off[k] = o;
        o += align_up(std::max<size_t>(sizes[k], 16), 256);
    }
    L.total = o;
    return L;
}

void bind(sphx_handle *h, char *a, const Layout &L) {
    h->arena = a;
    h->pos[0] = (float4 *)(a + L.off[Layout::kPos0]);
    h->pos[1] = (float4 *)(a + L.off[Layout::kPos1]);
    h->vel[0] = (float4 *)(a + L.off[Layout::kVel0]);
    h->vel[1] = (float4 *)(a + L.off[Layout::kVel1]);
    h->id[0] = (uint32_t *)(a + L.off[Layout::kId0]);
    h->id[1] = (uint32_t *)(a + L.off[Layout::kId1]);
    h->rp = (float4 *)(a + L.off[Layout::kRp]);
    h->force = (float4 *)(a + L.off[Layout::kForce]);
    h->sb.key = (uint32_t *)(a + L.off[Layout::kKey]);
    h->sb.rank = (uint32_t *)(a + L.off[Layout::kRank]);
    h->sb.order = (uint32_t *)(a + L.off[Layout::kOrder]);
    h->sb.scat = (uint2 *)(a + L.off[Layout::kScat]);
    h->sb.count = (uint32_t *)(a + L.off[Layout::kCount]);
    h->sb.start = (uint32_t *)(a + L.off[Layout::kStart]);
    h->sb.tile_sum = (uint32_t *)(a + L.off[Layout::kTiles]);
    h->sb.status = (uint32_t *)(a + L.off[Layout::kStatus]);
    h->staging = (float *)(a + L.off[Layout::kStaging]);
    h->d_params = (sphx::StepParams *)(a + L.off[Layout::kParams]);
    h->d_pofs = (uint32_t *)(a + L.off[Layout::kPofs]);
    h->d_sofs = (uint32_t *)(a + L.off[Layout::kSofs]);
    h->sb.large = (uint2 *)(a + L.off[Layout::kLarge]);
    h->sb.deferred = (uint32_t *)(a + L.off[Layout::kDeferred]);
    h->sb.cflags = (const uint8_t *)(a + L.off[Layout::kCflags]);
    h->fr = (float4 *)(a + L.off[Layout::kFr]);
    h->nbr = (uint32_t *)(a + L.off[Layout::kNbr]);
    h->ncount = (uint32_t *)(a + L.off[Layout::kNcount]);
    h->d_rofs = (uint32_t *)(a + L.off[Layout::kRofs]);
    h->row_warps = sphx::RowWarps{(uint32_t *)(a + L.off[Layout::kRowOfs])};
}

// Allocates an arena for the capacities, zeroes its counts and status.
int alloc_arena(sphx_handle *h, size_t cn, size_t cs, size_t csc, char **out, Layout *L) {
    *L = layout_for(cn, cs, csc, h->opt.neighbor_slots);
    char *a = nullptr;
    if (cudaMalloc(&a, L->total) != cudaSuccess) {
        cudaGetLastError();
        return fail(SPHX_ERR_NOMEM, "device allocation of " + std::to_string(L->total) + " bytes failed");
    }
    if (cudaMemsetAsync(a + L->off[Layout::kCount], 0, 4 * (cs + 1), h->stream) != cudaSuccess ||
        cudaMemsetAsync(a + L->off[Layout::kStatus], 0, 256, h->stream) != cudaSuccess ||
        cudaMemsetAsync(a + L->off[Layout::kRp], 0, 16 * cn, h->stream) != cudaSuccess ||
        cudaMemsetAsync(a + L->off[Layout::kForce], 0, 16 * cn, h->stream) != cudaSuccess) {
        cudaFree(a);
        return fail(SPHX_ERR_CUDA, "arena initialisation failed");
    }
    *out = a;
    return SPHX_OK;
}

// Scene offsets -> device tables; the constants are re-uploaded on next use.
int upload_tables(sphx_handle *h) {
    std::vector<uint32_t> pofs(h->scenes.size() + 1), sofs(h->scenes.size() + 1),
        rofs(h->scenes.size() + 1);
    uint32_t rows = 0;
    for (size_t k = 0; k < h->scenes.size(); ++k) {
        pofs[k] = h->scenes[k].first;
        sofs[k] = h->scenes[k].slot0;
        rofs[k] = rows;  // cell rows (gy * gz per scene) before scene k
        rows += (uint32_t)(h->scenes[k].grid.gy * h->scenes[k].grid.gz);
    }
    pofs.back() = h->n;
    sofs.back() = h->slots;
    rofs.back() = rows;
    h->rows = rows;
    SPHX_CUDA(cudaMemcpyAsync(h->d_pofs, pofs.data(), 4 * pofs.size(), cudaMemcpyHostToDevice, h->stream));
    SPHX_CUDA(cudaMemcpyAsync(h->d_sofs, sofs.data(), 4 * sofs.size(), cudaMemcpyHostToDevice, h->stream));
    SPHX_CUDA(cudaMemcpyAsync(h->d_rofs, rofs.data(), 4 * rofs.size(), cudaMemcpyHostToDevice, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));  // host vectors go out of scope
    h->sb.slots = h->slots;
    h->params_valid = false;
    // every readout reads the constants (h, walls) from the device table
    const int rc = sphx::ensure_params(h, h->params_dt);
    if (rc != SPHX_OK) return rc;
    // the grids' cell flags, after the constants they are computed from
    SPHX_CUDA(sphx::launch_cell_flags(sphx::table_of(h), h->slots,
                                      const_cast<uint8_t *>(h->sb.cflags), h->stream));
    return SPHX_OK;
}

// Uploads one scene's host state into rows [first, first + n) of buffer
// parity (pv, idc), with scene-local ids.
int upload_scene(sphx_handle *h, const sphx::Scene &sc, const float *pos3, const float *vel3,
                 int pv, int idc, uint32_t *bad = nullptr, bool keep_order = false) {
    const size_t n = sc.n;
    float *sp = h->staging, *sv = h->staging + 3 * (size_t)h->cap_n;
    SPHX_CUDA(cudaMemcpyAsync(sp, pos3, 12 * n, cudaMemcpyHostToDevice, h->stream));
    if (vel3) SPHX_CUDA(cudaMemcpyAsync(sv, vel3, 12 * n, cudaMemcpyHostToDevice, h->stream));
    else SPHX_CUDA(cudaMemsetAsync(sv, 0, 12 * n, h->stream));
    SPHX_CUDA(sphx::launch_upload_rows(sc.first, sc.n, sp, sv, h->pos[pv], h->vel[pv], h->id[idc],
                                       sc.d.h, bad, keep_order, h->sb.status, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));  // staging is reused by the next scene
    return SPHX_OK;
}

// sphx_set_state's upload of one scene, in two halves.  The first puts the
// copies into staging on the copy stream, once the kernels queued before
// have released staging; the second queues the upload kernel on the kernel
// stream behind the copies.  Work queued on the kernel stream between the
// two runs beside the copies.  No host wait (the caller synchronises).
int upload_copies(sphx_handle *h, const sphx::Scene &sc, const float *pos3, const float *vel3) {
    const size_t n = sc.n;
    float *sp = h->staging, *sv = h->staging + 3 * (size_t)h->cap_n;
    SPHX_CUDA(cudaEventRecord(h->ev_kernels, h->stream));
    SPHX_CUDA(cudaStreamWaitEvent(h->copy_stream, h->ev_kernels, 0));
    SPHX_CUDA(cudaMemcpyAsync(sp, pos3, 12 * n, cudaMemcpyHostToDevice, h->copy_stream));
    if (vel3) SPHX_CUDA(cudaMemcpyAsync(sv, vel3, 12 * n, cudaMemcpyHostToDevice, h->copy_stream));
    else SPHX_CUDA(cudaMemsetAsync(sv, 0, 12 * n, h->copy_stream));
    SPHX_CUDA(cudaEventRecord(h->ev_copies, h->copy_stream));
    return SPHX_OK;
}

int upload_rows_after_copies(sphx_handle *h, const sphx::Scene &sc, uint32_t *bad, bool keep_order) {
    float *sp = h->staging, *sv = h->staging + 3 * (size_t)h->cap_n;
    SPHX_CUDA(cudaStreamWaitEvent(h->stream, h->ev_copies, 0));
    SPHX_CUDA(sphx::launch_upload_rows(sc.first, sc.n, sp, sv, h->pos[h->pv], h->vel[h->pv],
                                       h->id[h->idc], sc.d.h, bad, keep_order, h->sb.status,
                                       h->stream));
    return SPHX_OK;
}

// Lattice corners (jitter included) as two points, for the grid choice and
// the domain check.
void lattice_corners(const sphx_lattice_desc &L, float *pts) {
    const uint32_t nn[3] = {L.nx, L.ny, L.nz};
    const float j = std::fabs(L.jitter);
    for (int a = 0; a < 3; ++a) {
        pts[a] = L.origin[a] - j;
        pts[3 + a] = L.origin[a] + (float)(nn[a] ? nn[a] - 1 : 0) * L.spacing + j;
    }
}

// A new scene from host positions or a device-generated lattice: validated,
// constants derived, grid chosen.
int new_scene(const sphx::SceneInit &in, const sphx_options &o, sphx::Scene &sc) {
    if (!finite_args(in.s)) return fail(SPHX_ERR_INVALID, "settings must be finite with h > 0");
    if (!box_ok(in.box)) return fail(SPHX_ERR_INVALID, "box bounds must be ordered and finite");
    const float *pts = in.pos3;
    uint32_t n = in.n, npts = in.n;
    float corners[6];
    if (in.lattice) {
        const sphx_lattice_desc &L = *in.lattice;
        const uint64_t nl = (uint64_t)L.nx * L.ny * L.nz;
        if (nl == 0 || nl >= (1ull << 31) || !std::isfinite(L.spacing) || !std::isfinite(L.jitter))
            return fail(SPHX_ERR_INVALID, "lattice must be non-empty with finite spacing and jitter");
        for (int a = 0; a < 3; ++a)
            if (!std::isfinite(L.origin[a])) return fail(SPHX_ERR_INVALID, "lattice origin must be finite");
        lattice_corners(L, corners);
        pts = corners;
        npts = 2;
        n = (uint32_t)nl;
    } else {
        if (!in.pos3) return fail(SPHX_ERR_INVALID, "null positions");
        if (in.vel3) {
            unsigned bad = 0;
            for (size_t i = 0; i < 3 * (size_t)in.n; ++i) bad |= !(std::fabs(in.vel3[i]) <= FLT_MAX);
            if (bad) return fail(SPHX_ERR_DOMAIN, "non-finite velocity");
        }
    }
    if (n == 0) return fail(SPHX_ERR_INVALID, "scene without particles");
    const int rc = check_positions(pts, npts, in.s.h);
    if (rc) return rc;
    sc.s = in.s;
    sc.d = sphx::derive_constants(in.s.mass, in.s.rest_density, in.s.gas_const, in.s.viscosity,
                                  in.s.h, in.s.g, in.s.tension);
    sc.box = in.box;
    sc.grid = choose_grid(in.box, o, in.s.h, pts, npts);
    sc.n = n;
    const uint64_t sl = (uint64_t)sc.grid.gx * sc.grid.gy * sc.grid.gz;
    if (sl >= (1ull << 31)) return fail(SPHX_ERR_INVALID, "cell grid too large");
    sc.slots = (uint32_t)sl;
    return SPHX_OK;
}

// Writes a new scene's initial state into rows [first, first + n).
int place_scene(sphx_handle *h, const sphx::Scene &sc, const sphx::SceneInit &in, int pv, int idc) {
    if (in.lattice) {
        const sphx_lattice_desc &L = *in.lattice;
        sphx::LatticeGen g{L.nx, L.ny, L.nz, {L.origin[0], L.origin[1], L.origin[2]}, L.spacing,
                           L.jitter, L.seed};
        SPHX_CUDA(sphx::launch_lattice_rows(sc.first, g, h->pos[pv], h->vel[pv], h->id[idc], h->stream));
        return SPHX_OK;
    }
    return upload_scene(h, sc, in.pos3, in.vel3, pv, idc);
}

cudaError_t enqueue_step(sphx_handle *h, bool reorder, int &pv, int &idc, cudaEvent_t *ev) {
    cudaStream_t st = h->stream;
    cudaError_t e;
    const sphx::SceneTable T = sphx::table_of(h);
    if (ev) cudaEventRecord(ev[0], st);
    if ((e = sphx::launch_sort(T, h->sb, h->pos[pv], st)) != cudaSuccess) return e;
    if (reorder) {
        if ((e = sphx::launch_gather(T.n, h->sb, h->pos[pv], h->vel[pv], h->id[idc],
                                     h->pos[pv ^ 1], h->vel[pv ^ 1], h->id[idc ^ 1], st)) !=
            cudaSuccess)
            return e;
        pv ^= 1;
        idc ^= 1;
    }
    if (ev) cudaEventRecord(ev[1], st);
    const sphx::NbrList L{h->nbr, h->ncount, h->opt.neighbor_slots};
    if ((e = sphx::launch_density(T, h->sb, h->pos[pv], h->vel[pv], h->rp, h->fr, L, !reorder,
                                  st, h->tune.density_threads, h->row_warps)) != cudaSuccess)
        return e;
    if (ev) cudaEventRecord(ev[2], st);
    if ((e = sphx::launch_force(T, h->sb, h->pos[pv], h->vel[pv], h->rp, h->fr, L,
                                h->pos[pv ^ 1], h->vel[pv ^ 1], h->force, !reorder, st,
                                h->tune.force_threads)) != cudaSuccess)
        return e;
    if (ev) cudaEventRecord(ev[3], st);
    pv ^= 1;
    return cudaSuccess;
}

int run_graph_step(sphx_handle *h, bool reorder) {
    sphx::GraphEntry *hit = nullptr;
    for (auto &g : h->graphs)
        if (g.reorder == reorder && g.pv == h->pv && g.idc == h->idc &&
            g.tune.density_threads == h->tune.density_threads &&
            g.tune.force_threads == h->tune.force_threads)
            hit = &g;
    if (!hit) {
        if (h->graphs.size() >= 16) sphx::destroy_graphs(h);
        int pv = h->pv, idc = h->idc;
        cudaGraph_t graph;
        SPHX_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const cudaError_t e = enqueue_step(h, reorder, pv, idc, nullptr);
        const cudaError_t e2 = cudaStreamEndCapture(h->stream, &graph);
        if (e != cudaSuccess) return fail(SPHX_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
        if (e2 != cudaSuccess) return fail(SPHX_ERR_CUDA, std::string("end capture: ") + cudaGetErrorString(e2));
        sphx::GraphEntry g{reorder, h->pv, h->idc, h->tune, nullptr};
        const cudaError_t e3 = cudaGraphInstantiate(&g.exec, graph, 0ULL);
        cudaGraphDestroy(graph);
        if (e3 != cudaSuccess) return fail(SPHX_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e3));
        h->graphs.push_back(g);
        hit = &h->graphs.back();
    }
    SPHX_CUDA(cudaGraphLaunch(hit->exec, h->stream));
    if (reorder) h->idc ^= 1;
    if (!reorder) h->pv ^= 1;  // reorder flips pv twice (gather, force)
    return SPHX_OK;
}

int normalise_threads(int t) { return t == 256 ? 256 : 128; }

#define HANDLE_CHECK(h)                                                 \
    do {                                                                \
        if (!(h)) return fail(SPHX_ERR_INVALID, "null handle");          \
        SPHX_CUDA(cudaSetDevice((h)->opt.device));                       \
    } while (0)

}  // namespace

// ---------------------------------------------------------------- internals

void sphx::destroy_graphs(sphx_handle *h) {
    for (auto &g : h->graphs) cudaGraphExecDestroy(g.exec);
    h->graphs.clear();
}

int sphx::read_status(sphx_handle *h) {
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

int sphx::ensure_params(sphx_handle *h, float dt) {
    if (h->params_valid && h->params_dt == dt) return SPHX_OK;
    h->params.resize(h->scenes.size());
    for (size_t k = 0; k < h->scenes.size(); ++k) h->params[k] = make_params(h->scenes[k], dt);
    // pageable source: the copy is staged before this returns
    SPHX_CUDA(cudaMemcpyAsync(h->d_params, h->params.data(),
                              sizeof(sphx::StepParams) * h->params.size(), cudaMemcpyHostToDevice,
                              h->stream));
    h->params_dt = dt;
    h->params_valid = true;
    return SPHX_OK;
}

int sphx::run_steps(sphx_handle *h, float dt, int nsteps) {
    const int prc = sphx::ensure_params(h, dt);
    if (prc) return prc;
    for (int k = 0; k < nsteps; ++k) {
        const bool reorder =
            (h->step_count % (uint64_t)std::max(1, h->tune.reorder_interval)) == 0;
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
            // sort 6 (7 past 1024 scan tiles), gather, row warps (1, 2 past
            // 4095 rows), density and its deferred particles, force over
            // lists, walkers, deferred
            const uint32_t tiles = (h->slots + 1u + 4095u) / 4096u;
            h->launches_per_step[h->events_used / 4] =
                (reorder ? 12u : 11u) + (tiles > 1024u) +
                1u + (h->rows >= 4096u);
            h->events_used += 4;
            int pv = h->pv, idc = h->idc;
            SPHX_CUDA(enqueue_step(h, reorder, pv, idc, ev));
            h->pv = pv;
            h->idc = idc;
        } else if (h->opt.use_graph) {
            const int rc = run_graph_step(h, reorder);
            if (rc) return rc;
        } else {
            int pv = h->pv, idc = h->idc;
            SPHX_CUDA(enqueue_step(h, reorder, pv, idc, nullptr));
            h->pv = pv;
            h->idc = idc;
        }
        ++h->step_count;
    }
    return SPHX_OK;
}

int sphx::create_handle(const SceneInit *inits, size_t nscenes, const sphx_options *opt,
                        sphx_handle **out) {
    if (!out) return fail(SPHX_ERR_INVALID, "null argument");
    *out = nullptr;
    if (nscenes == 0) return fail(SPHX_ERR_INVALID, "no scenes");
    sphx_options o;
    if (opt) o = *opt;
    else sphx_options_default(&o);
    if (o.reorder_interval < 1) return fail(SPHX_ERR_INVALID, "reorder_interval must be >= 1");
    if (o.max_cell_occupancy == 0 || o.max_cell_occupancy > sphx::kLargeCell)
        o.max_cell_occupancy = sphx::kLargeCell;
    if (o.neighbor_slots == 0) o.neighbor_slots = sphx::kNbrSlotsDefault;
    if (o.neighbor_slots > sphx::kNbrSlotsMax)
        return fail(SPHX_ERR_INVALID, "neighbor_slots must be at most 1024");
    o.neighbor_slots = (o.neighbor_slots + 3u) & ~3u;  // 16-byte list rows
    uint64_t total_n = 0, total_slots = 0;
    std::vector<sphx::Scene> scenes(nscenes);
    for (size_t k = 0; k < nscenes; ++k) {
        sphx::Scene &sc = scenes[k];
        const int rc = new_scene(inits[k], o, sc);
        if (rc) return rc;
        sc.first = (uint32_t)total_n;
        sc.slot0 = (uint32_t)total_slots;
        total_n += sc.n;
        total_slots += sc.slots;
        if (total_n >= (1ull << 31) || total_slots >= (1ull << 31))
            return fail(SPHX_ERR_INVALID, "particle or cell-grid total exceeds 2^31");
    }
    int ndev = 0;
    SPHX_CUDA(cudaGetDeviceCount(&ndev));
    if (o.device < 0 || o.device >= ndev) return fail(SPHX_ERR_CUDA, "no such CUDA device");
    SPHX_CUDA(cudaSetDevice(o.device));
    SPHX_CUDA(sphx::prepare_device());

    sphx_handle *h = new sphx_handle();
    h->opt = o;
    h->scenes = scenes;
    h->n = (uint32_t)total_n;
    h->slots = (uint32_t)total_slots;
    h->cap_n = h->n;
    h->cap_slots = h->slots;
    h->cap_scenes = (uint32_t)nscenes;
    h->tune.density_threads = normalise_threads(o.density_threads);
    h->tune.force_threads = normalise_threads(o.force_threads);
    h->tune.reorder_interval = o.reorder_interval;
    h->sb.max_cell = o.max_cell_occupancy;
    h->sb.large_cap = sphx::large_list_cap(h->cap_n);
    if (o.stream) {
        h->stream = (cudaStream_t)o.stream;
    } else {
        if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete h;
            return fail(SPHX_ERR_CUDA, "stream creation failed");
        }
        h->own_stream = true;
    }
    if (cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_kernels, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_copies, cudaEventDisableTiming) != cudaSuccess) {
        sphx_destroy(h);
        return fail(SPHX_ERR_CUDA, "copy stream creation failed");
    }
    char *arena = nullptr;
    Layout L;
    int rc = alloc_arena(h, h->cap_n, h->cap_slots, h->cap_scenes, &arena, &L);
    if (rc == SPHX_OK) {
        bind(h, arena, L);
        if (cudaMallocHost(&h->h_status, 4) != cudaSuccess) rc = fail(SPHX_ERR_NOMEM, "pinned allocation failed");
    }
    if (rc == SPHX_OK) rc = upload_tables(h);
    for (size_t k = 0; rc == SPHX_OK && k < nscenes; ++k)
        rc = place_scene(h, h->scenes[k], inits[k], h->pv, h->idc);
    if (rc) {
        const std::string msg = sphx_last_error();
        sphx_destroy(h);
        return fail(rc, msg);
    }
    *out = h;
    return SPHX_OK;
}

int sphx::relayout(sphx_handle *h, const std::vector<SceneInit> &inits) {
    SPHX_CUDA(cudaSetDevice(h->opt.device));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    std::vector<sphx::Scene> scenes(inits.size());
    uint64_t total_n = 0, total_slots = 0;
    for (size_t k = 0; k < inits.size(); ++k) {
        const SceneInit &in = inits[k];
        sphx::Scene &sc = scenes[k];
        if (in.keep >= 0) {
            if ((size_t)in.keep >= h->scenes.size()) return fail(SPHX_ERR_INVALID, "no such scene");
            sc = h->scenes[(size_t)in.keep];
            if (in.resettle) {
                if (!finite_args(in.s) || !box_ok(in.box))
                    return fail(SPHX_ERR_INVALID, "settings must be finite with h > 0 and ordered box");
                sc.s = in.s;
                sc.d = sphx::derive_constants(in.s.mass, in.s.rest_density, in.s.gas_const,
                                              in.s.viscosity, in.s.h, in.s.g, in.s.tension);
                sc.box = in.box;
                sc.grid = in.grid;
                sc.slots = (uint32_t)((uint64_t)sc.grid.gx * sc.grid.gy * sc.grid.gz);
            }
        } else {
            const int rc = new_scene(in, h->opt, sc);
            if (rc) return rc;
        }
        sc.first = (uint32_t)total_n;
        sc.slot0 = (uint32_t)total_slots;
        total_n += sc.n;
        total_slots += sc.slots;
    }
    if (total_n >= (1ull << 31) || total_slots >= (1ull << 31))
        return fail(SPHX_ERR_INVALID, "particle or cell-grid total exceeds 2^31");
    // Destination: the other buffer parity of this arena, or a larger arena.
    const bool grow = total_n > h->cap_n || total_slots > h->cap_slots || inits.size() > h->cap_scenes;
    char *old_arena = h->arena;
    float4 *src_pos = h->pos[h->pv], *src_vel = h->vel[h->pv];
    uint32_t *src_id = h->id[h->idc];
    int dpv = h->pv ^ 1, didc = h->idc ^ 1;
    if (grow) {
        const size_t cn = std::max<size_t>(total_n, (size_t)(1.5 * h->cap_n));
        const size_t cs = std::max<size_t>(total_slots, (size_t)(1.5 * h->cap_slots));
        const size_t csc = std::max<size_t>(inits.size(), (size_t)(1.5 * h->cap_scenes));
        char *arena = nullptr;
        Layout L;
        int rc = alloc_arena(h, cn, cs, csc, &arena, &L);
        if (rc) return rc;
        bind(h, arena, L);  // the old sources stay valid until freed below
        h->cap_n = (uint32_t)cn;
        h->cap_slots = (uint32_t)cs;
        h->cap_scenes = (uint32_t)csc;
        h->sb.large_cap = sphx::large_list_cap(h->cap_n);
        dpv = 0;
        didc = 0;
    }
    for (size_t k = 0; k < inits.size(); ++k) {
        if (inits[k].keep < 0) continue;
        const sphx::Scene &from = h->scenes[(size_t)inits[k].keep];
        const sphx::Scene &to = scenes[k];
        SPHX_CUDA(cudaMemcpyAsync(h->pos[dpv] + to.first, src_pos + from.first, 16ull * to.n,
                                  cudaMemcpyDeviceToDevice, h->stream));
        SPHX_CUDA(cudaMemcpyAsync(h->vel[dpv] + to.first, src_vel + from.first, 16ull * to.n,
                                  cudaMemcpyDeviceToDevice, h->stream));
        SPHX_CUDA(cudaMemcpyAsync(h->id[didc] + to.first, src_id + from.first, 4ull * to.n,
                                  cudaMemcpyDeviceToDevice, h->stream));
    }
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    if (grow) cudaFree(old_arena);
    h->scenes = scenes;
    h->n = (uint32_t)total_n;
    h->slots = (uint32_t)total_slots;
    h->pv = dpv;
    h->idc = didc;
    sphx::destroy_graphs(h);
    int rc = upload_tables(h);
    for (size_t k = 0; rc == SPHX_OK && k < inits.size(); ++k)
        if (inits[k].keep < 0) rc = place_scene(h, h->scenes[k], inits[k], h->pv, h->idc);
    return rc;
}

int sphx::read_scene(sphx_handle *h, size_t k, float *pos3, float *vel3, float *rho, float *prs,
                     float *force3) {
    SPHX_CUDA(cudaSetDevice(h->opt.device));
    if (k >= h->scenes.size()) return fail(SPHX_ERR_INVALID, "no such scene");
    const sphx::Scene &sc = h->scenes[k];
    struct F {
        float *dst;
        int field;
        const float4 *src;
        size_t floats;
    } fields[] = {{pos3, 0, h->pos[h->pv], 3ull * sc.n},
                  {vel3, 1, h->vel[h->pv], 3ull * sc.n},
                  {force3, 2, h->force, 3ull * sc.n},
                  {rho, 3, nullptr, sc.n},
                  {prs, 4, nullptr, sc.n}};
    const size_t cap = 6ull * h->cap_n;
    size_t used = 0;
    for (const F &f : fields) {
        if (!f.dst) continue;
        if (used + f.floats > cap) {
            SPHX_CUDA(cudaStreamSynchronize(h->stream));
            used = 0;
        }
        float *out = h->staging + used;
        SPHX_CUDA(sphx::launch_read_rows(sc.first, sc.n, f.field, h->id[h->idc], f.src, h->rp, out,
                                         h->stream));
        SPHX_CUDA(cudaMemcpyAsync(f.dst, out, 4 * f.floats, cudaMemcpyDeviceToHost, h->stream));
        used += f.floats;
    }
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    return SPHX_OK;
}

// ---------------------------------------------------------------- C-ABI

extern "C" {

int sphx_create(const sphx_settings *s, const sphx_box *box, const sphx_options *opt, size_t n,
                const float *pos3, const float *vel3, sphx_handle **out) {
    if (!s || !pos3 || !out) return fail(SPHX_ERR_INVALID, "null argument");
    if (n == 0 || n >= (size_t)1 << 31) return fail(SPHX_ERR_INVALID, "particle count must be in [1, 2^31)");
    sphx::SceneInit in{};
    in.s = *s;
    if (box) in.box = *box;
    else sphx_box_reference(&in.box);
    in.n = (uint32_t)n;
    in.pos3 = pos3;
    in.vel3 = vel3;
    in.keep = -1;
    return sphx::create_handle(&in, 1, opt, out);
}

int sphx_create_batch(const sphx_scene_desc *scenes, size_t nscenes, const sphx_options *opt,
                      sphx_handle **out) {
    if (!scenes || !out) return fail(SPHX_ERR_INVALID, "null argument");
    std::vector<sphx::SceneInit> in(nscenes);
    for (size_t k = 0; k < nscenes; ++k) {
        if (scenes[k].n >= (size_t)1 << 31) return fail(SPHX_ERR_INVALID, "scene too large");
        in[k].s = scenes[k].settings;
        in[k].box = scenes[k].box;
        in[k].n = (uint32_t)scenes[k].n;
        in[k].pos3 = scenes[k].pos3;
        in[k].vel3 = scenes[k].vel3;
        in[k].keep = -1;
    }
    return sphx::create_handle(in.data(), nscenes, opt, out);
}

int sphx_create_lattice(const sphx_settings *s, const sphx_box *box, const sphx_options *opt,
                        const sphx_lattice_desc *lattice, sphx_handle **out) {
    if (!s || !lattice || !out) return fail(SPHX_ERR_INVALID, "null argument");
    sphx::SceneInit in{};
    in.s = *s;
    if (box) in.box = *box;
    else sphx_box_reference(&in.box);
    in.lattice = lattice;
    in.keep = -1;
    return sphx::create_handle(&in, 1, opt, out);
}

int sphx_replace_scene(sphx_handle *h, size_t scene, const sphx_scene_desc *desc,
                       const sphx_lattice_desc *lattice) {
    HANDLE_CHECK(h);
    if (!desc || scene >= h->scenes.size()) return fail(SPHX_ERR_INVALID, "no such scene");
    std::vector<sphx::SceneInit> inits(h->scenes.size());
    for (size_t k = 0; k < inits.size(); ++k) inits[k].keep = (int)k;
    sphx::SceneInit &in = inits[scene];
    in = sphx::SceneInit{};
    in.keep = -1;
    in.s = desc->settings;
    in.box = desc->box;
    in.n = (uint32_t)desc->n;
    in.pos3 = desc->pos3;
    in.vel3 = desc->vel3;
    in.lattice = lattice;
    if (!lattice && (desc->n == 0 || desc->n >= (size_t)1 << 31))
        return fail(SPHX_ERR_INVALID, "particle count must be in [1, 2^31)");
    const int rc = sphx::relayout(h, inits);
    if (rc == SPHX_OK) h->error = 0;
    return rc;
}

int sphx_set_settings(sphx_handle *h, size_t scene, const sphx_settings *s, const sphx_box *box) {
    HANDLE_CHECK(h);
    if (!s || scene >= h->scenes.size()) return fail(SPHX_ERR_INVALID, "no such scene");
    if (h->error) return fail(SPHX_ERR_STATE, "handle is in an error state");
    const sphx::Scene &cur = h->scenes[scene];
    std::vector<sphx::SceneInit> inits(h->scenes.size());
    for (size_t k = 0; k < inits.size(); ++k) inits[k].keep = (int)k;
    sphx::SceneInit &in = inits[scene];
    in.resettle = true;
    in.s = *s;
    in.box = box ? *box : cur.box;
    in.grid = cur.grid;
    if (s->h != cur.s.h || box) {  // the cells change: size the grid to the current particles
        std::vector<float> pos(3ull * cur.n);
        int rc = sphx_synchronize(h);
        if (rc == SPHX_OK) rc = sphx::read_scene(h, scene, pos.data(), nullptr, nullptr, nullptr, nullptr);
        if (rc) return rc;
        if (!finite_args(*s)) return fail(SPHX_ERR_INVALID, "settings must be finite with h > 0");
        rc = check_positions(pos.data(), cur.n, s->h);
        if (rc) return rc;
        in.grid = choose_grid(in.box, h->opt, s->h, pos.data(), cur.n);
    }
    return sphx::relayout(h, inits);
}

int sphx_destroy(sphx_handle *h) {
    if (!h) return SPHX_OK;
    cudaSetDevice(h->opt.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
    sphx::destroy_graphs(h);
    for (cudaEvent_t e : h->events) cudaEventDestroy(e);
    if (h->transforms) cudaFree(h->transforms);
    if (h->arena) cudaFree(h->arena);
    if (h->h_status) cudaFreeHost(h->h_status);
    if (h->ev_kernels) cudaEventDestroy(h->ev_kernels);
    if (h->ev_copies) cudaEventDestroy(h->ev_copies);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return SPHX_OK;
}

size_t sphx_count(const sphx_handle *h) { return h ? h->n : 0; }
size_t sphx_scene_count(const sphx_handle *h) { return h ? h->scenes.size() : 0; }

int sphx_scene_range(const sphx_handle *h, size_t scene, size_t *first, size_t *count) {
    if (!h || scene >= h->scenes.size()) return fail(SPHX_ERR_INVALID, "no such scene");
    if (first) *first = h->scenes[scene].first;
    if (count) *count = h->scenes[scene].n;
    return SPHX_OK;
}

int sphx_set_state(sphx_handle *h, const float *pos3, const float *vel3) {
    HANDLE_CHECK(h);
    if (!pos3) return fail(SPHX_ERR_INVALID, "null positions");
    // the domain check runs in the upload kernel: status word 3 ends as the
    // first offending row, or stays all ones
    uint32_t *bad = h->sb.status + 3;
    // Rows keep their particles, so that the storage stays in the last
    // step's cell order, which the next step's sort then finds sorted; but
    // only while every step so far completed: a step that stopped on an
    // error did not move the ids with the data, and the state is then
    // rewritten in id order instead (the upload kernel checks the device's
    // error bits itself).
    const bool keep = h->error == 0;
    SPHX_CUDA(cudaMemsetAsync(bad, 0xFF, 4, h->stream));
    for (size_t k = 0; k < h->scenes.size(); ++k) {
        const sphx::Scene &sc = h->scenes[k];
        int rc = upload_copies(h, sc, pos3 + 3ull * sc.first, vel3 ? vel3 + 3ull * sc.first : nullptr);
        // the last step's outputs are cleared while the first scene's
        // copies run
        if (rc == SPHX_OK && k == 0 && cudaMemsetAsync(h->rp, 0, 16ull * h->n, h->stream) != cudaSuccess)
            rc = fail(SPHX_ERR_CUDA, "clearing densities failed");
        if (rc == SPHX_OK && k == 0 && cudaMemsetAsync(h->force, 0, 16ull * h->n, h->stream) != cudaSuccess)
            rc = fail(SPHX_ERR_CUDA, "clearing forces failed");
        if (rc == SPHX_OK) rc = upload_rows_after_copies(h, sc, bad, keep);
        if (rc) {
            cudaStreamSynchronize(h->copy_stream);
            cudaStreamSynchronize(h->stream);
            return rc;
        }
    }
    SPHX_CUDA(cudaMemsetAsync(h->sb.status, 0, 8, h->stream));
    SPHX_CUDA(cudaMemcpyAsync(h->h_status, bad, 4, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    const uint32_t row = *h->h_status;
    if (row != 0xffffffffu) {
        // the state now holds the rejected positions: refuse to step on it
        h->error = SPHX_ERR_DOMAIN;
        size_t k = 0;
        while (k + 1 < h->scenes.size() && row >= h->scenes[k + 1].first) ++k;
        return fail(SPHX_ERR_DOMAIN, "scene " + std::to_string(k) + " position " +
                                         std::to_string(row - h->scenes[k].first) +
                                         " is non-finite or too far from the origin");
    }
    h->error = 0;
    return SPHX_OK;
}

int sphx_step(sphx_handle *h, float dt, int nsteps) {
    HANDLE_CHECK(h);
    if (h->error) return fail(SPHX_ERR_STATE, "handle is in an error state; call sphx_set_state");
    if (nsteps < 0 || !std::isfinite(dt)) return fail(SPHX_ERR_INVALID, "bad dt or step count");
    return sphx::run_steps(h, dt, nsteps);
}

int sphx_synchronize(sphx_handle *h) {
    HANDLE_CHECK(h);
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    if (h->error) return fail(h->error, "handle is in an error state; call sphx_set_state");
    return sphx::read_status(h);
}

int sphx_read_state(sphx_handle *h, float *pos3, float *vel3, float *rho, float *prs,
                    float *force3) {
    HANDLE_CHECK(h);
    if (h->error) return fail(h->error, "handle is in an error state; call sphx_set_state");
    const size_t n = h->n;
    const sphx::SceneTable T = sphx::table_of(h);
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
    // Each field is gathered into id order in staging on the kernel stream
    // (behind the queued steps) and copied out on the copy stream, so that
    // one field's copy runs beside the next field's gather.  Fields share
    // staging (6 floats per particle of capacity) and wait only when it is
    // full.  The step's status word comes back last; a step that stopped on
    // an error makes the call return that error (the arrays then hold
    // whatever the failed state gave).
    const size_t cap = 6ull * h->cap_n;
    size_t used = 0;
    int rc = SPHX_OK;
    for (const F &f : fields) {
        if (!f.dst) continue;
        if (used + f.floats > cap) {
            if (cudaStreamSynchronize(h->copy_stream) != cudaSuccess) {
                rc = fail(SPHX_ERR_CUDA, "readout copy failed");
                break;
            }
            used = 0;
        }
        float *out = h->staging + used;
        if (sphx::launch_read_field(T, f.field, h->id[h->idc], f.src, h->rp, out, h->sb.status,
                                    h->stream) !=
                cudaSuccess ||
            cudaEventRecord(h->ev_kernels, h->stream) != cudaSuccess ||
            cudaStreamWaitEvent(h->copy_stream, h->ev_kernels, 0) != cudaSuccess ||
            cudaMemcpyAsync(f.dst, out, 4 * f.floats, cudaMemcpyDeviceToHost, h->copy_stream) !=
                cudaSuccess) {
            rc = fail(SPHX_ERR_CUDA, "readout failed");
            break;
        }
        used += f.floats;
    }
    const cudaError_t e1 = cudaStreamSynchronize(h->copy_stream);
    if (rc) {
        cudaStreamSynchronize(h->stream);
        return rc;
    }
    if (e1 != cudaSuccess) return fail(SPHX_ERR_CUDA, std::string("readout: ") + cudaGetErrorString(e1));
    return sphx::read_status(h);
}

int sphx_read_scene(sphx_handle *h, size_t scene, float *pos3, float *vel3, float *rho,
                    float *prs, float *force3) {
    const int rc = sphx_synchronize(h);
    if (rc) return rc;
    return sphx::read_scene(h, scene, pos3, vel3, rho, prs, force3);
}

int sphx_read_transforms(sphx_handle *h, float *mat16) {
    const int rc = sphx_synchronize(h);
    if (rc) return rc;
    if (!mat16) return fail(SPHX_ERR_INVALID, "null output");
    if (h->transforms_cap < h->n) {
        if (h->transforms) cudaFree(h->transforms);
        h->transforms = nullptr;
        h->transforms_cap = 0;
        if (cudaMalloc(&h->transforms, 64 * (size_t)h->n) != cudaSuccess) {
            h->transforms = nullptr;
            cudaGetLastError();
            return fail(SPHX_ERR_NOMEM, "transform buffer allocation failed");
        }
        h->transforms_cap = h->n;
    }
    SPHX_CUDA(sphx::launch_transforms(sphx::table_of(h), h->id[h->idc], h->pos[h->pv],
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
    uint16_t *dh = reinterpret_cast<uint16_t *>(h->staging + 3 * (size_t)h->cap_n);
    SPHX_CUDA(sphx::launch_cells(sphx::table_of(h), h->id[h->idc], h->pos[h->pv], dc, dh, h->stream));
    if (cells3) SPHX_CUDA(cudaMemcpyAsync(cells3, dc, 12 * n, cudaMemcpyDeviceToHost, h->stream));
    if (hash16) SPHX_CUDA(cudaMemcpyAsync(hash16, dh, 2 * n, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    return SPHX_OK;
}

int sphx_neighbor_digest(sphx_handle *h, uint32_t *count, uint64_t *digest) {
    int rc = sphx_synchronize(h);
    if (rc) return rc;
    if (!count || !digest) return fail(SPHX_ERR_INVALID, "null output");
    rc = sphx::ensure_params(h, h->params_valid ? h->params_dt : 0.f);
    if (rc) return rc;
    const size_t n = h->n;
    const sphx::SceneTable T = sphx::table_of(h);
    uint32_t *dcount = reinterpret_cast<uint32_t *>(h->staging);
    uint64_t *ddig = reinterpret_cast<uint64_t *>(h->staging + 2 * (size_t)h->cap_n);
    // The walk of a reordering step: the state moved into cell order (into
    // the other half of the ping-pong buffers, free between steps), walked
    // with direct addressing.  (sphx_walk_stats walks through the
    // permutation instead, as the steps between reorders do.)
    const int pv = h->pv, idc = h->idc;
    SPHX_CUDA(sphx::launch_sort(T, h->sb, h->pos[pv], h->stream));
    SPHX_CUDA(sphx::launch_gather(T.n, h->sb, h->pos[pv], h->vel[pv], h->id[idc], h->pos[pv ^ 1],
                                  h->vel[pv ^ 1], h->id[idc ^ 1], h->stream));
    SPHX_CUDA(sphx::launch_digest(T, h->sb, h->pos[pv ^ 1], h->id[idc ^ 1], dcount, ddig, nullptr,
                                  false, h->stream));
    rc = sphx::read_status(h);
    if (rc) return rc;
    SPHX_CUDA(cudaMemcpyAsync(count, dcount, 4 * n, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaMemcpyAsync(digest, ddig, 8 * n, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    return SPHX_OK;
}

int sphx_walk_stats(sphx_handle *h, uint64_t *r2_tests, uint64_t *accepted) {
    int rc = sphx_synchronize(h);
    if (rc) return rc;
    if (!r2_tests || !accepted) return fail(SPHX_ERR_INVALID, "null output");
    rc = sphx::ensure_params(h, h->params_valid ? h->params_dt : 0.f);
    if (rc) return rc;
    const size_t n = h->n;
    const sphx::SceneTable T = sphx::table_of(h);
    // staging holds 24 bytes per particle: counts, tests, then 8-byte digests
    uint32_t *dcount = reinterpret_cast<uint32_t *>(h->staging);
    uint32_t *dtests = dcount + h->cap_n;
    uint64_t *ddig = reinterpret_cast<uint64_t *>(h->staging + 2 * (size_t)h->cap_n);
    SPHX_CUDA(sphx::launch_sort(T, h->sb, h->pos[h->pv], h->stream));
    SPHX_CUDA(sphx::launch_digest(T, h->sb, h->pos[h->pv], h->id[h->idc], dcount, ddig, dtests,
                                  true, h->stream));
    rc = sphx::read_status(h);
    if (rc) return rc;
    std::vector<uint32_t> c(n), t(n);
    SPHX_CUDA(cudaMemcpyAsync(c.data(), dcount, 4 * n, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaMemcpyAsync(t.data(), dtests, 4 * n, cudaMemcpyDeviceToHost, h->stream));
    SPHX_CUDA(cudaStreamSynchronize(h->stream));
    uint64_t st = 0, sa = 0;
    for (size_t k = 0; k < n; ++k) {
        st += t[k];
        sa += c[k];
    }
    *r2_tests = st;
    *accepted = sa;
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

int sphx_get_tuning(const sphx_handle *h, sphx_tuning *out) {
    if (!h || !out) return fail(SPHX_ERR_INVALID, "null argument");
    out->density_threads = h->tune.density_threads;
    out->force_threads = h->tune.force_threads;
    out->reorder_interval = h->tune.reorder_interval;
    out->ms_per_step = 0.0;
    return SPHX_OK;
}

int sphx_set_tuning(sphx_handle *h, const sphx_tuning *t) {
    if (!h || !t) return fail(SPHX_ERR_INVALID, "null argument");
    if (t->reorder_interval < 1) return fail(SPHX_ERR_INVALID, "reorder_interval must be >= 1");
    h->tune.density_threads = normalise_threads(t->density_threads);
    h->tune.force_threads = normalise_threads(t->force_threads);
    h->tune.reorder_interval = t->reorder_interval;
    return SPHX_OK;
}

int sphx_autotune(sphx_handle *h, float dt, int trial_steps, const char *cache_path,
                  sphx_tuning *out) {
    HANDLE_CHECK(h);
    if (h->error) return fail(SPHX_ERR_STATE, "handle is in an error state");
    if (trial_steps < 1) trial_steps = 4;
    cudaDeviceProp prop;
    SPHX_CUDA(cudaGetDeviceProperties(&prop, h->opt.device));
    std::ostringstream sig;
    sig << prop.name << "|n=" << h->n << "|scenes=" << h->scenes.size();
    std::string name = sig.str();
    for (char &c : name)
        if (c == ' ') c = '_';
    sphx_tuning best{h->tune.density_threads, h->tune.force_threads, h->tune.reorder_interval, 0.0};
    if (cache_path) {  // "signature density force reorder ms" per line
        std::ifstream f(cache_path);
        std::string line;
        while (std::getline(f, line)) {
            std::istringstream is(line);
            std::string key;
            sphx_tuning t{};
            if ((is >> key >> t.density_threads >> t.force_threads >> t.reorder_interval >> t.ms_per_step) &&
                key == name)
                best = t;
        }
        if (best.ms_per_step > 0.0) {
            sphx_set_tuning(h, &best);
            if (out) *out = best;
            return SPHX_OK;
        }
    }
    // Snapshot the state so that every trial starts from it.
    const size_t n = h->n;
    void *snap = nullptr;
    if (cudaMalloc(&snap, 36 * n) != cudaSuccess) {
        cudaGetLastError();
        return fail(SPHX_ERR_NOMEM, "autotune snapshot allocation failed");
    }
    char *sp = static_cast<char *>(snap);
    SPHX_CUDA(cudaMemcpyAsync(sp, h->pos[h->pv], 16 * n, cudaMemcpyDeviceToDevice, h->stream));
    SPHX_CUDA(cudaMemcpyAsync(sp + 16 * n, h->vel[h->pv], 16 * n, cudaMemcpyDeviceToDevice, h->stream));
    SPHX_CUDA(cudaMemcpyAsync(sp + 32 * n, h->id[h->idc], 4 * n, cudaMemcpyDeviceToDevice, h->stream));
    const int pv0 = h->pv, idc0 = h->idc;
    const uint64_t step0 = h->step_count;
    const bool prof0 = h->profiling;
    h->profiling = false;
    cudaEvent_t e0, e1;
    SPHX_CUDA(cudaEventCreate(&e0));
    SPHX_CUDA(cudaEventCreate(&e1));
    auto restore = [&]() -> int {
        h->pv = pv0;
        h->idc = idc0;
        h->step_count = step0;
        SPHX_CUDA(cudaMemcpyAsync(h->pos[h->pv], sp, 16 * n, cudaMemcpyDeviceToDevice, h->stream));
        SPHX_CUDA(cudaMemcpyAsync(h->vel[h->pv], sp + 16 * n, 16 * n, cudaMemcpyDeviceToDevice, h->stream));
        SPHX_CUDA(cudaMemcpyAsync(h->id[h->idc], sp + 32 * n, 4 * n, cudaMemcpyDeviceToDevice, h->stream));
        return SPHX_OK;
    };
    double best_ms = 1e30;
    int rc = SPHX_OK;
    const int threads[2] = {128, 256}, intervals[3] = {1, 2, 4};
    for (int dt_i = 0; dt_i < 2 && rc == SPHX_OK; ++dt_i)
        for (int ft_i = 0; ft_i < 2 && rc == SPHX_OK; ++ft_i)
            for (int r_i = 0; r_i < 3 && rc == SPHX_OK; ++r_i) {
                h->tune = sphx::Tuning{threads[dt_i], threads[ft_i], intervals[r_i]};
                if ((rc = restore())) break;
                if ((rc = sphx::run_steps(h, dt, 2))) break;  // warm-up, graph capture
                cudaEventRecord(e0, h->stream);
                if ((rc = sphx::run_steps(h, dt, trial_steps))) break;
                cudaEventRecord(e1, h->stream);
                if ((rc = sphx::read_status(h))) break;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                const double per = ms / trial_steps;
                if (per < best_ms) {
                    best_ms = per;
                    best = sphx_tuning{threads[dt_i], threads[ft_i], intervals[r_i], per};
                }
            }
    const int rc2 = restore();
    cudaStreamSynchronize(h->stream);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(snap);
    h->profiling = prof0;
    if (rc) return rc;
    if (rc2) return rc2;
    sphx_set_tuning(h, &best);
    if (cache_path) {
        std::ofstream f(cache_path, std::ios::app);
        f << name << " " << best.density_threads << " " << best.force_threads << " "
          << best.reorder_interval << " " << best.ms_per_step << "\n";
    }
    if (out) *out = best;
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
