// The reference's GPU seam as a C-ABI call: sphx_update_particles takes the
// caller's array of 60-byte Particle records and mat4 transforms, exactly
// what updateParticlesGPU (src/kernels/sphGPU.h:8-11, sphGPU.cu:244-309)
// takes, and updates both in place for one step.
//
// Differences from the reference backend, each deliberate:
//   * the device state is cached between calls (one resident scene per
//     process, re-created only when n, settings or box change) instead of
//     device_vector + cudaMalloc/cudaFree on every call;
//   * walls follow the reference's CPU path (the GPU backend used other
//     constants, sphGPU.cu:8-10, and is therefore not a parity target);
//   * records keep the caller's order (the reference permutes the array by
//     hash every step, sph.cpp:227 / sphGPU.cu:263), and every record's
//     `hash` field holds hash16 of its pre-step cell as the reference's does.
#include <cstring>
#include <mutex>
#include <vector>

#include "sphx_internal.h"

namespace {

struct DropInCache {
    std::mutex mu;
    sphx_handle *h = nullptr;
    size_t n = 0;
    sphx_settings s{};
    sphx_box box{};
    void *d_rec = nullptr;       // 60 * n bytes
    uint16_t *d_hash = nullptr;  // n
    float *d_tr = nullptr;       // 16 * n floats
};

DropInCache &cache() {
    static DropInCache c;
    return c;
}

void release_locked(DropInCache &c) {
    if (c.h) sphx_destroy(c.h);
    if (c.d_rec) cudaFree(c.d_rec);
    if (c.d_hash) cudaFree(c.d_hash);
    if (c.d_tr) cudaFree(c.d_tr);
    c.h = nullptr;
    c.d_rec = nullptr;
    c.d_hash = nullptr;
    c.d_tr = nullptr;
    c.n = 0;
}

constexpr size_t kRec = 60;

}  // namespace

extern "C" {

int sphx_update_particles(void *particles, float *transforms16, size_t n,
                          const sphx_settings *s, const sphx_box *box, float dt) {
    using sphx::fail;
    if (!particles || !s) return fail(SPHX_ERR_INVALID, "null argument");
    if (n == 0) return SPHX_OK;
    DropInCache &c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    sphx_box b;
    if (box) b = *box;
    else sphx_box_reference(&b);
    const bool same = c.h && c.n == n && std::memcmp(&c.s, s, sizeof *s) == 0 &&
                      std::memcmp(&c.box, &b, sizeof b) == 0;
    if (!same) {
        release_locked(c);
        std::vector<float> pos3(3 * n);
        const unsigned char *rec = static_cast<const unsigned char *>(particles);
        for (size_t i = 0; i < n; ++i) std::memcpy(&pos3[3 * i], rec + kRec * i, 12);
        sphx_options o;
        sphx_options_default(&o);
        o.use_graph = 1;
        int rc = sphx_create(s, &b, &o, n, pos3.data(), nullptr, &c.h);
        if (rc) return rc;
        if (cudaMalloc(&c.d_rec, kRec * n) != cudaSuccess ||
            cudaMalloc(&c.d_hash, 2 * n) != cudaSuccess ||
            cudaMalloc(&c.d_tr, 64 * n) != cudaSuccess) {
            cudaGetLastError();
            release_locked(c);
            return fail(SPHX_ERR_NOMEM, "drop-in device buffers");
        }
        c.n = n;
        c.s = *s;
        c.box = b;
    }
    sphx_handle *h = c.h;
    SPHX_CUDA(cudaSetDevice(h->opt.device));
    cudaStream_t st = h->stream;
    SPHX_CUDA(cudaMemcpyAsync(c.d_rec, particles, kRec * n, cudaMemcpyHostToDevice, st));
    SPHX_CUDA(sphx::launch_aos_unpack((uint32_t)n, h->scenes[0].d.h, c.d_rec, h->pos[h->pv], h->vel[h->pv],
                                      h->id[h->idc], c.d_hash, st));
    SPHX_CUDA(cudaMemsetAsync(h->sb.status, 0, 8, st));
    h->error = 0;
    int rc = sphx::run_steps(h, dt, 1);
    if (rc) return rc;
    SPHX_CUDA(sphx::launch_aos_pack((uint32_t)n, h->scenes[0].d.h / 2.f, c.d_rec, h->id[h->idc],
                                    h->pos[h->pv], h->vel[h->pv], h->force, h->rp, c.d_hash,
                                    transforms16 ? c.d_tr : nullptr, st));
    SPHX_CUDA(cudaMemcpyAsync(particles, c.d_rec, kRec * n, cudaMemcpyDeviceToHost, st));
    if (transforms16)
        SPHX_CUDA(cudaMemcpyAsync(transforms16, c.d_tr, 64 * n, cudaMemcpyDeviceToHost, st));
    return sphx::read_status(h);
}

int sphx_update_particles_release(void) {
    DropInCache &c = cache();
    std::lock_guard<std::mutex> lock(c.mu);
    release_locked(c);
    return SPHX_OK;
}

}  // extern "C"
