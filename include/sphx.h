/*
 * sphx — GB300-native SPH step (C-ABI).
 *
 * Drop-in replacement for the per-step hot path of lijenicol/SPH-Fluid-Simulator:
 * SPHSystem::update (src/SPHSystem.cpp:110-117) -> updateParticles
 * (src/sph.cpp:277-290) -> updateParticlesCPU / updateParticlesGPU
 * (src/sph.cpp:195-275, src/kernels/sphGPU.cu:244-309).  State stays resident
 * on one GPU between steps; every entry point returns an int status
 * (SPHX_OK = 0, negative on error, message in sphx_last_error()) where the
 * reference returns void and checks nothing.
 *
 * Arrays crossing this boundary are host arrays unless named "device".  Vec3
 * arrays hold 3 floats per particle (x, y, z); per-particle outputs are in id
 * order (row i = the particle passed in row i at create / set_state), unlike
 * the reference, whose particle array is permuted by its sort every step
 * (src/sph.cpp:227).
 */
#ifndef SPHX_H
#define SPHX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHX_OK 0
#define SPHX_ERR_INVALID (-1)  /* bad argument */
#define SPHX_ERR_CUDA (-2)     /* CUDA runtime / no usable GPU */
#define SPHX_ERR_NOMEM (-3)    /* device or pinned allocation failed */
#define SPHX_ERR_DOMAIN (-4)   /* non-finite position or |x/h| >= 2^30 */
#define SPHX_ERR_OVERFLOW (-5) /* a cell holds more particles than the limit */
#define SPHX_ERR_STATE (-6)    /* handle state invalid after an earlier error */

/* Constructor arguments of SPHSettings (src/SPHSystem.h:15-17). */
typedef struct sphx_settings {
    float mass, rest_density, gas_const, viscosity, h, g, tension;
} sphx_settings;

/* The fields SPHSettings derives (src/SPHSystem.h:19-21, SPHSystem.cpp:8-26),
 * bit-identical to the reference's. sphere_scale is column-major. */
typedef struct sphx_derived {
    float poly6, spiky_grad, spiky_lap, gas_constant, mass, h2, self_dens,
        rest_density, viscosity, h, g, tension, mass_poly6_product;
    float sphere_scale[16];
} sphx_derived;

/* Wall geometry.  The reference hard-codes x, z in [-8, 8], a floor at y = 0,
 * no ceiling, damping 0.5 and offset 1e-4 (src/sph.cpp:139-176); reflection
 * happens at bound +- h.  sphx_box_reference() fills exactly that. */
typedef struct sphx_box {
    float xmin, xmax, ymin, ymax, zmin, zmax;
    float damping; /* velocity factor on reflection (reference 0.5) */
    float offset;  /* position offset on reflection (reference 1e-4) */
    int has_ceiling; /* 0 in the reference: ymax unused */
} sphx_box;

typedef struct sphx_options {
    int reorder_interval;  /* permute particle data into cell order every R steps (>= 1) */
    int use_graph;         /* replay each step as a captured CUDA graph */
    int device;            /* CUDA device ordinal */
    void *stream;          /* cudaStream_t to run on; NULL: the handle owns one */
    float grid_ymax;       /* top of the cell grid without a ceiling; <= ymin: automatic */
    int grid_dims[3];      /* cell-grid dimensions; 0: automatic (each >= 5) */
    int grid_origin[3];    /* cell coordinates of grid slot 0 (used when grid_dims set) */
    uint32_t max_cell_occupancy; /* particles per cell before a step fails (0 or > 16384: 16384) */
    int density_threads;   /* block size of the density kernel: 128 or 256 (0: 128) */
    int force_threads;     /* block size of the force kernel: 128 or 256 (0: 128) */
    uint32_t neighbor_slots; /* accepted neighbours the density pass records per particle for
                                the force pass (0: 256, at most 1024); particles with more are
                                walked again by the force pass */
} sphx_options;

/* One scene of a batch: its settings, walls and initial host state. */
typedef struct sphx_scene_desc {
    sphx_settings settings;
    sphx_box box;
    size_t n;
    const float *pos3;
    const float *vel3; /* NULL: zero */
} sphx_scene_desc;

/* Launch configuration of the step kernels; ms_per_step is what the
 * autotuner measured for it (0 if not measured). */
typedef struct sphx_tuning {
    int density_threads;
    int force_threads;
    int reorder_interval;
    double ms_per_step;
} sphx_tuning;

/* Dam-break lattice block: index i + nx*(j + ny*k), position
 * origin + (i, j, k) * spacing + jitter, jitter uniform in [-amp, amp) per
 * axis from a SplitMix64 stream (counter 3*index + axis) seeded by `seed`. */
typedef struct sphx_lattice_desc {
    uint32_t nx, ny, nz;
    float origin[3];
    float spacing;
    float jitter;
    uint64_t seed;
} sphx_lattice_desc;

typedef struct sphx_handle sphx_handle;

/* Device-resident state of a handle (float4 rows: x, y, z, 0), in the
 * handle's current storage order; id[k] is the id of storage row k. */
typedef struct sphx_device_view {
    const void *pos;   /* float4[n] */
    const void *vel;   /* float4[n] */
    const void *force; /* float4[n], force of the last step */
    const void *rho_prs; /* float4[n]: density, pressure, 1/density, 0 of the last step */
    const uint32_t *id; /* uint32[n] */
    size_t n;
    void *stream;      /* cudaStream_t the handle runs on */
} sphx_device_view;

/* Per-phase device time accumulated while profiling is on (ms, CUDA events
 * on the handle's stream). */
typedef struct sphx_kernel_times {
    double sort_ms;    /* keys + scan + scatter + cell sort + reorder */
    double density_ms; /* row warps + density (+ its deferred particles) */
    double force_ms;   /* force over lists, walkers, deferred (+ integrate, walls) */
    uint64_t steps;
    uint64_t launches; /* kernels launched by those steps */
} sphx_kernel_times;

const char *sphx_version(void);
/* Message of the last error on the calling thread ("" if none). */
const char *sphx_last_error(void);

/* Tester.cpp:90: SPHSettings(0.02, 1000, 1, 1.04, 0.15, -9.8, 0.2). */
void sphx_settings_reference(sphx_settings *s);
void sphx_box_reference(sphx_box *b);
void sphx_options_default(sphx_options *o);

/* SPHSettings::SPHSettings (src/SPHSystem.cpp:8-26). */
int sphx_derive(const sphx_settings *s, sphx_derived *out);
/* getHash (src/neighborTable.cpp:5-12): the 18-bit value; the reference
 * stores its low 16 bits (Particle.h:9). */
uint32_t sphx_hash(int32_t cx, int32_t cy, int32_t cz);
/* getCell (src/neighborTable.cpp:14-17): ivec3(p / h), truncating. */
void sphx_cell(float x, float y, float z, float h, int32_t out[3]);
/* Bucket-collision flags of the 27 cells around a cell (host evaluation of
 * the test the kernels use): bit 0 = two neighbour cells share a bucket;
 * bit 1+f = a cell two away across face f (-x,+x,-y,+y,-z,+z, only faces in
 * face_mask) shares a visited bucket.  Both bits are exact. */
uint32_t sphx_collision_flags(int32_t cx, int32_t cy, int32_t cz, uint32_t face_mask);

/* Fills 3*nx*ny*nz floats. */
int sphx_lattice(const sphx_lattice_desc *d, float *pos3);
/* SPHSystem::initParticles (src/SPHSystem.cpp:76-108): srand(1024), spacing
 * h + 0.01, one-sided jitter; fills 3*W^3 floats (index i + (j + W*k)*W). */
int sphx_reference_scene(size_t cube_width, float h, float *pos3);

/* A resident scene of n particles (n >= 1).  vel3 may be NULL (zero).
 * box NULL: the reference box; opt NULL: sphx_options_default. */
int sphx_create(const sphx_settings *s, const sphx_box *box, const sphx_options *opt, size_t n,
                const float *pos3, const float *vel3, sphx_handle **out);
/* Batched form (no counterpart in the reference, which simulates one scene):
 * nscenes independent scenes of uneven sizes and settings, resident in one
 * handle and advanced together, each kernel launch covering every scene.
 * All handle functions apply; arrays are the scenes concatenated in order,
 * each in its own id order (sphx_scene_range gives a scene's rows). */
int sphx_create_batch(const sphx_scene_desc *scenes, size_t nscenes, const sphx_options *opt,
                      sphx_handle **out);
/* A scene whose dam-break lattice (sphx_lattice_desc) is generated on the
 * device, bit-identical to sphx_lattice: no host positions, no upload. */
int sphx_create_lattice(const sphx_settings *s, const sphx_box *box, const sphx_options *opt,
                        const sphx_lattice_desc *lattice, sphx_handle **out);
/* Replaces scene `scene` of a handle with a new one (desc->settings, box and
 * either host state or, when lattice is not NULL, a device-generated
 * lattice), as the reference GUI's RESET re-creates its system
 * (Tester.cpp:148-173); the other scenes keep their state.  The arena is
 * reused while the new layout fits it. */
int sphx_replace_scene(sphx_handle *h, size_t scene, const sphx_scene_desc *desc,
                       const sphx_lattice_desc *lattice);
/* Changes a scene's settings (and walls, if box is not NULL) keeping its
 * particles; the cell grid is re-sized when h or the box changes. */
int sphx_set_settings(sphx_handle *h, size_t scene, const sphx_settings *s, const sphx_box *box);
int sphx_destroy(sphx_handle *h);
size_t sphx_count(const sphx_handle *h);
size_t sphx_scene_count(const sphx_handle *h);
int sphx_scene_range(const sphx_handle *h, size_t scene, size_t *first, size_t *count);
/* One scene's state, host, scene-local id order; any pointer may be NULL. */
int sphx_read_scene(sphx_handle *h, size_t scene, float *pos3, float *vel3, float *rho,
                    float *prs, float *force3);
/* Replaces positions / velocities (host, id order, vel3 may be NULL) and
 * clears an error state.  A non-finite position, or one whose cell quotient
 * x / h reaches 2^30, returns SPHX_ERR_DOMAIN and leaves the handle in the
 * error state until a valid replacement. */
int sphx_set_state(sphx_handle *h, const float *pos3, const float *vel3);
/* Enqueues nsteps steps of dt (asynchronous; errors raised by the kernels
 * surface at the next sphx_synchronize or read). */
int sphx_step(sphx_handle *h, float dt, int nsteps);
int sphx_synchronize(sphx_handle *h);
/* Host readout in id order; any pointer may be NULL.  force3 / rho / prs are
 * the values of the last step (what it integrated with).  Waits for the
 * queued steps; if one of them stopped on an error, returns that error and
 * the arrays' contents are unspecified. */
int sphx_read_state(sphx_handle *h, float *pos3, float *vel3, float *rho, float *prs,
                    float *force3);
/* translate(position) * scale(h/2) per particle, 16 floats column-major, id
 * order (src/sph.cpp:178-179) — the instanced renderer's input. */
int sphx_read_transforms(sphx_handle *h, float *mat16);
/* Cell (3 ints) and stored uint16 hash of each particle's current position,
 * id order; either pointer may be NULL. */
int sphx_read_cells(sphx_handle *h, int32_t *cells3, uint16_t *hash16);
/* For the current positions: per particle, the number of accepted neighbour
 * visits of the reference walk (src/sph.cpp:40-66) and the wrapping sum of
 * SplitMix64-finalised ids over them (a multiset fingerprint), id order. */
int sphx_neighbor_digest(sphx_handle *h, uint32_t *count, uint64_t *digest);
/* Work of one neighbour walk over the current positions, summed over all
 * particles: candidates whose r^2 the step's walk evaluates, and accepted
 * neighbour visits.  No counterpart in the reference (a diagnostic for the
 * r^2-test and FP32 operation rates). */
int sphx_walk_stats(sphx_handle *h, uint64_t *r2_tests, uint64_t *accepted);
int sphx_device_state(sphx_handle *h, sphx_device_view *out);

/* The reference's GPU seam, updateParticlesGPU(Particle*, glm::mat4*, size_t,
 * const SPHSettings&, float) (src/kernels/sphGPU.h:8-11): one step over the
 * caller's host array of n 60-byte Particle records (Particle.h:4-10) and,
 * if transforms16 is not NULL, its n column-major mat4 transforms, both
 * updated in place.  Records keep their order; `hash` holds hash16 of each
 * record's pre-step cell; `acceleration` is left untouched.  Device state is
 * cached across calls (re-created when n, settings or box change).  box NULL:
 * the reference CPU path's walls (src/sph.cpp:139-176). */
int sphx_update_particles(void *particles, float *transforms16, size_t n,
                          const sphx_settings *s, const sphx_box *box, float dt);
/* Frees the state cached by sphx_update_particles. */
int sphx_update_particles_release(void);

/* No counterpart in the reference.  Density and pressure (the values one
 * step would compute, src/sph.cpp:28-76) of n particles whose positions are
 * already on the device (d_pos4: n float4 rows x, y, z, unused), written to
 * the caller's device arrays d_rho and d_prs, on `stream` (NULL: the default
 * stream), without allocating any memory: for callers that cannot allocate
 * device memory when they need the result (a plugin inside a frame with a
 * fixed GPU memory budget, or a host that gives the library buffers but no
 * right to call cudaMalloc).  Its scratch is one static device array of about
 * 7 MiB per GPU, held until the process exits; n may be at most 131,072
 * (larger n: SPHX_ERR_INVALID).  Calls share that array, so calls whose work
 * overlaps on the GPU race.  It synchronises `stream` and reads a status
 * word back, so it cannot be called while that stream is being captured into
 * a CUDA graph.  The array's device address is looked up the first time a
 * call runs in a CUDA context of a device, and again in any other context. */
int sphx_density_static(const sphx_settings *s, const void *d_pos4, size_t n, float *d_rho,
                        float *d_prs, void *stream);

int sphx_get_tuning(const sphx_handle *h, sphx_tuning *out);
int sphx_set_tuning(sphx_handle *h, const sphx_tuning *t);
/* Times every candidate configuration (density / force block size 128 or
 * 256, reorder interval 1, 2 or 4) over trial_steps steps of dt on this
 * handle's scenes, applies the fastest and returns it.  The handle's state
 * is restored afterwards.  With cache_path set, a configuration recorded
 * there for the same device and workload signature (particle count, scene
 * count) is applied without timing, and new results are appended. */
int sphx_autotune(sphx_handle *h, float dt, int trial_steps, const char *cache_path,
                  sphx_tuning *out);

int sphx_set_profiling(sphx_handle *h, int enable);
/* Synchronises, then returns the accumulated per-phase times and resets them. */
int sphx_get_kernel_times(sphx_handle *h, sphx_kernel_times *out);

/* ---- Served form (no counterpart in the reference): a continuous-batching
 * request loop.  Each request is a scene plus a step count; a worker thread
 * admits queued requests in arrival order while their device footprint fits
 * the HBM budget, advances every admitted scene together in one batch,
 * retires each scene when it reaches its step count and admits the next
 * ones as memory frees up.  A result equals that of the same scene run
 * alone with the same dt. */
#define SPHX_REQ_QUEUED 0
#define SPHX_REQ_RUNNING 1
#define SPHX_REQ_DONE 2
#define SPHX_REQ_FAILED 3

typedef struct sphx_server sphx_server;

typedef struct sphx_server_options {
    size_t hbm_budget_bytes; /* admission budget (default 150 GB) */
    int steps_per_tick;      /* steps between admission/retirement points (default 10) */
    int max_scenes;          /* resident scene limit, 0: none */
    float dt;                /* step size of every request (default 0.002) */
    int device;
} sphx_server_options;

typedef struct sphx_request {
    sphx_settings settings;
    sphx_box box;
    size_t n;
    const float *pos3; /* host, copied at submission */
    const float *vel3; /* NULL: zero */
    int nsteps;
} sphx_request;

typedef struct sphx_request_status {
    int state;       /* SPHX_REQ_* */
    int steps_done;
    double submit_s; /* seconds since the server started */
    double admit_s;
    double done_s;
} sphx_request_status;

typedef struct sphx_server_stats {
    uint64_t submitted, completed, ticks, relayouts, particle_steps;
    size_t live_scenes, queued, bytes_in_use;
    double elapsed_s;
    /* worker time laying scenes out (admission, retirement), stepping (to
     * the end of each tick's steps on the device) and copying finished
     * scenes' results back */
    double layout_s, step_s, readout_s;
} sphx_server_stats;

void sphx_server_options_default(sphx_server_options *o);
int sphx_server_create(const sphx_server_options *opt, sphx_server **out);
int sphx_server_submit(sphx_server *s, const sphx_request *r, uint64_t *ticket);
int sphx_server_status(sphx_server *s, uint64_t ticket, sphx_request_status *out);
/* Blocks until the request is done (SPHX_OK), failed, or timeout_s passes
 * (SPHX_ERR_STATE). */
int sphx_server_wait(sphx_server *s, uint64_t ticket, double timeout_s);
/* Copies a finished request's final state (id order; any pointer may be
 * NULL) and releases it. */
int sphx_server_result(sphx_server *s, uint64_t ticket, float *pos3, float *vel3, float *rho,
                       float *prs);
int sphx_server_stats_get(sphx_server *s, sphx_server_stats *out);
/* Fault injection on the host, for tests of the failure path (no
 * counterpart in the reference): the worker's next tick fails with `code`
 * (negative, an SPHX_ERR_*) as if a CUDA call had.  The server then stops:
 * every running and queued request ends SPHX_REQ_FAILED with that code, and
 * waits on them return it at once.  No GPU work is faulted. */
int sphx_server_inject_failure(sphx_server *s, int code);
int sphx_server_destroy(sphx_server *s);

#ifdef __cplusplus
}
#endif

#endif /* SPHX_H */
