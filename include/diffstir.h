/*
 * diffstir.h - C ABI of the GB300 (sm_103a) differentiable MLS-MPM stirring
 * simulator.
 *
 * The reference (denzelzheng/DiffStir) is a Python/Taichi program with no FFI
 * of its own: its callers (src/gradient_descent_module.py,
 * src/force_calculation_and_animation_module.py) drive the module-level
 * Taichi kernels of src/simulator/simulation_functions.py.  Every entry point
 * below replaces one group of those kernels or one of the field accesses the
 * callers make; the reference line each one stands in for is cited beside it.
 * The Python package diffstir_gb300 (ctypes) binds exactly these symbols.
 *
 * Conventions
 *  - All float / int pointers passed to compute entry points are DEVICE
 *    pointers owned by the caller (for instance torch CUDA tensors), unless a
 *    parameter says "host".
 *  - `stream` is a cudaStream_t passed as void*; NULL means the legacy default
 *    stream.  A handle may be used from one host thread at a time.
 *  - Return value: DSTIR_OK (0) or a negative DSTIR_E* code; the message of the
 *    last failure is kept per handle (dstir_last_error).  No C++ exception
 *    crosses this boundary.
 *  - Particle order inside a handle is scene-major and, inside a scene,
 *    [liquid | rod | container], with counts from DstirSceneDesc.
 */
#ifndef DIFFSTIR_H
#define DIFFSTIR_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DSTIR_OK 0
#define DSTIR_EINVAL (-1)   /* bad argument */
#define DSTIR_ENOMEM (-2)   /* device allocation failed */
#define DSTIR_ECUDA (-3)    /* a CUDA call failed */
#define DSTIR_ESTATE (-4)   /* call order, e.g. backward without a recorded forward */
#define DSTIR_ERANGE (-5)   /* size beyond a fixed limit */

/* bits of the device status word (dstir_status) */
#define DSTIR_STATUS_NAN 1u          /* a non-finite particle state was produced */
#define DSTIR_STATUS_OUT_OF_GRID 2u  /* a particle stencil left the grid; it was skipped */
#define DSTIR_STATUS_TIMEOUT 4u      /* a grid barrier of a persistent launch waited past its limit;
                                        the launch stopped early and its results are void */

/* viscosity models: src/simulator/simulation_functions.py:118-146 */
#define DSTIR_MODEL_CARREAU 0   /* params [eta0, eta_inf, n, lambda] */
#define DSTIR_MODEL_CROSS 1     /* params [eta0, eta_inf, n, lambda] */
#define DSTIR_MODEL_HB 2        /* params [K, tau_y, n, unused]; power law = HB with tau_y 0 */

/* rod representation */
#define DSTIR_ROD_PARTICLES 0   /* kinematic rod particles, reference :165-180, :250-270 */
#define DSTIR_ROD_CYLINDER 1    /* analytic moving cylinder in the grid update */

/* J used by the bulk term */
#define DSTIR_J_DET 0           /* J = det(F_tmp), reference :113 */
#define DSTIR_J_SVD 1           /* J = s1*s2*s3 from the per-particle 3x3 SVD */

/* One scene.  Field names follow src/simulator/initialization.py:14-54. */
typedef struct DstirSceneDesc {
    int32_t n_grid;          /* nodes per axis, dx = 1/n_grid (initialization.py:22-24) */
    int32_t bound;           /* wall layers (initialization.py:15) */
    int32_t n_liquid;        /* n_particles */
    int32_t n_rod;           /* n_operator_particles (0 in cylinder mode) */
    int32_t n_container;     /* n_container_particles */
    int32_t model;           /* DSTIR_MODEL_* (model_index) */
    int32_t rod_mode;        /* DSTIR_ROD_* */
    int32_t j_mode;          /* DSTIR_J_* */
    int32_t container_wall;  /* 1: cylindrical container projection in the grid update (:204-210) */
    int32_t reserved;
    float dt;                /* substep (arguments.json simulation_setting.dt) */
    float gravity;           /* y acceleration added to liquid velocity in P2G (:152), -9.81*scale */
    float bulk_modulus;      /* k of (k/2)(J-1/J-1)J (:112, 20000 in the reference) */
    float liquid_p_vol;      /* liquid_p_vol */
    float liquid_p_mass;     /* liquid_p_mass */
    float rod_p_mass;        /* operator_p_mass */
    float container_p_mass;  /* container_p_mass */
    float force_scale;       /* particle rod: force = sum(dv) * force_scale (= V_o*rho_o/dt, :335-336) */
    float container_cx;      /* container axis x (0.5 in the reference, :206) */
    float container_cz;      /* container axis z (0.5) */
    float container_r;       /* projection radius (0.0415 - dx/2, :205) */
    float rod_radius;        /* cylinder mode: rod radius; the rod occupies y >= trajectory y */
} DstirSceneDesc;

typedef struct DstirHandle DstirHandle;

/* Create a simulator for `batch` scenes able to run up to `max_steps`
 * substeps per rollout.  Replaces the field allocation of
 * src/simulator/initialization.py:123-165 (time-indexed fields become K-step
 * checkpoints owned by the handle).  Each scene has 4 <= n_grid <= 1024, and
 * the batch's grid nodes together (sum of n_grid^3) must not exceed INT_MAX,
 * else DSTIR_ERANGE with *out NULL. */
int dstir_create(const DstirSceneDesc* scenes, int32_t batch, int32_t max_steps,
                 DstirHandle** out);
void dstir_destroy(DstirHandle* h);
const char* dstir_last_error(const DstirHandle* h);
/* total particles (all scenes, all kinds) and scene count */
int dstir_num_particles(const DstirHandle* h, int64_t* n_total, int32_t* batch);

/* Upload the step-0 particle state, AoS: x,v [N,3], C,F [N,3,3] row-major.
 * v/C may be NULL (zero) and F may be NULL (identity).  Replaces
 * initialize_objects / initialize_ti_field, simulation_functions.py:293-319. */
int dstir_set_state(DstirHandle* h, const float* x, const float* v, const float* C,
                    const float* F, void* stream);
/* Read the current particle state back, same layout (any pointer may be NULL).
 * Replaces x/operator_x/container_x .to_numpy(), gradient_descent_module.py:131-132. */
int dstir_get_state(DstirHandle* h, float* x, float* v, float* C, float* F, void* stream);

/* params [batch,4] (constitutive_parameters, initialization.py:134), models
 * [batch] or NULL to keep the scene descriptors' model (model_index). */
int dstir_set_params(DstirHandle* h, const float* params, const int32_t* models, void* stream);

/* Rod reference-point trajectory [batch, max_steps+1, 3]; substep f uses
 * entries f and f+1 (operator_kinematic_seq, simulation_functions.py:266;
 * for the cylinder the point is (axis x, lowest y, axis z)). */
int dstir_set_trajectory(DstirHandle* h, const float* traj, void* stream);

/* Advance `nsteps` substeps starting at substep index t0 (which selects the
 * trajectory entries).  force_out [batch, nsteps, 3] receives the rod reaction
 * force of each substep: entry f is the reference's force at frame t0+f+1
 * (compute_loss, :330-339).  With record != 0 the state is checkpointed every
 * `ckpt_every` substeps for dstir_backward.  With the "resort" option on, the
 * particle order is rebuilt every `ckpt_every` substeps, recorded or not
 * (ckpt_every <= 0 without record: never).  Replaces forward(s), :341-348. */
int dstir_forward(DstirHandle* h, int32_t t0, int32_t nsteps, int32_t ckpt_every,
                  int32_t record, float* force_out, void* stream);

/* One substep without recording (the reference's forward(s) called alone,
 * src/force_calculation_and_animation_module.py:8-9). force_out [batch,3] or NULL. */
int dstir_substep(DstirHandle* h, int32_t f, float* force_out, void* stream);

/* Reverse pass of the last recorded dstir_forward: given dL/dforce
 * [batch, nsteps, 3] it writes dL/dparams [batch,4] and optionally dL/d(step-0
 * state) (x,v [N,3], C,F [N,9]; NULL to skip).  Segments are recomputed from
 * the checkpoints.  Replaces backward(s) (:351-365) driven by ti.ad.Tape
 * (gradient_descent_module.py:103-107) and constitutive_parameters.grad. */
int dstir_backward(DstirHandle* h, const float* dL_dforce, float* dL_dparams,
                   float* dL_dx0, float* dL_dv0, float* dL_dC0, float* dL_dF0,
                   void* stream);

/* OR of DSTIR_STATUS_* raised on the device since the last call; clears it.
 * Synchronises `stream`.  (The reference only prints NaNs,
 * gradient_descent_module.py:51-54.) */
int dstir_status(DstirHandle* h, uint32_t* flags, void* stream);

/* Tuning knobs (defaults in brackets): "p2g" [4] (0 scalar atomics per
 * particle, 1 vector atomics per particle, 3 brick-binned shared-memory tiles
 * with one CTA per 4x4x4-cell brick, 4 vector atomics after summing
 * neighbouring lanes' contributions to shared stencil nodes by warp shuffles;
 * 3 and 4 also select the matching G2P-adjoint scatter; 2 is not a variant),
 * "block" [256] (threads per particle block: 64, 128 or 256), "gblock" [1024]
 * (threads per grid block: 64 to 1024), "graph" [1] (1:
 * replay each rollout and each reverse pass as a cached CUDA graph), "fuse" /
 * "fuse_adj" [0] (1: G2P of substep f fused with P2G of f+1 / P2G adjoint of
 * f fused with the G2P adjoint of f-1), "resort" [1] (re-sort the particle
 * order every ckpt_every substeps of a rollout; states and state adjoints
 * still cross the ABI in the order given to dstir_set_state), "tight" [3]
 * (register-cap level of the particle kernels, 0..3), "box" [1] (P2G records
 * each scene's occupied node box and the grid update and its adjoint skip the
 * nodes outside it; per-particle variants only), "store_grids" [0] (a recorded rollout keeps
 * the P2G and velocity grids of every substep, 32 bytes per grid node and
 * substep, and the reverse pass recomputes the states of each segment with
 * G2P alone instead of rerunning P2G and the grid update), "overlap" [1] (the
 * reverse pass recomputes segment s-1 on a second stream while it runs the
 * adjoint of segment s; per-particle variants),
 * "lsort" [1] (variant 4: each block of liquid particles rebuilds the
 * interleaved order over its own particles before the P2G scatter and the
 * G2P-adjoint scatter, so the lane-to-lane summation keeps working as
 * particles drift between re-sorts), "lstage" [3] (with "lsort": the
 * block's inputs are loaded coalesced into shared memory while the block
 * sorts, and its outputs go back the same way; bit 0 P2G, bit 1 the G2P
 * adjoint), "prefetch" [100] (each block of the P2G adjoint and of the G2P
 * adjoint hints L2, with prefetch.global.L2, to fetch the state that the
 * block this many block indices later reads: the whole state and the F part
 * of the next state's adjoint for the P2G adjoint, the positions and the x,
 * v, C parts of the next state's adjoint for the G2P adjoint; 0: no hints),
 * "gprio" [1] (the grid update and its adjoint are launched
 * at the device's greatest priority, and graphs are instantiated with node
 * priorities, so that in the overlapped reverse pass these short kernels,
 * which each gate the next kernel of their stream, get SM slots ahead of the
 * other stream's particle kernels; 0: default priority), "pdl" [1]
 * (programmatic dependent
 * launch of the substep kernels: a kernel's blocks may start while the
 * previous kernel of the stream drains and wait in hardware for its
 * completion before touching memory; 1 in forward rollouts, 2 also in the
 * reverse pass, 0 never), "brick_scatter" /
 * "brick_gather" (scatter and gather forms of variant 3), "persist" [0] (1:
 * with p2g 1, 256-thread particle blocks and no fusion or processing order,
 * each chunk of a forward rollout and each segment of the reverse pass runs
 * as cooperative launches of up to 50 substeps, the phases of a substep
 * separated by grid-wide barriers, instead of one launch per phase; for
 * scenes too small to fill the GPU; the reverse pass then runs on one
 * stream), "barrier_limit_us" [2000000] (longest wait at a grid barrier of a
 * persistent launch; past it the launch stops early and raises
 * DSTIR_STATUS_TIMEOUT), "barrier_test" [0] (1: every grid barrier waits for
 * one arrival more than the launch has blocks, so that every wait runs out;
 * for tests of the timeout path), "profile" [0] (1:
 * time every launch with CUDA events; totals via dstir_get_option
 * "prof_ns:<kernel>" / "prof_count:<kernel>"), "launches" (reset the launch
 * counter). */
int dstir_set_option(DstirHandle* h, const char* key, int64_t value);
int dstir_get_option(const DstirHandle* h, const char* key, int64_t* value);

/* Batched 3x3 SVD, A = U diag(S) V^T with det U = det V = +1 (the last
 * singular value carries the sign of det A), A/U/V [n,3,3], S [n,3].
 * Replaces the svd kernel (ti.svd), simulation_functions.py:55-58. */
int dstir_svd3(const float* A, float* U, float* S, float* V, int64_t n, void* stream);
/* SVD backward, simulation_functions.py:61-93 (backward_svd with the clamped
 * 1/(s_j^2 - s_i^2) terms evaluated in FP64): gA = f(gU, gS, gV, U, S, V).
 * gS is [n,3] (the diagonal of the reference's sig.grad). */
int dstir_svd3_backward(const float* gU, const float* gS, const float* gV, const float* U,
                        const float* S, const float* V, float* gA, int64_t n, void* stream);

/* One substep of one scene that allocates no device memory.  No counterpart in
 * the reference: it exists for callers that may not call cudaMalloc (a host
 * framework that owns the device pool and forbids allocations in its
 * callbacks, or a stepping loop that cannot take the synchronisation an
 * allocation may cause).  It runs the same kernels as dstir_substep, with its
 * grids, tables and reduction scratch in one static device array of about
 * 8.3 MB that every GPU loading the library keeps until exit.
 *  - scene: one descriptor (host pointer); n = n_liquid + n_rod + n_container.
 *  - params [4], traj2 [2][3] (rod reference point at frames f and f+1),
 *    state_in / state_out [24][n] (component-major: x0..2 v0..2 C00..C22
 *    F00..F22, component c of particle p at c*n + p; must not overlap),
 *    force_out [3] (the substep's rod reaction force): device pointers.
 *  - Limits: n_grid <= 64 and n <= 1048576, else DSTIR_ERANGE (checked
 *    before anything is queued).
 *  - Calls share the static array: calls that overlap on the GPU race.  Every
 *    call looks up the array's device address on the current device
 *    (cudaGetSymbolAddress, which allocates nothing); the first call on a
 *    device may load the module and should precede any stream capture.
 *  - A CUDA error still pending on the calling thread from earlier work is
 *    reported as DSTIR_ECUDA before anything is queued and left pending for
 *    the caller.  Device status flags are not reported. */
int dstir_substep_static(const DstirSceneDesc* scene, const float* params, const float* traj2,
                         const float* state_in, float* state_out, float* force_out, void* stream);

/* Diagnostics, no counterpart in the reference: the rate at which this GPU
 * retires 16-byte vector float reductions (red.global.add.v4.f32) when each
 * warp instruction covers 32 consecutive grid nodes (16 sectors of 32 bytes)
 * of an L2-resident grid of n_nodes nodes.  This is the roofline of the
 * warp-aggregated P2G and G2P-adjoint scatters.  Allocates and frees its own
 * grid; synchronises the stream.  sectors_per_s: host pointer. */
int dstir_measure_red_rate(int64_t n_nodes, int32_t reps, double* sectors_per_s, void* stream);
/* Diagnostics: FP32 FMA throughput of this GPU (flop/s, an FMA counting two),
 * from eight independent FMA chains per thread over 8 blocks of 256 threads
 * per SM.  Synchronises the stream.  flops_per_s: host pointer. */
int dstir_measure_fp32_rate(int32_t iters, double* flops_per_s, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DIFFSTIR_H */
