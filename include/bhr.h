/*
 * bhr.h - C ABI of the GB300 Schwarzschild ray tracer.
 *
 * This is the drop-in boundary for the per-pixel march of the reference renderer
 * (DeepjotG/BlackHoleRender). The reference drives that march as a GLSL program:
 *   Renderer::tracePass        src/Renderer.cpp:369-387   (one full-screen draw)
 *   Renderer::setTraceUniforms src/Renderer.cpp:242-356   (the uniforms below)
 *   blackhole.frag main()      shaders/blackhole.frag:67-253 (ray gen + march loop)
 * The reference has no FFI of its own; this header splits blackhole.frag at the end of
 * its march loop and returns, per pixel, the state the shading after the loop reads
 * (status, escape direction, disk-plane crossings, bAxis).
 *
 * Conventions (all entry points):
 *   - return BHR_OK (0) or a negative BHR_ERR_* code; no C++ exception crosses the ABI;
 *     bhr_last_error() gives the message of the last failure on a context.
 *   - GPU calls are stream-ordered and asynchronous on the caller's cudaStream_t
 *     (passed as void*, NULL = legacy default stream); the caller synchronises.
 *   - a context is not thread-safe: one context per host thread.
 *   - output buffers are owned by the caller (device memory for bhr_trace*).
 *   - frame: black hole at the origin, +Y = disk normal (src/Units.h:5-7), units G=c=M=1.
 *   - hit records are row-major, row 0 = bottom row (gl_FragCoord convention).
 */
#ifndef BHR_H
#define BHR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BHR_ABI_VERSION 1

/* ---- return codes ---------------------------------------------------------------- */
#define BHR_OK 0
#define BHR_ERR_INVALID_ARG (-1)
#define BHR_ERR_OOM (-2)
#define BHR_ERR_CUDA (-3)
#define BHR_ERR_TIMEOUT (-4)      /* a bounded device-side wait ran out */
#define BHR_ERR_UNSUPPORTED (-5)  /* e.g. DISK_VOLUMETRIC, no sm_103 device */
#define BHR_ERR_NOT_READY (-6)    /* surrogate used before it was trained or loaded */
#define BHR_ERR_IO (-7)

/* ---- hit status (low bits of bhr_hit.status) -------------------------------------- */
#define BHR_STATUS_ESCAPED 1   /* blackhole.frag status 1 */
#define BHR_STATUS_CAPTURED 2  /* blackhole.frag status 2 (horizon test) */
#define BHR_STATUS_BUDGET 3    /* step budget ran out; blackhole.frag:252 shades it as captured */
#define BHR_STATUS_OPAQUE 4    /* volumetric disk: transmittance fell below 0.004 (blackhole.frag:234 status 3) */
#define BHR_STATUS_BODY 5      /* the march hit a body (blackhole.frag status 4) */

/* ---- bhr_hit.flags ----------------------------------------------------------------- */
#define BHR_FLAG_FP64 0x01       /* some or all of the march ran in FP64 (mixed precision) */
#define BHR_FLAG_SURROGATE 0x02  /* record produced by the learned orbit surrogate */
#define BHR_FLAG_FALLBACK 0x04   /* surrogate declined the ray; the integrator produced it */
#define BHR_FLAG_NONFINITE 0x08  /* a non-finite state was met (blackhole.frag:367 NaN view) */

/* ---- disk modes (src/Settings.h:7, shaders/common.glsl:12-14) ---------------------- */
#define BHR_DISK_NONE 0
#define BHR_DISK_THIN 1
#define BHR_DISK_VOLUMETRIC 2 /* marched by bhr_trace_volumetric (bhr_trace refuses it) */

/* ---- termination rules ------------------------------------------------------------- */
/* SHADER: blackhole.frag:144,151-155 - capture r < 2.02, tolerance escape
 *         0.75 b^3/r^4 < esc_tol once outgoing beyond r_esc_min = max(1.25 r_out, 12),
 *         steps ds = max(step_scale * r * farMul, 0.02) plus the disk-slab clamp.
 * CONFIG: same step rule; capture r < capture_r (2.0001), escape once outgoing with
 *         r > escape_r (1000); farFieldDirection is still applied at the exit.
 * CPU:    src/physics/Geodesic.h:107-140 trace() - capture r < 2.01, tolerance escape with
 *         esc_tol / r_esc_min, ds = max(step_scale * r, 1e-4), no farMul, no slab clamp. */
#define BHR_TERM_SHADER 0
#define BHR_TERM_CONFIG 1
#define BHR_TERM_CPU 2

/* ---- precision / method selectors for bhr_trace ------------------------------------- */
#define BHR_PREC_FP32 0   /* plain FP32 march */
#define BHR_PREC_MIXED 1  /* FP32 bulk, FP64 for the photon-sphere band and r < promote_r */
#define BHR_METHOD_PLAIN 0
#define BHR_METHOD_SURROGATE 1

/* One camera view: the tracer uniforms of blackhole.frag:27-37 and disk.glsl:8-10, plus the
 * termination rule. bhr_view_init() fills the reference defaults. 160 bytes. */
typedef struct bhr_view {
    float cam_pos[3];      /* uCamPos = vec3(Camera::position())             Renderer.cpp:249 */
    float cam_basis[9];    /* uCamBasis, column-major, columns right, up, back Renderer.cpp:250 */
    float tan_half_fov;    /* uTanHalfFov = tan(radians(fovDeg) * 0.5f)       Renderer.cpp:246 */
    float jitter[2];       /* uJitter (pixels), 0 for parity                   Renderer.cpp:248 */
    int32_t width;         /* uResolution.x */
    int32_t height;        /* uResolution.y */
    int32_t max_steps;     /* uMaxSteps                                         Renderer.cpp:314 */
    float step_scale;      /* uStepScale */
    float disk_step;       /* uDiskStep */
    float disk_inner;      /* uDiskInner */
    float disk_outer;      /* uDiskOuter */
    float disk_thickness;  /* uDiskThickness (H/r) */
    int32_t disk_mode;     /* uDiskMode: BHR_DISK_* */
    int32_t lensing;       /* uLensing */
    int32_t far_mode;      /* uFarMode (camera radius > 1e7, App.cpp:506) */
    int32_t term_mode;     /* BHR_TERM_* */
    float capture_r;       /* horizon test radius */
    float escape_r;        /* CONFIG escape radius */
    float esc_tol;         /* tolerance escape (ESC_TOL, geodesic.glsl:8) */
    float r_esc_min;       /* CPU rule's rEscMin; SHADER derives max(1.25 disk_outer, 12) (frag:89) */
    float ds_floor;        /* smallest step (0.02 shader, 1e-4 CPU mirror) */
    float promote_band;    /* MIXED: |b - sqrt(27)| below this runs in FP64 (1e-2) */
    float promote_r;       /* MIXED: march continues in FP64 once r < promote_r (2.5) */
    int32_t reserved[6];
} bhr_view;

/* Per-pixel hit record: the march state blackhole.frag's shading reads after the loop
 * (status/escDir :97-98, the crossing points handed to thinDiskSample :209-216, bAxis :88)
 * plus the fields of the CPU mirror's TraceResult (Geodesic.h:97-103). 64 bytes = four
 * 16-byte words: the first two are written when the ray ends, the last two when it starts
 * (b_axis, b) and at each recorded crossing. */
typedef struct bhr_hit {
    uint8_t status;        /* BHR_STATUS_* */
    uint8_t ncross;        /* crossings recorded below (r in [disk_inner, disk_outer]), 0..3 */
    uint8_t flags;         /* BHR_FLAG_* */
    uint8_t nplane;        /* all y = 0 plane crossings (TraceResult::equatorCrossings), saturating */
    uint32_t steps;        /* march steps executed */
    float dir[3];          /* escDir (unit) when status is ESCAPED, else zero (as TraceResult::dir) */
    float min_r;           /* smallest r seen at the loop head (TraceResult::minR) */
    float reserved[2];
    float b_axis;          /* impactParameterAboutAxis(camPos, dir, +Y) */
    float b;               /* impact parameter h / |v_inf| (Geodesic.h:50-54 impactParameter) */
    float cross_r[3];      /* |hit.xz| of recorded crossings, march order (disk.glsl:114) */
    float cross_phi[3];    /* atan(hit.z, hit.x) of recorded crossings (disk.glsl:116) */
} bhr_hit;

typedef struct bhr_ctx bhr_ctx;

typedef struct bhr_options {
    int32_t device;        /* CUDA device ordinal */
    int32_t block_size;    /* 0 = autotuned / default */
    int32_t blocks_per_sm; /* 0 = autotuned / default */
    int32_t chunk;         /* rays a warp takes from the work queue at once, 0 = default */
    int32_t refill;        /* idle lanes before a warp refills, 0 = default */
    int32_t tile_w;        /* pixel tile of a warp's 32 work items: 32 (32x1 rows), 16 (16x2), 8 (8x4); 0 = 32 */
    int32_t reserved[2];
} bhr_options;

/* Launch shape of the FP32 march (block and tile shapes). bhr_autotune measures candidates;
 * every shape gives bit-identical hit records, only the speed differs. */
typedef struct bhr_launch_shape {
    int32_t block_size;    /* threads per block: 256 or 512 */
    int32_t blocks_per_sm; /* resident blocks per SM, 0 = as many as fit */
    int32_t chunk;         /* work items a warp claims at once (rounded up to a multiple of 32) */
    int32_t refill;        /* idle lanes of a warp that trigger its refill, 1..32 */
    int32_t tile_w;        /* pixel tile of 32 consecutive work items: 32, 16 or 8 pixels wide */
    float ms;              /* bhr_autotune: median time of one trace with this shape, else 0 */
} bhr_launch_shape;

typedef struct bhr_plan bhr_plan;

/* Per-call statistics, filled by bhr_trace_stats after the stream work completed. */
typedef struct bhr_stats {
    uint64_t rays;           /* rays traced */
    uint64_t steps;          /* sum of executed march steps */
    uint64_t fp64_rays;      /* rays that ran (partly) in FP64 */
    uint64_t fp64_steps;     /* steps taken in FP64 */
    uint64_t surrogate_rays; /* rays answered by the surrogate */
    uint64_t fallback_rays;  /* rays the surrogate sent to the integrator */
    uint64_t nonfinite;      /* rays with a non-finite state */
    uint64_t reserved;
} bhr_stats;

/* ---- context ----------------------------------------------------------------------- */
int bhr_abi_version(void);
int bhr_create(bhr_ctx** ctx, const bhr_options* opts); /* opts may be NULL */
int bhr_destroy(bhr_ctx* ctx);
const char* bhr_last_error(const bhr_ctx* ctx); /* ctx may be NULL: last global error */

/* ---- host helpers mirroring Settings / Camera / setTraceUniforms --------------------- */
/* Fills v with the reference defaults (Settings.h:19-37,82: High preset, thin disk [6,20],
 * H/r 0.035, FOV 60) and the given termination rule's constants. */
int bhr_view_init(bhr_view* v, int term_mode);
/* Applies Settings::applyPreset's trace fields (Settings.cpp:12-35): preset 0..3 = Low..Ultra
 * (max_steps, step_scale, disk_step; disk mode is left as it is). */
int bhr_view_apply_preset(bhr_view* v, int preset);
/* Camera pose from a position and a target, as Camera::lookAt / lookRotation
 * (Camera.cpp:12-23,67): float basis through a unit quaternion, up (0,1,0) with the
 * (0,0,-1) fallback when |dot(f, up)| > 0.999. Sets cam_pos and cam_basis. */
int bhr_view_look_at(bhr_view* v, const double pos[3], const double target[3]);
/* Camera.cpp:12-23 lookRotation(from, target, up): unit quaternion (w, x, y, z) of a camera at
 * `from` looking at `target` (up NULL = +Y). */
int bhr_look_rotation(const double from[3], const double target[3], const float up[3], float quat_wxyz[4]);
/* Camera pose -> uCamPos / uCamBasis (Renderer.cpp:249-250): position, and the basis
 * mat3_cast(orientation) with columns right, up, back. */
int bhr_view_set_pose(bhr_view* v, const double pos[3], const float quat_wxyz[4]);
/* tan_half_fov from a vertical FOV in degrees, as Renderer.cpp:246 (float arithmetic). */
int bhr_view_set_fov(bhr_view* v, float fov_deg);
/* Pose on a sphere: pos = r (sin i sin a, cos i, sin i cos a), looking at the hole. */
int bhr_view_orbit_pose(bhr_view* v, double r, double incl_rad, double azim_rad);
/* Rays of a view (width * height). */
int64_t bhr_view_rays(const bhr_view* v);

/* ---- tracing ------------------------------------------------------------------------- */
/* Traces nviews views. out_dev[k] is a caller-owned device buffer of width*height records
 * for view k. precision: BHR_PREC_*; method: BHR_METHOD_*. One view runs the plain kernel
 * with the view in constant memory; several views run one persistent launch over a
 * shared work queue. Work memory (queue counters, FP64 hand-off queue) is owned by ctx.
 * BHR_METHOD_SURROGATE (BHR_PREC_FP32 only) needs a surrogate bound with
 * bhr_ctx_set_surrogate (else BHR_ERR_NOT_READY): the views it answers (lensing on, not far
 * mode, thin disk or none, every termination rule) go through bhr_surrogate_trace, rays it
 * declines included, and the other views through the plain march, in the same call. */
int bhr_trace(bhr_ctx* ctx, const bhr_view* views, int nviews, bhr_hit* const* out_dev,
              int precision, int method, void* cuda_stream);
/* Host-memory variant for callers without device buffers (the CPU mirror's trace() callers):
 * traces into context-owned device staging and copies every view's records to out_host[k]
 * (width*height records each), overlapping the copies of one group of views with the trace
 * of the next. Synchronous: returns after all records are on the host. Pinned host buffers
 * (cudaHostAlloc) let the copies run asynchronously. */
int bhr_trace_host(bhr_ctx* ctx, const bhr_view* views, int nviews, bhr_hit* const* out_host,
                   int precision, int method);
/* Mixed-precision trace of one view (as bhr_trace with BHR_PREC_MIXED, BHR_METHOD_PLAIN) for
 * callers that cannot allocate device memory: a render loop that must not stall on cudaMalloc
 * and cudaFree (they synchronise the device), a host whose memory pool owns all device memory,
 * or code recording a CUDA graph. This entry point has no counterpart in the reference. It needs
 * no context and allocates nothing: its work memory is one static device array of about 15 MB,
 * held by every GPU that loads the library until the process exits, and sized for at most
 * 262144 rays (e.g. 512x512 or 640x360) per call; larger views are rejected with
 * BHR_ERR_INVALID_ARG. Runs on the current device and on cuda_stream; errors are reported by
 * bhr_last_error(NULL). Every call shares that array: calls that overlap on the GPU (other
 * streams or host threads) race, calls on one stream are ordered. The first call on a device
 * resolves the array's device address (cudaGetSymbolAddress, which may load the module): make
 * it before any stream capture. */
int bhr_trace_noalloc(const bhr_view* view, bhr_hit* out_dev, void* cuda_stream);
/* ---- learned orbit surrogate ------------------------------------------------------------
 * A small MLP (3 -> 64 -> 64 -> 64 -> 2, SiLU; BF16 tensor-core hidden layers with FP32
 * accumulation) corrects a closed-form elliptic-integral skeleton of the orbital-plane orbit
 * u(phi; r_cam, b) and predicts the capture flag; it is trained on orbits the FP64 integrator
 * generates. Captured orbits are answered too (the network's capture flag, crossings from the
 * exact one-real-root elliptic form). Rays near b = sqrt(27), outgoing at the camera, outside
 * the trained range, or whose learned capture flag disagrees with b fall back to the plain
 * integrator. No counterpart in the reference (the reference only integrates). */
typedef struct bhr_surrogate bhr_surrogate;
typedef struct bhr_surrogate_config {
    float rc_lo, rc_hi;    /* trained camera radii (6, 200) */
    float b_max;           /* trained impact parameters [0, b_max] (60) */
    float band;            /* |b - sqrt(27)| below this falls back to the integrator (2e-3) */
    float t_eps, t_scale;  /* input transform of b (1e-3, 0.125) */
    float y_scale;         /* output scale of the polar-angle residual (0.02) */
    float escape_r;        /* exit radius of the training orbits (1000, the CONFIG rule) */
    int32_t reserved[8];
} bhr_surrogate_config;
int bhr_surrogate_default_config(bhr_surrogate_config* cfg);
/* Binds a surrogate to a context for bhr_trace / bhr_trace_host with BHR_METHOD_SURROGATE
 * (NULL unbinds). The context does not own it: it must stay alive, on the context's device,
 * while it is bound. The reference's Renderer::tracePass (src/Renderer.cpp:369-387) has one
 * trace method; this selects the second. */
int bhr_ctx_set_surrogate(bhr_ctx* ctx, bhr_surrogate* s);
int bhr_surrogate_create(bhr_surrogate** s, int device, const bhr_surrogate_config* cfg, uint64_t seed);
int bhr_surrogate_destroy(bhr_surrogate* s);
/* Integrates n_orbits orbits (FP64 RK4 in the orbital plane) and keeps samples_per_orbit (2..8)
 * training samples of each; counts (may be NULL): escaped, captured, unusable orbits. */
int bhr_surrogate_generate(bhr_surrogate* s, int64_t n_orbits, int samples_per_orbit, uint64_t seed,
                           void* cuda_stream, uint64_t* counts);
/* Adam with a cosine learning-rate schedule; loss_out (may be NULL): 2 floats per step (mean
 * squared error of the scaled residual, mean capture cross-entropy). */
int bhr_surrogate_train(bhr_surrogate* s, int steps, int batch, float lr_max, float lr_min, float w_capture,
                        uint64_t seed, void* cuda_stream, float* loss_out);
/* Copies generated samples [offset, offset + n) to the host: n x {x1, x2, sigma, y}, labels. */
int bhr_surrogate_samples(bhr_surrogate* s, int64_t offset, int64_t n, float* out, int8_t* labels);
int bhr_surrogate_param_count(void);
int bhr_surrogate_params(bhr_surrogate* s, float* out, int n);
int bhr_surrogate_set_params(bhr_surrogate* s, const float* in, int n);
/* One forward + backward pass over exactly these samples (n x {x1, x2, sigma, y}, labels 0
 * escaped / 1 captured / 2 ignored; n a multiple of 32): the summed gradients of
 * mean(w_u (y_pred - y)^2) + w_capture mean(BCE), and loss sums {sum err^2, sum BCE, n_y}. */
int bhr_surrogate_gradients(bhr_surrogate* s, const float* samples, const int8_t* labels, int n, float w_capture,
                            float* grad_out, float* loss_out);
/* Forward pass: n queries {x1, x2, sigma} -> n x {y, capture logit} (tensor-core kernel with
 * bounded completion waits; BHR_ERR_TIMEOUT if one ran out). */
int bhr_surrogate_eval(bhr_surrogate* s, const float* queries, int n, float* out);
/* Self-test of the device-side timeout path (no reference counterpart): one tile of the forward
 * pass with its MMAs withheld, so that every completion wait runs out after about 1e8 SM clocks
 * with nothing in flight. Returns BHR_ERR_TIMEOUT when the kernel reported the expired waits (the
 * expected result) and BHR_ERR_CUDA if it did not; the context stays usable either way. */
int bhr_surrogate_wait_selftest(bhr_surrogate* s);
int bhr_surrogate_save(bhr_surrogate* s, const char* path);
int bhr_surrogate_load(bhr_surrogate* s, const char* path);
/* Selects the variant bhr_surrogate_trace runs (no counterpart in the reference): use_network 1
 * (the default) is the learned surrogate, whose network corrects a cheap closed form; 0 is the
 * same pass with its per-view tables built from the converged closed form (Carlson R_F with three
 * duplication steps) and no network: the non-learned orbit table the learned part is measured
 * against. The fallback rays are the same. */
int bhr_surrogate_use_network(bhr_surrogate* s, int use_network);
/* Surrogate-plus-fallback trace, stream-ordered like bhr_trace. Views: lensing on, not far mode,
 * thin disk or none; the CONFIG rule at the trained exit radius (escape_r), or the SHADER / CPU
 * rule's tolerance escape (0 < esc_tol <= 0.01), which the surrogate applies where the march's
 * escape test first passes in the limit of small steps (beyond rEscMin, at the radius where
 * 0.75 b'^3 / r^4 reaches esc_tol, b' the impact parameter at the current speed), then
 * farFieldDirection there. Other views: BHR_ERR_UNSUPPORTED (bhr_trace with
 * BHR_METHOD_SURROGATE sends them to the plain march instead).
 * The rays of the photon-sphere band (|b - sqrt 27| < band) are found before the surrogate pass
 * and marched by the plain integrator beside it (views sharing one rule, up to 64); the rays the
 * pass itself sends back are marched after it. Either way a ray's record is the plain march's. */
int bhr_surrogate_trace(bhr_surrogate* s, const bhr_view* views, int nviews, bhr_hit* const* out_dev,
                        void* cuda_stream);
/* Host-memory variant (records copied to out_host[k]; synchronous), as bhr_trace_host. Groups of
 * views are traced on two pipelines in turn, each with its own work memory, so that one group's
 * copy to the host overlaps the next group's trace. */
int bhr_surrogate_trace_host(bhr_surrogate* s, const bhr_view* views, int nviews, bhr_hit* const* out_host);
/* The same trace of a fixed batch of views captured once into a CUDA graph and replayed: the
 * launches of a trace (the band search and march, the tables, one pass per view, the fallback
 * march) become one graph launch. The plan uses the surrogate's work
 * memory and outputs: replays and traces on the same surrogate must not overlap on the GPU, and a
 * later trace that needs more work memory (more rays or views) reallocates it, after which
 * bhr_surrogate_plan_launch returns BHR_ERR_NOT_READY (recreate the plan).
 * bhr_surrogate_trace_stats covers replays too; bhr_surrogate_trace_times only eager traces.
 * No counterpart in the reference. */
typedef struct bhr_surrogate_plan bhr_surrogate_plan;
int bhr_surrogate_plan_create(bhr_surrogate* s, const bhr_view* views, int nviews, bhr_hit* const* out_dev,
                              bhr_surrogate_plan** plan);
int bhr_surrogate_plan_launch(bhr_surrogate_plan* plan, void* cuda_stream);
/* New cameras (and any other fields but the sizes) for the plan's views, as bhr_plan_update: the
 * trace is re-captured with the same outputs and the instantiated graph updated in place. */
int bhr_surrogate_plan_update(bhr_surrogate_plan* plan, const bhr_view* views, int nviews);
int bhr_surrogate_plan_destroy(bhr_surrogate_plan* plan);
/* Device time of the last bhr_surrogate_trace: ms2[0] from its start to the end of the views'
 * passes (the tables and passes; the band march runs beside them), ms2[1] from there to its end
 * (the fallback march of the rays the passes sent back, and the rest of the band march if that
 * was still running). */
int bhr_surrogate_trace_times(bhr_surrogate* s, float* ms2);
/* Of the last bhr_surrogate_trace: rays answered by the surrogate, rays marched by the
 * integrator (band march and fallback), capture-flag disagreements (also sent to the
 * integrator), integrator steps of those rays, network rows (the views' exit and crossing
 * tables: 2 x 2048 exit points, 2048 more for the tolerance escape's second branch, and
 * 256 x 64 crossing points per view; the rays read them by interpolation), network rows
 * evaluated (the same: whole 128-row tiles). */
int bhr_surrogate_trace_stats(bhr_surrogate* s, uint64_t* out6);

/* Statistics of the last bhr_trace on ctx (synchronises that call's stream). */
int bhr_trace_stats(bhr_ctx* ctx, bhr_stats* stats);
/* Per-view latency of the last multi-view bhr_trace: milliseconds from the start of the
 * launch to the moment the view's last ray finished (synchronises that call's stream). */
int bhr_trace_view_times(bhr_ctx* ctx, double* ms, int nviews);

/* ---- lens table (the second consumer of the integrator) ------------------------------ */
/* The star-disruption renderer's lens table (shaders/gas_lens.comp:10-43, gas_lens.glsl:13-21,
 * built by GasParticleRenderer::buildLensTable, src/GasParticles.cpp:161-171): for a camera at
 * radius cam_r, a fan of BHR_LENS_RAYS rays in one plane through the hole at local angles
 * alpha = bhr_lens_alpha((i + 0.5) / BHR_LENS_RAYS, bhr_shadow_angular_radius(cam_r)), and
 * table[j * BHR_LENS_RAYS + i] = log r of ray i after sweeping j 2 pi / (BHR_LENS_PHIS - 1)
 * around the hole (log 2 once captured, log 2e5 once escaped). method BHR_METHOD_PLAIN: the
 * reference's RK4 construction (FP32); BHR_METHOD_SURROGATE: every texel from the closed-form
 * orbit, in parallel (cam_r > 3, outside the photon sphere). table_dev: device memory, 4 MiB. */
#define BHR_LENS_RAYS 1024
#define BHR_LENS_PHIS 1024
int bhr_lens_table(bhr_ctx* ctx, float cam_r, int method, float* table_dev, void* cuda_stream);
float bhr_lens_alpha(float u, float alpha_crit);         /* lensAlpha, gas_lens.glsl:13-17 */
double bhr_shadow_angular_radius(double r);              /* shadowAngularRadius, Geodesic.h:78-82 */

/* ---- shading: hit records -> image (the consumer of the hit records) ------------------ */
/* What blackhole.frag does with the march's result when the disk is thin and no bodies, gas
 * or universe sky are on screen (uUniverse = 0, BHS_BODIES 0, BHS_GAS 0):
 *   - each recorded crossing shaded by thinDiskSample (disk.glsl:113-129) and composited front
 *     to back (blackhole.frag:209-216), the ray turning opaque below transmittance 0.004 (:234);
 *   - escaped, non-opaque rays get the sky (sky.glsl:105-118) with the footprint built from the
 *     screen-space derivatives of escDir (blackhole.frag:297-310; fine 2x2-quad differences,
 *     the unlensed footprint where a quad mixes escaped and other pixels);
 *   - the shadow overlay (:354-359), the NaN clear and the clamp at 0 (:377-379).
 * The sky cube (textureGrad(uSkyCube, ...) in sampleSky: galaxies, nebulae and the Milky Way
 * that SkyBaker bakes) is the caller's: rgba[3] is the weight of that term, transmittance x
 * skyBrightness x g^4 (x the overlay's 1 - k), so the reference's fragColor.rgb is
 * rgba.rgb + rgba.a * skyCube(escDir). The analytic star layers are included in rgba.rgb.
 * Disk noise comes from the context's 128^3 R16F noise volume (noise_bake.comp, baked on first
 * use and again when noise_seed changes) and colours from the blackbody LUT
 * (DiskTextures.cpp:65-91). Texture filtering uses exact weights (GL's hardware rounds the
 * linear-filter weights to 8 bits). Output: float4 per pixel, row-major with row 0 at the
 * bottom like the hit records, 16-byte aligned device memory. */
#define BHR_NOISE_SIZE 128    /* DiskTextures::kNoiseSize */
#define BHR_BLACKBODY_LUT 256 /* DiskTextures::kLutSize: rgb of luminance 1, a = Y / Y(6500 K) */
typedef struct bhr_shade_params {
    float disk_density;        /* uDiskDensity        Settings.h:38  (1.0) */
    float disk_opacity;        /* uDiskOpacity        diskOpacity x fade strength (2.0) */
    float disk_peak_temp;      /* uDiskPeakTemp       Kelvin (6000) */
    float disk_brightness;     /* uDiskBrightness     diskBrightness x fade strength (5.5) */
    float disk_noise_scale;    /* uDiskNoiseScale     (1.0) */
    float disk_noise_strength; /* uDiskNoiseStrength  (0.85) */
    float disk_time;           /* uDiskTime           flow clock in M, [0, 60) */
    float disk_warmth;         /* uDiskWarmth         (0.4) */
    float disk_inflow;         /* uDiskInflow         (0; 0.08 for the debris disk) */
    float doppler_strength;    /* uDopplerStrength    0 film look, 1 physical (0) */
    float sky_brightness;      /* uSkyBrightness      weight of the caller's sky cube (1.0) */
    float star_density;        /* uStarDensity        (1.0) */
    float star_brightness;     /* uStarBrightness     (1.0) */
    int32_t shadow_overlay;    /* uShadowOverlay      (0) */
    uint32_t noise_seed;       /* noise_bake.comp uSeed, DiskTextures.cpp:106 (7) */
    float time;                /* uTime (Renderer.cpp:253): cloud drift and stellar granulation of bodies (0) */
    int32_t reserved[4];
} bhr_shade_params;
int bhr_shade_default_params(bhr_shade_params* p);
/* Shades nviews views: hits_dev[k] holds view k's records (from any trace entry point),
 * rgba_dev[k] gets width x height float4. Stream-ordered like bhr_trace. A volumetric view
 * (disk_mode BHR_DISK_VOLUMETRIC) is shaded in place: rgba_dev[k] holds what
 * bhr_trace_volumetric gathered (rgb, transmittance) and gets the finished pixel. */
int bhr_shade(bhr_ctx* ctx, const bhr_view* views, int nviews, const bhr_hit* const* hits_dev,
              const bhr_shade_params* params, float* const* rgba_dev, void* cuda_stream);
/* The volumetric disk (the reference's default disk, Settings.h:22): blackhole.frag's march
 * with uDiskMode == DISK_VOLUMETRIC. Inside the disk slab the step is clamped to 6 diskStep
 * and each RK4 segment is sub-sampled along its cubic Hermite interpolant; every sample in
 * the disk's volume adds emission and absorption (volumetricDiskStep, disk.glsl:88-110) with
 * the look in `params`, and the ray turns opaque (BHR_STATUS_OPAQUE) once the transmittance
 * falls below 0.004 (blackhole.frag:169-181,217-234). hits_dev[k] gets the records (no
 * crossing slots), rgbt_dev[k] width x height float4 = (gathered rgb, transmittance); pass
 * rgbt_dev[k] to bhr_shade as that view's rgba to add the sky. FP32; views must have
 * disk_mode BHR_DISK_VOLUMETRIC and the SHADER or CONFIG rule. Stream-ordered. */
int bhr_trace_volumetric(bhr_ctx* ctx, const bhr_view* views, int nviews, bhr_hit* const* hits_dev,
                         const bhr_shade_params* params, float* const* rgbt_dev, void* cuda_stream);
/* The disk's noise volume (noise_bake.comp): BHR_NOISE_SIZE^3 IEEE half values, texel
 * (x, y, z) at (z N + y) N + x, into device memory. */
int bhr_noise_bake(bhr_ctx* ctx, uint32_t seed, uint16_t* out_dev, void* cuda_stream);
/* The blackbody table (DiskTextures::bakeBlackbodyLut) into host memory: BHR_BLACKBODY_LUT x 4
 * floats, entry i at T = exp(log 1000 + (log 40000 - log 1000) i / 255). */
int bhr_blackbody_lut(float* out_host);

/* ---- bodies: planets and stars in the march (the BHS_BODIES variant) ------------------ */
/* Spheres the march can hit (blackhole.frag:101-121,146-150,182-190,236-250): near-field
 * bodies settled by a straight camera-relative ray while the geodesic has not bent away from
 * it; short steps near the others and an intersection test on each step's chord. The layout is
 * the reference's BodyGpu (src/Bodies.h:40-49, shaders/bodies.glsl:12-21), as packBodies fills
 * it: at most BHR_MAX_BODIES per view (the shader's 32-bit masks). */
#define BHR_MAX_BODIES 32
typedef struct bhr_body {
    float pos_radius[4];   /* xyz centre relative to the hole (M), w radius */
    float rel_pos[4];      /* xyz centre relative to the camera, w kind (0 planet, 1 star) */
    float look[4];         /* x look id, y seed, z atmosphere / plumes, w rotation (rad) */
    float tint[4];         /* rgb albedo tint, w turbulence (stars) */
    float light[4];        /* xyz unit direction towards its light, w intensity */
    float light_color[4];  /* rgb light colour, a effective temperature (stars, K) */
    float axis[4];         /* xyz unit spin / ring axis */
    float ring[4];         /* x inner, y outer ring radius (0: none), z phase, w opacity */
} bhr_body;
/* What the shading after the loop needs of a body-aware march, per pixel (64 bytes). */
typedef struct bhr_body_hit {
    int32_t body;          /* hitBody: the body the march hit, -1 none */
    float t;               /* hitT: distance along the hit chord */
    float ro[3];           /* hitRo: start of the hit chord (hole frame) */
    float rd[3];           /* hitRd: unit direction of the hit chord */
    float x[3];            /* the ray's last position (the far-side straight test starts there) */
    uint32_t near_mask;    /* bodies settled by the near-field test */
    int32_t near_idx;      /* body the near-field straight ray hits, -1 none */
    float near_t;          /* its distance along that ray */
    float travelled;       /* path length marched */
    float reserved;
} bhr_body_hit;
/* Marches one view (thin or no disk, SHADER or CONFIG rule) with `nbodies` bodies (host
 * array): hits_dev gets the records (status BHR_STATUS_BODY when a body stopped the ray),
 * body_dev width x height bhr_body_hit. Stream-ordered. */
int bhr_trace_bodies(bhr_ctx* ctx, const bhr_view* view, const bhr_body* bodies, int nbodies, bhr_hit* hits_dev,
                     bhr_body_hit* body_dev, void* cuda_stream);
/* The same with the volumetric disk (the reference's default disk with BHS_BODIES 1,
 * blackhole.frag:101-121,146-150,169-190,217-250): the march of bhr_trace_volumetric with the body
 * tests of bhr_trace_bodies, the disk sampled on each step before the ray can turn opaque
 * (BHR_STATUS_OPAQUE) and before the step's chord meets a body, so a ray stopped by a body keeps
 * the disk's light gathered in front of it. rgbt_dev gets width x height float4 (gathered rgb,
 * transmittance); pass it to bhr_shade_bodies as rgba_dev, which shades it in place. The view
 * must have disk_mode BHR_DISK_VOLUMETRIC; params is the disk's look. FP32. Stream-ordered. */
int bhr_trace_bodies_volumetric(bhr_ctx* ctx, const bhr_view* view, const bhr_body* bodies, int nbodies,
                                const bhr_shade_params* params, bhr_hit* hits_dev, bhr_body_hit* body_dev,
                                float* rgbt_dev, void* cuda_stream);
/* Shades one view marched by bhr_trace_bodies (bhr_shade plus blackhole.frag:255-296): the hit
 * body's surface (shadeBodySurface, bodies.glsl:224-292: nine planet looks, stars, an exploding
 * photosphere), a body turning transparent letting the ray on, the bodies along the straight
 * stretches before and after the march (with their rings), and the halos of the bodies the ray
 * just missed; then the sky. params->time is uTime. rgba_dev as bhr_shade's: a volumetric view
 * (marched by bhr_trace_bodies_volumetric) is shaded in place, rgba_dev holding its rgbt. */
int bhr_shade_bodies(bhr_ctx* ctx, const bhr_view* view, const bhr_hit* hits_dev, const bhr_body_hit* body_dev,
                     const bhr_body* bodies, int nbodies, const bhr_shade_params* params, float* rgba_dev,
                     void* cuda_stream);

/* ---- launch shapes and the autotuner ------------------------------------------------ */
/* No counterpart in the reference (its march is one fragment-shader draw whose scheduling the
 * GL driver owns); these choose how the persistent march kernel covers a batch of views. */
int bhr_get_launch_shape(const bhr_ctx* ctx, bhr_launch_shape* shape);
int bhr_set_launch_shape(bhr_ctx* ctx, const bhr_launch_shape* shape);
/* Times candidate shapes on this workload (staged search over block size and chunk, then
 * refill, tile and blocks per SM; one warm-up and `reps` timed traces each, CUDA events, the
 * median), makes the fastest the context's shape and returns it in `best` (may be NULL).
 * Synchronous; writes the outputs. A repeated call with the same workload signature (views'
 * sizes, budgets and rules, precision) returns the cached result without measuring. */
int bhr_autotune(bhr_ctx* ctx, const bhr_view* views, int nviews, bhr_hit* const* out_dev, int precision, int reps,
                 bhr_launch_shape* best);

/* ---- plans: a fixed batch of views replayed as one CUDA graph ------------------------- */
/* The batched launch of many views (uneven sizes and budgets, one persistent kernel per rule
 * and 64 views) captured once into a CUDA graph with its own device scratch, then replayed by
 * bhr_plan_launch. autotune != 0 runs bhr_autotune first. The output buffers stay bound to the
 * plan. bhr_plan_update changes camera and budget fields of the views (same count, sizes,
 * rules and outputs) by re-capturing and updating the instantiated graph in place. The
 * reference's closest counterpart is one Renderer::render per frame (src/Renderer.h:61). */
int bhr_plan_create(bhr_ctx* ctx, const bhr_view* views, int nviews, bhr_hit* const* out_dev, int precision,
                    int autotune, bhr_plan** plan);
int bhr_plan_update(bhr_plan* plan, const bhr_view* views, int nviews);
int bhr_plan_launch(bhr_plan* plan, void* cuda_stream);
int bhr_plan_launch_shape(const bhr_plan* plan, bhr_launch_shape* shape);
/* after the launch's stream work completed: */
int bhr_plan_stats(bhr_plan* plan, bhr_stats* stats);
int bhr_plan_view_times(bhr_plan* plan, double* ms, int nviews); /* completion of each view after launch start */
int bhr_plan_destroy(bhr_plan* plan);

#ifdef __cplusplus
}
#endif
#endif /* BHR_H */
