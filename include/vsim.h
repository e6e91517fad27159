/*
 * vsim.h -- C ABI of the GB300-native XPBD soft-body solver.
 *
 * This is the drop-in boundary for the solver/step interface of the
 * visionary-sim kernel package. Every entry point below replaces one method
 * of the reference's ES class `Simulator`
 * (packages/visionary-sim/src/sim/simulator.js:35-518) or of the seams under
 * it; the citation beside each names the exact method. A Node N-API shim (or
 * any other FFI) binds these 1:1.
 *
 * Conventions
 *   - Opaque handles, `int` status codes (VSIM_OK == 0), caller-owned output
 *     buffers, no exceptions across the ABI.
 *   - A handle is thread-compatible: calls on one handle must not overlap;
 *     different handles may be used from different threads.
 *   - Status codes map onto the reference's throws: VSIM_ERR_RANGE is its
 *     `RangeError` (timing and material values, timestep.js:38-45,183-187,
 *     material.js:80-85), VSIM_ERR_INVALID its `Error` (limits, a static
 *     hold, kinematicDrive.js:158-160). `vsim_last_error()` returns the
 *     message of the most recent failure on the calling thread.
 *   - Node indices are the reference's: bodies are concatenated in scene
 *     order, each body's nodes are its dense lattice grid
 *     `i + nx * (j + ny * k)` (lattice.js:55-57, particles.js:55-65).
 *   - Positions cross the ABI as xyzw float quadruples per node, w written as
 *     0 on reads (state.wgsl:16-19, particles.js:227-231).
 *   - All device work is issued on the handle's stream; calls that return
 *     host data synchronise that stream.
 */
#ifndef VSIM_H
#define VSIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VSIM_ABI_VERSION 1

/* Status codes. */
#define VSIM_OK 0
#define VSIM_ERR_RANGE 1      /* a value outside its documented range (RangeError) */
#define VSIM_ERR_INVALID 2    /* a request the simulator cannot honour (Error) */
#define VSIM_ERR_CUDA 3       /* the CUDA runtime reported a failure */
#define VSIM_ERR_NOMEM 4      /* device or host allocation failed, or a budget is full */
#define VSIM_ERR_DESTROYED 5  /* the handle was already destroyed */
#define VSIM_ERR_CAPACITY 6   /* a fixed-capacity buffer is too small */
#define VSIM_ERR_TIMEOUT 7    /* a bounded device wait gave up */

/* Drive laws (kinematicDrive.js:35, `DriveLaw`). */
#define VSIM_DRIVE_HARD 0
#define VSIM_DRIVE_COMPLIANT 1

/* Nodes one hold can carry (kinematicDrive.js:49, MAX_DRIVEN). */
#define VSIM_MAX_DRIVEN 4096

/*
 * A material, in the reference's units (material.js:11-28). Defaults are
 * DEFAULT_MATERIAL (material.js:69-77): E 1.2e5 Pa, nu 0.40, rho 1000,
 * friction 0.4, damping 0.6 /s, relaxation 0.012 s, maxStretch 0 (off).
 */
typedef struct vsim_material {
    double youngs_modulus;  /* E, Pa; values below 1 are read as 1 (material.js:103) */
    double poisson_ratio;   /* nu, clamped to [0.25, 0.49] (material.js:66,102) */
    double density;         /* rho, kg/m^3 */
    double friction;        /* Coulomb coefficient for the tank and contact */
    double damping;         /* velocity drag, 1/s */
    double relaxation;      /* Kelvin-Voigt relaxation time, s */
    double max_stretch;     /* 0 (off) or a finite ratio > 1 (material.js:80-85) */
} vsim_material;

/*
 * One soft body, given as the occupancy grid its voxeliser produced: the
 * input `buildLattice(grid, {density})` takes (lattice.js:161-166). Cell
 * (i, j, k) is occupancy[i + cx * (j + cy * k)] != 0. Nodes are the dense
 * (cx+1)(cy+1)(cz+1) corner grid; node (i, j, k) rests at origin + (i, j, k) h.
 */
typedef struct vsim_body_desc {
    uint32_t cell_dims[3];
    double origin[3];
    double h;                       /* cell edge, metres */
    const uint8_t* occupancy;
    vsim_material material;
    const uint32_t* static_nodes;   /* body-local nodes held in place, or NULL
                                       (staticPrescription.js:9-20) */
    uint32_t static_count;
} vsim_body_desc;

/* Tank interior; the tank is open at the top (finalize.wgsl:61-67). */
typedef struct vsim_tank {
    double min[3];
    double max[3];
} vsim_tank;

typedef struct vsim_sim vsim_sim;

/* Simulator.stats() (simulator.js:194-230), the numeric part. */
typedef struct vsim_stats {
    uint32_t body_count;
    uint32_t nodes;            /* dense node slots, inactive included */
    uint32_t active_nodes;     /* nodes with material */
    uint32_t cells;            /* occupied cells over all bodies */
    uint32_t contact_nodes;    /* surface records */
    int32_t contact;           /* body contact enabled */
    int32_t self_contact;      /* same-body contact enabled (no reference counterpart) */
    uint32_t iterations;       /* Gauss-Seidel sweeps per substep */
    uint64_t steps;            /* total fixed steps taken */
    uint32_t last_steps;       /* steps in the last frame */
    uint32_t max_steps_per_frame;
    double step_duration;      /* seconds per substep */
    double simulated_time;
    double backlog_time;
    double frame_dropped_time;
    double dropped_time;
    int32_t overloaded;
    double cfl;                /* wave rate x step duration (simulator.js:149-151) */
    int32_t limited_by;        /* body index setting the CFL, -1 with no bodies */
    uint32_t driven;           /* nodes currently held */
    uint32_t drive_capacity;   /* VSIM_MAX_DRIVEN */
} vsim_stats;

/* ---- errors ---------------------------------------------------------- */

/* Message of the last failure on this thread ("" if none). */
const char* vsim_last_error(void);
int vsim_abi_version(void);

/* ---- lifecycle (simulator.js:44-115, :505-517) ----------------------- */

/*
 * `new Simulator(device, bodies, tank)`. Builds every lattice, uploads the
 * node state and allocates everything the solver needs on the current CUDA
 * device. On failure nothing is leaked (simulator.js:111-114).
 * `stream` is a cudaStream_t to issue work on, or NULL for a stream the
 * handle creates and owns.
 */
int vsim_create(const vsim_body_desc* bodies, uint32_t body_count,
                const vsim_tank* tank, void* stream, vsim_sim** out);
/* Flags of vsim_create_ex. */
#define VSIM_CREATE_ISOLATED 1u  /* bodies never touch each other: each bins its
                                    surface into its own contact grid around it,
                                    and only same-body (self) contact exists */

/* vsim_create with options. With VSIM_CREATE_ISOLATED every body is an
   independent world (no counterpart in the reference, whose bodies all share
   one grid, bodyContact.js:343): what a batch of unrelated bodies or a pool
   of serving sessions needs. */
int vsim_create_ex(const vsim_body_desc* bodies, uint32_t body_count,
                   const vsim_tank* tank, void* stream, uint32_t flags, vsim_sim** out);
/* `destroy()`; idempotent on a NULL handle. */
int vsim_destroy(vsim_sim* sim);
/* Which bodies take part in subsequent frames (`active[b]` nonzero), NULL for
   all. A body that sits out is left exactly as it is. No counterpart in the
   reference. */
int vsim_set_bodies_active(vsim_sim* sim, const uint8_t* active, uint32_t count);

/* ---- stepping (simulator.js:239-318, :495-500) ----------------------- */

/* `step(dt)`: bank wall time on the fixed clock and dispatch its steps.
   Non-finite or negative dt counts as 0 (simulator.js:256). */
int vsim_step(vsim_sim* sim, double dt);
/* `requestStep()`: the next vsim_step takes one step even when paused. */
int vsim_request_step(vsim_sim* sim);
/* `dispatch(steps)`: run `steps` fixed substeps now. */
int vsim_dispatch(vsim_sim* sim, uint32_t steps);
/* `reset()`: release the grab, return every node to rest, clear the clock. */
int vsim_reset(vsim_sim* sim);
/* Block until all work issued on the handle's stream has finished. */
int vsim_synchronize(vsim_sim* sim);

/* ---- state transfer (simulator.js:503, particles.js:227-231) --------- */

/* `readPositions()`: xyzw per node, w = 0. `node_count` must equal the
   simulator's node count. */
int vsim_read_positions(vsim_sim* sim, float* xyzw, size_t node_count);
/* Full state read/write (xyzw each; any pointer may be NULL). Used by
   parity harnesses to start the solver and a reference from one state. */
int vsim_read_state(vsim_sim* sim, float* pos, float* prev, float* vel, size_t node_count);
int vsim_write_state(vsim_sim* sim, const float* pos, const float* prev, const float* vel,
                     size_t node_count);
uint32_t vsim_node_count(const vsim_sim* sim);
/* Where body `b`'s nodes start (Particles.offsetOf, particles.js:119-121). */
uint32_t vsim_body_node_offset(const vsim_sim* sim, uint32_t body);
/* Material inverse mass per node (Particles.invMass), static nodes included. */
int vsim_read_inv_mass(vsim_sim* sim, float* inv_mass, size_t node_count);

/* ---- grab / drive (simulator.js:383-492, kinematicDrive.js:155-264) -- */

/* KinematicDrive.hold(nodes, offsets): hold global nodes, offsets xyz per
   node from the anchor. Holding a static node fails with VSIM_ERR_INVALID and
   leaves the current hold unchanged; more than VSIM_MAX_DRIVEN keeps the
   first VSIM_MAX_DRIVEN; an empty set releases. */
int vsim_hold(vsim_sim* sim, const uint32_t* nodes, const float* offsets, uint32_t count);
/* Simulator.moveGrab(position): the grab target; its velocity for a frame is
   derived at dispatch from how far it moved (simulator.js:309-315). */
int vsim_move_grab(vsim_sim* sim, const double position[3]);
/* Place the grab target without implying motion (Simulator.grab's
   `position = previousPosition = anchor`, simulator.js:419-422). */
int vsim_place_grab(vsim_sim* sim, const double position[3]);
/* Simulator.releaseGrab() / KinematicDrive.release(). */
int vsim_release(vsim_sim* sim);

/* Simulator.grab(origin, direction) (simulator.js:383-425) without reading
   the node positions back: the nearest grabbable node along the ray within
   1.2 x the coarsest node spacing of it (pick.js:41-68), then the grip --
   the anchor alone, or every grabbable node of the anchor's body within
   `grip_radius` of it, nearest first, ties by index, at most
   VSIM_MAX_DRIVEN (grip.js:58-136) -- is held and the grab target placed
   on the anchor. Picking and gripping run on the device in double
   precision, as the reference's JavaScript does; only the anchor and the
   candidates within the radius come back. A ray that hits nothing holds
   nothing: out->body = -1. */
#define VSIM_GRIP_SINGLE_NODE 0
#define VSIM_GRIP_WITHIN_RADIUS 1
typedef struct vsim_grab_result {
    int32_t body;        /* the anchor's body, -1 when the ray missed */
    uint32_t anchor;     /* global node */
    double position[3];  /* the anchor's position: the grab target */
    uint32_t held;       /* nodes held */
    uint32_t found;      /* grabbable nodes within the grip radius, anchor included */
} vsim_grab_result;
int vsim_grab(vsim_sim* sim, const double origin[3], const double direction[3], int grip, double grip_radius,
              vsim_grab_result* out);
/* Simulator.setDriveLaw(law). */
int vsim_set_drive_law(vsim_sim* sim, int law);
/* Simulator.setDriveResponseTime(seconds): finite and > 0, else RANGE. */
int vsim_set_drive_response_time(vsim_sim* sim, double seconds);

/* ---- settings (simulator.js:332-366) --------------------------------- */

/* Bits of `fields` for vsim_set_material. */
#define VSIM_MAT_YOUNGS     (1u << 0)
#define VSIM_MAT_POISSON    (1u << 1)
#define VSIM_MAT_DENSITY    (1u << 2)
#define VSIM_MAT_FRICTION   (1u << 3)
#define VSIM_MAT_DAMPING    (1u << 4)
#define VSIM_MAT_RELAXATION (1u << 5)
#define VSIM_MAT_MAX_STRETCH (1u << 6)
/* Simulator.setMaterial(bodyIndex, changes): `fields` selects which members
   of `changes` apply. Density rescales node masses; the step duration is
   recomputed from the new wave rate. */
int vsim_set_material(vsim_sim* sim, uint32_t body, const vsim_material* changes, uint32_t fields);
/* Simulator.setContact(enabled). */
int vsim_set_contact(vsim_sim* sim, int enabled);
/* Same-body contact between nodes that share no cell. No counterpart in the
   reference (its contact skips same-body pairs, collide.wgsl:66); off by
   default. */
int vsim_set_self_contact(vsim_sim* sim, int enabled);
/* `params.gravity` (simulator.js:30-33). */
int vsim_set_gravity(vsim_sim* sim, const double gravity[3]);
/* `params.paused`. */
int vsim_set_paused(vsim_sim* sim, int paused);
/* Override the fixed step duration the clock chose from the CFL rule
   (FixedTimestep.setStepDuration, timestep.js:56-59). RANGE unless finite
   and > 0. */
int vsim_set_step_duration(vsim_sim* sim, double seconds);
/* Gauss-Seidel sweeps of the elastic colour passes per substep (1 in the
   reference; each sweep restarts lambda at zero, xpbdCouple.wgsl:9-13). */
int vsim_set_iterations(vsim_sim* sim, uint32_t iterations);
/* Record each frame's substep sequence once as a CUDA graph and replay it
   (default on). Off issues every kernel individually. */
int vsim_set_graph(vsim_sim* sim, int enabled);
/* Threads per block of the elastic colour pass (128, 256 or 512) and the
   cell order inside each colour (0: lattice order, 4 or 8: bricks of that
   many cells per axis). Chosen by vsim_tune; settable for sweeps. */
int vsim_set_launch_shape(vsim_sim* sim, uint32_t block, uint32_t brick);
/* The large colour passes (a dense pass of at least two cells per resident
   thread) through tensor-memory-accelerator brick tiles: each block takes
   bricks of 8 x 4 x 4 same-colour cells, loads their 16 x 8 x 8 node boxes
   of positions and previous positions with bulk tensor copies, solves in
   shared memory and stores the position box back. Results equal the other
   forms bit for bit. For scenes of 1 to 4 bodies (else VSIM_ERR_RANGE); off
   by default. A block whose copies never arrive (bounded wait) makes the
   next vsim_synchronize fail. */
int vsim_set_tma_pass(vsim_sim* sim, int enabled);
/* The small colour passes (under two cells per resident thread, dense) with
   each cell split over four lanes: every lane runs the tetrahedra's serial
   spine, lane q its corner's products and update, exchanged by shuffles.
   Results equal the one-lane form bit for bit. `lanes` 1 (default) or 4
   (else VSIM_ERR_RANGE). */
int vsim_set_cell_lanes(vsim_sim* sim, uint32_t lanes);
/* Time every {brick 0,4,8} x {block 128,256,512} shape on `frames` frames of
   the live state (which is saved and restored) and keep the fastest.
   Writes the chosen shape to *block and *brick when non-NULL. */
int vsim_tune(vsim_sim* sim, uint32_t frames, uint32_t* block, uint32_t* brick);

/* Launch every substep kernel with programmatic dependent launch (default
   on): the next kernel's launch overlaps the tail of the one before it. */
int vsim_set_pdl(vsim_sim* sim, int enabled);

/* How the contact gather maps surface records to GPU threads: AUTO (default)
   gives each record a warp while the substep has fewer than 2048 records
   per SM and a thread otherwise; WARP and THREAD force one mapping. All three
   give the same results (each record's hits are summed in the reference's
   order); the setting exists for tests and sweeps. No reference counterpart. */
#define VSIM_GATHER_AUTO 0
#define VSIM_GATHER_WARP 1
#define VSIM_GATHER_THREAD 2
int vsim_set_gather_mapping(vsim_sim* sim, int mapping);

/* ---- readout ---------------------------------------------------------- */

/* The six Kuhn rest shape inverses of the unit cube the kernels use,
   column-major 3x3 each (kuhn.js:78-80 as elasticCells.js:85-107 emits
   them). */
int vsim_kuhn_rest_inverse(float out[54]);

/* Simulator.stats(). */
int vsim_get_stats(vsim_sim* sim, vsim_stats* out);
/* Simulator.cflNumber(). */
int vsim_cfl_number(vsim_sim* sim, double* out);

/*
 * The contact pairs of the current positions: every pair of surface records
 * (a < b) that the broadphase puts in neighbouring buckets (with the
 * reference's 32-per-bucket visibility, contacts.wgsl:75), that the body rule
 * admits and that overlap (distance < r_a + r_b). Written as (a, b) surface
 * indices, in no particular order; *count receives the total even when it
 * exceeds `capacity` (then VSIM_ERR_CAPACITY).
 */
int vsim_contact_pairs(vsim_sim* sim, uint32_t* pairs, size_t capacity, size_t* count);
/* The contact gather's work on the current positions, for measurement (no
   reference counterpart): one contact chain is run on the handle's stream
   with each kernel bracketed by events, its grid is counted, and the grid is
   emptied again without moving any node. `candidates` sums, over the live
   records, the visible entries (at most 32 per bucket) of the record's 27
   neighbour buckets -- what the gather reads. `ms` are the device times of
   the five kernels: bin, segment, scatter, order, gather. */
typedef struct vsim_census {
    uint64_t records;           /* live surface records binned */
    uint64_t occupied_buckets;
    uint64_t candidates;
    double ms[5];
} vsim_census;
int vsim_contact_census(vsim_sim* sim, vsim_census* out);
/* Surface record table (node, body) of the contact constraint
   (bodyContact.js:325-340), `capacity` records at most. */
int vsim_contact_surface(vsim_sim* sim, uint32_t* nodes, uint32_t* bodies, size_t capacity,
                         size_t* count);

/* ---- profiling ---------------------------------------------------------- */

/* Kernel groups a frame is made of. */
#define VSIM_KIND_PREDICT 0
#define VSIM_KIND_DRIVE 1     /* unused: the drive runs inside the pass that predicts each substep */
#define VSIM_KIND_ELASTIC 2   /* the colour passes */
#define VSIM_KIND_LIMIT 3     /* limit-only stretch sweeps */
#define VSIM_KIND_CONTACT 4   /* bin, segment, scatter, order, collide, settle */
#define VSIM_KIND_FINALIZE 5
#define VSIM_KIND_SPLAT 6     /* splat deformation */
#define VSIM_KIND_SORT 7      /* splat depth sort */
#define VSIM_KIND_COUNT 8

typedef struct vsim_profile {
    double ms[VSIM_KIND_COUNT];          /* summed device time per group */
    uint32_t launches[VSIM_KIND_COUNT];  /* kernels launched per group */
} vsim_profile;

/* Run one frame of `steps` substeps (plus the splat deformation and sort
   when `with_splats`) with every kernel launched on its own, bracketed by
   CUDA events on the handle's stream, and report the device time of each
   kernel group. The frame advances the simulation like vsim_dispatch. */
int vsim_profile_frame(vsim_sim* sim, uint32_t steps, int with_splats, const float view_dir[3],
                       vsim_profile* out);
/* Time `sweeps` Gauss-Seidel sweeps of the elastic colour passes (8 passes
   each, the frame's launch shapes) run back to back as one captured graph,
   with events only at its two ends; *ms receives the total. The positions
   the passes move are saved first and restored after, so the state is
   unchanged. For roofline measurement: the bracketed launches in
   vsim_profile_frame cannot overlap one another. No reference counterpart. */
int vsim_time_colour_passes(vsim_sim* sim, uint32_t sweeps, float* ms);
/* Occupied cells per colour over all bodies (a colour pass's work). */
int vsim_color_counts(const vsim_sim* sim, uint32_t out[8]);
/* Kernels a frame of `steps` substeps launches (splats excluded). */
uint32_t vsim_frame_launches(const vsim_sim* sim, uint32_t steps);
/* Kernels one splat deformation plus sort launches. */
uint32_t vsim_splat_launches(const vsim_sim* sim);

/* ---- splats (sample.wgsl:40-80, covariance.wgsl:30-42) ---------------- */

/*
 * Bind Gaussian splats to body `body`'s lattice: rest means xyz, rotations
 * xyzw, scales xyz (standard deviations), `count` splats. Replaces whatever
 * was bound to that body. The embedding (cell and local coordinates,
 * sample.wgsl:45-51) is computed here once.
 */
int vsim_splats_bind(vsim_sim* sim, uint32_t body, const float* means, const float* quats,
                     const float* scales, uint32_t count);
/* Total splats bound over all bodies. */
uint32_t vsim_splats_count(const vsim_sim* sim);
/* Deform every bound splat from the live node positions (device side):
   mean' = x(rest) and covariance' = (F R S)(F R S)^T, and compute its depth
   key along `view_dir` (larger depth sorts first: back to front). */
int vsim_splats_deform(vsim_sim* sim, const float view_dir[3]);
/* vsim_splats_deform, and each deformed covariance taken apart into the
   ellipsoid's orientation and axis lengths in the same launch -- what a
   renderer that stores rotation + scale wants (ellipsoid.wgsl:20-91, four
   sweeps of cyclic Jacobi; apps/simulator/src/render/ellipsoid.js is its CPU
   twin). */
int vsim_splats_deform_axes(vsim_sim* sim, const float view_dir[3]);
/* The axes of the last vsim_splats_deform_axes: unit quaternions xyzw and
   axis lengths xyz, splats in bind order (either pointer may be NULL). */
int vsim_splats_read_axes(vsim_sim* sim, float* rotation, float* scale, size_t count);
/* Stable radix sort of the depth keys: the draw order, back to front. */
int vsim_splats_sort(vsim_sim* sim);
/* Copy results to the host (any pointer may be NULL): means xyz, covariance
   (xx, xy, xz, yy, yz, zz) and the draw order, splats in bind order (body
   by body). */
int vsim_splats_read(vsim_sim* sim, float* means, float* cov6, uint32_t* order, size_t count);

/* ---- device radix sort -------------------------------------------------- */

/*
 * Stable LSD radix sort of `n` 32-bit keys in device memory (the splat depth
 * sort's engine; PlayCanvas 2.21.3's GPU sorter is the reference's,
 * apps/simulator/src/scene/app.js:71-75). Writes to `d_order` the
 * permutation that sorts `d_keys` ascending, ties in index order; `d_keys`
 * is not modified. Only the low `key_bits` bits take part (1..32).
 * `d_keys` and `d_order` must not overlap (VSIM_ERR_INVALID if they do).
 * Scratch: call once with d_temp == NULL to receive the size in *temp_bytes.
 */
int vsim_radix_sort_u32(const uint32_t* d_keys, uint32_t* d_order, uint32_t n, uint32_t key_bits,
                        void* d_temp, size_t* temp_bytes, void* stream);

/*
 * The same sort for callers that cannot allocate device memory -- an engine
 * that owns the whole GPU through its own pool, a frame loop that may not
 * stall on cudaMalloc, a binding holding only raw device pointers. No
 * counterpart in the reference. It allocates and frees nothing: its scratch
 * is a fixed array of about 17 MiB inside this library, held on every GPU
 * that loads the library until the process exits, and it sorts at most
 * 1048576 keys (more fails with VSIM_ERR_CAPACITY). The first call on each
 * device looks up the array's device address; make that first call before
 * any stream capture. The address is remembered per device and context: after
 * a device reset (cudaDeviceReset, or the primary context made again) the
 * next call looks it up once more, so make that call outside a capture too.
 * All calls share the array: calls that overlap on the GPU race, so
 * serialise them. `d_keys` and `d_order` must not overlap. Same results as
 * vsim_radix_sort_u32.
 */
int vsim_radix_sort_u32_noalloc(const uint32_t* d_keys, uint32_t* d_order, uint32_t n,
                                uint32_t key_bits, void* stream);

/* ---- serving: many sessions stepped in shared frames ------------------ */
/*
 * No counterpart in the reference (one simulator per page). A server holds a
 * pool of sessions -- one body each, isolated from one another -- resident on
 * the device, admitted in order while their state fits an HBM budget; which
 * sessions are resident can be changed between ticks (eviction: the state of
 * a session that leaves is kept on the host and restored when it returns).
 * Requests ask a session to advance some frames, optionally dragging one of
 * its nodes (hard law) toward a target moving along a cubic Bezier curve.
 * Every tick runs one frame for every session with a pending request, in one
 * batched launch sequence: a request submitted while others are running
 * joins at the next frame boundary (continuous batching). A session's
 * result does not depend on which other sessions share its frames.
 */
typedef struct vsim_server vsim_server;

typedef struct vsim_server_config {
    double hbm_budget_bytes;  /* admit sessions while their device state fits; 0 = no limit */
    double step_duration;     /* seconds per substep */
    uint32_t substeps;        /* substeps per frame */
    int32_t self_contact;     /* same-body contact inside each session */
} vsim_server_config;

typedef struct vsim_drag {
    uint32_t node;            /* session-local node to hold */
    float control[4][3];      /* cubic Bezier control points of the target's path */
    double speed;             /* metres per second along the path */
} vsim_drag;

typedef struct vsim_completion {
    uint64_t request;
    uint32_t session;
    uint32_t frames;
    double submitted;         /* server clock, seconds */
    double completed;
    uint64_t first_tick;      /* tick that ran the request's first frame */
    uint64_t last_tick;
} vsim_completion;

typedef struct vsim_server_stats {
    uint32_t sessions;        /* resident */
    uint32_t rejected;        /* not admitted at creation: over the budget */
    double resident_bytes;    /* device bytes the resident sessions hold */
    uint64_t ticks;
    uint64_t session_frames;  /* frames run, summed over sessions */
    uint64_t cell_updates;    /* occupied cells x substeps, summed over frames run */
    uint32_t pending;         /* requests queued or running */
    double tick_seconds;      /* wall time inside vsim_server_tick, summed */
    double prepare_seconds;   /* of which host work before the frame's launch */
    double frame_seconds;     /* device time of the frames (CUDA events), summed */
} vsim_server_stats;

/* `stream` (a cudaStream_t, or NULL): the stream the ticks run on. NULL: the
   server makes its own at the device's greatest priority, so that a tick's
   launches start before the session engine's, whose streams are made at
   the least; a stream given should have a priority above the least too
   (cudaStreamCreateWithPriority). */
int vsim_server_create(const vsim_body_desc* sessions, uint32_t count, const vsim_tank* tank,
                       const vsim_server_config* config, void* stream, vsim_server** out);
int vsim_server_destroy(vsim_server* server);
/* How many sessions are resident. At creation they are sessions
   0 .. admitted-1 (the rest did not fit the budget). */
uint32_t vsim_server_admitted(const vsim_server* server);
/* The resident sessions, in the order of the device pool (NULL sessions:
   only *count). VSIM_ERR_CAPACITY when `capacity` is smaller. */
int vsim_server_resident(const vsim_server* server, uint32_t* sessions, uint32_t capacity, uint32_t* count);
/* Makes exactly `sessions` resident, in that order. Every session leaving
   the device must be idle (no request queued or running, else
   VSIM_ERR_INVALID); its state is kept on the host and written back when it
   is made resident again -- it then continues exactly as if it had stayed
   (a session never run starts at rest). The set must fit the budget (else
   VSIM_ERR_NOMEM, nothing changed). Drags still held from finished requests
   are let go. The device pool is rebuilt: the cost is that of creating it
   (lattices, uploads), paid once per call. */
int vsim_server_set_resident(vsim_server* server, const uint32_t* sessions, uint32_t count);
/* Seconds on the server's monotonic clock. */
double vsim_server_clock(const vsim_server* server);
/* Queue `frames` frames for `session` (FIFO per session); drag may be NULL.
   The session must be resident (else VSIM_ERR_RANGE). */
int vsim_server_submit(vsim_server* server, uint32_t session, uint32_t frames, const vsim_drag* drag,
                       uint64_t* request);
/* Run one frame for every session with a pending request (within the tick
   budget, vsim_server_set_tick_budget) and wait for it; *stepped receives
   how many sessions it advanced (0: nothing to do). */
int vsim_server_tick(vsim_server* server, uint32_t* stepped);
/* Caps the occupied cells one tick steps (0, the default: every session with
   a pending request runs). Under a cap a tick first takes the sessions whose
   requests have already started, oldest first, then waiting requests in
   arrival order, each while its cells still fit; the first always runs. The
   rest wait for the next tick: admission by slots as they free up, which
   bounds a tick's length -- and so the frame latency under load -- at some
   cost in throughput. No reference counterpart. */
int vsim_server_set_tick_budget(vsim_server* server, uint64_t cells);
/* One request of a run (vsim_server_run). */
typedef struct vsim_scheduled_request {
    double arrival;       /* seconds after the run starts (unused in a closed-loop run) */
    uint32_t session;     /* (unused in a closed-loop run) */
    uint32_t frames;
    uint32_t drag;        /* nonzero: the request drags along drags[session] */
    uint32_t pad;
} vsim_scheduled_request;

/* Open loop: the whole run. Closed loop: the measured span, from the start
   to the first tick that ends after closed_loop_seconds (the drain after it
   not counted). */
typedef struct vsim_run_report {
    uint64_t requests;    /* completed */
    uint64_t frames;      /* session-frames run */
    uint64_t ticks;
    uint32_t returned;    /* completions written to `out` (all of the run's, up to capacity) */
    uint32_t pad;
    double seconds;       /* wall time */
} vsim_run_report;

/* The server's request loop, run in the library against its own clock (no
   caller round trips between ticks). Open loop (closed_loop_seconds == 0):
   each request is submitted when its arrival time comes -- its completion
   records that scheduled time as `submitted` -- ticks run while anything is
   pending, and the loop returns once every request has completed. Closed
   loop (closed_loop_seconds > 0): as many requests as sessions are resident
   are submitted at once, the list's first (cycling), and each completion
   submits the list's next one (its arrival unused) to the session it
   names, for that long; then the loop drains. With sessions drawn
   uniformly the outstanding requests gather where service is slowest, so
   the rate measured is the capacity for that mix. Completions go to `out` (up to `capacity`; NULL: counts only),
   not to vsim_server_poll. Needs no request pending at the start. A drag
   request drags drags[session] (indexed by session id: one per session
   offered). How requests run is the server's engine
   (vsim_server_set_engine); a tick of the session engine is one launch.
   No reference counterpart. */
int vsim_server_run(vsim_server* server, const vsim_scheduled_request* requests, uint32_t n,
                    const vsim_drag* drags, double closed_loop_seconds, vsim_completion* out,
                    uint32_t capacity, vsim_run_report* report);
/* Engines of vsim_server_run. FRAMES: ticks, one frame at a time for every
   session with a request, as vsim_server_tick runs them. SESSIONS (the
   default): a session whose largest colour has at most `block_cells` cells
   (32 is the server's default) runs each request whole -- all its frames --
   in one block of the session kernel, else, with at most `cluster_cells`
   (default 512), in one cluster of 8 blocks; every such session that has a
   request and none running starts in the next launch, launches overlap,
   and a request completes when its own job ends. Larger sessions run in
   ticks of shared frames on the server's stream at the same time. Every
   engine gives every session the same result, bit for bit. The session
   engine, once used, keeps its own contact arrays (60 B a surface record
   of the resident pool, outside the admission budget) until the resident
   set changes or the server is destroyed. The session engine keeps ten
   streams busy (eight launch slots, the pool's stream and its capture
   stream); the CUDA driver feeds streams to the GPU through
   CUDA_DEVICE_MAX_CONNECTIONS hardware queues (8 unless set), and where a
   slot shares the pool stream's queue the ticks wait behind session jobs.
   Set CUDA_DEVICE_MAX_CONNECTIONS=32 in the environment before the
   process's first CUDA call (the Python package sets it when imported
   first, unless already set). */
#define VSIM_SERVE_FRAMES 0
#define VSIM_SERVE_SESSIONS 1
int vsim_server_set_engine(vsim_server* server, int engine, uint32_t block_cells, uint32_t cluster_cells);
/* Requests completed since the last poll (at most `capacity`). */
int vsim_server_poll(vsim_server* server, vsim_completion* out, uint32_t capacity, uint32_t* count);
int vsim_server_get_stats(const vsim_server* server, vsim_server_stats* out);
uint32_t vsim_server_node_count(const vsim_server* server, uint32_t session);
/* The session's node positions, xyzw, w = 0. */
int vsim_server_read_positions(vsim_server* server, uint32_t session, float* xyzw, size_t node_count);
/* Checkpoint and restore of one session (any pointer may be NULL): its
   positions, previous positions and velocities, xyzw per node (w = 0 out,
   ignored in). Writing or resetting needs the session idle (no request
   queued or running, else VSIM_ERR_INVALID); a drag still held from its last
   request is let go first. A session written back continues exactly as the
   one read out would have. Reset returns it to its rest state. */
int vsim_server_read_state(vsim_server* server, uint32_t session, float* pos, float* prev, float* vel,
                           size_t node_count);
int vsim_server_write_state(vsim_server* server, uint32_t session, const float* pos, const float* prev,
                            const float* vel, size_t node_count);
int vsim_server_reset_session(vsim_server* server, uint32_t session);

/* ---- fixed timestep clock (timestep.js:17-180), host only ------------- */

typedef struct vsim_clock vsim_clock;
typedef struct vsim_clock_report {
    double step_duration;
    uint32_t max_steps_per_frame;
    uint32_t steps;
    double elapsed;
    uint64_t total_steps;
    double simulated_time;
    double backlog_time;
    double frame_dropped_time;
    double dropped_time;
    int32_t overloaded;
} vsim_clock_report;

/* stableStepDuration(waveRate). RANGE for negative or non-finite rates. */
int vsim_stable_step_duration(double wave_rate, double* out);
/* new FixedTimestep(stepDuration, {maxStepsPerFrame}) (0 = 24). */
int vsim_clock_create(double step_duration, uint32_t max_steps_per_frame, vsim_clock** out);
int vsim_clock_destroy(vsim_clock* clock);
int vsim_clock_consume(vsim_clock* clock, double elapsed, int force_step, vsim_clock_report* out);
int vsim_clock_idle(vsim_clock* clock, vsim_clock_report* out);
int vsim_clock_single_step(vsim_clock* clock, vsim_clock_report* out);
int vsim_clock_set_step_duration(vsim_clock* clock, double step_duration);
int vsim_clock_reset(vsim_clock* clock);
int vsim_clock_snapshot(const vsim_clock* clock, vsim_clock_report* out);

/* ---- Gaussian-cloud voxeliser (cloudVolume.js:101-397) ----------------
 *
 * voxelizeCloud(cloud, {elementSize, padding, sigma, seal, fill}) on the
 * device: the occupancy grid of a cloud of Gaussians (centres xyz, unit
 * quaternions x-y-z-w, per-axis standard deviations, float32 as the
 * reference's arrays), the same cell for cell as the reference's CPU
 * voxeliser -- each Gaussian stamped as a solid ellipsoid at `sigma`
 * standard deviations with the cell holding its centre always material; with
 * `fill`, the shell dilated `seal` times, every cell the outside cannot
 * reach through face neighbours filled, eroded back and the stamp put back.
 * The reference's defaults are padding 2 (voxelize.js), sigma 2, seal 2,
 * fill on (cloudVolume.js:70,83). A cloud with no Gaussians or no extent
 * fails with VSIM_ERR_INVALID (the reference's `Error`), a bad element size
 * with VSIM_ERR_RANGE. Runs on the calling thread's current device and
 * returns when the grid is built; the result stays on the device in the
 * returned volume until it is destroyed.
 */
typedef struct vsim_cloud_options {
    double element_size; /* cell edge, metres */
    double sigma;        /* standard deviations counted as material */
    uint32_t padding;    /* empty cells added on every side */
    uint32_t seal;       /* cells the shell is thickened by before the fill */
    int32_t fill;        /* nonzero: make everything the outside cannot reach material */
} vsim_cloud_options;

typedef struct vsim_cloud_grid {
    uint32_t dims[3];  /* cells per axis; occupancy is x fastest */
    double origin[3];  /* world position of the grid's min corner */
    double h;          /* cell edge */
    uint64_t occupied; /* material cells */
    uint64_t filled;   /* cells the fill made material (fillEnclosed's count) */
} vsim_cloud_grid;

typedef struct vsim_cloud_volume vsim_cloud_volume;

/* Host arrays: positions 3 x count, rotations 4 x count, scales 3 x count. */
int vsim_voxelize_cloud(const float* positions, const float* rotations, const float* scales, uint64_t count,
                        const vsim_cloud_options* options, vsim_cloud_volume** out);
/* The same arrays already on the device; `stream` (NULL: the legacy default
 * stream) is synchronised first, so work that wrote them has finished. */
int vsim_voxelize_cloud_device(const float* d_positions, const float* d_rotations, const float* d_scales,
                               uint64_t count, const vsim_cloud_options* options, void* stream,
                               vsim_cloud_volume** out);
int vsim_cloud_volume_grid(const vsim_cloud_volume* volume, vsim_cloud_grid* out);
/* Copies the grid's occupancy (one byte per cell, 0 or 1) to `occupancy`;
 * VSIM_ERR_CAPACITY when `cells` is smaller than the grid. */
int vsim_cloud_volume_read(vsim_cloud_volume* volume, uint8_t* occupancy, size_t cells);
/* Frees the volume; NULL is accepted. */
int vsim_cloud_volume_destroy(vsim_cloud_volume* volume);
/* The fill finds what the outside reaches by rounds of sweeps over the grid
 * until a round adds nothing, and past a cap of rounds by a union-find over
 * the empty cells instead; both give the flood's set. Sets the cap for the
 * whole process (default 24; 0: always the union-find) and returns the
 * previous one. For tests of both paths; no reference counterpart. */
uint32_t vsim_cloud_set_flood_rounds(uint32_t rounds);

/* ---- material arithmetic (material.js:101-140, compliance.js:30-109) -- */

/* Lame parameters after the reference's clamps. */
int vsim_lame_parameters(const vsim_material* m, double* mu, double* lambda);
/* Element compliances for a rest volume, and gamma = 1 + mu/lambda. */
int vsim_element_compliance(const vsim_material* m, double rest_volume, double* deviatoric,
                            double* hydrostatic, double* gamma);
/* The collapse barrier of the stable Neo-Hookean energy under uniform scale. */
double vsim_collapse_scale(double gamma);
/* Longitudinal wave speed. */
double vsim_wave_speed(const vsim_material* m);

#ifdef __cplusplus
}
#endif

#endif /* VSIM_H */
