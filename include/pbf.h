/*
 * pbf.h — C ABI of the GB300 (sm_103a) Position Based Fluids substep library.
 *
 * This is the drop-in boundary for pbf's per-substep simulation path: the
 * SPH class (src/SPH.h, src/SPH.cpp), its RadixSort (src/RadixSort.h) and its
 * NeighbourCellFinder (src/NeighbourCellFinder.h).  Every entry point below
 * names the reference member it replaces.
 *
 * Conventions
 *  - Plain C types only: pointers, sizes, POD structs.  No exceptions cross
 *    the ABI; every call returns a pbf_status, and pbf_last_error() gives the
 *    message of the last failure on a handle.
 *  - The library owns all device memory of a handle (the reference's SPH owns
 *    its GL buffers, src/SPH.cpp:96-133).  Caller pointers are borrowed for the
 *    duration of the call only.
 *  - Particle state crosses the ABI as float4 per particle (x, y, z, w) in
 *    particle-id order, exactly like the reference's position and velocity
 *    buffers (src/SPH.h:49,181; shaders/sph/update.glsl:26-27).  The w lane is
 *    written as 0 and ignored on input.
 *  - A handle is bound to the CUDA device that was current at creation and
 *    to one CUDA stream (default: a non-blocking stream the handle owns).
 *    Calls on one handle are not thread-safe, matching the reference's
 *    single GL context.
 *  - Stepping is asynchronous.  Device-side failures (non-finite positions, a
 *    sort lookback that ran out of its spin budget) are latched in a device
 *    status word and reported by the next synchronising call (pbf_synchronize,
 *    pbf_get_state, the pbf_get_* debug reads).
 */
#ifndef PBF_GB300_PBF_H
#define PBF_GB300_PBF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Bumped whenever a struct passed across the ABI changes layout (2: pbf_tuning
 * gained coop_candidates and auto_period; 3: adjoint_warp_candidates).  A
 * caller compiled against another version must not pass its structs to this
 * library. */
#define PBF_ABI_VERSION 3

typedef enum pbf_status {
    PBF_OK = 0,
    PBF_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or parameter */
    PBF_ERR_OUT_OF_MEMORY = 2,    /* a device or pinned-host allocation failed */
    PBF_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    PBF_ERR_DEVICE_FAULT = 4,     /* the device status word latched an error */
    PBF_ERR_NO_DEVICE = 5,        /* no CUDA device is visible */
    PBF_ERR_UNSUPPORTED = 6       /* the request is outside what this build does */
} pbf_status;

/* Bits of the device status word (pbf_device_status). */
#define PBF_DEV_NONFINITE 0x1u       /* a predicted or solved position was NaN/Inf */
#define PBF_DEV_SORT_TIMEOUT 0x2u    /* a radix-sort lookback exceeded its spin limit */
#define PBF_DEV_RUN_OVER_127 0x4u    /* a 3-cell neighbour run held >= 128 particles; the
                                        reference's packed 8-bit count
                                        (shaders/sph/foreachneighbour.glsl:5) would have
                                        dropped it.  Informational only. */
#define PBF_DEV_INDEX 0x8u           /* a bounds check of the bounds-checked build
                                        (compiled with -DPBF_CHECK) failed; the access
                                        was skipped */

/* Where a caller pointer lives. */
#define PBF_HOST 0
#define PBF_DEVICE 1

/*
 * Simulation parameters.  The first eight floats are the reference's
 * sphparams_t uniform block (src/SPH.h:252-285) in the same order; the rest
 * are the host fields and constants the reference keeps elsewhere.
 */
typedef struct pbf_params {
    float one_over_rho_0;            /* SPH::SetRestDensity stores 1/rho (src/SPH.cpp:166-169) */
    float epsilon;                   /* SPH::SetCFMEpsilon (src/SPH.h:79) */
    float gravity;                   /* SPH::SetGravity (src/SPH.h:93) */
    float timestep;                  /* SPH::SetTimestep (src/SPH.h:107) */
    float tensile_instability_k;     /* SPH::SetTensileInstabilityK (src/SPH.h:131) */
    float tensile_instability_scale; /* SPH::SetTensileInstabilityScale (src/SPH.h:144), = 1/Wpoly6(dq) */
    float xsph_viscosity_c;          /* SPH::SetXSPHViscosity (src/SPH.h:159) */
    float vorticity_epsilon;         /* SPH::SetVorticityEpsilon (src/SPH.h:175) */
    float h;                         /* kernel radius; a shader constant in the reference (src/SPH.cpp:58) */
    uint32_t num_solver_iterations;  /* SPH::SetNumSolverIterations (src/SPH.h:197) */
    uint32_t vorticity_confinement;  /* SPH::SetVorticityConfinementEnabled (src/SPH.h:220); also gates XSPH */
    uint32_t external_force;         /* SPH::SetExternalForce (src/SPH.h:230) */
    uint32_t grid[3];                /* cell grid (x, y, z), the SPH ctor's gridsize (src/SPH.h:40); cell edge = 1 */
    float wall_lo[3];                /* position clamp box; the reference hard-codes (16,0,16) .. */
    float wall_hi[3];                /* .. GRID_SIZE-(16,0,16) (shaders/sph/updatepos.glsl:98-100) */
} pbf_params;

typedef struct pbf_sim pbf_sim;

/* ---- parameters and scenes (host only, no GPU needed) ---------------------- */

/* Reference defaults (src/SPH.cpp:24-26,136-144, src/SPH.h:40) for a grid of
 * the given size, except h = 1 (one cell edge) so the 27-cell stencil covers
 * the kernel support.  Walls as in shaders/sph/updatepos.glsl:98-100. */
pbf_status pbf_params_default(const uint32_t grid[3], pbf_params* out);

/* Poly6 kernel W(r; h) as the reference's host helper SPH::Wpoly6
 * (src/SPH.cpp:159-164), evaluated in double. */
double pbf_wpoly6(double r, double h);

/* Poly6 density of an interior point of a cubic lattice of the given spacing,
 * self term excluded (the neighbour loop skips j == i,
 * shaders/sph/foreachneighbour.glsl:9), in double. */
double pbf_rest_density_lattice(double h, double spacing);

/* Seeded block scene: lattice[0] x lattice[1] x lattice[2] particles at
 * origin + spacing * (i, j, k), each coordinate jittered by U(-jitter, jitter),
 * velocities U(-vel_uniform, vel_uniform) per component, plus N(0, vel_sigma^2)
 * when vel_sigma > 0.  Particle ids run x outermost, then z, then y, as in
 * Simulation::ResetParticleBuffer (src/Simulation.cpp:214-229).  Random
 * numbers come from a 64-bit Mersenne twister (mt19937_64) with explicit
 * uniform / Box-Muller transforms, so every platform generates the same bytes.
 * x4 and v4 receive lattice[0]*lattice[1]*lattice[2] float4 each. */
pbf_status pbf_scene_block(const uint32_t lattice[3], float spacing, const float origin[3],
                           float jitter, float vel_uniform, float vel_sigma, uint64_t seed,
                           float* x4, float* v4);

/* ---- single-scene handle: the SPH class ------------------------------------ */

/* SPH::SPH (src/SPH.h:40, src/SPH.cpp:24-151).  Any n >= 1 (the reference
 * needs a multiple of 512).  Uses the current CUDA device. */
pbf_status pbf_create(const pbf_params* params, uint32_t n, pbf_sim** out);

/* Several independent scenes in one handle (no reference counterpart: the
 * reference steps one scene).  Scene k has scene_counts[k] particles and its
 * own parameters (grid, walls, constants); all scenes share the iteration
 * count and the vorticity flag.  Particle state is the scenes' float4 arrays
 * concatenated in scene order; every other call (state, stepping, timing,
 * tuning, debug reads) works on a batch as on a single scene, and each stage
 * is one launch over all scenes.  A scene in a batch steps bit-identically to
 * the same scene in its own handle. */
pbf_status pbf_create_batch(const pbf_params* scene_params, const uint32_t* scene_counts,
                            uint32_t num_scenes, pbf_sim** out);
uint32_t pbf_num_scenes(const pbf_sim* sim);
/* First particle and particle count of a scene in the concatenated arrays. */
pbf_status pbf_scene_range(const pbf_sim* sim, uint32_t scene, uint32_t* first, uint32_t* count);
/* Parameters of one scene (the grid must not change). */
pbf_status pbf_set_scene_params(pbf_sim* sim, uint32_t scene, const pbf_params* params);
pbf_status pbf_get_scene_params(const pbf_sim* sim, uint32_t scene, pbf_params* out);
/* Cells of all scenes: the length of the pbf_get_cells tables. */
uint32_t pbf_num_cells(const pbf_sim* sim);

/* SPH::~SPH (src/SPH.h:43, src/SPH.cpp:153-157). */
void pbf_destroy(pbf_sim* sim);

/* All SPH::Set* parameter setters at once (src/SPH.cpp:166-204, uploaded by
 * SPH::UploadSPHParams :206-216).  The grid must not change.  Single-scene
 * handles only (a batch takes pbf_set_scene_params); pbf_get_params returns
 * scene 0's parameters. */
pbf_status pbf_set_params(pbf_sim* sim, const pbf_params* params);
pbf_status pbf_get_params(const pbf_sim* sim, pbf_params* out);
uint32_t pbf_num_particles(const pbf_sim* sim);

/* Binds the handle to a CUDA stream (cudaStream_t passed as void*); NULL
 * restores the handle's own stream.  The substep is captured as a CUDA graph,
 * so the legacy default stream cannot be used. */
pbf_status pbf_set_stream(pbf_sim* sim, void* stream);

/* Initial particle state, float4 per particle in id order; what the
 * reference's Simulation::ResetParticleBuffer writes into the SPH buffers
 * (src/Simulation.cpp:248-268).  where = PBF_HOST or PBF_DEVICE. */
pbf_status pbf_set_state(pbf_sim* sim, const float* x4, const float* v4, int where);

/* Reads positions / velocities (id order), the contents of
 * GetPositionBuffer / GetVelocityBuffer (src/SPH.h:49,181).  Either pointer
 * may be NULL.  Synchronises and reports the device status word. */
pbf_status pbf_get_state(pbf_sim* sim, float* x4, float* v4, int where);

/* Zero-copy device pointers to the id-order position and velocity arrays
 * (float4[n]), the CUDA counterpart of the GL buffer names returned by
 * GetPositionBuffer / GetVelocityBuffer. */
pbf_status pbf_device_buffers(pbf_sim* sim, float** x4, float** v4);

/* SPH::Run (src/SPH.h:235, src/SPH.cpp:246-334), `substeps` times:
 * predict, cell keys, stable radix sort, cell ranges, num_solver_iterations
 * x (lambda, delta-p + wall clamp), velocity commit, and, when
 * vorticity_confinement is set, XSPH viscosity + vorticity confinement.
 * Asynchronous on the handle's stream.  After the first call the substep is
 * replayed from a captured CUDA graph (one per sweep configuration).  Under
 * PBF_SWEEP_AUTO, a call in which a trial completes waits on the host for the
 * trial's substeps (at most once per trial period, 32 to 256 substeps). */
pbf_status pbf_step(pbf_sim* sim, uint32_t substeps);

/* Performance knobs of a handle.  None of them changes any result: every
 * setting produces the same bits (the tests check this). */
typedef struct pbf_tuning {
    uint32_t use_neighbour_lists; /* 1: the first lambda sweep of a substep records each
                                     particle's candidates within h + skin (in the
                                     reference's visit order) and later sweeps replay
                                     them while a displacement guard proves no other
                                     candidate can be within h; 0 (default): every
                                     scanning sweep walks the full 27-cell stencil (the
                                     reference's loop) */
    uint32_t list_capacity;       /* entries per particle; longer lists fall back to the
                                     full stencil scan for that particle */
    float skin_h;                 /* list radius is h * (1 + skin_h) */
    uint32_t block_size;          /* threads per block of the neighbour sweeps: a
                                     multiple of 32 in [32, 256]; 0 = 256 */
    uint32_t sweep_mode;          /* PBF_SWEEP_DIRECT: a full stencil scan evaluates each
                                     candidate within h where it finds it;
                                     PBF_SWEEP_MASKED (default): it scans each run in
                                     chunks of 32 candidates, marks the ones within h in
                                     a bit mask, then evaluates the marked ones, in the
                                     same order (a warp's lanes stay converged);
                                     PBF_SWEEP_COOP: a warp per particle, its lanes
                                     testing 32 candidates at once and computing their
                                     pair terms in parallel, folded in the same order
                                     (for scenes too small to fill the GPU with a
                                     thread per particle, and clumped states; the
                                     default below 32,768 particles per handle) */
    uint32_t pair_list_capacity;  /* with PBF_SWEEP_MASKED and > 0: each lambda sweep
                                     records every particle's candidates within h (in
                                     visit order, up to this many), evaluates its own
                                     pairs from that list, and the delta-p sweep over
                                     the same positions replays it instead of scanning
                                     the stencil; the same between the two vorticity
                                     passes.  Longer lists fall back to scans.  0 = off;
                                     default 128; PBF_SWEEP_DIRECT records none */
    uint32_t coop_candidates;     /* with PBF_SWEEP_DIRECT or PBF_SWEEP_MASKED and no skin
                                     lists: particles whose 27-cell stencil holds more
                                     than this many candidates are swept by the
                                     warp-cooperative kernels, the rest a thread each
                                     (clumped states); 0 = off */
    uint32_t auto_period;         /* PBF_SWEEP_AUTO: substeps before the first trial and
                                     between trials while the choice or its measured
                                     time keeps changing (doubling up to 256 substeps
                                     while both hold); 0 = 32 */
    uint32_t adjoint_warp_candidates; /* pbf_backward: particles whose stencil holds more
                                     than this many candidates get a warp each in the
                                     reverse neighbour sweeps (their pair terms summed
                                     across its lanes), the others a thread; 0 = 512;
                                     0xFFFFFFFF: a thread for every particle */
} pbf_tuning;

/* PBF_SWEEP_AUTO (default): the solver sweeps (lambda + delta-p) and the two
 * vorticity passes each run one of the PBF_PASS_* configurations.  A trial
 * steps one real substep under each candidate configuration with stage
 * events, and the handle keeps the fastest solver and vorticity
 * configurations.  Every configuration gives the same bits, so trials change
 * no result; skin lists are not used.  Handles start with PBF_PASS_COOP below
 * 32,768 particles and from there with PBF_PASS_MIXED (a thread per particle,
 * and a warp for each particle in a dense stencil) for one scene and
 * PBF_PASS_MASKED for a batch. */
enum { PBF_SWEEP_DIRECT = 0, PBF_SWEEP_MASKED = 1, PBF_SWEEP_COOP = 2, PBF_SWEEP_AUTO = 3 };
enum {
    PBF_PASS_MASKED = 0,      /* masked scans (with pair lists when pair_list_capacity > 0) */
    PBF_PASS_DIRECT = 1,      /* direct stencil loops */
    PBF_PASS_COOP = 2,        /* warp-cooperative sweeps */
    PBF_PASS_DIRECT_COOP = 3, /* direct first sweep (lambda, vorticity a), cooperative second
                                 (delta-p, vorticity b); not among the automatic mode's
                                 candidates (its cooperative sweeps walk piles pair by pair) */
    PBF_PASS_MIXED = 4        /* masked scans, and warp-cooperative sweeps for the particles
                                 with more than coop_candidates (0: 256) stencil candidates */
};

/* No reference counterpart (the reference has no tuning surface). */
pbf_status pbf_set_tuning(pbf_sim* sim, const pbf_tuning* tuning);
pbf_status pbf_get_tuning(const pbf_sim* sim, pbf_tuning* out);
/* The PBF_PASS_* configurations the next substep runs for the solver sweeps
 * (out[0]) and the vorticity passes (out[1]), and the number of
 * PBF_SWEEP_AUTO trials since the last state upload or tuning change
 * (out[2]).  No reference counterpart. */
pbf_status pbf_get_sweep_choice(const pbf_sim* sim, uint32_t out[3]);

/* Autotuner: times `trial_substeps` substeps from the current state under
 * each candidate tuning (sweep block size 128 / 256; direct or masked
 * sweeps; neighbour lists off, or on with skin 0.05h / 0.1h / 0.2h),
 * restoring the state before every trial
 * and after the last, and keeps the fastest, which it also writes to `best`
 * (may be NULL).  The state is unchanged on return.  Since no tuning changes
 * any result, tuning never changes a simulation. */
pbf_status pbf_autotune(pbf_sim* sim, uint32_t trial_substeps, pbf_tuning* best);

/* Waits for the handle's stream and reports the device status word. */
pbf_status pbf_synchronize(pbf_sim* sim);
pbf_status pbf_device_status(pbf_sim* sim, uint32_t* bits);

/* Per-phase timers, the counterpart of SPH's GL_TIME_ELAPSED queries
 * (src/SPH.cpp:218-240): predict, sort, neighbour cells, solver,
 * commit + vorticity.  When enabled, pbf_step runs each substep eagerly
 * with CUDA events between the stages and waits for it; ms[5] receives the
 * last substep's times.  Enabling (or re-enabling) resets the sums below. */
pbf_status pbf_enable_timing(pbf_sim* sim, int enable);
pbf_status pbf_get_timing(pbf_sim* sim, float ms[5]);

/* Stage sums (ms) over all substeps run since timing was last enabled:
 * predict, sort, cell ranges, lambda (all iterations), delta-p (all
 * iterations), commit, XSPH/vorticity pass A, vorticity pass B.  *substeps
 * receives how many substeps the sums cover.  No reference counterpart; the
 * per-kernel split of the phases above. */
pbf_status pbf_get_stage_times(pbf_sim* sim, double ms_sum[8], uint32_t* substeps);

/* Number of kernels one substep launches under the current sweep
 * configuration (for launch accounting). */
uint32_t pbf_kernels_per_substep(const pbf_sim* sim);
/* Kernels launched by all substeps of this handle so far (graph replays,
 * automatic-mode trials and timed substeps, each counted under the
 * configuration it ran); the difference around a window counts its
 * launches.  No reference counterpart. */
uint64_t pbf_kernels_launched(const pbf_sim* sim);

/* ---- debug reads of the last substep's intermediates (synchronising) -------- */

/* Cell key of every particle in id order (the key GetHash computes,
 * shaders/radixsort/counting.glsl:53-57), sorted keys and the sort
 * permutation (perm[i] = id of the i-th particle in sorted order,
 * the w lane of RadixSort's output records).  Any pointer may be NULL. */
pbf_status pbf_get_sort(pbf_sim* sim, uint32_t* keys_by_id, uint32_t* sorted_keys, uint32_t* perm);

/* Dense cell tables of NeighbourCellFinder (findcells.glsl:34-53):
 * start[c] = first sorted index in cell c, end[c] = one past its last, both
 * -1 for empty cells.  Each array has pbf_num_cells() entries (the scenes'
 * grids one after the other). */
pbf_status pbf_get_cells(pbf_sim* sim, int32_t* start, int32_t* end);

/* Lambda of the last solver iteration and the predicted positions (float4,
 * sorted order) the neighbour runs were built from.  Either may be NULL. */
pbf_status pbf_get_solver(pbf_sim* sim, float* lambda_sorted, float* xpred4_sorted);

/* ---- standalone stages on caller device buffers ----------------------------- */

/* RadixSort::Run (src/RadixSort.h:57, src/RadixSort.cpp:124-133): stable sort
 * of n 32-bit keys on their low `numbits` bits (1..32), onesweep with
 * decoupled lookback.  perm_out[i] = input index of the i-th smallest key,
 * ties in input order; keys_out (may be NULL) receives the sorted keys.
 * keys_out and perm_out must not alias keys_in or each other.
 * Device pointers; runs on `stream` and synchronises before returning.
 * Scratch memory is allocated by the library on first use and cached. */
pbf_status pbf_radix_sort(const uint32_t* keys_in, uint32_t* keys_out, uint32_t* perm_out,
                          uint32_t n, uint32_t numbits, void* stream);

/* Allocation-free variant of pbf_radix_sort, with the same arguments and
 * results.  No counterpart in the reference (its RadixSort allocates its GL
 * buffers in the constructor, where allocation is always allowed).  For
 * callers that cannot call cudaMalloc: a host application whose own
 * allocator has reserved all of the GPU's memory (a cudaMalloc from this
 * library would fail or steal from its pool), or a real-time loop that must
 * not stall on the allocator's implicit synchronisation.  It allocates
 * nothing: its scratch is one device array inside the library, sized for at
 * most 1,048,576 keys (larger n returns PBF_ERR_INVALID_ARGUMENT), which every
 * GPU that loads the library holds (about 13.6 MB) until the process exits.
 * The first call on a device looks up that array's device address (once per
 * device, cached for the life of the process, so cudaDeviceReset after it is
 * not supported); make the first call on each device before any stream
 * capture.  All calls share the array, and each call clears what must start
 * at zero; calls whose work overlaps on the GPU (other streams, other host
 * threads) race and corrupt each other: serialise them.  keys_out and
 * perm_out must not alias keys_in or each other.  Device pointers; runs on
 * `stream` and synchronises before returning. */
pbf_status pbf_radix_sort_noalloc(const uint32_t* keys_in, uint32_t* keys_out, uint32_t* perm_out,
                                  uint32_t n, uint32_t numbits, void* stream);

/* NeighbourCellFinder's findcells pass (shaders/neighbourcellfinder/findcells.glsl:34-53)
 * on n sorted keys below num_cells: fills start/end (num_cells entries each,
 * -1 for empty cells).  Device pointers; synchronises before returning. */
pbf_status pbf_find_cells(const uint32_t* sorted_keys, uint32_t n, uint32_t num_cells,
                          int32_t* start, int32_t* end, void* stream);

/* ---- differentiation (no reference counterpart) ------------------------------ */

/* Gradient of a scalar loss with respect to the scalar parameters; one per
 * scene (an array of pbf_num_scenes() entries). */
typedef struct pbf_param_grads {
    double epsilon;                /* CFM relaxation epsilon */
    double tensile_instability_k;  /* s_corr k */
    double xsph_viscosity_c;       /* XSPH c */
    double vorticity_epsilon;      /* vorticity confinement epsilon */
} pbf_param_grads;

/* Runs `substeps` substeps from the current state like pbf_step and keeps
 * what pbf_backward needs: the state every `checkpoint_every` substeps (the
 * substeps in between are recomputed during the backward pass) and the final
 * state.  Parameters must not change until pbf_backward; pbf_set_params and
 * pbf_set_scene_params drop the recording. */
pbf_status pbf_forward_record(pbf_sim* sim, uint32_t substeps, uint32_t checkpoint_every);

/* Reverse-mode gradient of a loss L(x_final, v_final) through the recorded
 * substeps: dL_dx4 / dL_dv4 (float4 per particle, id order; NULL = zero) are
 * the loss gradients at the end of the run; dL_dx0_4 / dL_dv0_4 receive the
 * gradients with respect to the state at the start (either may be NULL), and
 * grads (NULL or one entry per scene) those with respect to the scalar
 * parameters.  The sort permutation and neighbour candidates are frozen from
 * the forward pass (piecewise constant); the wall clamp contributes its
 * subgradient.  Hand-written adjoint kernels, FP32, deterministic.  Leaves the
 * state at the end of the recorded run. */
pbf_status pbf_backward(pbf_sim* sim, const float* dL_dx4, const float* dL_dv4, int where,
                        float* dL_dx0_4, float* dL_dv0_4, pbf_param_grads* grads);

/* Frees the recording of pbf_forward_record. */
pbf_status pbf_release_record(pbf_sim* sim);

/* SPH's highlight pass (clearhighlight.glsl:7, highlight.glsl:16-30, run from
 * src/SPH.cpp:288-297): flags (one uint32 per particle, id order) have bit 0
 * set on selected particles; bit 1 is cleared everywhere and then set on every
 * stencil candidate of a selected particle (the 27-cell candidates, as the
 * reference's FOR_EACH_NEIGHBOUR, not distance-filtered), using the last
 * substep's sort.  Synchronising. */
pbf_status pbf_highlight_neighbours(pbf_sim* sim, uint32_t* flags, int where);

/* ---- headless splatting ---------------------------------------------------------- */

/* The camera of SurfaceReconstruction's particle passes: the two matrices of
 * the reference's TransformationBlock (shaders/particledepth/vertex.glsl:29-32),
 * column-major as GL and glm store them. */
typedef struct pbf_view {
    float viewmat[16];
    float projmat[16];
} pbf_view;

enum { PBF_SPLAT_DEPTH = 0, PBF_SPLAT_THICKNESS = 1 };

/* SurfaceReconstruction::Render's particle passes (src/SurfaceReconstruction.cpp:
 * 176-231) into a device buffer out[height][width] (row 0 at the bottom, as GL
 * window coordinates), without a GL context:
 *   PBF_SPLAT_DEPTH      shaders/particledepth: per pixel the smallest sphere
 *                        depth clip z / clip w, clamped to [0, 1], of the
 *                        particle sprites covering it; 1 where none does;
 *   PBF_SPLAT_THICKNESS  shaders/thickness with noise off: per pixel the
 *                        number of sprites covering it (as float).
 * positions: float4[n] on the device (xyz used, the layout of the position
 * buffer).  The reference renders depth at 1280 x 720 and thickness at
 * 512 x 512 with the same matrices.  Runs on `stream` and synchronises. */
pbf_status pbf_splat(int pass, const float* positions, uint32_t n, const pbf_view* view,
                     uint32_t width, uint32_t height, float* out, void* stream);

/* Binary snapshot of the state (no reference counterpart: the reference only
 * resets to its initial blocks, src/Simulation.cpp:303-305): "PBFSTATE",
 * u32 version 1, u32 particle count, u32 scene count, u32 0, then x and v as
 * float4[n] in id order, little-endian.  Loading checks the particle count. */
pbf_status pbf_save_state(pbf_sim* sim, const char* path);
pbf_status pbf_load_state(pbf_sim* sim, const char* path);

/* ---- diagnostics ------------------------------------------------------------- */

typedef struct pbf_diagnostics {
    double mean_density_error; /* mean over particles of |rho_i / rho_0 - 1| */
    double max_density_error;  /* max over particles of |rho_i / rho_0 - 1| */
    double kinetic_energy;     /* 0.5 * sum |v|^2, unit mass */
    double candidate_pairs;    /* sum over particles of (27-cell candidates - 1) */
} pbf_diagnostics;

/* Density error (self term excluded, as the lambda kernel computes it),
 * kinetic energy and neighbour-candidate count of the current state, with a
 * fresh cell sort of the current positions.  Synchronising. */
pbf_status pbf_compute_diagnostics(pbf_sim* sim, pbf_diagnostics* out);

/* ---- errors ------------------------------------------------------------------ */

const char* pbf_status_string(pbf_status status);

/* Host-side fault injection for tests (no reference counterpart): the
 * `after`-th device allocation made by the library from now on (0 = the next
 * one) fails as out of memory, without reaching the device; negative disarms. */
void pbf_debug_fail_allocation(int after);
/* Device-side timeout test hook (no reference counterpart): with spins > 0,
 * every radix-sort pass launched (or captured into a graph) after the call
 * waits on a word nothing sets instead of its predecessor tile, gives up after
 * `spins` polls and latches PBF_DEV_SORT_TIMEOUT; the sort's results are then
 * invalid and the call that synchronises reports PBF_ERR_DEVICE_FAULT.  No
 * wait is unbounded and every write stays in bounds.  0 disarms. */
void pbf_debug_sort_stall(uint32_t spins);
/* Message of the last failed call on `sim`, or of the last failed call
 * without a handle when sim is NULL.  Never NULL. */
const char* pbf_last_error(const pbf_sim* sim);
/* PBF_ABI_VERSION of the built library. */
int pbf_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PBF_GB300_PBF_H */
