/*
 * xpbi.h — C ABI of libxpbi, the GB300 (sm_103a) XPBI substep.
 *
 * The ABI mirrors the `Simulation` class of Chiplis/xpbi-webgpu
 * (web/js/sim.js:9-273) and the frame loop that drives it
 * (web/js/main.js:385-415). Every entry point is `extern "C"`, takes plain
 * pointers and sizes, returns an int status (XPBI_OK == 0) and records a
 * message retrievable with xpbi_last_error(). A handle is confined to one host
 * thread at a time. All device work is ordered on the handle's CUDA stream.
 *
 * Layouts at this boundary are the reference's buffer layouts
 * (sim.js:32-82): positions and velocities are vec4 x N (pos.w = material
 * index + colour seed in [0, 0.49); vel.w = V^n), the deformation gradient and
 * the kernel-gradient correction are mat3x3f x N (3 columns padded to vec4:
 * 12 floats per particle), aux is vec4 x N (V^n, lambda, plastic state,
 * PBF lambda), sortedIdx is u32 x N and the cell table u32 x numCells.
 */
#ifndef XPBI_H
#define XPBI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  XPBI_OK = 0,
  XPBI_ERR_INVALID = 1, /* bad argument or scene descriptor */
  XPBI_ERR_CUDA = 2,    /* a CUDA runtime call failed */
  XPBI_ERR_OOM = 3,     /* device allocation failed */
  XPBI_ERR_DEVICE = 4   /* a kernel raised its error word (bounded wait expired) */
};

/* Material kinds, sim.js:4-7 (MAT). */
enum {
  XPBI_ELASTIC = 0,
  XPBI_DP = 1,
  XPBI_NACC = 2,
  XPBI_VM = 3,
  XPBI_HB = 4,
  XPBI_SNOW = 5,
  XPBI_WATER = 6
};

#define XPBI_MAX_MATERIALS 8 /* MATS : array<Material, 8>, simkernels.js:19 */
#define XPBI_PARAMS_WORDS 64 /* 256-byte Params uniform, sim.js:160 */
#define XPBI_MATERIAL_WORDS 16 /* MAT_STRIDE, sim.js:4 */

/* One material parameter set as written by the scene factories
 * (web/js/scenes.js:40-80) and consumed by writeMaterials (sim.js:84-99):
 * DP (p0 = alpha, p1 = cohesion), NACC (p1 = beta, p2 = xi, p3 = M),
 * VM (p0 = sigmaY), HB (p0 = sigmaY, p1 = h, p2 = eta),
 * SNOW (p0 = thetaC, p1 = thetaS, p2 = xi). */
typedef struct xpbi_material {
  uint32_t kind;
  double E, nu, density; /* f64 like the JS numbers they replace; */
  double p0, p1, p2, p3; /* derived values are rounded to f32 once */
  float color[3];
  double bound_friction; /* scenes default 0.4 (sim.js:95) */
} xpbi_material;

/* A scene as handed to `new Simulation(device, scene)` (sim.js:10-30, 52-81).
 * states, velocities and color_seeds may be NULL (zeros; seeds 0). */
typedef struct xpbi_scene_desc {
  uint32_t n;                /* particles */
  const float* positions;    /* 3N */
  const uint32_t* mat_ids;   /* N, each < n_materials */
  const float* states;       /* N or NULL: initial plastic state (aux.z) */
  const float* velocities;   /* 3N or NULL */
  const float* color_seeds;  /* N or NULL: fraction added to pos.w, [0, 0.49) */
  double h;                  /* particle spacing r; support = 2h (f64 as in JS) */
  double domain_min[3];      /* grid sizing runs in f64 (sim.js:20-26) */
  double domain_max[3];
  uint32_t n_materials;      /* 1..8 */
  const xpbi_material* materials;
} xpbi_scene_desc;

/* Per-frame parameters of writeParams (sim.js:159-186, main.js:392-402).
 * pbf_iterations < 0 keeps the reference schedule (one PBF pass after every
 * XPBI iteration); k >= 0 runs PBF after the first k iterations only. */
typedef struct xpbi_params {
  float dt;
  float domain_min[3];
  float domain_max[3];
  float gravity[3];
  float collider_pos[3];
  float collider_r;
  float collider_vel[3];
  int32_t collider_active;
  float xsph_c;        /* scenes.js:88 default 0.01 */
  float omega;         /* 0.5 */
  float contact_omega; /* 0.4 */
  float pbf_eps;       /* 100 */
  float s_corr_k;      /* 1e-4 */
  float time;          /* written, never read by a kernel (sim.js:185) */
  float k_damp;        /* 0.4 (sim.js:184) */
  int32_t pbf_iterations;
} xpbi_params;

typedef struct xpbi_sim xpbi_sim;

/* Text of the last error raised on this thread ("" if none). */
const char* xpbi_last_error(void);

/* Host-only: grid sizing (sim.js:20-26), material packing (sim.js:84-99) and
 * Params packing (sim.js:159-186) into the reference's uniform words. No GPU
 * needed. params may be NULL (dt and friends left 0). */
int xpbi_pack_uniforms(const xpbi_scene_desc* scene, const xpbi_params* params,
                       uint32_t params_words[XPBI_PARAMS_WORDS],
                       uint32_t material_words[XPBI_MAX_MATERIALS * XPBI_MATERIAL_WORDS]);

/* constructor + createBuffers + createPipelines (sim.js:10-30, 32-82, 101-156).
 * Allocates all device buffers on the current CUDA device. */
int xpbi_create(const xpbi_scene_desc* scene, xpbi_sim** out);

/* Batched form: many independent scenes (uneven sizes, mixed materials) in one
 * handle; every stage runs as one launch over all scenes. Not in the
 * reference (one scene per Simulation). */
int xpbi_batch_create(const xpbi_scene_desc* scenes, uint32_t n_scenes, xpbi_sim** out);

void xpbi_destroy(xpbi_sim* sim);

/* writeMaterials (sim.js:84-99); scene < 0 applies to every scene. */
int xpbi_write_materials(xpbi_sim* sim, int32_t scene, const xpbi_material* materials, uint32_t n);

/* writeParams (sim.js:159-186); scene < 0 applies to every scene. */
int xpbi_write_params(xpbi_sim* sim, int32_t scene, const xpbi_params* params);

/* Per-scene solver schedule for batched handles (each scene of a batch may
 * use its own iteration count and water flag). */
int xpbi_set_schedule(xpbi_sim* sim, int32_t scene, int32_t iterations, int32_t has_water);

/* encodeSubstep (sim.js:220-272): enqueue one substep for every scene with
 * the given iteration count and water flag (iterations < 0: per-scene
 * schedule from xpbi_set_schedule). Asynchronous. */
int xpbi_encode_substep(xpbi_sim* sim, int32_t iterations, int32_t has_water);

/* The frame loop's substep loop (main.js:406-413): `substeps` substeps,
 * replayed from a captured CUDA graph of one substep. Asynchronous. */
int xpbi_step(xpbi_sim* sim, int32_t substeps, int32_t iterations, int32_t has_water);

/* Wait for the handle's stream and report device-side errors. */
int xpbi_synchronize(xpbi_sim* sim);

/* Run subsequent work on a caller's cudaStream_t (NULL: the handle's own). */
int xpbi_set_stream(xpbi_sim* sim, void* cuda_stream);

/* __XPBI.readPos / readVel (main.js:291-312): vec4 x N of scene `scene`
 * (0 for single-scene handles), in the current (cell-sorted) order. */
int xpbi_read_positions(xpbi_sim* sim, uint32_t scene, float* out_pos4);

/* Asynchronous form of xpbi_read_positions, like the reference's mapAsync
 * read-back (main.js:291-312): enqueues the copy of the scene's current
 * positions into out_pos4 behind the work enqueued so far and returns at
 * once. out_pos4 should be page-locked host memory, and it holds the
 * positions once xpbi_synchronize returns. Later substeps wait for the copy
 * before they move the particles, so read-back overlaps the next substep.
 * No counterpart in the reference's C surface. */
int xpbi_read_positions_async(xpbi_sim* sim, uint32_t scene, float* out_pos4);
int xpbi_read_velocities(xpbi_sim* sim, uint32_t scene, float* out_vel4);

/* Full state of one scene in the reference layouts; any pointer may be NULL.
 * cell_tab receives the scene's numCells cell start offsets after the last
 * substep's scatter (simkernels.js:131-147), sorted_idx its permutation. */
int xpbi_read_state(xpbi_sim* sim, uint32_t scene, float* pos4, float* vel4, float* F12, float* L12,
                    float* aux4, uint32_t* sorted_idx, uint32_t* cell_tab);

/* Overwrite one scene's state (pos4, vel4, F12, aux4; NULL keeps a field). */
int xpbi_write_state(xpbi_sim* sim, uint32_t scene, const float* pos4, const float* vel4, const float* F12,
                     const float* aux4);

/* The uniform words the kernels of scene `scene` consume (as packed by
 * xpbi_pack_uniforms after the last write_params / write_materials). */
int xpbi_read_uniforms(xpbi_sim* sim, uint32_t scene, uint32_t params_words[XPBI_PARAMS_WORDS],
                       uint32_t material_words[XPBI_MAX_MATERIALS * XPBI_MATERIAL_WORDS]);

/* Sizes: total particles, total cells, scenes; dims of scene 0 (may be NULL). */
int xpbi_info(xpbi_sim* sim, uint32_t* n_particles, uint32_t* n_cells, uint32_t* n_scenes, int32_t dims[3]);

/* profileSubstep (sim.js:199-215): runs one substep with a CUDA event around
 * every launch; ms[k] is launch k's time, labels (may be NULL) receives
 * "label: x.xxxms" lines. *count = number of launches recorded. */
int xpbi_profile_substep(xpbi_sim* sim, int32_t iterations, int32_t has_water, float* ms, int32_t cap,
                         int32_t* count, char* labels, size_t labels_cap);

/* Borrowed device pointers for a renderer (posBuf, velA, matsBuf bound in
 * main.js:189-199): float4 positions, float4 velocities (both cell-sorted,
 * all scenes concatenated) and the packed material table. */
int xpbi_device_ptrs(xpbi_sim* sim, void** pos4, void** vel4, void** materials);

/* Number of kernel launches one substep issues with this schedule. */
int xpbi_launches_per_substep(xpbi_sim* sim, int32_t iterations, int32_t has_water, int32_t* out);

/* Failure-path check (no counterpart in the reference): enqueues, on the
 * handle's stream, the prefix scan's bounded look-back wait on a descriptor
 * that nothing publishes. The wait gives up after `polls` polls (1..2^20,
 * ~0.1 us each) and raises the device error word, so the next
 * xpbi_synchronize returns XPBI_ERR_DEVICE and clears it; the handle stays
 * usable. No kernel faults, traps or waits without a limit. */
int xpbi_test_wait_expiry(xpbi_sim* sim, uint32_t polls);

/* ---- headless renderer (web/js/shaders/render.js, main.js:232-272) ----
 * The reference draws each frame through WebGPU: the ground plane with its
 * grid, the domain box, and every particle as a depth-correct sphere
 * impostor (material colour with a per-particle shade, diffuse +
 * hemisphere + specular lighting, water rims and speed whitening). This
 * rasterises the same frame with CUDA kernels into a device RGBA8 image,
 * with no graphics API. The camera is the reference's look-at camera
 * (main.js:24-32 gives eye from its orbit angles; fov_y pi/4, near 0.02,
 * far 50, light (0.5, 0.9, 0.35)); particle_radius <= 0 uses 0.62 h. */
typedef struct xpbi_camera {
  float eye[3];
  float target[3];
  float fov_y;             /* radians */
  float near_z, far_z;
  float light_dir[3];      /* world; normalised here */
  float particle_radius;   /* world units; <= 0: 0.62 h of the scene */
  int32_t draw_ground;     /* ground quad with grid lines at domain_min.y */
  int32_t draw_box;        /* the 12 edges of the scene's domain */
} xpbi_camera;

/* Render scene `scene` at width x height (row 0 at the top, RGBA8). rgba_out
 * (host, 4 * width * height bytes) and device_rgba (receives the device
 * image, valid until the next xpbi_render or xpbi_destroy) may be NULL.
 * Enqueued on the handle's stream; synchronous when rgba_out is given. */
int xpbi_render(xpbi_sim* sim, uint32_t scene, const xpbi_camera* cam, uint32_t width, uint32_t height,
                uint8_t* rgba_out, void** device_rgba);

/* ---- autotuner (no counterpart in the reference) ----
 * solveA and solveB are built in several launch shapes: block size (64,
 * 128 or 256 threads) and register allocation (resident blocks per SM traded
 * against registers). xpbi_autotune runs the
 * substep's preparation (sort, reorder, Bonet-Lok correction) on the current
 * state and times iteration 0 of every variant `repeats` times on this
 * handle's own data, then keeps the fastest of each for the handle (the
 * default on a tie within 1%). Everything xpbi_read_state reports is left
 * as it was (the working buffers it overwrites are saved and restored); it
 * synchronises the handle's stream and allocates temporary device memory. chosen[2] (may be NULL)
 * receives the variant indices, ms (may be NULL) the mean time of each
 * variant: XPBI_SOLVEA_VARIANTS entries for solveA, then solveB's. All
 * variants compute the same results; only their speed differs. */
#define XPBI_SOLVEA_VARIANTS 6
#define XPBI_SOLVEB_VARIANTS 5
int xpbi_autotune(xpbi_sim* sim, int32_t iterations, int32_t has_water, int32_t repeats, int32_t* chosen, float* ms,
                  int32_t cap);

/* Select variants directly (-1 keeps the current one); 0 is the default. */
int xpbi_set_variants(xpbi_sim* sim, int32_t solve_a, int32_t solve_b);

/* Lanes per particle in solveA / solveB: 1, 2, 4, or 0 (the default) to
 * choose by the handle's solid particle count (four up to 24,576 solids, two
 * up to 49,152). Small scenes leave most of the GPU idle with one thread per
 * particle; several lanes split each particle's neighbour sweep and add their
 * partial sums, which changes the summation order (results agree with one
 * lane to rounding, not bit for bit). The register variants above apply to
 * the one-lane kernels. */
int xpbi_set_lanes(xpbi_sim* sim, int32_t lanes);

/* ---- solver modes (no counterpart in the reference) ----
 * mode 0: the reference solve (every XPBI iteration starts from lambda = 0).
 * mode 1: iteration 0 starts from the particle's previous-substep multiplier
 *   plus the increment the warm-start network predicts.
 * mode 2: iteration 0 starts from the particle's previous-substep multiplier.
 * rel_tol > 0: a scene stops iterating (its remaining passes skip) once its
 *   constraint residual |C + alpha_tilde lambda + gamma dt dC/dt| (0 for an
 *   inactive constraint, C = 0) falls to rel_tol times its value at
 *   lambda = 0 and its contact residual (the contact correction solveB would
 *   apply) to contact_rel_tol times its value entering iteration 0
 *   (contact_rel_tol < 0: rel_tol); rel_tol <= 0 keeps the fixed iteration
 *   count. With a warm start the earliest stop is after
 *   iteration 0. Scheduled PBF passes run whether or not the scene stopped.
 * track_residual: record the residual norm of every iteration and of the
 *   final state (xpbi_read_residuals).
 * log_features: compute the network features every substep
 *   (xpbi_read_training). */
int xpbi_set_solver(xpbi_sim* sim, int32_t mode, float rel_tol, float contact_rel_tol, int32_t track_residual,
                    int32_t log_features);

/* Active set (no counterpart in the reference): work skipping for a solve
 * with an early stop (rel_tol > 0, one lane per slot; ignored otherwise).
 * Iterations 0 and 1 run every particle (iteration 0 moves them all).
 * From iteration 2 on, a solid is
 * re-evaluated only if its own velocity or a solid neighbour's moved since
 * its last evaluation (otherwise its residuals are unchanged), takes an
 * impulse only if its squared constraint residual exceeds share / nSolid of
 * the scene's squared budget (rel_tol^2 times the iteration-0 sum), and
 * applies a contact correction only above the same share of the contact
 * budget; a particle's velocity is updated only if it was re-evaluated or a
 * neighbour's impulse reaches it. A velocity change counts as a move if its
 * square exceeds share * rel_tol^2 times the mean squared velocity change of
 * iteration 0 (smaller ones shift a neighbour's residual by about its settle
 * threshold or less). Settled particles hold about `share` of each budget,
 * and the scene stops once the residual sums over all particles (the
 * settled ones with their last values) are within tolerance; with
 * track_residual the final state's residuals are re-measured over every
 * particle. share = 0 turns it off (the default); 0 < share <= 1. */
int xpbi_set_active_set(xpbi_sim* sim, float share);

/* Iteration cap of an early-stopped solve (rel_tol > 0; no counterpart in
 * the reference): each scene iterates until both of its residuals reach
 * their tolerances or max_iterations iterations ran, whichever is first, so
 * a solve that needs a few more iterations than the plain budget to reach
 * the plain solve's residual still reaches it. PBF passes keep the scene's
 * own schedule. 0 (the default) caps at the scene's own iteration count;
 * at most 128. The residual histories then hold max(cap, iterations) + 2
 * entries (the final state's residual last). */
int xpbi_set_max_iterations(xpbi_sim* sim, int32_t max_iterations);

/* The judge of an early-stopped solve that differs from the reference (a
 * warm start, or the active set; no counterpart in the reference): a scene
 * whose constraint or contact residual has not reached its tolerance when
 * its iteration cap runs out is re-solved in the same substep with the
 * reference solve (lambda from 0, its own iteration count and PBF passes)
 * from the velocities that entered iteration 0, and keeps that result.
 * *resolved = 1 if scene `scene` was re-solved in the last substep. In a
 * graph the re-solve sits behind a conditional node, so it costs nothing
 * when every scene stopped. */
int xpbi_read_fallback(xpbi_sim* sim, uint32_t scene, int32_t* resolved);

/* Particles visited per iteration of the last substep, summed over scenes:
 * solve_a[k] = solids solveA re-evaluated, solve_b[k] = particles solveB
 * updated, for k >= 2 (iterations 0 and 1 visit every particle and record
 * 0).
 * Either pointer may be NULL; cap entries at most. */
int xpbi_read_active_counts(xpbi_sim* sim, uint32_t* solve_a, uint32_t* solve_b, int32_t cap);

/* Load the warm-start network's 9473 parameters (layout of xpbi_mlp_*).
 * Its output is alpha_tilde times the multiplier increment over the previous
 * substep's final multiplier. */
int xpbi_set_network(xpbi_sim* sim, const float* params, uint32_t count);

/* Residual norms of the last substep of one scene: norms[0] = |C(v_pred)|,
 * norms[1 + k] = |r_k| entering iteration k (NaN after an early stop),
 * norms[1 + K] = |r| of the final state (with track_residual);
 * *iterations_run = iterations whose update was applied. */
int xpbi_read_residuals(xpbi_sim* sim, uint32_t scene, double* norms, int32_t cap, int32_t* iterations_run);

/* Contact residual norms of the last substep of one scene, in the slots of
 * xpbi_read_residuals: the norm of the contact position correction solveB
 * would apply at each iteration's velocities (norms[0] = iteration 0's). */
int xpbi_read_contact_residuals(xpbi_sim* sim, uint32_t scene, double* norms, int32_t cap);

/* Per-particle residuals of the last substep of one scene, in its cell
 * order (the order of xpbi_read_state), squared: r2 = the constraint
 * residual and c2 = the contact correction of the last pass that recorded
 * them (with track_residual: the pass after the last iteration, i.e. of the
 * final state), r0sq = the constraint residual at lambda = 0 entering
 * iteration 0. Zeros for water and inactive constraints. Any pointer may be
 * NULL. No counterpart in the reference. */
int xpbi_read_particle_residuals(xpbi_sim* sim, uint32_t scene, float* r2, float* c2, float* r0sq);

/* Training rows of the last substep of one scene (cell-sorted order):
 * features16 [n][16] (zeros for water; feature 4 is alpha_tilde times the
 * previous substep's multiplier), target [n] = alpha_tilde * final lambda,
 * *alpha_tilde (may be NULL). Needs log_features or mode 1. */
int xpbi_read_training(xpbi_sim* sim, uint32_t scene, float* features16, float* target, float* alpha_tilde);

/* ---- warm-start network (no counterpart in the reference) ----
 * A per-particle MLP 16 -> 64 -> 64 -> 64 -> 1 (SiLU), BF16 weights, FP32
 * accumulate, run on the tcgen05 tensor cores. Parameters are one f32 vector:
 * W1[64][16] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] w4[64] b4. */
int xpbi_mlp_param_count(void);

/* y[r] = net(X[r]) for rows of 16 features (host buffers, synchronous). */
int xpbi_mlp_forward(const float* X, uint32_t rows, const float* params, float* y);

/* Gradient of the mean squared error (1/rows) sum_r (net(X[r]) - T[r])^2
 * with respect to params; *loss (may be NULL) receives the error. */
int xpbi_mlp_grad(const float* X, const float* T, uint32_t rows, const float* params, float* grad, float* loss);

/* `steps` Adam steps (lr, betas 0.9 / 0.999) on consecutive mini-batches of
 * `batch` rows, cycling through the rows in the given order; params is
 * updated in place, loss_history (may be NULL) gets each step's loss. */
int xpbi_mlp_train(const float* X, const float* T, uint32_t rows, float* params, int32_t steps, uint32_t batch,
                   float lr, float* loss_history);

/* ---- scene sampling on the device (web/js/scenes.js:7-38) ----
 * The reference samples its scenes in JavaScript: sampleBox puts a lattice
 * point at every cell centre lo + (i + 0.5) h, i < max(1, Math.round(extent
 * / h)) per axis; sampleSphere keeps the points c - r + i h, i <= ceil(2 r /
 * h), with Math.hypot(p - c) <= r; each coordinate gets
 * (Math.random() - 0.5) * jitter * h. xpbi_sample_shapes runs the same loops
 * on the GPU for scenes too large to sample quickly on the host: the lattice
 * points are the reference's bit for bit (f64, one rounding per operation,
 * Math.hypot as V8 evaluates it), numbered in its loop order (z outer, x
 * inner; shapes in order), and the jitter's uniforms come from
 * Philox-4x32-10 keyed by `seed` (low word, high word) with counter
 * (particle number, 0 or 1, 0, 0): x and y from the first block, z from the
 * second, each as a 53-bit double from two words. */
enum { XPBI_SHAPE_BOX = 0, XPBI_SHAPE_SPHERE = 1 };
typedef struct xpbi_shape {
  int32_t kind;          /* XPBI_SHAPE_BOX or XPBI_SHAPE_SPHERE */
  double lo[3], hi[3];   /* box corners (sampleBox's min, max) */
  double centre[3];      /* sphere centre */
  double radius;         /* sphere radius */
  uint32_t mat_id;       /* material index of every particle of the shape */
  float state0;          /* initial plastic state */
  double jitter;         /* fraction of h (scenes.js default 0.2) */
} xpbi_shape;

/* Samples the shapes at spacing h. *count receives the particle count;
 * with positions NULL nothing else is written (a sizing call). Otherwise
 * capacity must be at least the count, and positions (3 floats per
 * particle), mat_ids and states (either may be NULL) receive the particles
 * in host memory. Synchronous; allocates temporary device memory. */
int xpbi_sample_shapes(const xpbi_shape* shapes, uint32_t n_shapes, double h, uint64_t seed, uint32_t capacity,
                       float* positions, uint32_t* mat_ids, float* states, uint32_t* count);

/* Philox-4x32-10 (Salmon et al., SC 2011) on the host, the generator
 * xpbi_sample_shapes uses: out = the block for `counter` under `key`. */
int xpbi_philox4x32_10(const uint32_t counter[4], const uint32_t key[2], uint32_t out[4]);

/* ---- cell sort without allocation (no counterpart in the reference) ----
 * For callers that own every byte of device memory and cannot let a library
 * allocate: engines and plugins that hand out buffers from their own fixed
 * pool, and code that records work into a CUDA graph, where a cudaMalloc
 * would break the recording. It runs the substep's first stage alone (cell
 * key, histogram, scan, bucket fill, deterministic ranks: the same results
 * as xpbi_encode_substep's sort) on the caller's device buffers, with all
 * scratch in one fixed array inside this library (about 10 MB per device,
 * held until the process exits). Nothing is allocated.
 *   pos4        device, n float4 (x, y, z, any w), 16-byte aligned
 *   origin, cell_size, dims   host; the grid of xpbi_read_uniforms words
 *               0..6 (cell = clamp(floor((p - origin) / cell_size), 0, dim-1))
 *   cell_start  device, out, dims[0]*dims[1]*dims[2] + 1 words, 16-byte
 *               aligned: start of each cell's run; the last word is n
 *   sorted_idx  device, out, n words: particle indices in cell order, within
 *               a cell by descending index
 *   cuda_stream the stream to enqueue on (NULL: the legacy default stream)
 * Limits: 1 <= n <= XPBI_NOALLOC_MAX_PARTICLES and at most
 * XPBI_NOALLOC_MAX_CELLS cells; larger inputs return XPBI_ERR_INVALID.
 * The first call on a device (with that device current) looks up the
 * scratch array's address; make it before any stream capture. Each call
 * clears the parts of the scratch that must start at zero (cell counters,
 * scan descriptors) itself. Calls share the one array per device: two calls
 * whose work can overlap on the GPU (other streams, other host threads)
 * race and corrupt each other's results, so serialise them. Returns after
 * enqueueing; synchronise the stream before reading the outputs. */
#define XPBI_NOALLOC_MAX_PARTICLES 262144u
#define XPBI_NOALLOC_MAX_CELLS 1048576u
int xpbi_sort_cells_noalloc(const float* pos4, uint32_t n, const float origin[3], float cell_size,
                            const int32_t dims[3], uint32_t* cell_start, uint32_t* sorted_idx, void* cuda_stream);

/* Status of the last xpbi_sort_cells_noalloc call on the current device
 * (no counterpart in the reference). Its prefix scan waits, with a bounded
 * number of polls, for earlier tiles to publish their sums; a wait that runs
 * out raises an error word inside the same fixed scratch array, and the
 * outputs of that call are then not valid. This synchronises cuda_stream
 * (the stream the sort was enqueued on), reads the word and clears it:
 * XPBI_OK, or XPBI_ERR_DEVICE with the word in xpbi_last_error(). It
 * allocates nothing. The next sort call clears the word itself, so ask
 * before making it. */
int xpbi_sort_cells_noalloc_status(void* cuda_stream);

/* Failure-path check of the above (no counterpart in the reference): runs
 * the scan's bounded look-back wait on a descriptor of the fixed scratch
 * array that nothing publishes, with a limit of `polls` polls (1..2^20,
 * ~0.1 us each), on cuda_stream. The wait gives up and raises the error word
 * that xpbi_sort_cells_noalloc_status reports. Nothing faults or waits
 * without a limit. */
int xpbi_test_noalloc_wait_expiry(uint32_t polls, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* XPBI_H */
