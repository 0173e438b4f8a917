/*
 * diaphane_gb300 — C ABI of a GB300-native (sm_103a) Yee leapfrog time step.
 *
 * This is the drop-in boundary for the step / source-injection / field
 * read-back API that the reference's two solvers share (src/cpu.rs:97-714 and
 * src/gpu.rs:180-730, trait Steppable in src/timeline.rs:63-72).  Every entry
 * point below names the reference interface it replaces.
 *
 * Conventions
 *   - Plain pointers and sizes only.  The caller owns every host buffer it
 *     passes; the library owns the device buffers behind a handle.
 *   - Errors come back as dp_status codes where the reference panics
 *     (assert!/expect).  dp_last_error() returns a message for the calling
 *     thread.
 *   - One handle is used from one thread at a time.  Each simulation owns one
 *     CUDA stream; dp_sim_advance and dp_sim_reverse are asynchronous on it,
 *     exactly as gpu::Simulation::advance_by returns after submit.  Reads wait.
 *   - Fields are component-major and x-major inside a component: component a
 *     of a field occupies [a*cells, (a+1)*cells), cell (x,y,z) sits at
 *     (z*ny + y)*nx + x (src/grid.rs:119-126, src/gpu.rs:25-30).
 *   - There is no CPU fallback: every dp_sim_* call runs on the GPU and fails
 *     with DP_ERR_CUDA when no device is usable.
 */
#ifndef DIAPHANE_GB300_H
#define DIAPHANE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status                                                                   */
/* ------------------------------------------------------------------------ */

typedef enum dp_status {
    DP_OK = 0,
    DP_ERR_INVALID = 1,     /* a scene or argument the reference would panic on */
    DP_ERR_LOSSY = 2,       /* reverse on a lossy scene (src/cpu.rs:253-260) */
    DP_ERR_CUDA = 3,        /* a CUDA runtime or driver call failed */
    DP_ERR_TIMEOUT = 4,     /* dp_sim_wait deadline passed (src/gpu.rs:616-622) */
    DP_ERR_OOM = 5,         /* device memory or an admission budget exhausted */
    DP_ERR_UNSUPPORTED = 6, /* a scene outside this build's limits */
    DP_ERR_RANGE = 7,       /* step past the start, size mismatch, bad index */
    DP_ERR_BUSY = 8,        /* a request slot or arena region is in use */
    DP_ERR_NONFINITE = 9    /* a batch scene's field became NaN or infinite (is_finite, src/cpu.rs:707-713) */
} dp_status;

/* Message for the last error on the calling thread ("" when none). */
const char *dp_last_error(void);
const char *dp_status_string(dp_status status);

/* ------------------------------------------------------------------------ */
/* Scene recipe — flat C mirror of Scene (src/scene.rs:116-122)              */
/* ------------------------------------------------------------------------ */

enum { DP_AXIS_X = 0, DP_AXIS_Y = 1, DP_AXIS_Z = 2 };

/* Refinement (src/grid.rs:313-320): metres from the domain centre. */
typedef struct dp_refinement {
    float center[3];
    float size[3]; /* non-positive: that axis is not refined */
    float cell_size;
} dp_refinement;

/* GridSpec (src/grid.rs:381-392): the recipe, not the resolved arrays. */
typedef struct dp_grid_spec {
    uint32_t extent[3]; /* cells at cell_size; refinements only subdivide */
    float cell_size;    /* metres */
    float courant;      /* S = c*dt/d_ref, in (0, 1/sqrt(3)] */
    float max_ratio;    /* growth cap between neighbouring cells, > 1 */
    uint32_t refinement_count;
    const dp_refinement *refinements;
} dp_grid_spec;

enum { DP_BOUNDARY_PEC = 0, DP_BOUNDARY_ABSORBING = 1 };

/* Boundary (src/boundary.rs:53-67). */
typedef struct dp_boundary {
    uint32_t kind;
    uint32_t thickness;      /* cells, absorbing only */
    float target_reflection; /* absorbing only, in (0, 1) */
} dp_boundary;

/* Material (src/material.rs:29-39).  Infinite conductivity is a PEC. */
typedef struct dp_material {
    float relative_permittivity;
    float relative_permeability;
    float conductivity;
    float magnetic_loss;
} dp_material;

enum { DP_SHAPE_BLOCK = 0, DP_SHAPE_SPHERE = 1, DP_SHAPE_SLAB = 2 };

/* Shape (src/scene.rs:32-56).  Later shapes overwrite earlier ones. */
typedef struct dp_shape {
    uint32_t kind;
    uint32_t material; /* index into dp_scene_desc.materials */
    float center[3];   /* block, sphere */
    float size[3];     /* block: full side lengths */
    float radius;      /* sphere */
    uint32_t axis;     /* slab */
    float offset;      /* slab */
    float thickness;   /* slab */
} dp_shape;

enum { DP_WAVE_RICKER = 0, DP_WAVE_GAUSSIAN_PULSE = 1, DP_WAVE_CONTINUOUS = 2 };

/* Waveform (src/source.rs:31-52). */
typedef struct dp_waveform {
    uint32_t kind;
    float frequency;       /* peak (Ricker), centre (Gaussian), carrier (CW) */
    float duration_cycles; /* Gaussian: envelope FWHM in carrier periods */
    float ramp_cycles;     /* CW */
    float delay;           /* Ricker, Gaussian: seconds */
} dp_waveform;

enum { DP_SOURCE_POINT = 0, DP_SOURCE_SHEET = 1, DP_SOURCE_PLANE_WAVE = 2, DP_SOURCE_PLANE_WAVE_BOX = 3 };

/* Source (src/source.rs:136-195).  DP_SOURCE_PLANE_WAVE_BOX is an extension
 * the reference does not have: a plane wave travelling toward +axis through a
 * total-field box, with the scattered field alone outside the box on every
 * side.  Its incident field is a 1-D Yee line along the travel axis stepped
 * with the grid's own gains, driven by the plane-wave corrections of
 * src/source.rs:334-401; the box faces must lie in vacuum.  Time reversal
 * refuses it (DP_ERR_UNSUPPORTED: the line absorbs at its far end). */
typedef struct dp_source {
    uint32_t shape;
    uint32_t polarization; /* driven E component */
    float at[3];           /* point: metres from the domain centre */
    float velocity[3];     /* point: metres per second */
    uint32_t axis;         /* sheet, plane wave, box: travel axis */
    float offset;          /* sheet, plane wave: metres along axis */
    float waist;           /* sheet: metres */
    float amplitude;
    dp_waveform waveform;
    float box_low[3];      /* box: corners in metres from the domain centre; the */
    float box_high[3];     /* cells containing them bound the total field */
} dp_source;

/* Scene (src/scene.rs:116-122).  materials[0] must be vacuum
 * (MaterialTable invariant, src/material.rs:160-176). */
typedef struct dp_scene_desc {
    dp_grid_spec grid;
    dp_boundary boundary;
    uint32_t material_count;
    const dp_material *materials;
    uint32_t shape_count;
    const dp_shape *shapes;
    uint32_t source_count;
    const dp_source *sources;
} dp_scene_desc;

/* ------------------------------------------------------------------------ */
/* Grid queries (host only): what a scene author reads off a Grid            */
/* ------------------------------------------------------------------------ */

typedef struct dp_grid_info {
    uint32_t extent[3];        /* resolved cell counts (graded axes differ) */
    float size[3];             /* Grid::size, src/grid.rs:587-589 */
    float time_step;           /* Grid::time_step, src/grid.rs:592-594 */
    float finest;              /* Grid::finest, src/grid.rs:554-559 */
    float coarsest;            /* Grid::coarsest, src/grid.rs:561-566 */
    float worst_ratio;         /* Grid::worst_ratio, src/grid.rs:541-546 */
    float reference_cell_size; /* src/grid.rs:575-584 */
} dp_grid_info;

/* Grid::build (src/grid.rs:466-508) then the queries above. */
dp_status dp_grid_resolve(const dp_grid_spec *spec, dp_grid_info *out);

enum {
    DP_MAP_TO_CELL = 0,         /* Grid::to_cell, src/grid.rs:695-697 */
    DP_MAP_TO_POSITION = 1,     /* Grid::to_position, src/grid.rs:700-702 */
    DP_MAP_CELL_CONTAINING = 2, /* Grid::cell_containing, src/grid.rs:710-714 */
    DP_MAP_CELL_CENTER = 3      /* Grid::cell_center, src/grid.rs:718-720 (in: integer coords) */
};
dp_status dp_grid_map(const dp_grid_spec *spec, uint32_t op, const float in[3], float out[3]);

/* ------------------------------------------------------------------------ */
/* Resolved scene (host setup): what Simulation::new builds before upload    */
/* (src/cpu.rs:100-120, src/gpu.rs:190-319).  Host only, needs no GPU.      */
/* ------------------------------------------------------------------------ */

typedef struct dp_scene dp_scene;

typedef struct dp_scene_info {
    uint32_t extent[3];
    uint32_t material_count;
    float time_step;       /* Grid::time_step, src/grid.rs:592-594 */
    float courant;
    float absorber_peak;   /* AbsorbingProfile::peak, src/boundary.rs:215-221 */
    int32_t reversible;    /* Simulation::is_reversible, src/cpu.rs:209-215 */
    uint32_t index_bytes;  /* bytes per cell of the material index: 1 up to 256 materials, else 2 */
} dp_scene_info;

/* Grid::cell_lookup (src/grid.rs:635-646): three sections of `samples` values
 * (0 = the reference GPU solver's count, dp_scene_lookup_samples), each the
 * fractional cell coordinate of a uniformly spaced world position — the
 * renderer's world-to-cell map (gpu::Simulation::lookup_buffer). */
dp_status dp_scene_cell_lookup(const dp_scene *scene, uint32_t samples, float *host, size_t count);
/* gpu::Simulation::lookup_samples (src/gpu.rs:225-228, 349-351). */
uint32_t dp_scene_lookup_samples(const dp_scene *scene);

/* Tables a kernel consumes, readable for parity checks. */
enum {
    DP_TABLE_MAGNETIC_GAINS = 0, /* f32 nx+ny+nz: Grid::magnetic_gains, src/grid.rs:602-604 */
    DP_TABLE_ELECTRIC_GAINS = 1, /* f32 nx+ny+nz: Grid::electric_gains, src/grid.rs:606-608 */
    DP_TABLE_CELL_CENTERS = 2,   /* f32 nx+ny+nz: Grid::cell_centers, src/grid.rs:649-654 */
    DP_TABLE_ABSORBER = 3,       /* f32 2*(nx+ny+nz): AbsorbingProfile::packed, src/boundary.rs:203-212 */
    DP_TABLE_COEFFICIENTS = 4,   /* f32 4*materials: MaterialTable::coefficients, src/material.rs:207-212 */
    DP_TABLE_MATERIAL_INDEX = 5, /* u8 cells: Scene::material_indices, src/scene.rs:181-206 */
    DP_TABLE_PRIMARY = 6,        /* f32 nx+ny+nz: Spacing::primary, src/grid.rs:221-223 */
    DP_TABLE_DUAL = 7            /* f32 nx+ny+nz: Spacing::dual, src/grid.rs:226-228 */
};

/* Injection (src/source.rs:409-427), flattened for a kernel. */
typedef struct dp_injection {
    uint32_t origin[3];
    uint32_t extent[3];
    uint32_t component;
    uint32_t magnetic;
    float value;                 /* amplitude * waveform(t) */
    float inverse_waist_squared; /* 0: every cell weighs 1 */
    float center[3];
} dp_injection;

/* Replaces the setup half of cpu::Simulation::new / gpu::Simulation::new
 * (src/cpu.rs:100-120, src/gpu.rs:190-271): grid resolve, coefficient table,
 * gains, absorber profile, rasterized material index.  Material indices are
 * stored as u8, so a scene may hold at most 256 materials. */
dp_status dp_scene_create(const dp_scene_desc *desc, dp_scene **out);
void dp_scene_destroy(dp_scene *scene);
dp_status dp_scene_info_get(const dp_scene *scene, dp_scene_info *out);
/* Copies one table; bytes must equal the table's size exactly. */
dp_status dp_scene_table(const dp_scene *scene, uint32_t table, void *host, size_t bytes);
/* Scene::material_indices (src/scene.rs:181-206) on the GPU: writes the
 * index (index_bytes per cell: u8, or u16 past 256 materials) into
 * caller-owned device memory with rows of `row_pitch` cells (0 = nx; padding
 * cells are set to 0), asynchronously on `stream` (a cudaStream_t, or null
 * for the default stream).  Identical to the DP_TABLE_MATERIAL_INDEX table,
 * which is rasterized on the host. */
dp_status dp_scene_raster(const dp_scene *scene, void *device_out, uint32_t row_pitch, void *stream);
/* Source::injections (src/source.rs:280-403) for every source at `time`,
 * silenced slots included: 2 per source, in source order. */
dp_status dp_scene_injections(const dp_scene *scene, float time, dp_injection *out,
                              uint32_t capacity, uint32_t *count);

/* ------------------------------------------------------------------------ */
/* Simulation — gpu::Simulation (src/gpu.rs:159-763)                         */
/* ------------------------------------------------------------------------ */

typedef struct dp_sim dp_sim;

enum {
    DP_KERNEL_AUTO = 0,  /* fused z-streaming step where the scene allows it */
    DP_KERNEL_FUSED = 1, /* fused H+E step, TMA plane staging, ping-pong fields */
    DP_KERNEL_NAIVE = 2  /* one thread per cell, H pass then E pass, in place */
};

typedef struct dp_options {
    int32_t device;          /* CUDA ordinal */
    uint32_t kernel;         /* DP_KERNEL_* */
    uint32_t tile_y;         /* fused: rows per tile (8 or 16); 0 = default */
    uint32_t z_chunk;        /* fused: planes per CTA; 0 = fill whole waves */
    uint32_t cells_per_lane; /* fused: x cells per thread (1, 2 or 4); 0 = default */
    uint32_t ring_slots;     /* fused: z-planes in the shared-memory ring; 0 = default */
} dp_options;

enum { DP_FIELD_ELECTRIC = 0, DP_FIELD_MAGNETIC = 1, DP_FIELD_INTENSITY = 2 };

/* gpu::Simulation::new (src/gpu.rs:190-340).  opts may be NULL. */
dp_status dp_sim_create(const dp_scene *scene, const dp_options *opts, dp_sim **out);
/* Drop for gpu::Simulation (src/gpu.rs:779-799). */
void dp_sim_destroy(dp_sim *sim);
/* advance_by (src/gpu.rs:393-484, src/cpu.rs:200-204): asynchronous. */
dp_status dp_sim_advance(dp_sim *sim, uint64_t steps);
/* reverse_by (src/gpu.rs:499-576, src/cpu.rs:275-279): DP_ERR_LOSSY on a
 * lossy scene, DP_ERR_RANGE past step 0. */
dp_status dp_sim_reverse(dp_sim *sim, uint64_t steps);
/* reset (src/gpu.rs:625-637). */
dp_status dp_sim_reset(dp_sim *sim);
/* wait (src/gpu.rs:616-622): polls the stream, never traps. */
dp_status dp_sim_wait(dp_sim *sim, uint32_t timeout_ms);
/* step_count (src/gpu.rs:357-359). */
uint64_t dp_sim_step_count(const dp_sim *sim);
/* time (src/gpu.rs:362-364): step as f32 * dt. */
float dp_sim_time(const dp_sim *sim);
/* read_electric / read_magnetic / read_intensity (src/gpu.rs:644-729).
 * count = 3*cells for E and H, cells for intensity. */
dp_status dp_sim_read_field(dp_sim *sim, uint32_t field, float *host, size_t count);
/* Steppable::restore's upload (src/gpu.rs:663-695, 756-762); also seeds an
 * initial condition like cpu::Simulation::electric_mut (src/cpu.rs:145-151). */
dp_status dp_sim_write_field(dp_sim *sim, uint32_t field, const float *host, size_t count);
/* restore (src/gpu.rs:756-762): both fields, the step, intensity cleared. */
dp_status dp_sim_restore(dp_sim *sim, uint64_t step, const float *electric,
                         const float *magnetic, size_t count);
/* set_accumulate_intensity / accumulated_steps (src/gpu.rs:584-594). */
dp_status dp_sim_set_accumulate_intensity(dp_sim *sim, int on);
uint64_t dp_sim_accumulated_steps(const dp_sim *sim);
/* electric_buffer / magnetic_buffer / intensity_buffer (src/gpu.rs:366-374,
 * 596-599): the live device allocation, valid until the next advance,
 * reverse or destroy.  Rows are dp_sim_row_pitch cells apart (nx rounded up
 * to a multiple of 4, so equal to nx — the reference's dense layout — when nx
 * is a multiple of 4); component a starts at a * pitch * ny * nz. */
dp_status dp_sim_device_ptr(dp_sim *sim, uint32_t field, void **ptr);
/* The simulation's CUDA stream (cudaStream_t), for zero-copy consumers. */
dp_status dp_sim_stream(dp_sim *sim, void **stream);
/* bytes_per_step (src/gpu.rs:386-388) = 48 * cells; field_bytes (:377-379). */
uint64_t dp_sim_bytes_per_step(const dp_sim *sim);
uint64_t dp_sim_field_bytes(const dp_sim *sim);
/* energy (src/cpu.rs:654-687), reduced on the device in f64. */
dp_status dp_sim_energy(dp_sim *sim, double *electric, double *magnetic);
/* is_finite (src/cpu.rs:707-713), reduced on the device. */
dp_status dp_sim_is_finite(dp_sim *sim, int32_t *finite);
/* is_reversible (src/cpu.rs:209-215). */
int32_t dp_sim_is_reversible(const dp_sim *sim);
/* ------------------------------------------------------------------------ */
/* Batched form: many scenes of uneven sizes advanced together              */
/* ------------------------------------------------------------------------ */
/* No single counterpart in the reference, which runs one scene per
 * gpu::Simulation: a batch is many Simulation::advance_by calls
 * (src/gpu.rs:393-484) merged into one launch per step over a work list of
 * (scene, tile, z-chunk) units, with K-step chunks replayed as CUDA graphs.
 * Each scene's results are bit-identical to its solo run. */

typedef struct dp_batch dp_batch;

typedef struct dp_batch_options {
    int32_t device;
    uint32_t chunk_steps; /* steps per graph replay (K); 0 = 50 */
    uint64_t arena_bytes; /* device memory for every scene's state */
    uint32_t max_scenes;  /* scene slots; 0 = 256 */
    uint32_t use_graphs;  /* 0: launch each chunk's kernels directly */
    uint32_t cells_per_lane; /* tile width 32·this for every scene (1, 2 or 4); 0 = per scene, least waste */
    uint32_t unit_planes;    /* z-planes per work unit; 0 = chosen when the work list is rebuilt:
                                64 when the batch holds 16 units per SM at that depth, else 24 */
    uint32_t skip_finite_check; /* nonzero: no per-scene NaN/infinity check after each chunk */
    uint32_t axis_order; /* 0: each scene stored in the axis order whose tiles cover the fewest cells;
                            k in 1-6: order k-1 of (xyz, yxz, xzy, zyx, yzx, zxy) for every scene
                            (scenes with sheet or total-field-box sources keep xyz, and so does a scene
                            whose order would move its x off the stored x while cells_per_lane asks
                            for 64- or 128-wide tiles).  Results do not depend on it: reads and
                            probes come back in the scene's own axes. */
} dp_batch_options;

dp_status dp_batch_create(const dp_batch_options *opts, dp_batch **out);
void dp_batch_destroy(dp_batch *batch);
/* Admits a scene for `steps` steps, or DP_ERR_OOM when the arena cannot hold
 * it now, DP_ERR_BUSY when every slot is taken.  probes: probe_count
 * (x, y, z) cells whose Ez and Hy are recorded after every step.  Takes
 * effect at the next chunk. */
dp_status dp_batch_add(dp_batch *batch, const dp_scene *scene, uint64_t steps, int32_t accumulate_intensity,
                       const uint32_t *probes, uint32_t probe_count, uint64_t *id);
/* Frees a scene's slot and arena block (waits for the running chunk). */
dp_status dp_batch_remove(dp_batch *batch, uint64_t id);
/* One chunk for every scene with steps left (asynchronous). */
dp_status dp_batch_advance_chunk(dp_batch *batch, uint32_t *stepping);
dp_status dp_batch_wait(dp_batch *batch, uint32_t timeout_ms);
dp_status dp_batch_status(dp_batch *batch, uint64_t id, uint64_t *step, uint64_t *target);
/* Per-scene failure (is_finite, src/cpu.rs:707-713, on the device): after
 * every chunk each stepping scene's fields are checked for NaN and infinity.
 * A scene found non-finite stops stepping within two chunks (its target
 * becomes the steps issued for it, so dp_batch_status shows it finished);
 * *fault then reads DP_ERR_NONFINITE and *at_step its step count when it
 * stopped.  DP_OK (and 0) otherwise.  Does not wait: marks of chunks still
 * running are taken by dp_batch_wait and by later chunks.  The other scenes
 * run on unaffected. */
dp_status dp_batch_fault(dp_batch *batch, uint64_t id, dp_status *fault, uint64_t *at_step);
/* read_electric / read_magnetic / read_intensity of one scene, dense. */
dp_status dp_batch_read_field(dp_batch *batch, uint64_t id, uint32_t field, float *host, size_t count);
/* Probe series: step-major, then probe, then (Ez, Hy). */
dp_status dp_batch_read_probes(dp_batch *batch, uint64_t id, float *host, size_t count);
dp_status dp_batch_memory(const dp_batch *batch, uint64_t *used, uint64_t *capacity);
/* Arena bytes a scene would take (for admission control: the most of any
 * axis order the batch may store it in); UINT64_MAX when
 * its probe series (probe_count x steps x 2 values) would exceed 2^40 values,
 * which no arena holds (dp_batch_add then returns DP_ERR_OOM). */
uint64_t dp_scene_batch_bytes(const dp_scene *scene, uint32_t probe_count, uint64_t steps);
uint64_t dp_batch_launch_count(const dp_batch *batch);
/* How the batch stores a scene (no reference counterpart; diagnostics):
 * its axis order (0-5: xyz, yxz, xzy, zyx, yzx, zxy, stored axis i holding
 * the scene's axis named i-th) and the width of its tiles in cells. */
dp_status dp_batch_layout(dp_batch *batch, uint64_t id, uint32_t *axis_order, uint32_t *tile_width);

/* Field energy of caller-owned device arrays, allocating nothing.  No
 * counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc where they need the energy (cudaMalloc may synchronize the
 * device or fail under memory pressure; some hosts own all device memory
 * through their own allocator).  Computes what dp_sim_energy does, on the
 * calling thread's current device and the given stream (NULL: default
 * stream).  All pointers are device pointers:
 *   electric, magnetic  3 components of f32 with rows of field_pitch cells
 *                       (0 = nx): cell (x, y, z) of component a at
 *                       a*field_pitch*ny*nz + (z*ny + y)*field_pitch + x,
 *                       the layout dp_sim_device_ptr / dp_sim_row_pitch give;
 *   material_index      index_bytes (1: u8, 2: u16 for scenes of more than
 *                       256 materials) per cell, rows of index_pitch cells
 *                       (0 = nx);
 *   eps_mu              2 f32 (relative permittivity, permeability) for each
 *                       of material_count materials; an index at or past
 *                       material_count makes both sums NaN;
 *   primary, dual       nx+ny+nz f32 each;
 *   out                 2 f64 (electric, magnetic).
 * Its partial sums live in a fixed 64 KiB array inside the library, so it
 * covers at most 2^28 cells (DP_ERR_RANGE beyond).  The first call on a
 * device loads the library's device code there; make it before any stream
 * capture.  Every call shares the array: calls whose kernels overlap on the
 * GPU race and must be serialized by the caller. */
dp_status dp_energy_noalloc(const float *electric, const float *magnetic, uint32_t field_pitch,
                            const void *material_index, uint32_t index_bytes, uint32_t index_pitch,
                            const float *eps_mu, uint32_t material_count, const float *primary,
                            const float *dual, const uint32_t extent[3], double *out, void *stream);
/* Row stride of the device field buffers, in cells. */
uint32_t dp_sim_row_pitch(const dp_sim *sim);
/* Kernel the handle actually runs (DP_KERNEL_FUSED or DP_KERNEL_NAIVE). */
uint32_t dp_sim_kernel(const dp_sim *sim);
/* Kernel launches issued by this handle so far (every kernel of this library). */
uint64_t dp_sim_launch_count(const dp_sim *sim);

/* ---- Autotuning ---------------------------------------------------------
 * Times every fused-step tile shape (cells per lane × rows per tile, with its
 * ring depth) at several z-chunk depths, `steps` steps each (0 = 8), from the
 * simulation's current state, and keeps the fastest.  The fields, intensity
 * and step count are restored exactly, so tuning changes no result.  On the
 * one-thread-per-cell path there is nothing to tune (candidates = 0). */
typedef struct dp_tuning {
    uint32_t cells_per_lane, tile_y, ring_slots, z_chunk; /* the chosen plan */
    float ms_per_step;                                    /* its time per step in the trial */
    uint32_t candidates;                                  /* plans timed */
} dp_tuning;
dp_status dp_sim_autotune(dp_sim *sim, uint32_t steps, dp_tuning *out);
/* The plan the handle runs now (ms_per_step and candidates 0); every field
 * 0 on the one-thread-per-cell path. */
dp_status dp_sim_plan(const dp_sim *sim, dp_tuning *out);
/* Tuned plans are kept per process, keyed by the grid's extent and the
 * device's SM count: a simulation created later for a grid of that shape,
 * with the plan fields of dp_options left at 0, starts from the tuned plan,
 * and a batch scene of that shape (cells_per_lane 0) takes its tile width.
 * Export writes the cache as text, one line per shape ("nx ny nz sms
 * cells_per_lane tile_y ring_slots z_chunk ms_per_step"), into buf
 * (capacity cap, NUL-terminated); *len gets the length it needs without the
 * NUL, even when cap is too small (DP_ERR_RANGE then).  Import adds such
 * lines (DP_ERR_INVALID at a malformed line or a tile shape this build
 * lacks; the lines before it are kept), so tuning can outlive the process. */
dp_status dp_tune_cache_export(char *buf, size_t cap, size_t *len);
dp_status dp_tune_cache_import(const char *text);
void dp_tune_cache_clear(void);

/* ---- Probes and asynchronous read-back ----------------------------------
 * Probes record Ez and Hy at given cells after every step into a device ring
 * of `capacity` steps (one small gather launch per step while set); count 0
 * removes them.  A restore, reset or field write starts a new history, and
 * only steps recorded since are readable.  A ring of more than 2^40 values
 * (capacity x count x 2) is refused with DP_ERR_OOM before anything is
 * allocated. */
dp_status dp_sim_set_probes(dp_sim *sim, const uint32_t *cells_xyz, uint32_t count, uint64_t capacity);
/* Steps first_step .. first_step+steps-1 (step k = the state after k steps),
 * steps × probes × (Ez, Hy) floats; DP_ERR_RANGE outside the ring. */
dp_status dp_sim_read_probes(dp_sim *sim, uint64_t first_step, uint64_t steps, float *host, size_t count);
/* dp_sim_read_field without the wait: the copy is queued on the handle's
 * stream behind the steps already issued; the host buffer (pinned for true
 * overlap) is valid after dp_sim_wait. */
dp_status dp_sim_read_field_async(dp_sim *sim, uint32_t field, float *host, size_t count);
/* cpu::Simulation::energy_density (src/cpu.rs:689-703): ½(E² + H²) per cell,
 * summed over the three components, in f32. */
dp_status dp_sim_energy_density(dp_sim *sim, float *host, size_t count);
/* cpu::Simulation::sample_electric / sample_magnetic (src/cpu.rs:154-161):
 * one component at one cell (DP_FIELD_INTENSITY with axis 0 reads the
 * accumulated intensity). */
dp_status dp_sim_sample(dp_sim *sim, uint32_t field, uint32_t axis, const uint32_t coord[3], float *out);

/* ---- Device keyframes (Timeline, src/timeline.rs:76-213) -----------------
 * A ring of `capacity` field snapshots kept in device memory (24 bytes per
 * cell each, allocated at creation) for a simulation that must outlive it.
 * observe records a keyframe when the step has crossed into a later interval
 * than the newest one; seek goes to a step by the cheapest route: forward by
 * stepping, backward by restoring the newest keyframe at or before it and
 * replaying, or from a reset when the window has slid past it.  Snapshots and
 * restores are device-to-device copies on the simulation's stream. */
typedef struct dp_keyframes dp_keyframes;
enum { DP_SEEK_UNCHANGED = 0, DP_SEEK_FORWARD = 1, DP_SEEK_KEYFRAME = 2, DP_SEEK_START = 3 };
/* Seek (src/timeline.rs:83-106): what a seek had to do. */
typedef struct dp_seek {
    uint32_t kind;     /* DP_SEEK_* */
    uint64_t replayed; /* steps run */
    uint64_t at;       /* the keyframe restored (DP_SEEK_KEYFRAME) */
} dp_seek;
dp_status dp_keyframes_create(dp_sim *sim, uint64_t interval, uint32_t capacity, dp_keyframes **out);
void dp_keyframes_destroy(dp_keyframes *keyframes);
dp_status dp_keyframes_observe(dp_keyframes *keyframes);
dp_status dp_keyframes_seek(dp_keyframes *keyframes, uint64_t target, dp_seek *out);
dp_status dp_keyframes_clear(dp_keyframes *keyframes);
uint32_t dp_keyframes_count(const dp_keyframes *keyframes);
dp_status dp_keyframes_earliest(const dp_keyframes *keyframes, uint64_t *step);
/* Bytes the recorded keyframes stand for, 24 per cell each (Timeline::bytes). */
uint64_t dp_keyframes_bytes(const dp_keyframes *keyframes);

/* ---- Headless volume renderer -------------------------------------------
 * The reference viewer's volume pass (examples/common/shaders/volume.wgsl)
 * and exposure control (examples/common/render.rs) on a simulation's own
 * device buffers, into an RGBA8 image (sRGB-encoded, row 0 at the top) in
 * device memory.  No window, swapchain or graphics API: the image can be
 * read back or used in place.  The renderer borrows the simulation, which
 * must outlive it; work is queued on the simulation's stream. */
typedef struct dp_renderer dp_renderer;
/* ViewMode (render.rs:12-47), with the shader's mode codes. */
enum {
    DP_VIEW_ENERGY = 0,
    DP_VIEW_ELECTRIC = 1,
    DP_VIEW_MAGNETIC = 2,
    DP_VIEW_MAGNITUDE = 3,
    DP_VIEW_FIELDS = 4,
    DP_VIEW_GRID = 5,
    DP_VIEW_RIBBONS = 6,
    DP_VIEW_INTENSITY = 7
};
/* Camera (examples/common/camera.rs) and ViewSettings (render.rs:118-137). */
typedef struct dp_view {
    float yaw, pitch;   /* orbit angles, radians */
    float distance;     /* from the box centre, in longest sides */
    float fov;          /* vertical field of view, radians */
    uint32_t mode;      /* DP_VIEW_* */
    float gain;         /* multiplies the auto-ranged exposure */
    float log_strength; /* signed-log compression, 0 = linear */
    int32_t scrub;      /* nonzero: draw the scrub bar */
    float played;       /* scrub bar playhead, 0..1 */
    float window_start; /* start of the keyframed window, 0..1 */
} dp_view;
/* Camera::new and ViewSettings::new: yaw 0.9, pitch 0.45, distance 1.9,
 * fov 0.8, the E-and-H view, gain 1, log strength 6, no scrub bar. */
dp_view dp_view_default(void);
dp_status dp_renderer_create(dp_sim *sim, uint32_t width, uint32_t height, dp_renderer **out);
void dp_renderer_destroy(dp_renderer *renderer);
/* The peak reduction on its own (Renderer::measure): run once before the
 * first draw, whose exposure comes from the previous reduction. */
dp_status dp_renderer_measure(dp_renderer *renderer);
/* Renderer::draw: folds the previous reduction into the exposure (only when
 * `advanced`), reduces again, and ray-marches the frame. */
dp_status dp_renderer_draw(dp_renderer *renderer, const dp_view *view, int32_t advanced);
dp_status dp_renderer_pixels(dp_renderer *renderer, uint8_t *host_rgba, size_t bytes);
dp_status dp_renderer_image(dp_renderer *renderer, void **device_rgba);
/* The last reduction's eight slots (energy-density peak, |E| and |H| per
 * component, averaged intensity), the exposure scale, and the components of
 * E and H the signed views read; any pointer may be null. */
dp_status dp_renderer_state(dp_renderer *renderer, float peaks[8], float *scale, uint32_t components[2]);

/* ---- FP64 instance ------------------------------------------------------
 * The same time step in double on the GPU: fields, curls, updates, drive
 * values and time in f64 over the f32 setup tables, i.e. the reference's
 * Simulation instantiated at f64 (src/cpu.rs:174-198, 283-434, 606-633 with
 * T = f64).  It is what the f32 step's error is measured against; it has no
 * reverse, intensity or fused path.  advance is asynchronous like
 * dp_sim_advance; reads and the energy wait. */
typedef struct dp_sim64 dp_sim64;
dp_status dp_sim64_create(const dp_scene *scene, int32_t device, dp_sim64 **out);
void dp_sim64_destroy(dp_sim64 *sim);
dp_status dp_sim64_advance(dp_sim64 *sim, uint64_t steps);
dp_status dp_sim64_wait(dp_sim64 *sim, uint32_t timeout_ms);
uint64_t dp_sim64_step_count(const dp_sim64 *sim);
/* DP_FIELD_ELECTRIC or DP_FIELD_MAGNETIC, 3 * cells doubles, component-major. */
dp_status dp_sim64_read_field(dp_sim64 *sim, uint32_t field, double *host, size_t count);
/* energy, src/cpu.rs:654-687, over the f64 fields. */
dp_status dp_sim64_energy(dp_sim64 *sim, double *electric, double *magnetic);

#ifdef __cplusplus
}
#endif

#endif /* DIAPHANE_GB300_H */
