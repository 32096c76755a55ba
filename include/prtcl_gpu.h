/*
 * prtcl_gpu.h -- C ABI of the GB300 (sm_103a) implementation of prtcl's
 * SPH hot path: the uniform-grid neighbourhood, the generated IISPH
 * pressure-solve procedures, the WKBB18 implicit-viscosity PCG solver and
 * the small per-step procedures around them.
 *
 * Every entry point returns 0 on success and a negative status on failure;
 * the message of the last failure on the calling thread is available from
 * prtcl_gpu_last_error().  Plain pointers and sizes only.  `stream` may be
 * NULL (the model's own stream) or a cudaStream_t cast to void*.
 *
 * Host layouts follow the reference (data/varying_field.hpp:26-58): a field
 * of type real[3] is 3 contiguous floats per item, real[3][3] is 9 floats per
 * item in column-major order.  Component types: "f32" (the reference's
 * `real` for T=f32) and "i32" (the generated schemes' `integer`).
 */
#ifndef PRTCL_GPU_H
#define PRTCL_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct prtcl_gpu_model prtcl_gpu_model;
typedef struct prtcl_gpu_nhood prtcl_gpu_nhood;
typedef struct prtcl_gpu_scheme prtcl_gpu_scheme;

/* Status codes. */
#define PRTCL_GPU_OK 0
#define PRTCL_GPU_ERROR -1          /* see prtcl_gpu_last_error() */
#define PRTCL_GPU_NOT_FOUND -2      /* unknown group / field / procedure / scheme */
#define PRTCL_GPU_INVALID -3        /* invalid argument */

/* Message of the last failure on this thread (never NULL). */
const char *prtcl_gpu_last_error(void);

/* Library version string. */
const char *prtcl_gpu_version(void);

/* Number of CUDA kernels this library has launched in this process,
 * including the kernels its device-side loops (CUDA graphs) executed; call
 * after the work has completed (no counterpart in the reference; used to
 * account for device work). */
uint64_t prtcl_gpu_launch_count(void);

/* ---- model: replaces prtcl::Model (data/model.hpp, data/model.cpp:13-34) ---- */

int prtcl_gpu_model_create(prtcl_gpu_model **out);
int prtcl_gpu_model_destroy(prtcl_gpu_model *model);

/* Model::AddGroup (data/model.cpp:13-34): creates the group (or returns the
 * existing one of the same type).  Group indices are the alphabetical rank
 * of the group names and change when a group is added. */
int prtcl_gpu_group_add(prtcl_gpu_model *model, const char *name, const char *type);
/* Group::AddTag (data/group.hpp) */
int prtcl_gpu_group_add_tag(prtcl_gpu_model *model, const char *group, const char *tag);
/* Group::Resize (data/group.hpp): resizes every varying field, keeping the
 * first min(old, new) items */
int prtcl_gpu_group_resize(prtcl_gpu_model *model, const char *group, int64_t count);
int prtcl_gpu_group_count(prtcl_gpu_model *model, const char *group, int64_t *count_out);
int prtcl_gpu_group_index(prtcl_gpu_model *model, const char *group, int32_t *index_out);
int prtcl_gpu_model_group_count(prtcl_gpu_model *model, int32_t *count_out);
/* Model::GetGroups: the group names in index order, '\n'-separated (written
 * to `buf` as prtcl_gpu_scheme_full_name does). */
int prtcl_gpu_model_group_names(prtcl_gpu_model *model, char *buf, int64_t size, int64_t *needed_out);

/* VaryingManager::AddFieldImpl (data/varying_manager.hpp:33-46): adds a
 * field (or checks the type of an existing one).  rank 0..2, extents[rank]. */
int prtcl_gpu_field_add(prtcl_gpu_model *model, const char *group, const char *field, const char *ctype, int32_t rank,
                        const int32_t *extents);
/* Copy `count` items (== the group's item count) from host memory in the
 * reference layout.  Synchronous: returns after the copy completed. */
int prtcl_gpu_field_upload(prtcl_gpu_model *model, const char *group, const char *field, const void *host,
                           int64_t count, void *stream);
/* As above but stream-ordered: `host` must stay valid (pinned memory for
 * overlap) until the stream reaches the copy. */
int prtcl_gpu_field_upload_async(prtcl_gpu_model *model, const char *group, const char *field, const void *host,
                                 int64_t count, void *stream);
/* Upload a varying field like prtcl_gpu_field_upload, but without allocating
 * device memory.  No counterpart in the reference (its fields live in host
 * memory).  For callers that cannot allocate when they upload: a host that
 * hands all free device memory to its own pool, or code that must not enter
 * the device allocator inside a time-critical section.  real[3] and
 * real[3][3] fields are staged through one fixed 8 MiB device array of the
 * library (at most 699,050 vector or 233,016 matrix items per call; larger
 * counts return PRTCL_GPU_ERROR and change nothing); other fields are copied
 * directly and have no limit.  prtcl_gpu_model_create makes the array and
 * its kernels resident on the current device, so create the model before
 * the host takes the remaining device memory (a model used on another device
 * does this on its first call there).  Synchronous, hence not capturable: a
 * call on a stream under capture returns PRTCL_GPU_ERROR.  The array is
 * shared by the whole process and keeps the last call's bytes: calls that
 * overlap in time, from different threads, race on it. */
int prtcl_gpu_field_upload_noalloc(prtcl_gpu_model *model, const char *group, const char *field, const void *host,
                                   int64_t count, void *stream);
/* Copy the field to host memory in the reference layout (synchronous). */
int prtcl_gpu_field_download(prtcl_gpu_model *model, const char *group, const char *field, void *host, int64_t count,
                             void *stream);
/* Type of a varying field; ctype_out receives "f32" or "i32" (>= 4 bytes). */
int prtcl_gpu_field_info(prtcl_gpu_model *model, const char *group, const char *field, char *ctype_out,
                         int32_t *rank_out, int32_t *extents_out /* [2] */);

/* UniformManager (data/uniform_manager.hpp): one value per group.  `value`
 * holds prod(extents) components of the field's component type. */
int prtcl_gpu_uniform_add(prtcl_gpu_model *model, const char *group, const char *field, const char *ctype,
                          int32_t rank, const int32_t *extents);
int prtcl_gpu_uniform_set(prtcl_gpu_model *model, const char *group, const char *field, const void *value);
int prtcl_gpu_uniform_get(prtcl_gpu_model *model, const char *group, const char *field, void *value);

/* Global fields of the model (data/model.hpp, Model::AddGlobalFieldImpl). */
int prtcl_gpu_global_add(prtcl_gpu_model *model, const char *field, const char *ctype, int32_t rank,
                         const int32_t *extents);
int prtcl_gpu_global_set(prtcl_gpu_model *model, const char *field, const void *value);
int prtcl_gpu_global_get(prtcl_gpu_model *model, const char *field, void *value);
/* Stream-ordered set of a global field of at most 64 bytes: returns without
 * waiting; the value is applied in `stream` order (NULL: the model's
 * stream).  For per-step values such as current_time. */
int prtcl_gpu_global_set_async(prtcl_gpu_model *model, const char *field, const void *value, void *stream);

/* Statistics of the device-side loops since the last reset (no counterpart
 * in the reference, whose script prints the iteration counts per step):
 * out[0] Jacobi solves, [1] Jacobi iterations, [2] solves stopped at the
 * iteration cap, [3] largest final aprde / nprde, [4] PCG solves, [5] PCG
 * iterations, [6] PCG solves stopped by the iteration limit.  Waits for the
 * model's stream; `reset` != 0 zeroes them afterwards. */
int prtcl_gpu_model_stats(prtcl_gpu_model *model, double *out, int32_t n, int32_t reset);

/* Model::Save / Model::Load (data/model.cpp:54-75) in the reference's native
 * binary archive format (util/archive.cpp:5-40): global fields, then per
 * group its name, type, tags, varying fields and uniform fields.  Load adds
 * the groups and fields it finds (resizing the groups to the archive's item
 * counts) and uploads the values; f32 and s32 components only.  Synchronous. */
int prtcl_gpu_model_save(prtcl_gpu_model *model, const char *path);
int prtcl_gpu_model_load(prtcl_gpu_model *model, const char *path);

/* SaveVTK (util/save_vtk.cpp:57-128): one group as a legacy ASCII VTK
 * polydata file (points from "position"; velocity, acceleration, mass,
 * volume, density, pressure, time_of_birth ... where present).  Synchronous. */
int prtcl_gpu_group_save_vtk(prtcl_gpu_model *model, const char *group, const char *path);

/* Types of uniform and global fields (ctype_out >= 4 bytes, extents_out[2]). */
int prtcl_gpu_uniform_info(prtcl_gpu_model *model, const char *group, const char *field, char *ctype_out,
                           int32_t *rank_out, int32_t *extents_out);
int prtcl_gpu_global_info(prtcl_gpu_model *model, const char *field, char *ctype_out, int32_t *rank_out,
                          int32_t *extents_out);

/* The model's own CUDA stream (a cudaStream_t), used when a call gets
 * stream == NULL. */
int prtcl_gpu_model_stream(prtcl_gpu_model *model, void **stream_out);

/* Wait for all work queued on the model's stream (and `stream`, if given). */
int prtcl_gpu_model_synchronize(prtcl_gpu_model *model, void *stream);

/* Per-kernel timing with CUDA events on the launching stream (no
 * counterpart in the reference, whose only tracing is a disabled scope
 * macro, schemes/iisph.hpp:35).  While enabled, every procedure and grid
 * kernel launch records an event pair; read returns lines
 * "name count total_ms" for the launches since the last reset. */
int prtcl_gpu_profile_enable(prtcl_gpu_model *model, int32_t enable);
int prtcl_gpu_profile_read(prtcl_gpu_model *model, char *buf, int64_t size, int64_t *needed_out);
int prtcl_gpu_profile_reset(prtcl_gpu_model *model);

/* Launch-shape knobs of the neighbour sweeps and the relaxed-Jacobi loop
 * (no counterpart in the reference, whose loops are OpenMP-scheduled).
 * Every value gives bit-identical results; they change only speed.  Knobs
 * carry the kernels' profile names: density, iisph_setup, iisph_accel,
 * iisph_pressure, wkbb18_diag, pcg_init, pcg_q (values 0..3, a launch
 * shape each; pcg_q 4: a cell-tile sweep without neighbour lists, for
 * unbatched models), jacobi_unroll (1, 2 or 4 relaxed-Jacobi iterations per
 * iteration of the device loop's graph), staging (1: unbatched models with
 * one fluid and one boundary group build staged lists, and the
 * relaxed-Jacobi and PCG sweeps read their neighbours' records from shared
 * memory per tile of 128 items), grid_sort (1, the default: a grid of at
 * most 128,000 items is sorted in one launch of a thread-block cluster of 8
 * or 16 CTAs; 0: the tiled radix-sort launches at every size) and list_split
 * (1, the default: the lists of a query group of at most 65,536 items are
 * built by four threads per query, each walking a quarter of its cells; 0:
 * one thread per query at every size).  prtcl_gb300/tune.py searches them
 * per workload and caches the choice.  prtcl_gpu_tune_knobs returns one line
 * per knob: "name default value=shape ...", a shape written as threads per
 * block x blocks per SM / neighbour-walk batch.  An unknown knob gives
 * PRTCL_GPU_NOT_FOUND, a value outside its set PRTCL_GPU_INVALID. */
int prtcl_gpu_tune_knobs(char *buf, int64_t size, int64_t *needed_out);
int prtcl_gpu_model_tune_set(prtcl_gpu_model *model, const char *knob, int32_t value);
int prtcl_gpu_model_tune_get(prtcl_gpu_model *model, const char *knob, int32_t *value_out);

/* ---- neighbourhood: replaces prtcl::Neighborhood (util/neighborhood.hpp:23-42) ---- */

int prtcl_gpu_nhood_create(prtcl_gpu_nhood **out);
int prtcl_gpu_nhood_destroy(prtcl_gpu_nhood *nhood);
/* Neighborhood::SetRadius (util/neighborhood.cpp:61-65) */
int prtcl_gpu_nhood_set_radius(prtcl_gpu_nhood *nhood, double radius);
/* Neighborhood::Load (util/neighborhood.cpp:67-98): binds the groups'
 * "position" fields (real[3]) and their cannot_be_neighbor tags */
int prtcl_gpu_nhood_load(prtcl_gpu_nhood *nhood, prtcl_gpu_model *model);
/* Neighborhood::Update (util/neighborhood.cpp:100-104 ->
 * grouped_uniform_grid::update, util/grouped_uniform_grid.hpp:126-337) */
int prtcl_gpu_nhood_update(prtcl_gpu_nhood *nhood, void *stream);
/* Neighborhood::Permute (util/neighborhood.cpp:106-154): reorders every
 * varying field of each neighbour-capable group into cell order, then Update */
int prtcl_gpu_nhood_permute(prtcl_gpu_nhood *nhood, prtcl_gpu_model *model, void *stream);
/* The neighbour sets of every item of `query_group` (grouped_uniform_grid::
 * neighbors, util/grouped_uniform_grid.hpp:407-422, for all items at once):
 * builds the device lists the procedures read, without copying them out.
 * No counterpart as an entry point in the reference, which queries per item
 * inside each procedure.  *pairs_out (optional) receives the number of
 * (item, neighbour) pairs over all neighbour groups; it synchronises. */
int prtcl_gpu_nhood_query(prtcl_gpu_nhood *nhood, int32_t query_group, int64_t *pairs_out, void *stream);
/* Neighborhood::CopyNeighbors (util/neighborhood.cpp:156-166): neighbours of
 * item `index` of group `group`; counts_out[g] receives the number of
 * neighbours in group g (group-count entries), indices_out the raw indices
 * grouped by group in traversal order (at most `capacity` are written);
 * *total_out the total.  */
int prtcl_gpu_nhood_copy_neighbors(prtcl_gpu_nhood *nhood, int32_t group, int64_t index, int64_t *counts_out,
                                   int64_t *indices_out, int64_t capacity, int64_t *total_out);
/* Bulk form for parity checks: CSR of every item of `query_group` to the
 * neighbours in `neighbor_group`; offsets_out has count + 1 entries. */
int prtcl_gpu_nhood_copy_lists(prtcl_gpu_nhood *nhood, int32_t query_group, int32_t neighbor_group,
                               int64_t *offsets_out, uint32_t *indices_out, int64_t capacity);
/* Introspection of staged lists (the `staging` knob; no counterpart in the
 * reference): of the tiles of 128 consecutive items of `query_group`'s
 * last built lists, *staged_out receives those whose neighbours' records
 * fit the staged sweeps' shared memory, *tiles_out all of them; both 0 when
 * the lists were not built staged.  Synchronises. */
int prtcl_gpu_nhood_staged_tiles(prtcl_gpu_nhood *nhood, int32_t query_group, int64_t *staged_out,
                                 int64_t *tiles_out);
/* Grid introspection for parity checks: the sorted item handles
 * (group << 28 | raw index, util/grouped_uniform_grid.hpp:104-110), and per
 * cell its grid index (3 x int32), its [first, last) sorted range and its
 * 26 adjacent cells (-1 = none).  Any output pointer may be NULL. */
int prtcl_gpu_nhood_grid_size(prtcl_gpu_nhood *nhood, int64_t *sorted_count_out, int64_t *cell_count_out);
int prtcl_gpu_nhood_copy_grid(prtcl_gpu_nhood *nhood, uint32_t *sorted_out, int32_t *cell_grid_index_out,
                              int32_t *cell_range_out, int32_t *cell_adjacency_out);

/* ---- schemes: replaces prtcl::SchemeBase / SchemeRegistry (schemes/scheme_base.hpp:18-105) ---- */

/* SchemeRegistry::NewScheme (schemes/scheme_base.hpp:87-92) by full name,
 * e.g. "prtcl::schemes::iisph[T=f32, N=3, K=Cubic Spline]";
 * PRTCL_GPU_NOT_FOUND with "scheme is not registered" otherwise. */
int prtcl_gpu_scheme_new(const char *full_name, prtcl_gpu_scheme **out);
int prtcl_gpu_scheme_destroy(prtcl_gpu_scheme *scheme);
/* SchemeBase::Load (e.g. schemes/iisph.hpp:134-185): creates the global,
 * uniform and varying fields the scheme uses and binds the groups. */
int prtcl_gpu_scheme_load(prtcl_gpu_scheme *scheme, prtcl_gpu_model *model);
/* SchemeBase::RunProcedure (schemes/scheme_base.hpp:33-38): queues the
 * procedure on `stream`; PRTCL_GPU_NOT_FOUND with "procedure does not
 * exist" for an unknown name. */
int prtcl_gpu_scheme_run(prtcl_gpu_scheme *scheme, const char *procedure, prtcl_gpu_nhood *nhood, void *stream);
/* SchemeBase::GetFullName / GetProcedureNames / GetPrtclSourceCode and
 * SchemeRegistry::GetSchemeNames: '\n'-separated lists written to `buf`
 * (NUL-terminated, truncated to `size`); *needed_out gets the full length. */
int prtcl_gpu_scheme_full_name(prtcl_gpu_scheme *scheme, char *buf, int64_t size, int64_t *needed_out);
int prtcl_gpu_scheme_procedure_names(prtcl_gpu_scheme *scheme, char *buf, int64_t size, int64_t *needed_out);
int prtcl_gpu_scheme_source(prtcl_gpu_scheme *scheme, char *buf, int64_t size, int64_t *needed_out);
/* Load a scheme plugin: a shared library generated from the scheme language
 * (share/schemes/*.prtcl, compiled by prtcl_gb300.dsl), whose exported
 * prtcl_gpu_plugin_init registers its schemes by full name, after which
 * prtcl_gpu_scheme_new creates them like the built-in ones.  Counterpart of
 * the reference's generated scheme headers (lua/prtcl/generate/
 * cxx_openmp_impl_hpp.lua) compiled into the library. */
int prtcl_gpu_scheme_load_plugin(const char *path);
int prtcl_gpu_registry_scheme_names(char *buf, int64_t size, int64_t *needed_out);

/* ---- batched scenes (no single counterpart in the reference) ----
 *
 * A batch keeps many independent dam-break scenes resident on the device and
 * steps them together: every procedure of the reference's step loop
 * (share/scripts/prtcl-lua.example.lua:363-461: grid update with a permute
 * every `permute_every` steps of the scene, density, gravity, velocity
 * integration, IISPH set-up and relaxed-Jacobi pressure loop, optional WKBB18
 * implicit viscosity, position integration) runs as one launch over all
 * scenes.  The relaxed-Jacobi and PCG loops decide convergence per scene, so
 * each scene stops when its own criterion is met.  A scene's results are the
 * same, bit for bit, whether it runs alone or beside others, and whenever it
 * was added.  All scenes of a batch share the parameters below.  Scenes can be
 * added and removed between steps (continuous batching); added scenes are
 * set up as the reference's scripts do (update, permute, boundary volumes,
 * share/scripts/prtcl-lua.example.lua:196-316) at the next step or query. */
typedef struct prtcl_gpu_batch prtcl_gpu_batch;
typedef struct prtcl_gpu_batch_params {
  double smoothing_scale;            /* h; search radius 2 h */
  double time_step;
  double rest_density;
  double gravity[3];
  double relaxation;                 /* iisph_relaxation (omega) */
  double max_density_error;          /* eta of the Jacobi loop */
  int32_t max_iterations;            /* Jacobi cap */
  int32_t viscosity;                 /* nonzero: WKBB18 implicit viscosity each step */
  double dynamic_viscosity;          /* fluid */
  double boundary_dynamic_viscosity;
  double pcg_max_error;              /* wkbb18_maximum_error */
  int32_t pcg_max_iterations;        /* wkbb18_maximum_iterations */
  int32_t permute_every;             /* steps between permutes of a scene (>= 1) */
} prtcl_gpu_batch_params;
typedef struct prtcl_gpu_scene_info {
  int64_t fluid, boundary;           /* particle counts */
  int64_t steps;                     /* steps taken */
  int32_t slot;                      /* segment of the scene in the batch */
  int32_t last_jacobi_iterations;
  int32_t last_pcg_iterations;
  int32_t pad;
  double last_relative_density_error; /* aprde / nprde at the end of the last Jacobi loop */
  double max_relative_density_error;
  double jacobi_solves, jacobi_iterations, jacobi_capped; /* accumulated over the scene's steps */
  double pcg_solves, pcg_iterations, pcg_capped;
} prtcl_gpu_scene_info;

int prtcl_gpu_batch_create(const prtcl_gpu_batch_params *params, prtcl_gpu_batch **out);
int prtcl_gpu_batch_destroy(prtcl_gpu_batch *batch);
/* Add a scene: fluid particles (3 floats each, at rest, mass h^3 rho0) and
 * static boundary particles.  *scene_id_out is unique within the batch. */
int prtcl_gpu_batch_add_scene(prtcl_gpu_batch *batch, const float *fluid_xyz, int64_t fluid_count,
                              const float *boundary_xyz, int64_t boundary_count, int64_t *scene_id_out);
int prtcl_gpu_batch_remove_scene(prtcl_gpu_batch *batch, int64_t scene_id);
/* Advance every scene by `steps` steps (queued on the batch's stream; the
 * grid update synchronises once per step). */
int prtcl_gpu_batch_step(prtcl_gpu_batch *batch, int32_t steps);
int prtcl_gpu_batch_synchronize(prtcl_gpu_batch *batch);
int prtcl_gpu_batch_scene_info(prtcl_gpu_batch *batch, int64_t scene_id, prtcl_gpu_scene_info *out);
/* Copy a varying field of a scene's fluid particles ("position", "velocity",
 * "density", "pressure", ...) to host memory in the reference layout;
 * `count` must equal the scene's fluid count. */
int prtcl_gpu_batch_download(prtcl_gpu_batch *batch, int64_t scene_id, const char *field, void *host, int64_t count);
int prtcl_gpu_batch_scene_count(prtcl_gpu_batch *batch, int32_t *count_out);
int prtcl_gpu_batch_particles(prtcl_gpu_batch *batch, int64_t *fluid_out, int64_t *boundary_out);
/* Device bytes held by the batch's particle state, grid and neighbour lists. */
int prtcl_gpu_batch_device_bytes(prtcl_gpu_batch *batch, int64_t *bytes_out);
int prtcl_gpu_batch_profile_enable(prtcl_gpu_batch *batch, int32_t enable);
/* Per-kernel timing lines "name launches total_ms", as prtcl_gpu_profile_read. */
int prtcl_gpu_batch_profile_read(prtcl_gpu_batch *batch, char *buf, int64_t size, int64_t *needed_out);
/* The knobs of prtcl_gpu_model_tune_set for the batch's model; the tiled
 * sweeps of a batch use the batched shapes of prtcl_gpu_tune_knobs. */
int prtcl_gpu_batch_tune_set(prtcl_gpu_batch *batch, const char *knob, int32_t value);
int prtcl_gpu_batch_tune_get(prtcl_gpu_batch *batch, const char *knob, int32_t *value_out);

/* ---- Serving: continuous batching of simulation requests ----------------
 * The reference runs one scene per process (share/scripts/prtcl-lua.example.lua);
 * a server keeps every admitted request resident in one batch and advances
 * them together, one step per turn.  A turn:
 *   1. admits the submitted requests whose arrival time has come, in arrival
 *      order (ties in submission order), while a scene slot is free and the
 *      batch's device bytes plus the request's estimate (its particles times
 *      the largest bytes per particle seen so far) stay within the budget;
 *   2. steps every resident scene once;
 *   3. retires, in admission order, the requests that have taken all their
 *      steps: their scene information and (keep_results) final fluid
 *      positions are kept until read with prtcl_gpu_server_next_result.
 * Every scene converges on its own, so a request's result is the same, bit
 * for bit, alone and in the mix.  Times are seconds on the server's clock.
 *
 * Failures.  A request whose own estimate exceeds the budget is refused at
 * submit (PRTCL_GPU_ERROR), and one whose estimate has grown beyond the
 * budget by the time it could be admitted is retired unrun with status
 * PRTCL_GPU_REQUEST_REJECTED: no request reaches the device allocator with
 * more than the budget.  prtcl_gpu_server_cancel retires a queued or
 * resident request with status PRTCL_GPU_REQUEST_CANCELLED.  If a batch step
 * fails, every resident request is retired with status
 * PRTCL_GPU_REQUEST_FAILED (its scene removed from the batch) and the turn
 * returns the step's error; queued requests stay queued.  If reading a
 * finished request's results fails, that request alone is retired with
 * status PRTCL_GPU_REQUEST_FAILED and is never stepped again.  A scene the
 * batch failed to remove is removed again at the start of later turns. */
typedef struct prtcl_gpu_server prtcl_gpu_server;
typedef double (*prtcl_gpu_clock_fn)(void *user);
typedef struct prtcl_gpu_server_params {
  double budget_bytes;               /* admission limit on the batch's device bytes */
  int32_t max_scenes;                /* resident requests at most (>= 1) */
  int32_t keep_results;              /* nonzero: keep each request's final fluid positions */
  double bytes_per_particle;         /* admission estimate until the batch holds a scene */
  prtcl_gpu_clock_fn clock;          /* NULL: a steady clock started at creation */
  void *clock_user;
} prtcl_gpu_server_params;
/* The batch a server drives, supplied by the caller
 * (prtcl_gpu_server_create_custom): each operation returns 0 on success. */
typedef struct prtcl_gpu_server_batch_ops {
  int (*add_scene)(void *user, const float *fluid_xyz, int64_t fluid_count, const float *boundary_xyz,
                   int64_t boundary_count, int64_t *scene_id_out);
  int (*remove_scene)(void *user, int64_t scene_id);
  int (*step)(void *user, int32_t steps);
  int (*synchronize)(void *user);
  int (*device_bytes)(void *user, int64_t *bytes_out);
  int (*scene_info)(void *user, int64_t scene_id, prtcl_gpu_scene_info *out);
  int (*download_positions)(void *user, int64_t scene_id, float *host_xyz, int64_t count);
} prtcl_gpu_server_batch_ops;
enum {
  PRTCL_GPU_REQUEST_DONE = 0,       /* took all its steps */
  PRTCL_GPU_REQUEST_CANCELLED = 1,  /* prtcl_gpu_server_cancel */
  PRTCL_GPU_REQUEST_REJECTED = 2,   /* its estimate exceeded the budget at admission */
  PRTCL_GPU_REQUEST_FAILED = 3      /* a batch step, or reading its results, failed */
};
typedef struct prtcl_gpu_request_result {
  int64_t request_id;
  int64_t fluid, boundary, steps;    /* steps taken */
  double arrival, admitted, finished; /* admitted: -1 if never admitted */
  prtcl_gpu_scene_info info;         /* the scene's information at retirement (zero if never admitted) */
  int32_t status;                    /* PRTCL_GPU_REQUEST_* */
  int32_t pad;
} prtcl_gpu_request_result;
typedef struct prtcl_gpu_server_status {
  int64_t pending, running, results; /* submitted, resident, retired and not yet read */
  int64_t steps_run, particle_steps; /* turns that stepped; fluid particles x steps */
  int64_t held_bytes;                /* the batch's device bytes at the last admission or retirement */
  double next_arrival;               /* of the first pending request; +inf when none */
} prtcl_gpu_server_status;

/* A server over a batch of its own (prtcl_gpu_batch_create with `batch`). */
int prtcl_gpu_server_create(const prtcl_gpu_batch_params *batch, const prtcl_gpu_server_params *params,
                            prtcl_gpu_server **out);
/* A server over a caller's batch; `ops` and `user` must outlive the server. */
int prtcl_gpu_server_create_custom(const prtcl_gpu_server_batch_ops *ops, void *user,
                                   const prtcl_gpu_server_params *params, prtcl_gpu_server **out);
int prtcl_gpu_server_destroy(prtcl_gpu_server *server);
/* Queue a request (its particles are copied); request ids are the caller's. */
int prtcl_gpu_server_submit(prtcl_gpu_server *server, int64_t request_id, double arrival, const float *fluid_xyz,
                            int64_t fluid_count, const float *boundary_xyz, int64_t boundary_count, int64_t steps);
/* One turn; *stepped_out = 1 if the resident scenes were stepped, 0 if
 * nothing was resident (wait for status.next_arrival). */
int prtcl_gpu_server_turn(prtcl_gpu_server *server, int32_t *stepped_out);
int prtcl_gpu_server_status_get(prtcl_gpu_server *server, prtcl_gpu_server_status *out);
/* Cancel a queued or resident request: it is retired with status
 * PRTCL_GPU_REQUEST_CANCELLED (a resident one with the steps it took and
 * its scene removed).  *found_out = 0 if no queued or resident request has
 * that id (already retired, or never submitted). */
int prtcl_gpu_server_cancel(prtcl_gpu_server *server, int64_t request_id, int32_t *found_out);
/* The oldest unread result (*has_out = 0 when there is none).  Its final
 * fluid positions are copied to `positions_xyz` (NULL: not copied; otherwise
 * `capacity` >= the request's fluid count, in particles). */
int prtcl_gpu_server_next_result(prtcl_gpu_server *server, prtcl_gpu_request_result *out, float *positions_xyz,
                                 int64_t capacity, int32_t *has_out);

#ifdef __cplusplus
}
#endif

#endif /* PRTCL_GPU_H */
