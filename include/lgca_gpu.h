/*
 * lgca_gpu.h -- C ABI of the GB300 lattice-gas engine (liblgca_gpu.so).
 *
 * One handle = one lattice resident in GPU memory as multi-spin-coded
 * bit-planes (one bit per site and channel, 64 sites per uint64 word), plus
 * its geometry planes, its step counter and the CUDA stream it runs on.
 * Plain C types only; every call returns an lgca_status (0 = success) and
 * records a message retrievable with lgca_last_error().  Calls on one handle
 * must not overlap from several host threads, and a call on a batch counts
 * as a call on each of its members.  Host buffers are owned by the caller
 * and may be freed when the call returns.
 *
 * The entry points replace the backend half of the reference's Lattice<Model>
 * interface (keva92/lgca src/lattice.h:32-238, implemented by OMP_Lattice in
 * src/omp_lattice.{h,cpp}); each declaration names the reference member it
 * stands in for.  The reference state format -- one byte per cell, bit d =
 * channel d (src/lgca_bitset.h:31-245, bit dir + 8*cell) -- is the exchange
 * format of lgca_upload_state / lgca_download_state.
 *
 * Randomness: collision chirality and forcing draws come from the
 * counter-based generator in include/lgca/rng.h, keyed by the lattice seed
 * and the global step number, so a run is reproducible bit for bit.
 */
#ifndef LGCA_GPU_H_
#define LGCA_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LGCA_GPU_ABI_VERSION 1

typedef enum {
    LGCA_OK = 0,
    LGCA_ERR_INVALID = 1,  /* bad argument; nothing was changed             */
    LGCA_ERR_NOMEM = 2,    /* device allocation failed or over the budget   */
    LGCA_ERR_CUDA = 3,     /* CUDA runtime error (message has the details)  */
    LGCA_ERR_TIMEOUT = 4,  /* a bounded device-side wait gave up            */
    LGCA_ERR_BUSY = 5      /* resource in use                                */
} lgca_status;

/* Model and cell-type values are those of src/lgca_common.h:49-60. */
typedef enum { LGCA_HPP = 0, LGCA_FHP_I = 1, LGCA_FHP_II = 2, LGCA_FHP_III = 3 } lgca_model;
typedef enum { LGCA_FLUID = 0, LGCA_SOLID_NO_SLIP = 1, LGCA_SOLID_SLIP = 2 } lgca_cell_type;

typedef struct lgca_lattice *lgca_handle;

/* ABI version and the device the library was built for. */
int lgca_abi_version(void);
const char *lgca_status_string(int status);
const char *lgca_last_error(lgca_handle h); /* h may be NULL: last global error */

/* Allocate a dim_x x dim_y lattice of `model` on the current CUDA device,
 * all cells FLUID and empty, step counter 0 (the zeroing is queued on the
 * handle's stream; the call does not wait for it).  FHP models need an even dim_y
 * (src/lattice.cpp:141, src/omp_lattice.cpp:103-111).
 * Replaces: OMP_Lattice<M>::OMP_Lattice + allocate_memory
 *           (src/omp_lattice.cpp:75-88,457-471). */
int lgca_create(int model, int dim_x, int dim_y, uint64_t seed, lgca_handle *out);

/* Replaces: OMP_Lattice<M>::~OMP_Lattice + free_memory (src/omp_lattice.cpp:91-97,474-489). */
int lgca_destroy(lgca_handle h);

/* Lattice device memory comes from a per-device stream-ordered pool that
 * keeps freed blocks for the next lattice (no device-wide wait when lattices
 * are created or destroyed).  Return unused pool memory beyond keep_bytes to
 * the driver.  (No reference counterpart: the reference frees with
 * cudaFree/delete in free_memory.) */
int lgca_trim_memory(int device, uint64_t keep_bytes);

/* Dimensions, model, seed and step counter of a handle. */
int lgca_info(lgca_handle h, int *model, int *dim_x, int *dim_y, uint64_t *seed,
              uint64_t *step);

/* Set / read the global step number t that keys the step's random draws. */
int lgca_set_step(lgca_handle h, uint64_t t);

/* Cell-type map, dim_x*dim_y int32 values of lgca_cell_type in row-major
 * order (x fastest), the layout of the reference's m_cell_type_cpu
 * (src/lattice.h:80).  Any other value is rejected.
 * Replaces the effect of apply_cell_type_all / apply_boundary_cell_type_* /
 * apply_bc_* (src/lattice.cpp:221-395), which build that map on the host. */
int lgca_set_cell_types(lgca_handle h, const int32_t *types);
int lgca_get_cell_types(lgca_handle h, int32_t *types);

/* Shapes of lgca_paint_cells. */
typedef enum {
    LGCA_SHAPE_RECT = 0,       /* a <= x < c and b <= y < d (clipped to the lattice) */
    LGCA_SHAPE_DISC = 1,       /* (x-a)^2 + (y-b)^2 < c^2, exact integers */
    LGCA_SHAPE_DISC_FLOAT = 2  /* float(sqrt(dx^2 + dy^2)) < c / 2.0 with dx = x-a, dy = y-b:
                                  the obstacle of diameter c of apply_bc_karman_vortex_street */
} lgca_shape;

/* Set every cell of a shape to `type`, on the device and in stream order
 * (no host map, no wait).  Replaces apply_cell_type_all and
 * apply_boundary_cell_type_{north,south,east,west} (src/lattice.cpp:337-398;
 * rectangles) and the obstacle loop of apply_bc_karman_vortex_street
 * (src/lattice.cpp:252-280; LGCA_SHAPE_DISC_FLOAT), so that apply_bc_pipe,
 * _karman_vortex_street and _reflecting are a few calls.  |a|, |b|, |c|, |d|
 * must be below 2^29 and c >= 0 for discs.  The boundary kernels chosen
 * afterwards assume that every painted type may be present (painting FLUID
 * over all walls keeps the wall-aware kernels, which give the same result). */
int lgca_paint_cells(lgca_handle h, int shape, int32_t type, int64_t a, int64_t b, int64_t c,
                     int64_t d);

/* Whole state in the reference byte format: dim_x*dim_y bytes, bit d =
 * channel d.  Bits >= NUM_DIR are ignored on upload and zero on download.
 * Replaces: copy_data_to_device / copy_data_from_device
 * (src/lattice.h:206-211, src/lattice.cpp:422-435). */
int lgca_upload_state(lgca_handle h, const uint8_t *cells);
int lgca_download_state(lgca_handle h, uint8_t *cells);
/* Queued forms: lgca_upload_state returns once the copy is queued; from a
 * pinned buffer the copy runs later, so keep the buffer unchanged until
 * lgca_sync(h).  lgca_download_state_async queues the download; the bytes
 * are in `cells` after lgca_sync(h).  At most one queued download per handle
 * (both use the handle's scratch). */
int lgca_download_state_async(lgca_handle h, uint8_t *cells);

/* Occupy each channel of each FLUID cell independently with probability
 * p_move (moving channels) or p_rest (rest channel of FHP-II/III), drawn from
 * the INIT stream; other cells are emptied.
 * Replaces: Lattice::init_random (src/lattice.cpp:198-217, p = 1/NUM_DIR). */
int lgca_init_random(lgca_handle h, double p_move, double p_rest);

/* Empty lattice.  Replaces: Lattice::init_zero (src/lattice.cpp:166-170). */
int lgca_init_zero(lgca_handle h);

/* Forcing column: before each step, every FLUID cell (x, y) with a
 * west-moving particle and an empty east-moving channel reverses it with
 * probability p (FORCE stream); x < 0 or p <= 0 disables.  The reversal rule
 * is the reference's x body force (src/omp_lattice.cpp:295-300, :313-318). */
int lgca_set_forcing_column(lgca_handle h, int x, double p);

/* Chirality source.  field == NULL: counter-based draw per site and step
 * (default).  Otherwise dim_x*dim_y bytes (0/1) frozen for all later steps,
 * which is the reference's own model: a per-cell bit field drawn once
 * (m_rnd_cpu, src/omp_lattice.cpp:84,198). */
int lgca_set_chirality(lgca_handle h, const uint8_t *field);

/* Temporal blocking depth: steps advanced per pass over the state in global
 * memory (1..8).  Results do not depend on it. */
int lgca_set_temporal_depth(lgca_handle h, int depth);

/* Kernel family for the steps: 0 = automatic (default: the resident form 6
 * on lattices it holds, for calls of 16 or more steps on lattices of at
 * least 4 Mi sites with rows of at least 2048 sites, and for calls of 64 or
 * more steps on lattices of at least 1 Mi sites with rows of at least 4096
 * sites; the register
 * wavefront at 4 steps per pass for HPP lattices of 64 Mi sites or more and
 * at 4 (FHP-I) or 2 (FHP-II/III) for FHP lattices of 256 Mi sites or more;
 * else one step per pass; a temporal depth above 1 selects the wavefront),
 * 1 = one step per
 * pass only, 2 = register wavefront (several steps per pass), 3 = shared-
 * memory tiles (several steps per pass), 4 = persistent (all steps of a call
 * in one cooperative launch; each block owns a band of rows and waits, with a
 * bounded wait, only for its two neighbour bands between steps; a wait that
 * times out marks the handle failed: see lgca_clear_error),
 * 5 = one step per pass with two words per lane where dim_x is a multiple of
 * 128 (variant 1 keeps one word per lane), 6 = resident (all steps of a call
 * in one cooperative launch with the state held on chip between steps; for
 * dim_x a multiple of 128 and lattices whose rows, at one row of up to 4096
 * sites per warp, fit the GPU at once, e.g. 8192 x 2048; otherwise one step
 * per pass; waits as for 4).  Results do not depend on it.
 * No reference counterpart (a scheduling choice of this engine). */
int lgca_set_kernel_variant(lgca_handle h, int variant);

/* The kernels a call lgca_collide_and_propagate(h, nsteps) would run with the
 * handle's current settings: *family = 6 (resident), 4 (persistent bands) or
 * 1 (passes of one or more steps), *launches = the step-kernel launches of
 * the call (memory-set nodes not counted).  Either pointer may be NULL.
 * No reference counterpart (introspection of this engine's scheduling). */
int lgca_step_plan(lgca_handle h, int nsteps, int *family, int *launches);

/* lgca_step_plan for a lattice of model and dim_x x dim_y with a new handle's
 * settings (automatic kernel choice, one step per pass unless chosen
 * otherwise) on the current device, without creating it.  Either pointer may
 * be NULL.  Invalid dimensions as for lgca_create.
 * No reference counterpart (introspection of this engine's scheduling). */
int lgca_plan_shape(int model, int dim_x, int dim_y, int nsteps, int *family, int *launches);

/* Launch shape of the one-step kernels: warps per block (1, 2, 4 or 8), or 0
 * to choose per launch the largest block whose grid spreads over the SMs with
 * the least wave-quantisation loss.  A tuning knob: results do not depend on
 * it.  (No reference counterpart.) */
int lgca_set_block_warps(lgca_handle h, int warps);

/* Advance nsteps steps (forcing column, then pull-stream + collide by cell
 * type), enqueued on the handle's stream; the step counter advances by
 * nsteps.  Replaces: OMP_Lattice<M>::collide_and_propagate
 * (src/omp_lattice.cpp:100-249), called nsteps times; its `p` argument is
 * ignored there and has no counterpart. */
int lgca_collide_and_propagate(lgca_handle h, int nsteps);

/* nsteps steps, then the B x B block sums of the result into the device
 * arrays N, Jx2, Jy (as lgca_block_sums_device).  Where the resident kernel
 * runs the steps and B is 8, 16, 32 or 64, the sums are computed inside its
 * launch.  No reference counterpart beyond the two calls it stands for
 * (src/omp_lattice.cpp:100-249 and the block sums). */
int lgca_collide_and_propagate_sums(lgca_handle h, int nsteps, int B, int32_t *N, int32_t *Jx2,
                                    int32_t *Jy);

/* One job on the handle's stream, without waiting: the state from cells_in
 * (host, dim_x*dim_y bytes as lgca_upload_state; NULL keeps the current
 * state), nsteps steps, the result to cells_out (host, as
 * lgca_download_state_async; NULL: no download) and, for B > 0, the B x B
 * block sums of the result to the host arrays N, Jx2, Jy (as
 * lgca_block_sums_async).  Outputs are valid after lgca_sync.  The same as
 * those calls in that order, but where the resident kernel runs the steps,
 * the byte-per-cell conversions (and the block sums for B = 8, 16, 32, 64)
 * happen inside its launch, so no other kernel runs between jobs.  Host
 * buffers should be pinned for the copies to overlap other work.
 * Reference counterpart: copy_data_to_device, collide_and_propagate (x
 * nsteps) and copy_data_from_device + copy_data_to_output_buffer
 * (src/lattice.cpp:422-441, src/omp_lattice.cpp:100-249). */
int lgca_run_job_async(lgca_handle h, const uint8_t *cells_in, int nsteps, uint8_t *cells_out,
                       int B, int32_t *N, int32_t *Jx2, int32_t *Jy);

/* Random-cell body force with the reference's semantics: candidate cells
 * are drawn (FSEQ stream, call counter of the handle) until `forcing`
 * particles were reverted or 2*num_cells draws were made; bf_dir is 'x', 'y'
 * or 0.  *reverted (may be NULL) receives the number of reversals.
 * Replaces: OMP_Lattice<M>::apply_body_force (src/omp_lattice.cpp:254-346). */
int lgca_apply_body_force(lgca_handle h, int forcing, int bf_dir, uint64_t *reverted);

/* Replaces: Lattice::get_n_particles (src/lattice.cpp:180-195). */
int lgca_count_particles(lgca_handle h, uint64_t *n);

/* Mean over FLUID cells of cell momentum / cell density (cells with density
 * 0 add nothing).  Replaces: OMP_Lattice<M>::get_mean_velocity
 * (src/omp_lattice.cpp:508-557). */
int lgca_mean_velocity(lgca_handle h, float *ux, float *uy);

/* Exact integer sums over non-overlapping B x B blocks (B >= 1; blocks at
 * the top/right edge are clipped): N = particles, Jx2 = x momentum in units
 * of 1/2, Jy = y momentum in units of sin(60 deg) (FHP) or 1 (HPP).  Each
 * output holds ceil(dim_y/B) rows of ceil(dim_x/B) int32 values.  Host
 * pointers; the _device variant takes device pointers and does not wait.
 * No reference counterpart: the integer form of the coarse-graining of
 * src/omp_lattice.cpp:397-454. */
int lgca_block_sums(lgca_handle h, int B, int32_t *N, int32_t *Jx2, int32_t *Jy);
int lgca_block_sums_device(lgca_handle h, int B, int32_t *N, int32_t *Jx2, int32_t *Jy);
/* As lgca_block_sums into host buffers, without waiting: the values are in
 * place after lgca_sync(h).  Host buffers should be pinned for the copies to
 * overlap; at most one outstanding call per handle before lgca_sync. */
int lgca_block_sums_async(lgca_handle h, int B, int32_t *N, int32_t *Jx2, int32_t *Jy);

/* Post-processing with the reference's arithmetic: per-cell density and FP32
 * momentum (dim_x*dim_y and 2*dim_x*dim_y floats, momentum interleaved x,y)
 * and the coarse means over radius r (coarse grid (dim_x/2r) x (dim_y/2r)).
 * Any output pointer may be NULL.  Host pointers.
 * Replaces: OMP_Lattice<M>::post_process = cell_post_process +
 * mean_post_process (src/omp_lattice.cpp:349-454). */
int lgca_post_process(lgca_handle h, int r, float *cell_density, float *cell_momentum,
                      float *mean_density, float *mean_momentum);

/* Allocation-free random-cell body force.  No counterpart in the reference:
 * an extra entry point of this library for callers that must not allocate
 * device memory during a run -- a host that has handed its whole device
 * budget to resident lattices, or one that cannot afford the device-wide
 * synchronisation of cudaMalloc/cudaFree between queued steps.  Same rule
 * and draws as lgca_apply_body_force (its FSEQ call index is `call`), on
 * caller-owned device buffers in the layout of lgca_state_device: `planes`
 * (NUM_DIR planes, `plane_stride` words apart, rows `row_pitch` words apart),
 * optional `solid` / `slip` planes of the same shape (NULL = none), and an
 * optional device counter `reverted`.  Enqueued on `stream` (NULL = default
 * stream); nothing is allocated or freed.  Its work arrays live in one fixed
 * device array of LGCA_NOALLOC_MAX_CELLS * 4 bytes + 4 KiB that every GPU
 * loading the library holds until exit; lattices above LGCA_NOALLOC_MAX_CELLS
 * cells are rejected with LGCA_ERR_INVALID.  The first call on a device looks
 * the array up (cudaGetSymbolAddress) and should come before any stream
 * capture.  All calls share the array: calls whose work overlaps on the GPU
 * race and must be ordered by the caller. */
#define LGCA_NOALLOC_MAX_CELLS 2097152ULL
int lgca_apply_body_force_noalloc(int model, int dim_x, int dim_y, uint64_t *planes,
                                  size_t plane_stride, int row_pitch, const uint64_t *solid,
                                  const uint64_t *slip, uint64_t seed, uint64_t call, int forcing,
                                  int bf_dir, unsigned long long *reverted, void *stream);

/* Wait for all work of the handle.  Returns LGCA_ERR_TIMEOUT while the
 * handle is marked failed (below). */
int lgca_sync(lgca_handle h);

/* Bounded waits of the persistent kernel (variant 4).  A neighbour wait that
 * runs past the handle's wait limit (lgca_set_wait_limit, 1 us .. 60 s,
 * default 2 s) makes the kernel stop early and marks the handle failed: its
 * step counter has advanced but its state is partly stepped.  From then on
 * every call that waits for the handle's stream (lgca_sync, downloads,
 * counts, sums, post-processing, checkpoints) returns LGCA_ERR_TIMEOUT, and
 * later persistent launches return at once without stepping, until
 * lgca_clear_error(h).  After clearing, load a state (lgca_upload_state or
 * lgca_checkpoint_load) before stepping on.
 * lgca_test_withhold_progress(h, b) is a test hook: block b (-1: none) of
 * the handle's persistent launches never publishes its progress, so its
 * neighbours' waits run out after the wait limit (every wait still ends).
 * No reference counterpart (the reference has no device-side waits). */
int lgca_clear_error(lgca_handle h);
int lgca_set_wait_limit(lgca_handle h, uint64_t wait_ns);
int lgca_test_withhold_progress(lgca_handle h, int block);

/* The cudaStream_t the handle enqueues on (as void*), and a way to replace
 * it by a caller-owned stream (NULL restores the handle's own stream).
 * lgca_stream also orders the stream after the lattice's queued batch steps
 * and marks it used, so that the lattice's next batch step runs after what
 * the caller queues on it: call it again after each batch call, rather than
 * keeping the pointer across batch calls.
 * Steps queued on a stream under CUDA graph capture are recorded with their
 * buffers and random keys fixed at capture time: a replay repeats steps
 * t .. t+k-1 of the capturing call, so capture an even number of steps to
 * replay it on the current state. */
void *lgca_stream(lgca_handle h);
int lgca_set_stream(lgca_handle h, void *stream);

/* Device view of the current state: base pointer of plane 0, words between
 * consecutive planes, words between consecutive rows.  Valid until the next
 * call that steps or replaces the state.  Everything that writes the state,
 * from lgca_create's zeroing on, is queued on the handle's stream: read it on
 * that stream (lgca_stream) or after lgca_sync. */
int lgca_state_device(lgca_handle h, const uint64_t **planes, size_t *plane_stride,
                      int *row_pitch);

/* Checkpoint / export of a lattice: state, geometry, frozen chirality, step
 * and body-force counters, seed and settings, into a caller-owned host
 * buffer of lgca_checkpoint_size bytes (a 96-byte header, then the planes
 * packed row by row).  lgca_checkpoint_load restores it into a handle of the
 * same model and dimensions, after which stepping continues bit for bit as
 * if uninterrupted.  No reference counterpart (the reference only writes
 * .vti output, src/lgca_io_vti.cpp:113-144). */
int lgca_checkpoint_size(lgca_handle h, size_t *bytes);
int lgca_checkpoint_save(lgca_handle h, void *buf, size_t bytes);
int lgca_checkpoint_load(lgca_handle h, const void *buf, size_t bytes);

/* Batches: many lattices (any sizes, models, geometries) advanced together,
 * one launch per step over a device work-list of the members' rows, the
 * steps captured in CUDA graphs.  A member whose kernel variant is 2 (the
 * register wavefront) with depth 2, 4 or 8 (8: HPP) and whose dim_x is a
 * multiple of 64 runs its steps as passes of `depth` steps over its state
 * (after nsteps % depth single steps with the others).  Members stay owned by
 * the caller and keep their own state, counters and settings; each member
 * gives exactly the bits it gives when stepped alone.  No reference
 * counterpart (the reference steps one lattice per object).
 *   lgca_batch_step_each: member i (in the order added) advances nsteps[i]
 *   steps (0 = not at all); members with fewer steps drop out of the
 *   work-list when done.  Work queued on a member's own stream before the
 *   call runs first; the member's later calls run after the batch.  Both
 *   orders are set up lazily: a call costs one stream wait per member whose
 *   stream was used since it last stepped, and none for the others; the
 *   member's stream waits for the batch at the member's next call.
 *   A lattice belongs to at most one batch; lgca_destroy removes it from
 *   its batch first. */
typedef struct lgca_batch *lgca_batch_handle;
int lgca_batch_create(lgca_batch_handle *out);
int lgca_batch_destroy(lgca_batch_handle b);
int lgca_batch_add(lgca_batch_handle b, lgca_handle lattice);
int lgca_batch_remove(lgca_batch_handle b, lgca_handle lattice);
int lgca_batch_size(lgca_batch_handle b, int *n);
int lgca_batch_step(lgca_batch_handle b, int nsteps);
int lgca_batch_step_each(lgca_batch_handle b, const int *nsteps);
int lgca_batch_set_graph_steps(lgca_batch_handle b, int steps_per_graph); /* 0: no graphs */
/* Warp tasks (32 lane items of one member) each warp of the batched kernel
 * takes per step: 1, 2, 4 or 8, or 0 (default) to choose per call: 2 when
 * the call's work fills at least four waves of resident warps at 2 tasks per
 * warp, 4 for calls 16 times larger, else 1.  More tasks per warp pay the
 * member lookup less often (2 ran 18 % faster than 1 on 512 lattices of
 * 1 G sites); fewer give more parallelism to small calls.  A tuning knob:
 * results do not depend on it.  (No reference counterpart.) */
int lgca_batch_set_warp_tasks(lgca_batch_handle b, int n);
/* Persistent form (on = 1, default): the one-step work of each call runs as
 * one cooperative launch per stretch of steps with an unchanged set of
 * members, the resident blocks walking the work-list with a grid barrier
 * between steps; on = 0 makes one launch per step, captured in CUDA graphs
 * (lgca_batch_set_graph_steps).  A barrier wait is bounded (2 s): when one
 * gives up, the next lgca_batch_sync returns LGCA_ERR_TIMEOUT once and the
 * members' states are unspecified.  Results do not depend on the form.
 * (No reference counterpart.) */
int lgca_batch_set_persistent(lgca_batch_handle b, int on);
int lgca_batch_sync(lgca_batch_handle b);
const char *lgca_batch_last_error(lgca_batch_handle b);
void *lgca_batch_stream(lgca_batch_handle b);

/* Bytes of device memory the handle holds. */
int lgca_device_bytes(lgca_handle h, size_t *bytes);

#ifdef __cplusplus
}
#endif

#endif /* LGCA_GPU_H_ */
