// Internal declarations shared by the CUDA translation units of
// liblgca_gpu.so.  Not part of the public interface (include/lgca_gpu.h).
//
// Device layout of one lattice (W x H sites, D channels):
//   state   D bit-planes, each H rows of `pitch` uint64 words; word w of row y
//           of plane d holds channel d of sites x = 64w .. 64w+63, bit i =
//           site 64w+i.  Bits at x >= W (the tail of the last word) are 0.
//           Plane d starts at base + d * plane_stride (words).
//   solid   one plane of the same shape, bit = SOLID_NO_SLIP (optional)
//   slip    one plane, bit = SOLID_SLIP (optional)
//   chir    one plane of frozen chirality bits (optional)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "collide.cuh"

namespace lgca_gpu {

// Programmatic dependent launch.  The step kernels are launched with
// programmatic stream serialisation: the next step's blocks may be scheduled
// while the previous step drains, and wait in pdl_wait() -- which returns
// once every earlier grid on the stream has completed and its writes are
// visible -- before they touch memory.  Launched without that attribute,
// pdl_wait() returns at once.
//
// Such kernels read the state through L2 only (ld.global.cg), never through
// the non-coherent L1/texture path: grids of consecutive steps share SMs, so
// an SM's L1 can still hold lines of a buffer that an older step read and the
// step in between has since rewritten.
// (Host builds of the kernel bodies -- the CPU emulation in the tests -- see
// no-ops.)
__device__ __forceinline__ void pdl_wait()
{
#ifdef __CUDA_ARCH__
    asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}
__device__ __forceinline__ void pdl_launch_dependents()
{
#ifdef __CUDA_ARCH__
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
}

//
// Not inside CUDA graphs: a stream under capture gets plain launches (the
// kernels' pdl_wait() then returns at once).  With programmatic edges in
// graphs that a batch call instantiates and releases while they run, the
// served loop stalled the device after about ten thousand calls; graphs
// already launch their kernels back to back.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t st, Args... args)
{
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr.val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = (cap == cudaStreamCaptureStatusNone) ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Number of SMs of the current device (cached per device).
int sm_count();

// Geometry modes of the step kernels: which cell-type planes exist.
enum : int { GEOM_NONE = 0, GEOM_NOSLIP = 1, GEOM_FULL = 2 };

struct PlaneGeom {
    int W, H;          // sites
    int nw;            // words per row = ceil(W / 64)
    int pitch;         // words between rows (>= nw, even)
    size_t ps;         // words between planes (= H * pitch)
    int L;             // bit index of site W-1 inside the last word
    uint64_t lastmask; // valid bits of the last word of a row
};

struct StepArgs {
    const uint64_t *__restrict__ src;
    uint64_t *__restrict__ dst;
    const uint64_t *__restrict__ solid;  // GEOM_NOSLIP / GEOM_FULL
    const uint64_t *__restrict__ slip;   // GEOM_FULL
    const uint64_t *__restrict__ chir;   // frozen chirality plane or nullptr
    PlaneGeom g;
    int chunks;         // 32-word chunks per row
    uint64_t chir_key;  // lgca_rng_key(seed, CHIR, t)
    uint64_t force_key; // lgca_rng_key(seed, FORCE, t)
    uint64_t force_thr; // 0 disables forcing
    int fx;             // forcing column (valid when force_thr > 0)
    int wpt;            // words per lane of the one-step kernel (1 or 2)
    int bw;             // warps per block of the one-step kernels (0: chosen per launch)
    uint32_t fmagic;    // flat_magic of the kernel's lane items (set by the launcher)
};

// One lattice of a batch (batch.cu): its step arguments (src/dst unused),
// its two buffers (buf0 holds the state at the start of the batch call), the
// keys' seed and first global step, the steps it advances in the call and
// its place in the work-list.
struct BatchEntry {
    StepArgs a;
    uint64_t *buf0, *buf1;
    uint64_t seed, t0;
    uint64_t *keys;  // 2 * nsteps keys (chirality, forcing) per step of the call
    int nsteps;
    int items;    // lane items per row (words, or word pairs when wpt == 2)
    int task0;    // first warp task (a multiple of the block's tasks) and real tasks
    int tasks;
    int gm, wpt;  // geometry mode, words per lane
    int code;     // model family * 9 + geometry mode * 3 + path (0 word, 1 pair, 2 pair, odd words)
    // members on the register wavefront (k_batch_wave): steps per pass K, the
    // single steps r that come before the passes, slab rows S and strips of
    // 30 words per row; tasks = strips x slabs
    int K, r, S, nstrips;
};
// total_tasks: warp tasks of the active members (each member's tasks padded
// to whole blocks of 8 * warp_tasks); block_lat[b] = member of block b;
// gmax: the largest geometry mode among the launch's members; warp_tasks:
// tasks per warp (1, 2, 4 or 8)
cudaError_t launch_batch(const BatchEntry *E, const int *block_lat, int total_tasks, int s_local,
                         const int *s_base, int gmax, int warp_tasks, cudaStream_t stream);
cudaError_t launch_batch_keys(const BatchEntry *E, int n, int max_steps, cudaStream_t stream);
// Persistent form of launch_batch: steps s0 .. s0 + nsteps - 1 (batch-local)
// in one cooperative launch with a grid barrier between steps; *bar must be
// zero before the launch; *err is set when a barrier wait passes wait_ns.
cudaError_t launch_batch_persist(const BatchEntry *E, const int *block_lat, int total_tasks, int s0,
                                 int nsteps, unsigned *bar, int *err, uint64_t wait_ns, int gmax,
                                 int warp_tasks, cudaStream_t stream);
// Pass j_base[0] + j_local of K steps for the wave members: total_tasks warp
// tasks (each member's padded to whole blocks of WAVE_BLOCK_WARPS warps),
// block_lat[b] = member of block b.
cudaError_t launch_batch_wave(const BatchEntry *E, const int *block_lat, int total_tasks, int j_local,
                              const int *j_base, int gmax, int K, cudaStream_t stream);
static constexpr int WAVE_BLOCK_WARPS = 4;
cudaError_t launch_advance(int *s_base, int by, cudaStream_t stream);
cudaError_t launch_set_base(int *s_base, int v, cudaStream_t stream);

// One lattice step of `a` (k = 1), launched on `stream`.
cudaError_t launch_step(int model, int geom_mode, const StepArgs &a, cudaStream_t stream);

// Multi-step pass: advances `depth` steps per pass over global memory.
// keys[i] / fkeys[i] are the chirality / forcing keys of step i of the pass.
struct MultiStepArgs {
    StepArgs base;  // src / dst of the whole pass; keys unused
    int depth;
    uint64_t chir_keys[8];
    uint64_t force_keys[8];
};
// Shared-memory tile form (multistep.cu) and register wavefront form (wave.cu).
cudaError_t launch_multistep(int model, int geom_mode, const MultiStepArgs &a,
                             cudaStream_t stream);
bool multistep_supported(int model, const PlaneGeom &g, int depth);
cudaError_t launch_wave(int model, int geom_mode, const MultiStepArgs &a, cudaStream_t stream);
bool wave_supported(int model, const PlaneGeom &g, int depth);

// Persistent band form (step.cu): nsteps steps in one cooperative launch,
// buf0 holding the input; the result is in buf0 if nsteps is even, else in
// buf1.  `flags` holds one int per block (at most max_blocks) and must be
// zero before the launch.  *err != 0 afterwards means a bounded neighbour
// wait gave up; it is never cleared by the kernel, and a launch that finds it
// set returns at once.  Each neighbour wait gives up after w.wait_ns (> 0)
// nanoseconds; block w.withhold (-1: none) never publishes its progress (a
// test hook that makes its neighbours' waits run out).
static constexpr int PERSIST_MAX_BLOCKS = 1024;
struct PersistWait {
    uint64_t wait_ns;
    int withhold;
};
cudaError_t launch_persistent(int model, int geom_mode, const StepArgs &a, uint64_t *buf0,
                              uint64_t *buf1, uint64_t seed, uint64_t t0, int nsteps, int *flags,
                              int *err, int max_blocks, const PersistWait &w, cudaStream_t stream);

// Resident form (resident.cu): nsteps steps in one cooperative launch with
// the state held on chip between steps; for lattices of whole word pairs per
// row whose one-row-per-warp tasks fit on the GPU at once.  The result is in
// `a.dst`.  `halo` holds halo_words words; *err as for launch_persistent.
struct ResidentShape {
    int nblk, wpr, rpb;  // blocks (bands), warps per row, most rows in a band
    size_t smem;         // dynamic shared memory per block
    size_t halo_words;
    bool rowsync;        // row barriers instead of a block barrier per step
};
static constexpr size_t RES_MAX_SMEM = 200 * 1024;
// the automatic choice gives the resident form calls of at least
// RESIDENT_MIN_STEPS steps on lattices of at least RESIDENT_MIN_SITES sites,
// and calls of at least RESIDENT_LONG_STEPS steps on lattices of at least
// RESIDENT_LONG_SITES sites whose rows fill whole warps (4096+ sites)
static constexpr int RESIDENT_MIN_STEPS = 16;
static constexpr long long RESIDENT_MIN_SITES = 4LL << 20;
static constexpr int RESIDENT_LONG_STEPS = 64;
static constexpr long long RESIDENT_LONG_SITES = 1LL << 20;
bool resident_shape(int model, const PlaneGeom &g, ResidentShape &out);
// aos_in / aos_out (device, H x W bytes, bit d = channel d; either may be
// null): the launch's input is read from aos_in instead of a.src, and its
// result is written to aos_out as well as to a.dst.  sums (or null): the
// B x B block sums of the result, fused into the launch, added into the
// device arrays N, Jx2, Jy (ceil(H/B) x ceil(W/B), zero before the launch);
// B in 8, 16, 32, 64 and resident_sums_fit true.
struct ResidentSums {
    int B;
    int32_t *N, *Jx2, *Jy;
};
bool resident_sums_fit(int model, const PlaneGeom &g, const ResidentShape &sh, int B);
// epoch (1..255) tags the launch's halo items: the slots must hold no item
// of that epoch (zero them, then use each epoch once); nsteps is at most
// RESIDENT_MAX_STEPS.
static constexpr int RESIDENT_MAX_STEPS = (1 << 24) - 2;
cudaError_t launch_resident(int model, int geom_mode, const StepArgs &a, const ResidentShape &sh,
                            uint64_t *halo, int *err, uint64_t seed, uint64_t t0,
                            int nsteps, const PersistWait &w, const uint8_t *aos_in,
                            uint8_t *aos_out, const ResidentSums *sums, unsigned epoch,
                            cudaStream_t stream);

// Kernel families selectable per handle.
enum : int {
    VARIANT_AUTO = 0,
    VARIANT_PLAIN = 1,
    VARIANT_WAVE = 2,
    VARIANT_TILE = 3,
    VARIANT_PERSIST = 4,
    VARIANT_PLAIN2 = 5,   // one step per pass, two words per lane
    VARIANT_RESIDENT = 6  // state held on chip across the steps of a call
};

// Layout conversion between the reference byte-per-cell format and planes.
cudaError_t launch_aos_to_planes(int D, const PlaneGeom &g, const uint8_t *aos, uint64_t *planes,
                                 cudaStream_t s);
cudaError_t launch_planes_to_aos(int D, const PlaneGeom &g, const uint64_t *planes, uint8_t *aos,
                                 cudaStream_t s);
// Cell types (int32) -> solid / slip planes; *bad set to 1 on invalid values.
cudaError_t launch_types_to_planes(const PlaneGeom &g, const int32_t *types, uint64_t *solid,
                                   uint64_t *slip, int *bad, cudaStream_t s);
cudaError_t launch_paint(const PlaneGeom &g, uint64_t *solid, uint64_t *slip, int shape, int type,
                         long long a, long long b, long long c, long long d, cudaStream_t s);
cudaError_t launch_planes_to_types(const PlaneGeom &g, const uint64_t *solid, const uint64_t *slip,
                                   int32_t *types, cudaStream_t s);
// Bernoulli initial occupation (fluid cells only).
cudaError_t launch_init_random(int D, const PlaneGeom &g, const uint64_t *solid,
                               const uint64_t *slip, uint64_t *planes, uint64_t seed,
                               uint64_t thr_move, uint64_t thr_rest, cudaStream_t s);
// Bytes (0/1) -> one plane.
cudaError_t launch_bytes_to_plane(const PlaneGeom &g, const uint8_t *bytes, uint64_t *plane,
                                  cudaStream_t s);
// Integer block sums.
cudaError_t launch_block_sums(int model, const PlaneGeom &g, const uint64_t *planes, int B,
                              int32_t *N, int32_t *Jx2, int32_t *Jy, cudaStream_t s);
// Reference-arithmetic post-processing.
cudaError_t launch_cell_post(int model, const PlaneGeom &g, const uint64_t *planes,
                             float *cell_density, float *cell_momentum, cudaStream_t s);
cudaError_t launch_mean_post(int model, const PlaneGeom &g, const uint64_t *planes, int r,
                             float *mean_density, float *mean_momentum, cudaStream_t s);
// Reductions: out[0] = particles; mean velocity sums into dsum[0..1] (double)
// and the fluid-cell count into out[1].
cudaError_t launch_count(int D, const PlaneGeom &g, const uint64_t *planes,
                         unsigned long long *out, cudaStream_t s);
cudaError_t launch_mean_velocity(int model, const PlaneGeom &g, const uint64_t *planes,
                                 const uint64_t *solid, const uint64_t *slip, double *dsum,
                                 unsigned long long *nfluid, cudaStream_t s);

// Random-cell body force (reference semantics), one cooperative launch.
// scratch holds body_force_scratch_bytes(num_cells) bytes (a first-occurrence
// table of one word per cell, then per-call state); `sticky` points to
// BODY_FORCE_STICKY_BYTES bytes at a place that stays the same from call to
// call for the same scratch, zero before the first call: it records how much
// of the table is known to be all ones, so that calls need not clear it.
// *reverted_dev receives the reversals (all ones if a grid barrier gave up,
// which also sets *err_out when err_out is not null).
size_t body_force_scratch_bytes(size_t num_cells);
static constexpr size_t BODY_FORCE_STICKY_BYTES = 64;
cudaError_t launch_body_force(int model, const PlaneGeom &g, uint64_t *planes,
                              const uint64_t *solid, const uint64_t *slip, uint64_t key,
                              long long forcing, int bf_dir, void *scratch, void *sticky,
                              unsigned long long *reverted_dev, int *err_out, cudaStream_t s);

// Lane mapping of the one-step kernels: the lane items (words, or pairs of
// words) of all even rows, then of all odd rows, are numbered row by row, and
// warp task k takes 32 consecutive numbers of one parity class.  Every lane
// is used except at the end of a class, and the rows of a warp share one
// parity (the step bodies' contract).  A lane whose left or right neighbour
// lane holds another row loads that neighbour word instead of shuffling.
__host__ __device__ __forceinline__ long long class_tasks(int H, int items, int parity)
{
    const long long rows = parity ? (H / 2) : ((H + 1) / 2);
    return (rows * items + 31) / 32;
}
__host__ __device__ __forceinline__ long long flat_tasks(int H, int items)
{
    return class_tasks(H, items, 0) + class_tasks(H, items, 1);
}
// Multiplier for dividing lane numbers by `items` without a divide: with
// m = ceil(2^32 / items), floor(l * m / 2^32) = l / items for every l with
// l * items < 2^32 (the rounding error l * (m * items - 2^32) / 2^32 stays
// below one step).  Lane numbers stay below rows-per-class * items + 32;
// 0 when that bound fails or items < 2 (then a divide is used).
__host__ __device__ __forceinline__ uint32_t flat_magic(int H, int items)
{
    if (items < 2) return 0u;
    const unsigned long long lmax = (unsigned long long)((H + 1) / 2) * (unsigned)items + 32u;
    if (lmax * (unsigned long long)items >= (1ull << 32)) return 0u;
    return (uint32_t)(((1ull << 32) + (unsigned)items - 1) / (unsigned)items);
}

// Row y and item of `lane` in warp task `task` (y >= H past a class's end);
// magic = flat_magic(H, items).  Host-callable for the mapping checks.
__host__ __device__ __forceinline__ void flat_site(long long task, int lane, int H, int items,
                                                   uint32_t magic, int &y, int &item)
{
    const long long even_tasks = class_tasks(H, items, 0);
    const int p = task >= even_tasks ? 1 : 0;
    const unsigned l = (unsigned)((p ? task - even_tasks : task) * 32 + lane);
#ifdef __CUDA_ARCH__
    const unsigned r = magic ? __umulhi(l, magic) : l / (unsigned)items;
#else
    const unsigned r = magic ? (unsigned)(((unsigned long long)l * magic) >> 32) : l / (unsigned)items;
#endif
    item = (int)(l - r * (unsigned)items);
    y = (int)(2 * r + p);
}

static inline int num_dir(int model) { return model == M_HPP ? 4 : (model == M_FHP_I ? 6 : 7); }

}  // namespace lgca_gpu
