// C ABI of the GB300 lattice-gas engine: handle management, host <-> device
// transfers and dispatch to the kernels.  Declarations and the reference
// interface each entry point replaces: include/lgca_gpu.h.
#include "internal.cuh"
#include "../../include/lgca_gpu.h"
#include "../../include/lgca/rng.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

using namespace lgca_gpu;

struct lgca_batch;

struct lgca_lattice {
    int model = 0, D = 0;
    PlaneGeom g{};
    uint64_t seed = 0, t = 0, fcall = 0;
    uint64_t *buf[2] = {nullptr, nullptr};
    int cur = 0;
    uint64_t *solid = nullptr, *slip = nullptr, *chir = nullptr;
    bool has_noslip = false, has_slip = false, frozen = false;
    int force_x = -1;
    uint64_t force_thr = 0;
    int depth = 1;
    int variant = VARIANT_AUTO;
    int wpt = 2;  // words per lane of the one-step kernel where the width allows
    int bw = 0;   // warps per block of the one-step kernels (0: chosen per launch)
    int device = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    void *scratch = nullptr;
    size_t scratch_bytes = 0;
    // random-cell body force: its first-occurrence table (kept all ones
    // between calls), per-call state, the table's clean mark and the count
    void *bf = nullptr;
    // resident form: the band edges' halo slots (resident_shape of the lattice)
    // and the epoch of the last launch's items (0: the slots need zeroing)
    void *res = nullptr;
    unsigned res_epoch = 0;
    // persistent kernel: sync[0] = error flag (sticky: set when a bounded
    // neighbour wait gave up, cleared only by lgca_clear_error), then one step
    // flag per block; sync_err_host is its pinned copy, refreshed after each
    // persistent call and checked by every call that waits for the stream
    int *sync = nullptr;
    int *sync_err_host = nullptr;
    uint64_t wait_ns = 2000000000ull;  // limit of one neighbour wait
    int withhold = -1;                 // test hook: block that never publishes its step
    size_t bytes = 0;
    lgca_batch *batch = nullptr;  // the batch this lattice belongs to, if any
    // Ordering against batch calls without stream calls per member and call:
    // `after_batch` -- batch steps of this lattice are queued on the batch's
    // stream and the handle's stream has not yet been made to wait for them
    // (done at the handle's next use, on `batch_done`); `used` -- work was
    // queued on the handle's stream since the last batch call that stepped it,
    // so the next such call orders its steps after that work.
    cudaEvent_t batch_done = nullptr;
    bool after_batch = false;
    bool used = true;
    std::string err;
};

namespace {

thread_local std::string g_err;

// The plane layout of a W x H lattice: 64 sites per word, rows padded to an
// even number of words.
void set_plane_geom(PlaneGeom &g, int W, int H)
{
    g.W = W;
    g.H = H;
    g.nw = (W + 63) / 64;
    g.pitch = (g.nw + 1) & ~1;
    g.ps = (size_t)H * g.pitch;
    g.L = (W - 1) & 63;
    g.lastmask = (g.L == 63) ? ~0ull : ((1ull << (g.L + 1)) - 1ull);
}

int fail(lgca_lattice *h, int status, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    if (h) h->err = buf;
    return status;
}

int cuda_fail(lgca_lattice *h, cudaError_t e, const char *what)
{
    return fail(h, e == cudaErrorMemoryAllocation ? LGCA_ERR_NOMEM : LGCA_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

#define CK(h, expr)                                                   \
    do {                                                              \
        cudaError_t e_ = (expr);                                      \
        if (e_ != cudaSuccess) return cuda_fail((h), e_, #expr);      \
    } while (0)

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// Lattice memory comes from one stream-ordered pool per device that keeps
// freed blocks for reuse: lattices are created and destroyed while others
// run without synchronising the device or returning memory to the driver
// (lgca_trim_memory hands unused blocks back).
constexpr int MAX_DEVICES = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pool[MAX_DEVICES] = {};

cudaError_t lattice_pool(int dev, cudaMemPool_t *out)
{
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (!g_pool[dev]) {
        cudaMemPoolProps props;
        memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        cudaError_t e = cudaMemPoolCreate(&p, &props);
        if (e != cudaSuccess) return e;
        uint64_t keep = ~0ull;
        e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
        if (e != cudaSuccess) {
            cudaMemPoolDestroy(p);
            return e;
        }
        g_pool[dev] = p;
    }
    *out = g_pool[dev];
    return cudaSuccess;
}

// stream-ordered allocation on the handle's stream (zeroed when asked)
int dalloc(lgca_lattice *h, void **p, size_t bytes, bool zero, const char *what)
{
    cudaMemPool_t pool;
    cudaError_t e = lattice_pool(h->device, &pool);
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync(p, bytes, pool, h->stream);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(h, e, what);
    }
    if (zero && (e = cudaMemsetAsync(*p, 0, bytes, h->stream)) != cudaSuccess)
        return cuda_fail(h, e, what);
    h->bytes += bytes;
    return LGCA_OK;
}

void dfree(lgca_lattice *h, void *p)
{
    if (p) cudaFreeAsync(p, h->stream);
}

int geometry_planes(lgca_lattice *h)
{
    if (h->solid) return LGCA_OK;
    const size_t plane_bytes = h->g.ps * sizeof(uint64_t);
    int st = dalloc(h, reinterpret_cast<void **>(&h->solid), plane_bytes, true, "solid plane");
    if (st == LGCA_OK)
        st = dalloc(h, reinterpret_cast<void **>(&h->slip), plane_bytes, true, "slip plane");
    return st;
}

int scratch_reserve(lgca_lattice *h, size_t bytes)
{
    if (h->scratch_bytes >= bytes) return LGCA_OK;
    if (h->scratch) {
        dfree(h, h->scratch);  // in stream order after its last use
        h->bytes -= h->scratch_bytes;
        h->scratch = nullptr;
        h->scratch_bytes = 0;
    }
    int st = dalloc(h, &h->scratch, bytes, false, "scratch");
    if (st) return st;
    h->scratch_bytes = bytes;
    return LGCA_OK;
}

int geom_mode(const lgca_lattice *h)
{
    if (h->has_slip) return GEOM_FULL;
    if (h->has_noslip) return GEOM_NOSLIP;
    return GEOM_NONE;
}

bool valid(lgca_handle h) { return h != nullptr && h->buf[0] != nullptr; }

// The device error flag of bounded device waits (persistent kernel, body
// force) and its pinned host copy, allocated at first use.
int error_flag(lgca_lattice *h)
{
    if (h->sync) return LGCA_OK;
    const size_t sync_bytes = (size_t)(PERSIST_MAX_BLOCKS + 1) * sizeof(int);
    int st = dalloc(h, reinterpret_cast<void **>(&h->sync), sync_bytes, true, "flags");
    if (st) return st;
    const cudaError_t e = cudaHostAlloc(&h->sync_err_host, sizeof(int), cudaHostAllocDefault);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaHostAlloc");
    *h->sync_err_host = 0;
    return LGCA_OK;
}

// Wait for the handle's stream, then report a persistent-kernel timeout that
// has not been cleared: the state the stream produced is then not the state
// of the handle's step counter.
int synced(lgca_lattice *h)
{
    const cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamSynchronize");
    if (h->sync_err_host && *h->sync_err_host)
        return fail(h, LGCA_ERR_TIMEOUT,
                    "a neighbour wait of the persistent kernel timed out; the state is partly "
                    "stepped until lgca_clear_error and a new state");
    return LGCA_OK;
}

#define SYNC(h)                                        \
    do {                                               \
        if (const int s_ = synced(h)) return s_;       \
    } while (0)

// Called before the handle's stream is used: the stream waits for the batch
// steps queued for the lattice (once per batch call), and is marked used.
int enter(lgca_lattice *h)
{
    if (h->after_batch) {
        const cudaError_t e = cudaStreamWaitEvent(h->stream, h->batch_done, 0);
        if (e != cudaSuccess) return cuda_fail(h, e, "cudaStreamWaitEvent (batch)");
        h->after_batch = false;
    }
    h->used = true;
    return LGCA_OK;
}

// Entry points that queue work on, or wait for, the handle's stream.
#define CHECK_HANDLE(h)                                                          \
    do {                                                                         \
        if (!valid(h)) return fail(nullptr, LGCA_ERR_INVALID, "invalid handle"); \
        if (const int st_ = enter(h)) return st_;                                \
    } while (0)

// Entry points that only read or set host-side fields.
#define CHECK_VALID(h)                                                           \
    do {                                                                         \
        if (!valid(h)) return fail(nullptr, LGCA_ERR_INVALID, "invalid handle"); \
    } while (0)

}  // namespace

namespace lgca_gpu {
// Error message for lgca_last_error(NULL) from entry points without a handle.
void record_error(const char *msg) { g_err = msg; }
}  // namespace lgca_gpu

extern "C" {

int lgca_abi_version(void) { return LGCA_GPU_ABI_VERSION; }

const char *lgca_status_string(int status)
{
    switch (status) {
    case LGCA_OK: return "ok";
    case LGCA_ERR_INVALID: return "invalid argument";
    case LGCA_ERR_NOMEM: return "out of device memory";
    case LGCA_ERR_CUDA: return "CUDA error";
    case LGCA_ERR_TIMEOUT: return "device wait timed out";
    case LGCA_ERR_BUSY: return "busy";
    default: return "unknown status";
    }
}

const char *lgca_last_error(lgca_handle h) { return h ? h->err.c_str() : g_err.c_str(); }

int lgca_create(int model, int W, int H, uint64_t seed, lgca_handle *out)
{
    if (!out) return fail(nullptr, LGCA_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (model < LGCA_HPP || model > LGCA_FHP_III)
        return fail(nullptr, LGCA_ERR_INVALID, "unknown model %d", model);
    if (W < 1 || H < 1) return fail(nullptr, LGCA_ERR_INVALID, "invalid dimensions %d x %d", W, H);
    if (model != LGCA_HPP && (H % 2) != 0)
        return fail(nullptr, LGCA_ERR_INVALID,
                    "FHP lattices need an even number of rows (dim_y = %d)", H);
    if ((unsigned long long)W * (unsigned long long)H > 0x7fffffffULL)
        return fail(nullptr, LGCA_ERR_INVALID, "lattice of %d x %d exceeds 2^31-1 cells", W, H);

    lgca_lattice *h = new (std::nothrow) lgca_lattice();
    if (!h) return fail(nullptr, LGCA_ERR_NOMEM, "host allocation failed");
    h->model = model;
    h->D = num_dir(model);
    h->seed = seed;
    PlaneGeom &g = h->g;
    set_plane_geom(g, W, H);
    cudaGetDevice(&h->device);

    cudaError_t e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        int st = cuda_fail(nullptr, e, "cudaStreamCreate");
        delete h;
        return st;
    }
    h->stream = h->own_stream;
    const size_t state_bytes = (size_t)h->D * g.ps * sizeof(uint64_t);
    int st = LGCA_OK;
    for (int i = 0; i < 2 && st == LGCA_OK; ++i)
        st = dalloc(h, reinterpret_cast<void **>(&h->buf[i]), state_bytes, true, "state buffer");
    // No wait here: the allocations and their zeroing are queued on the
    // handle's stream like all of its work.  Every call of this library uses
    // that stream, a batch orders its first call on a new member after the
    // member's queued work, lgca_set_stream synchronises first, and callers
    // order on lgca_stream.  (A wait here would stall admissions while a
    // persistent batch launch holds the SMs.)
    if (st != LGCA_OK) {
        dfree(h, h->buf[0]);
        dfree(h, h->buf[1]);
        cudaStreamSynchronize(h->stream);
        cudaStreamDestroy(h->own_stream);
        delete h;
        return st;
    }
    *out = h;
    return LGCA_OK;
}

int lgca_destroy(lgca_handle h)
{
    if (!h) return LGCA_OK;
    DeviceGuard dg(h->device);
    // the batch must not keep a dangling member; leaving orders the frees
    // below after the lattice's queued batch steps (a failed wait: a full
    // device sync instead)
    if (h->batch && lgca_batch_remove(h->batch, h) != LGCA_OK) cudaDeviceSynchronize();
    // memory goes back to the pool in stream order, after the handle's queued
    // work (batch steps of a member are ordered before it); no host wait
    void *mem[] = {h->buf[0], h->buf[1], h->solid, h->slip, h->chir, h->scratch, h->sync, h->bf,
                   h->res};
    for (void *p : mem) dfree(h, p);
    if (h->sync_err_host) {
        cudaStreamSynchronize(h->stream);
        cudaFreeHost(h->sync_err_host);
    }
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    delete h;
    return LGCA_OK;
}

int lgca_trim_memory(int device, uint64_t keep_bytes)
{
    cudaMemPool_t pool;
    cudaError_t e = lattice_pool(device, &pool);
    if (e == cudaSuccess) e = cudaMemPoolTrimTo(pool, (size_t)keep_bytes);
    return e == cudaSuccess ? LGCA_OK : cuda_fail(nullptr, e, "cudaMemPoolTrimTo");
}

int lgca_info(lgca_handle h, int *model, int *W, int *H, uint64_t *seed, uint64_t *step)
{
    CHECK_VALID(h);
    if (model) *model = h->model;
    if (W) *W = h->g.W;
    if (H) *H = h->g.H;
    if (seed) *seed = h->seed;
    if (step) *step = h->t;
    return LGCA_OK;
}

int lgca_set_step(lgca_handle h, uint64_t t)
{
    CHECK_VALID(h);
    h->t = t;
    return LGCA_OK;
}

int lgca_set_cell_types(lgca_handle h, const int32_t *types)
{
    CHECK_HANDLE(h);
    if (!types) return fail(h, LGCA_ERR_INVALID, "types is NULL");
    DeviceGuard dg(h->device);
    const PlaneGeom &g = h->g;
    const size_t n = (size_t)g.W * g.H;
    // scan on the host first: it decides which planes exist, and rejects
    // invalid values before anything changes
    bool any_noslip = false, any_slip = false;
    for (size_t i = 0; i < n; ++i) {
        const int32_t t = types[i];
        if (t < 0 || t > 2) return fail(h, LGCA_ERR_INVALID, "invalid cell type %d at cell %zu", t, i);
        any_noslip |= (t == 1);
        any_slip |= (t == 2);
    }
    {
        int gst = geometry_planes(h);
        if (gst) return gst;
    }
    int st = scratch_reserve(h, n * sizeof(int32_t) + 256);
    if (st) return st;
    int *bad = reinterpret_cast<int *>(static_cast<char *>(h->scratch) + n * sizeof(int32_t));
    CK(h, cudaMemcpyAsync(h->scratch, types, n * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemsetAsync(bad, 0, sizeof(int), h->stream));
    CK(h, launch_types_to_planes(g, static_cast<const int32_t *>(h->scratch), h->solid, h->slip, bad,
                                 h->stream));
    SYNC(h);
    h->has_noslip = any_noslip;
    h->has_slip = any_slip;
    return LGCA_OK;
}

int lgca_paint_cells(lgca_handle h, int shape, int32_t type, int64_t a, int64_t b, int64_t c,
                     int64_t d)
{
    CHECK_HANDLE(h);
    if (shape < LGCA_SHAPE_RECT || shape > LGCA_SHAPE_DISC_FLOAT)
        return fail(h, LGCA_ERR_INVALID, "unknown shape %d", shape);
    if (type < LGCA_FLUID || type > LGCA_SOLID_SLIP)
        return fail(h, LGCA_ERR_INVALID, "invalid cell type %d", type);
    const int64_t lim = 1ll << 29;
    if (a <= -lim || a >= lim || b <= -lim || b >= lim || c <= -lim || c >= lim || d <= -lim ||
        d >= lim || (shape != LGCA_SHAPE_RECT && c < 0))
        return fail(h, LGCA_ERR_INVALID, "shape parameters out of range");
    DeviceGuard dg(h->device);
    if (!h->solid) {
        if (type == LGCA_FLUID) return LGCA_OK;  // no geometry planes yet: all cells are fluid
        int gst = geometry_planes(h);
        if (gst) return gst;
    }
    CK(h, launch_paint(h->g, h->solid, h->slip, shape, type, a, b, c, d, h->stream));
    h->has_noslip |= (type == LGCA_SOLID_NO_SLIP);
    h->has_slip |= (type == LGCA_SOLID_SLIP);
    return LGCA_OK;
}

int lgca_get_cell_types(lgca_handle h, int32_t *types)
{
    CHECK_HANDLE(h);
    if (!types) return fail(h, LGCA_ERR_INVALID, "types is NULL");
    DeviceGuard dg(h->device);
    const size_t n = (size_t)h->g.W * h->g.H;
    if (!h->solid) {
        memset(types, 0, n * sizeof(int32_t));
        return LGCA_OK;
    }
    int st = scratch_reserve(h, n * sizeof(int32_t));
    if (st) return st;
    CK(h, launch_planes_to_types(h->g, h->solid, h->slip, static_cast<int32_t *>(h->scratch), h->stream));
    CK(h, cudaMemcpyAsync(types, h->scratch, n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    SYNC(h);
    return LGCA_OK;
}

int lgca_upload_state(lgca_handle h, const uint8_t *cells)
{
    CHECK_HANDLE(h);
    if (!cells) return fail(h, LGCA_ERR_INVALID, "cells is NULL");
    DeviceGuard dg(h->device);
    const size_t n = (size_t)h->g.W * h->g.H;
    int st = scratch_reserve(h, n + 64);
    if (st) return st;
    CK(h, cudaMemcpyAsync(h->scratch, cells, n, cudaMemcpyHostToDevice, h->stream));
    CK(h, launch_aos_to_planes(h->D, h->g, static_cast<const uint8_t *>(h->scratch), h->buf[h->cur],
                               h->stream));
    return LGCA_OK;
}

int lgca_download_state(lgca_handle h, uint8_t *cells)
{
    CHECK_HANDLE(h);
    if (!cells) return fail(h, LGCA_ERR_INVALID, "cells is NULL");
    DeviceGuard dg(h->device);
    const size_t n = (size_t)h->g.W * h->g.H;
    int st = scratch_reserve(h, n + 64);
    if (st) return st;
    CK(h, launch_planes_to_aos(h->D, h->g, h->buf[h->cur], static_cast<uint8_t *>(h->scratch),
                               h->stream));
    CK(h, cudaMemcpyAsync(cells, h->scratch, n, cudaMemcpyDeviceToHost, h->stream));
    SYNC(h);
    return LGCA_OK;
}

int lgca_download_state_async(lgca_handle h, uint8_t *cells)
{
    CHECK_HANDLE(h);
    if (!cells) return fail(h, LGCA_ERR_INVALID, "cells is NULL");
    DeviceGuard dg(h->device);
    const size_t n = (size_t)h->g.W * h->g.H;
    int st = scratch_reserve(h, n + 64);
    if (st) return st;
    CK(h, launch_planes_to_aos(h->D, h->g, h->buf[h->cur], static_cast<uint8_t *>(h->scratch),
                               h->stream));
    CK(h, cudaMemcpyAsync(cells, h->scratch, n, cudaMemcpyDeviceToHost, h->stream));
    return LGCA_OK;
}

int lgca_init_random(lgca_handle h, double p_move, double p_rest)
{
    CHECK_HANDLE(h);
    if (!(p_move >= 0.0 && p_move <= 1.0) || !(p_rest >= 0.0 && p_rest <= 1.0))
        return fail(h, LGCA_ERR_INVALID, "probabilities must lie in [0, 1]");
    DeviceGuard dg(h->device);
    CK(h, launch_init_random(h->D, h->g, h->has_noslip ? h->solid : nullptr,
                             h->has_slip ? h->slip : nullptr, h->buf[h->cur], h->seed,
                             lgca_prob_threshold(p_move), lgca_prob_threshold(p_rest), h->stream));
    return LGCA_OK;
}

int lgca_init_zero(lgca_handle h)
{
    CHECK_HANDLE(h);
    DeviceGuard dg(h->device);
    CK(h, cudaMemsetAsync(h->buf[h->cur], 0, (size_t)h->D * h->g.ps * sizeof(uint64_t), h->stream));
    return LGCA_OK;
}

int lgca_set_forcing_column(lgca_handle h, int x, double p)
{
    CHECK_VALID(h);
    if (x >= h->g.W) return fail(h, LGCA_ERR_INVALID, "forcing column %d outside 0..%d", x, h->g.W - 1);
    if (!(p >= 0.0 && p <= 1.0)) return fail(h, LGCA_ERR_INVALID, "probability must lie in [0, 1]");
    if (x < 0 || p <= 0.0) {
        h->force_x = -1;
        h->force_thr = 0;
    } else {
        h->force_x = x;
        h->force_thr = lgca_prob_threshold(p);
    }
    return LGCA_OK;
}

int lgca_set_chirality(lgca_handle h, const uint8_t *field)
{
    CHECK_HANDLE(h);
    DeviceGuard dg(h->device);
    if (!field) {
        h->frozen = false;
        return LGCA_OK;
    }
    const size_t n = (size_t)h->g.W * h->g.H;
    if (!h->chir) {
        int cst = dalloc(h, reinterpret_cast<void **>(&h->chir), h->g.ps * sizeof(uint64_t), true,
                         "chirality plane");
        if (cst) return cst;
    }
    int st = scratch_reserve(h, n + 64);
    if (st) return st;
    CK(h, cudaMemcpyAsync(h->scratch, field, n, cudaMemcpyHostToDevice, h->stream));
    CK(h, launch_bytes_to_plane(h->g, static_cast<const uint8_t *>(h->scratch), h->chir, h->stream));
    h->frozen = true;
    return LGCA_OK;
}

int lgca_set_temporal_depth(lgca_handle h, int depth)
{
    CHECK_VALID(h);
    if (depth < 1 || depth > 8) return fail(h, LGCA_ERR_INVALID, "depth %d outside 1..8", depth);
    h->depth = depth;
    return LGCA_OK;
}

int lgca_set_kernel_variant(lgca_handle h, int variant)
{
    CHECK_VALID(h);
    if (variant < VARIANT_AUTO || variant > VARIANT_RESIDENT)
        return fail(h, LGCA_ERR_INVALID, "unknown kernel variant %d", variant);
    h->variant = variant;
    return LGCA_OK;
}

int lgca_set_block_warps(lgca_handle h, int warps)
{
    CHECK_VALID(h);
    if (!(warps == 0 || warps == 1 || warps == 2 || warps == 4 || warps == 8))
        return fail(h, LGCA_ERR_INVALID, "warps per block must be 0, 1, 2, 4 or 8");
    h->bw = warps;
    return LGCA_OK;
}

}  // extern "C"

namespace {
// Which kernel family a call of nsteps steps runs (the resident form, the
// persistent band form, or the per-pass loop); shared by the call itself
// and lgca_step_plan.
int step_family(const lgca_lattice *h, int nsteps, ResidentShape *rs)
{
    if (h->variant == VARIANT_PERSIST && nsteps > 1) return VARIANT_PERSIST;
    // the resident form: asked for, or chosen for calls of enough steps to
    // repay its launch on lattices it holds that are large enough.  Measured
    // on GB300 (FHP-III, us per step, chained one-step launches / resident):
    //   2048 x 1024, 16 steps per call: 2.05 / 2.45; 100 steps: 2.05 / 2.09
    //   2048 x 2048, 16 steps: 3.96 / 3.06
    //   4096 x 256, 16 steps: 1.84 / 2.28; 100 steps: 1.86 / 1.77
    //   4096 x 512, 16 steps: 2.14 / 2.29; 100 steps: 2.06 / 1.77
    // so: 16+ steps from 4 Mi sites on rows of 2048+ sites (at least half of
    // every warp's lanes busy); 64+ steps from 1 Mi sites when the rows fill
    // whole warps (4096+ sites)
    ResidentShape tmp;
    ResidentShape &shape = rs ? *rs : tmp;
    if (nsteps <= 0 || nsteps > RESIDENT_MAX_STEPS || !resident_shape(h->model, h->g, shape))
        return VARIANT_PLAIN;
    // not into CUDA graphs: a resident call always leaves its result in the
    // other buffer and tags its halo items with the call's epoch, so a
    // replayed capture would neither chain (as an even number of one-step
    // launches does) nor start from clean halo slots
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(h->stream, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
        return VARIANT_PLAIN;
    if (h->variant == VARIANT_RESIDENT) return VARIANT_RESIDENT;
    // (np = pairs per row: lanes busy in a row's warps)
    const long long sites = (long long)h->g.W * h->g.H;
    const int np = h->g.nw / 2;
    if (h->variant == VARIANT_AUTO && h->depth == 1 &&
        ((nsteps >= RESIDENT_MIN_STEPS && sites >= RESIDENT_MIN_SITES && np >= 16) ||
         (nsteps >= RESIDENT_LONG_STEPS && sites >= RESIDENT_LONG_SITES && np >= 32)))
        return VARIANT_RESIDENT;
    return VARIANT_PLAIN;
}
// Steps per pass of the next pass of the per-pass loop, `left` steps to go.
int pass_depth(const lgca_lattice *h, int left)
{
    int k = std::min(h->depth, left);
    if (h->variant == VARIANT_AUTO && h->depth == 1) {
        // lattices far beyond L2, where one step per pass is bound by HBM,
        // take passes of several steps on the register wavefront (measured
        // on GB300: HPP from 64 Mi sites, 4 steps per pass, 1.45-2.4x;
        // FHP-I and FHP-II/III from 256 Mi sites, 4 and 2 steps, 1.34x and
        // 1.14x; smaller lattices run as fast or faster one step per pass)
        const long long sites = (long long)h->g.W * h->g.H;
        const int kauto = h->model == M_HPP     ? (sites >= (64LL << 20) ? 4 : 1)
                          : h->model == M_FHP_I ? (sites >= (256LL << 20) ? 4 : 1)
                                                : (sites >= (256LL << 20) ? 2 : 1);
        k = std::min(kauto, left);
    }
    const bool tile = h->variant == VARIANT_TILE;
    if (h->variant == VARIANT_PLAIN || h->variant == VARIANT_PLAIN2 ||
        h->variant == VARIANT_RESIDENT)
        k = 1;
    while (k > 1 && !(tile ? multistep_supported(h->model, h->g, k)
                           : wave_supported(h->model, h->g, k)))
        --k;
    return k;
}
// Step arguments of the handle (buffers and keys set by the caller).
StepArgs step_args(const lgca_lattice *h)
{
    StepArgs a;
    a.solid = h->solid;
    a.slip = h->slip;
    a.chir = h->frozen ? h->chir : nullptr;
    a.g = h->g;
    a.chunks = (h->g.nw + 31) / 32;
    a.force_thr = h->force_thr;
    a.fx = h->force_x;
    a.wpt = (h->variant == VARIANT_PLAIN) ? 1 : h->wpt;
    a.bw = h->bw;
    return a;
}
// nsteps steps on the resident kernel (shape rs); the input comes from the
// byte-per-cell device buffer aos_in when it is not null, and the result
// also goes to aos_out when that is not null.  RESIDENT_UNAVAILABLE when
// the device cannot hold the launch's blocks at once right now (e.g. a
// share of the SMs under MPS): nothing was stepped, and the caller takes
// one step per pass instead.
constexpr int RESIDENT_UNAVAILABLE = -1;
int run_resident(lgca_lattice *h, int nsteps, const ResidentShape &rs, const uint8_t *aos_in,
                 uint8_t *aos_out, const ResidentSums *sums = nullptr)
{
    if (const int fst = error_flag(h)) return fst;
    const size_t halo_bytes = rs.halo_words * sizeof(uint64_t);
    if (!h->res) {
        int st = dalloc(h, &h->res, halo_bytes, false, "resident halo");
        if (st) return st;
    }
    // items carry their launch's epoch and step: each launch takes the next
    // epoch, and the slots are zeroed once every 255 launches
    if (h->res_epoch == 0 || h->res_epoch >= 255) {
        CK(h, cudaMemsetAsync(h->res, 0, halo_bytes, h->stream));
        h->res_epoch = 1;
    } else {
        ++h->res_epoch;
    }
    StepArgs a = step_args(h);
    a.src = h->buf[h->cur];
    a.dst = h->buf[h->cur ^ 1];
    const PersistWait w{h->wait_ns, h->withhold};
    const cudaError_t e = launch_resident(h->model, geom_mode(h), a, rs,
                                          static_cast<uint64_t *>(h->res), h->sync, h->seed, h->t,
                                          nsteps, w, aos_in, aos_out, sums, h->res_epoch,
                                          h->stream);
    if (e == cudaErrorCooperativeLaunchTooLarge) {
        cudaGetLastError();  // (not sticky: the context stays usable)
        return RESIDENT_UNAVAILABLE;
    }
    CK(h, e);
    CK(h, cudaMemcpyAsync(h->sync_err_host, h->sync, sizeof(int), cudaMemcpyDeviceToHost,
                          h->stream));
    h->cur ^= 1;
    h->t += (uint64_t)nsteps;
    return LGCA_OK;
}
// The family and step-kernel launches of a call of nsteps steps on h.
void plan_counts(const lgca_lattice *h, int nsteps, int *family, int *launches)
{
    const int f = step_family(h, nsteps, nullptr);
    int n = 0;
    if (f == VARIANT_PLAIN) {
        for (int done = 0; done < nsteps; ++n) {
            const int k = pass_depth(h, nsteps - done);
            done += k;
        }
    } else {
        n = 1;
    }
    if (family) *family = f == VARIANT_PLAIN ? 1 : f;
    if (launches) *launches = n;
}
}  // namespace

extern "C" {

int lgca_step_plan(lgca_handle h, int nsteps, int *family, int *launches)
{
    CHECK_VALID(h);
    if (nsteps < 0) return fail(h, LGCA_ERR_INVALID, "nsteps < 0");
    DeviceGuard dg(h->device);
    plan_counts(h, nsteps, family, launches);
    return LGCA_OK;
}

int lgca_plan_shape(int model, int W, int H, int nsteps, int *family, int *launches)
{
    if (model < LGCA_HPP || model > LGCA_FHP_III)
        return fail(nullptr, LGCA_ERR_INVALID, "unknown model %d", model);
    if (W < 1 || H < 1) return fail(nullptr, LGCA_ERR_INVALID, "invalid dimensions %d x %d", W, H);
    if (model != LGCA_HPP && (H % 2) != 0)
        return fail(nullptr, LGCA_ERR_INVALID,
                    "FHP lattices need an even number of rows (dim_y = %d)", H);
    if ((unsigned long long)W * (unsigned long long)H > 0x7fffffffULL)
        return fail(nullptr, LGCA_ERR_INVALID, "lattice of %d x %d exceeds 2^31-1 cells", W, H);
    if (nsteps < 0) return fail(nullptr, LGCA_ERR_INVALID, "nsteps < 0");
    // a handle's default settings on the current device, with no memory
    lgca_lattice h;
    h.model = model;
    h.D = num_dir(model);
    set_plane_geom(h.g, W, H);
    if (cudaGetDevice(&h.device) != cudaSuccess) {
        cudaGetLastError();
        return fail(nullptr, LGCA_ERR_CUDA, "no CUDA device");
    }
    plan_counts(&h, nsteps, family, launches);
    return LGCA_OK;
}

int lgca_collide_and_propagate(lgca_handle h, int nsteps)
{
    CHECK_HANDLE(h);
    if (nsteps < 0) return fail(h, LGCA_ERR_INVALID, "nsteps < 0");
    DeviceGuard dg(h->device);
    StepArgs a = step_args(h);
    const int gm = geom_mode(h);
    ResidentShape rs;
    const int family = step_family(h, nsteps, &rs);
    if (family == VARIANT_PERSIST) {
        const size_t sync_bytes = (size_t)(PERSIST_MAX_BLOCKS + 1) * sizeof(int);
        if (const int fst = error_flag(h)) return fst;
        // step flags start at zero; the error flag keeps an earlier timeout
        CK(h, cudaMemsetAsync(h->sync + 1, 0, sync_bytes - sizeof(int), h->stream));
        const PersistWait w{h->wait_ns, h->withhold};
        CK(h, launch_persistent(h->model, gm, a, h->buf[h->cur], h->buf[h->cur ^ 1], h->seed, h->t,
                                nsteps, h->sync + 1, h->sync, PERSIST_MAX_BLOCKS, w, h->stream));
        CK(h, cudaMemcpyAsync(h->sync_err_host, h->sync, sizeof(int), cudaMemcpyDeviceToHost,
                              h->stream));
        if (nsteps & 1) h->cur ^= 1;
        h->t += (uint64_t)nsteps;
        return LGCA_OK;
    }
    if (family == VARIANT_RESIDENT) {
        const int st = run_resident(h, nsteps, rs, nullptr, nullptr);
        if (st != RESIDENT_UNAVAILABLE) return st;
    }
    int done = 0;
    while (done < nsteps) {
        // largest supported depth that fits, else one step per pass
        const int k = pass_depth(h, nsteps - done);
        const bool tile = h->variant == VARIANT_TILE;
        if (k > 1) {
            MultiStepArgs m;
            m.base = a;
            m.base.src = h->buf[h->cur];
            m.base.dst = h->buf[h->cur ^ 1];
            m.depth = k;
            for (int i = 0; i < k; ++i) {
                m.chir_keys[i] = lgca_rng_key(h->seed, LGCA_STREAM_CHIR, h->t + (uint64_t)i);
                m.force_keys[i] = lgca_rng_key(h->seed, LGCA_STREAM_FORCE, h->t + (uint64_t)i);
            }
            if (tile) CK(h, launch_multistep(h->model, gm, m, h->stream));
            else CK(h, launch_wave(h->model, gm, m, h->stream));
            h->cur ^= 1;
            h->t += (uint64_t)k;
            done += k;
            continue;
        }
        a.src = h->buf[h->cur];
        a.dst = h->buf[h->cur ^ 1];
        a.chir_key = lgca_rng_key(h->seed, LGCA_STREAM_CHIR, h->t);
        a.force_key = lgca_rng_key(h->seed, LGCA_STREAM_FORCE, h->t);
        CK(h, launch_step(h->model, gm, a, h->stream));
        h->cur ^= 1;
        h->t += 1;
        done += 1;
    }
    return LGCA_OK;
}

int lgca_collide_and_propagate_sums(lgca_handle h, int nsteps, int B, int32_t *N, int32_t *Jx2,
                                    int32_t *Jy)
{
    CHECK_HANDLE(h);
    if (nsteps < 0) return fail(h, LGCA_ERR_INVALID, "nsteps < 0");
    if (B < 1 || !N || !Jx2 || !Jy) return fail(h, LGCA_ERR_INVALID, "invalid block-sum arguments");
    DeviceGuard dg(h->device);
    ResidentShape rs;
    if (step_family(h, nsteps, &rs) == VARIANT_RESIDENT && resident_sums_fit(h->model, h->g, rs, B)) {
        // the sums fused into the step launch: its blocks add into zeroed arrays
        const size_t nb = (size_t)((h->g.W + B - 1) / B) * ((h->g.H + B - 1) / B);
        if (Jx2 == N + nb && Jy == Jx2 + nb)  // one array of three planes: one memset
            CK(h, cudaMemsetAsync(N, 0, 3 * nb * sizeof(int32_t), h->stream));
        else
            for (int32_t *p : {N, Jx2, Jy}) CK(h, cudaMemsetAsync(p, 0, nb * sizeof(int32_t), h->stream));
        const ResidentSums sums{B, N, Jx2, Jy};
        const int st = run_resident(h, nsteps, rs, nullptr, nullptr, &sums);
        if (st != RESIDENT_UNAVAILABLE) return st;
    }
    if (const int st = lgca_collide_and_propagate(h, nsteps)) return st;
    return lgca_block_sums_device(h, B, N, Jx2, Jy);
}

int lgca_run_job_async(lgca_handle h, const uint8_t *cells_in, int nsteps, uint8_t *cells_out,
                       int B, int32_t *N, int32_t *Jx2, int32_t *Jy)
{
    CHECK_HANDLE(h);
    if (nsteps < 0) return fail(h, LGCA_ERR_INVALID, "nsteps < 0");
    if (B < 0 || (B > 0 && (!N || !Jx2 || !Jy)))
        return fail(h, LGCA_ERR_INVALID, "invalid block-sum arguments");
    DeviceGuard dg(h->device);
    ResidentShape rs;
    if (step_family(h, nsteps, &rs) == VARIANT_RESIDENT && (cells_in || cells_out || B > 0)) {
        // one launch converts the input, steps, converts the result and (for
        // B in 8, 16, 32, 64) adds up the block sums: the byte-per-cell
        // buffer is read and rewritten row by row by the warp that owns the
        // row, so input and output share it; the sums follow it in scratch
        const size_t n = (size_t)h->g.W * h->g.H, aos_bytes = (n + 255) & ~(size_t)255;
        const size_t nb = B > 0 ? (size_t)((h->g.W + B - 1) / B) * ((h->g.H + B - 1) / B) : 0;
        int st = scratch_reserve(h, aos_bytes + 3 * nb * sizeof(int32_t) + 64);
        if (st) return st;
        uint8_t *aos = static_cast<uint8_t *>(h->scratch);
        int32_t *d = reinterpret_cast<int32_t *>(aos + aos_bytes);
        const bool fused = B > 0 && resident_sums_fit(h->model, h->g, rs, B);
        if (fused) CK(h, cudaMemsetAsync(d, 0, 3 * nb * sizeof(int32_t), h->stream));
        if (cells_in) CK(h, cudaMemcpyAsync(aos, cells_in, n, cudaMemcpyHostToDevice, h->stream));
        const ResidentSums sums{B, d, d + nb, d + 2 * nb};
        st = run_resident(h, nsteps, rs, cells_in ? aos : nullptr, cells_out ? aos : nullptr,
                          fused ? &sums : nullptr);
        if (st == RESIDENT_UNAVAILABLE) {  // the copied input converted here, then the plain path
            if (cells_in)
                CK(h, launch_aos_to_planes(h->D, h->g, aos, h->buf[h->cur], h->stream));
            if ((st = lgca_collide_and_propagate(h, nsteps))) return st;
            if (cells_out && (st = lgca_download_state_async(h, cells_out))) return st;
            return B > 0 ? lgca_block_sums_async(h, B, N, Jx2, Jy) : LGCA_OK;
        }
        if (st) return st;
        if (cells_out) CK(h, cudaMemcpyAsync(cells_out, aos, n, cudaMemcpyDeviceToHost, h->stream));
        if (B > 0) {
            if (!fused)
                CK(h, launch_block_sums(h->model, h->g, h->buf[h->cur], B, d, d + nb, d + 2 * nb,
                                        h->stream));
            CK(h, cudaMemcpyAsync(N, d, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
            CK(h, cudaMemcpyAsync(Jx2, d + nb, nb * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                  h->stream));
            CK(h, cudaMemcpyAsync(Jy, d + 2 * nb, nb * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                  h->stream));
        }
        return LGCA_OK;
    }
    if (cells_in) {
        if (const int st = lgca_upload_state(h, cells_in)) return st;
    }
    if (const int st = lgca_collide_and_propagate(h, nsteps)) return st;
    if (cells_out) {
        if (const int st = lgca_download_state_async(h, cells_out)) return st;
    }
    return B > 0 ? lgca_block_sums_async(h, B, N, Jx2, Jy) : LGCA_OK;
}

int lgca_apply_body_force(lgca_handle h, int forcing, int bf_dir, uint64_t *reverted)
{
    CHECK_HANDLE(h);
    if (!(bf_dir == 'x' || bf_dir == 'y' || bf_dir == 0))
        return fail(h, LGCA_ERR_INVALID, "bf_dir must be 'x', 'y' or 0");
    DeviceGuard dg(h->device);
    const size_t n = (size_t)h->g.W * h->g.H;
    const size_t work = body_force_scratch_bytes(n);
    if (const int fst = error_flag(h)) return fst;
    if (!h->bf) {  // zeroed: the table's clean mark says "not clean" until the first call
        int st = dalloc(h, &h->bf, work + 2 * BODY_FORCE_STICKY_BYTES, true, "body-force table");
        if (st) return st;
    }
    char *sticky = static_cast<char *>(h->bf) + work;
    unsigned long long *rev =
        reinterpret_cast<unsigned long long *>(sticky + BODY_FORCE_STICKY_BYTES);
    const uint64_t key = lgca_rng_key(h->seed, LGCA_STREAM_FSEQ, h->fcall);
    CK(h, launch_body_force(h->model, h->g, h->buf[h->cur], h->has_noslip ? h->solid : nullptr,
                            h->has_slip ? h->slip : nullptr, key, forcing, bf_dir, h->bf, sticky,
                            rev, h->sync, h->stream));
    CK(h, cudaMemcpyAsync(h->sync_err_host, h->sync, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    h->fcall += 1;
    if (reverted) {
        unsigned long long v = 0;
        CK(h, cudaMemcpyAsync(&v, rev, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
        SYNC(h);
        *reverted = v;
    }
    return LGCA_OK;
}

int lgca_count_particles(lgca_handle h, uint64_t *n)
{
    CHECK_HANDLE(h);
    if (!n) return fail(h, LGCA_ERR_INVALID, "n is NULL");
    DeviceGuard dg(h->device);
    int st = scratch_reserve(h, 64);
    if (st) return st;
    unsigned long long *d = static_cast<unsigned long long *>(h->scratch);
    CK(h, cudaMemsetAsync(d, 0, sizeof(*d), h->stream));
    CK(h, launch_count(h->D, h->g, h->buf[h->cur], d, h->stream));
    unsigned long long v = 0;
    CK(h, cudaMemcpyAsync(&v, d, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    SYNC(h);
    *n = v;
    return LGCA_OK;
}

int lgca_mean_velocity(lgca_handle h, float *ux, float *uy)
{
    CHECK_HANDLE(h);
    if (!ux || !uy) return fail(h, LGCA_ERR_INVALID, "output is NULL");
    DeviceGuard dg(h->device);
    int st = scratch_reserve(h, 64);
    if (st) return st;
    double *ds = static_cast<double *>(h->scratch);
    unsigned long long *nf = reinterpret_cast<unsigned long long *>(ds + 2);
    CK(h, cudaMemsetAsync(ds, 0, 3 * sizeof(double), h->stream));
    CK(h, launch_mean_velocity(h->model, h->g, h->buf[h->cur], h->has_noslip ? h->solid : nullptr,
                               h->has_slip ? h->slip : nullptr, ds, nf, h->stream));
    struct { double s[2]; unsigned long long n; } v;
    CK(h, cudaMemcpyAsync(&v, ds, sizeof(v), cudaMemcpyDeviceToHost, h->stream));
    SYNC(h);
    *ux = (float)(v.s[0] / (double)v.n);
    *uy = (float)(v.s[1] / (double)v.n);
    return LGCA_OK;
}

int lgca_block_sums_device(lgca_handle h, int B, int32_t *N, int32_t *Jx2, int32_t *Jy)
{
    CHECK_HANDLE(h);
    if (B < 1 || !N || !Jx2 || !Jy) return fail(h, LGCA_ERR_INVALID, "invalid block-sum arguments");
    DeviceGuard dg(h->device);
    CK(h, launch_block_sums(h->model, h->g, h->buf[h->cur], B, N, Jx2, Jy, h->stream));
    return LGCA_OK;
}

int lgca_block_sums(lgca_handle h, int B, int32_t *N, int32_t *Jx2, int32_t *Jy)
{
    CHECK_HANDLE(h);
    if (B < 1 || !N || !Jx2 || !Jy) return fail(h, LGCA_ERR_INVALID, "invalid block-sum arguments");
    DeviceGuard dg(h->device);
    const size_t nb = (size_t)((h->g.W + B - 1) / B) * ((h->g.H + B - 1) / B);
    int st = scratch_reserve(h, 3 * nb * sizeof(int32_t));
    if (st) return st;
    int32_t *d = static_cast<int32_t *>(h->scratch);
    CK(h, launch_block_sums(h->model, h->g, h->buf[h->cur], B, d, d + nb, d + 2 * nb, h->stream));
    CK(h, cudaMemcpyAsync(N, d, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(Jx2, d + nb, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(Jy, d + 2 * nb, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    SYNC(h);
    return LGCA_OK;
}

int lgca_block_sums_async(lgca_handle h, int B, int32_t *N, int32_t *Jx2, int32_t *Jy)
{
    CHECK_HANDLE(h);
    if (B < 1 || !N || !Jx2 || !Jy) return fail(h, LGCA_ERR_INVALID, "invalid block-sum arguments");
    DeviceGuard dg(h->device);
    const size_t nb = (size_t)((h->g.W + B - 1) / B) * ((h->g.H + B - 1) / B);
    int st = scratch_reserve(h, 3 * nb * sizeof(int32_t));
    if (st) return st;
    int32_t *d = static_cast<int32_t *>(h->scratch);
    CK(h, launch_block_sums(h->model, h->g, h->buf[h->cur], B, d, d + nb, d + 2 * nb, h->stream));
    CK(h, cudaMemcpyAsync(N, d, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(Jx2, d + nb, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaMemcpyAsync(Jy, d + 2 * nb, nb * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
    return LGCA_OK;
}

int lgca_post_process(lgca_handle h, int r, float *cell_density, float *cell_momentum,
                      float *mean_density, float *mean_momentum)
{
    CHECK_HANDLE(h);
    if (r < 1) return fail(h, LGCA_ERR_INVALID, "coarse-graining radius must be >= 1");
    DeviceGuard dg(h->device);
    const size_t n = (size_t)h->g.W * h->g.H;
    const int Wc = h->g.W / (2 * r), Hc = h->g.H / (2 * r);
    const size_t nc = (size_t)std::max(Wc, 0) * (size_t)std::max(Hc, 0);
    const size_t cell_bytes = (cell_density ? n : 0) * 4 + (cell_momentum ? 2 * n : 0) * 4;
    const size_t mean_bytes = (mean_density ? nc : 0) * 4 + (mean_momentum ? 2 * nc : 0) * 4;
    int st = scratch_reserve(h, cell_bytes + mean_bytes + 512);
    if (st) return st;
    char *p = static_cast<char *>(h->scratch);
    float *dcd = cell_density ? reinterpret_cast<float *>(p) : nullptr;
    p += cell_density ? ((n * 4 + 127) & ~(size_t)127) : 0;
    float *dcm = cell_momentum ? reinterpret_cast<float *>(p) : nullptr;
    p += cell_momentum ? ((2 * n * 4 + 127) & ~(size_t)127) : 0;
    float *dmd = mean_density ? reinterpret_cast<float *>(p) : nullptr;
    p += mean_density ? ((nc * 4 + 127) & ~(size_t)127) : 0;
    float *dmm = mean_momentum ? reinterpret_cast<float *>(p) : nullptr;
    if (dcd || dcm) CK(h, launch_cell_post(h->model, h->g, h->buf[h->cur], dcd, dcm, h->stream));
    if ((dmd || dmm) && nc > 0)
        CK(h, launch_mean_post(h->model, h->g, h->buf[h->cur], r, dmd, dmm, h->stream));
    if (dcd) CK(h, cudaMemcpyAsync(cell_density, dcd, n * 4, cudaMemcpyDeviceToHost, h->stream));
    if (dcm) CK(h, cudaMemcpyAsync(cell_momentum, dcm, 2 * n * 4, cudaMemcpyDeviceToHost, h->stream));
    if (dmd && nc) CK(h, cudaMemcpyAsync(mean_density, dmd, nc * 4, cudaMemcpyDeviceToHost, h->stream));
    if (dmm && nc) CK(h, cudaMemcpyAsync(mean_momentum, dmm, 2 * nc * 4, cudaMemcpyDeviceToHost, h->stream));
    SYNC(h);
    return LGCA_OK;
}

int lgca_sync(lgca_handle h)
{
    CHECK_HANDLE(h);
    DeviceGuard dg(h->device);
    SYNC(h);
    return LGCA_OK;
}

int lgca_clear_error(lgca_handle h)
{
    CHECK_HANDLE(h);
    DeviceGuard dg(h->device);
    CK(h, cudaStreamSynchronize(h->stream));
    if (h->sync) {
        CK(h, cudaMemsetAsync(h->sync, 0, sizeof(int), h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    if (h->sync_err_host) *h->sync_err_host = 0;
    h->err.clear();
    return LGCA_OK;
}

int lgca_set_wait_limit(lgca_handle h, uint64_t wait_ns)
{
    CHECK_VALID(h);
    if (wait_ns < 1000ull || wait_ns > 60000000000ull)
        return fail(h, LGCA_ERR_INVALID, "wait limit %llu ns outside 1 us .. 60 s",
                    (unsigned long long)wait_ns);
    h->wait_ns = wait_ns;
    return LGCA_OK;
}

int lgca_test_withhold_progress(lgca_handle h, int block)
{
    CHECK_VALID(h);
    if (block < -1 || block >= PERSIST_MAX_BLOCKS)
        return fail(h, LGCA_ERR_INVALID, "block %d outside -1 .. %d", block, PERSIST_MAX_BLOCKS - 1);
    h->withhold = block;
    return LGCA_OK;
}

void *lgca_stream(lgca_handle h)
{
    // the caller queues work on the stream: order it after the lattice's
    // batch steps and before its next ones
    if (!valid(h) || enter(h) != LGCA_OK) return nullptr;
    return (void *)h->stream;
}

int lgca_set_stream(lgca_handle h, void *stream)
{
    CHECK_HANDLE(h);
    DeviceGuard dg(h->device);
    SYNC(h);
    h->stream = stream ? static_cast<cudaStream_t>(stream) : h->own_stream;
    return LGCA_OK;
}

int lgca_state_device(lgca_handle h, const uint64_t **planes, size_t *plane_stride, int *row_pitch)
{
    CHECK_HANDLE(h);
    if (planes) *planes = h->buf[h->cur];
    if (plane_stride) *plane_stride = h->g.ps;
    if (row_pitch) *row_pitch = h->g.pitch;
    return LGCA_OK;
}

// ---- checkpoint: header + packed planes (rows of nw words, no padding)
namespace {
struct CkptHeader {
    char magic[8];  // "LGCAGB01"
    int32_t model, dim_x, dim_y, flags;  // flags: 1 noslip, 2 slip, 4 frozen chirality
    uint64_t seed, step, fcall;
    int32_t force_x, depth;
    uint64_t force_thr;
    int32_t variant, wpt;
    uint64_t reserved[3];
};
static_assert(sizeof(CkptHeader) == 96, "checkpoint header layout");

size_t ckpt_planes(const lgca_lattice *h)
{
    return (size_t)h->D + (h->solid ? 2 : 0) + (h->frozen ? 1 : 0);
}
}  // namespace

int lgca_checkpoint_size(lgca_handle h, size_t *bytes)
{
    CHECK_VALID(h);
    if (!bytes) return fail(h, LGCA_ERR_INVALID, "bytes is NULL");
    const size_t plane = (size_t)h->g.H * h->g.nw * sizeof(uint64_t);
    *bytes = sizeof(CkptHeader) + ckpt_planes(h) * plane;
    return LGCA_OK;
}

int lgca_checkpoint_save(lgca_handle h, void *buf, size_t bytes)
{
    CHECK_HANDLE(h);
    size_t need = 0;
    lgca_checkpoint_size(h, &need);
    if (!buf || bytes < need) return fail(h, LGCA_ERR_INVALID, "checkpoint buffer of %zu bytes < %zu", bytes, need);
    DeviceGuard dg(h->device);
    CkptHeader hd;
    memset(&hd, 0, sizeof(hd));
    memcpy(hd.magic, "LGCAGB01", 8);
    hd.model = h->model;
    hd.dim_x = h->g.W;
    hd.dim_y = h->g.H;
    hd.flags = (h->solid && h->has_noslip ? 1 : 0) | (h->solid && h->has_slip ? 2 : 0) |
               (h->frozen ? 4 : 0) | (h->solid ? 8 : 0);
    hd.seed = h->seed;
    hd.step = h->t;
    hd.fcall = h->fcall;
    hd.force_x = h->force_x;
    hd.force_thr = h->force_thr;
    hd.depth = h->depth;
    hd.variant = h->variant;
    hd.wpt = h->wpt;
    memcpy(buf, &hd, sizeof(hd));
    char *out = static_cast<char *>(buf) + sizeof(hd);
    const size_t row = (size_t)h->g.nw * sizeof(uint64_t), pitch = (size_t)h->g.pitch * sizeof(uint64_t);
    const size_t plane = row * h->g.H;
    auto copy_plane = [&](const uint64_t *src) -> cudaError_t {
        cudaError_t e = cudaMemcpy2DAsync(out, row, src, pitch, row, h->g.H, cudaMemcpyDeviceToHost,
                                          h->stream);
        out += plane;
        return e;
    };
    for (int d = 0; d < h->D; ++d) CK(h, copy_plane(h->buf[h->cur] + (size_t)d * h->g.ps));
    if (h->solid) {
        CK(h, copy_plane(h->solid));
        CK(h, copy_plane(h->slip));
    }
    if (h->frozen) CK(h, copy_plane(h->chir));
    SYNC(h);
    return LGCA_OK;
}

int lgca_checkpoint_load(lgca_handle h, const void *buf, size_t bytes)
{
    CHECK_HANDLE(h);
    if (!buf || bytes < sizeof(CkptHeader)) return fail(h, LGCA_ERR_INVALID, "checkpoint too short");
    CkptHeader hd;
    memcpy(&hd, buf, sizeof(hd));
    if (memcmp(hd.magic, "LGCAGB01", 8) != 0) return fail(h, LGCA_ERR_INVALID, "not a checkpoint of this engine");
    if (hd.model != h->model || hd.dim_x != h->g.W || hd.dim_y != h->g.H)
        return fail(h, LGCA_ERR_INVALID, "checkpoint of model %d, %d x %d does not match the lattice",
                    hd.model, hd.dim_x, hd.dim_y);
    // the settings pass the same checks as their setters before anything changes
    if ((hd.flags & ~15) != 0) return fail(h, LGCA_ERR_INVALID, "checkpoint flags 0x%x invalid", hd.flags);
    if (hd.variant < VARIANT_AUTO || hd.variant > VARIANT_RESIDENT)
        return fail(h, LGCA_ERR_INVALID, "checkpoint kernel variant %d invalid", hd.variant);
    if (hd.wpt != 1 && hd.wpt != 2)
        return fail(h, LGCA_ERR_INVALID, "checkpoint words per lane %d invalid", hd.wpt);
    if (hd.depth < 1 || hd.depth > 8)
        return fail(h, LGCA_ERR_INVALID, "checkpoint temporal depth %d invalid", hd.depth);
    const bool no_force = hd.force_x == -1 && hd.force_thr == 0;
    const bool force_ok = hd.force_x >= 0 && hd.force_x < h->g.W && hd.force_thr >= 1 &&
                          hd.force_thr <= (1ull << 32);
    if (!no_force && !force_ok)
        return fail(h, LGCA_ERR_INVALID, "checkpoint forcing column %d / threshold %llu invalid",
                    hd.force_x, (unsigned long long)hd.force_thr);
    const bool has_geom = (hd.flags & 8) != 0, frozen = (hd.flags & 4) != 0;
    if (!has_geom && (hd.flags & 3))
        return fail(h, LGCA_ERR_INVALID, "checkpoint cell types without geometry planes");
    const size_t row = (size_t)h->g.nw * sizeof(uint64_t), pitch = (size_t)h->g.pitch * sizeof(uint64_t);
    const size_t plane = row * h->g.H;
    const size_t need = sizeof(CkptHeader) + ((size_t)h->D + (has_geom ? 2 : 0) + (frozen ? 1 : 0)) * plane;
    if (bytes < need) return fail(h, LGCA_ERR_INVALID, "checkpoint of %zu bytes < %zu", bytes, need);
    DeviceGuard dg(h->device);
    const size_t plane_bytes = h->g.ps * sizeof(uint64_t);
    if (has_geom && !h->solid) {
        int gst = geometry_planes(h);
        if (gst) return gst;
    }
    if (frozen && !h->chir) {
        int cst = dalloc(h, reinterpret_cast<void **>(&h->chir), plane_bytes, true, "chirality plane");
        if (cst) return cst;
    }
    const char *in = static_cast<const char *>(buf) + sizeof(CkptHeader);
    auto copy_plane = [&](uint64_t *dst) -> cudaError_t {
        cudaError_t e = cudaMemcpy2DAsync(dst, pitch, in, row, row, h->g.H, cudaMemcpyHostToDevice,
                                          h->stream);
        in += plane;
        return e;
    };
    for (int d = 0; d < h->D; ++d) CK(h, copy_plane(h->buf[h->cur] + (size_t)d * h->g.ps));
    if (has_geom) {
        CK(h, copy_plane(h->solid));
        CK(h, copy_plane(h->slip));
    }
    if (frozen) CK(h, copy_plane(h->chir));
    SYNC(h);
    h->has_noslip = has_geom && (hd.flags & 1);
    h->has_slip = has_geom && (hd.flags & 2);
    h->frozen = frozen;
    h->seed = hd.seed;
    h->t = hd.step;
    h->fcall = hd.fcall;
    h->force_x = hd.force_x;
    h->force_thr = hd.force_thr;
    h->depth = hd.depth;
    h->variant = hd.variant;
    h->wpt = hd.wpt;
    return LGCA_OK;
}

int lgca_device_bytes(lgca_handle h, size_t *bytes)
{
    CHECK_VALID(h);
    if (bytes) *bytes = h->bytes;
    return LGCA_OK;
}


// ------------------------------------------------------------------ batches
}  // extern "C"

namespace {
// One launch sequence of a batch call: the device work-list (entries, task
// prefix and block -> entry map in one allocation, the key table), its
// pinned staging and the device counter of graph replays.  Entries come in
// descending order of their sort key `nsteps` (units to run: steps or
// passes), so the entries active at unit u are a prefix of the list.
struct WorkList {
    BatchEntry *dE = nullptr;
    int *dP = nullptr, *dB = nullptr;  // dB points into dP's allocation
    uint64_t *dK = nullptr;
    size_t capE = 0, capB = 0, capK = 0;
    std::vector<BatchEntry> E;
    std::vector<int> P, Bl, nsteps;
    // pinned staging of the work-list, two slots used in turn; a slot is
    // rewritten once the copies out of it (two calls back) have run
    struct Staging {
        void *host = nullptr;
        size_t cap = 0;
        cudaEvent_t copied = nullptr;
    } stage[2];
    int slot = 0;
    int *base = nullptr;  // device: first unit of a graph replay
};
constexpr int WAVE_DEPTHS[3] = {2, 4, 8};
constexpr int WAVE_SLAB_ROWS = 64;  // output rows per wavefront warp task
}  // namespace

struct lgca_batch {
    std::vector<lgca_lattice *> members;
    // one per member: its stream's work before a call, recorded only when the
    // member's stream was used since it last stepped
    std::vector<cudaEvent_t> ev;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;  // end of the latest call; members' streams wait on it lazily
    int graph_steps = 32;        // steps captured per CUDA graph (0: no graphs)
    int warp_tasks = 0;          // warp tasks per warp of the batched kernel (0: per call)
    int call_wt = 1;             // the value used by the current call
    WorkList main;               // one step per launch (k_batch), all members' keys
    WorkList wave[3];            // passes of 2, 4, 8 steps (k_batch_wave)
    // persistent form of the one-step work (the default: on the 512-lattice
    // mix a step took 0.257 ms against 0.274 ms with one launch per step):
    // one cooperative launch per segment, grid barrier counter and error flag
    // (device), the flag's pinned copy read by lgca_batch_sync
    int persistent = 1;
    unsigned *pbar = nullptr;
    int *perr = nullptr, *perr_host = nullptr;
    std::string err;
};

namespace {

int bfail(lgca_batch *b, int status, const char *msg)
{
    g_err = msg;
    if (b) b->err = msg;
    return status;
}

int bcuda(lgca_batch *b, cudaError_t e, const char *what)
{
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return bfail(b, e == cudaErrorMemoryAllocation ? LGCA_ERR_NOMEM : LGCA_ERR_CUDA, buf);
}

#define BCK(b, expr)                                                \
    do {                                                            \
        cudaError_t e_ = (expr);                                    \
        if (e_ != cudaSuccess) return bcuda((b), e_, #expr);        \
    } while (0)

template <class T> int grow(lgca_batch *b, T *&p, size_t &cap, size_t n)
{
    if (cap >= n) return LGCA_OK;
    BCK(b, cudaStreamSynchronize(b->stream));  // queued steps still read the old list
    cudaFree(p);
    p = nullptr;
    cap = 0;
    BCK(b, cudaMalloc(&p, n * sizeof(T)));
    cap = n;
    return LGCA_OK;
}

void wl_clear(WorkList &w)
{
    w.E.clear();
    w.P.assign(1, 0);
    w.nsteps.clear();
}

// Append an entry with `own` warp tasks (padded to whole blocks of
// per_block) and sort key n, not larger than the previous entry's.
int wl_add(lgca_batch *b, WorkList &w, BatchEntry e, long long own, int n, int per_block)
{
    e.task0 = w.P.back();
    e.tasks = (int)std::min(own, 0x7fffffffLL);
    const long long tasks = (long long)w.P.back() + (own + per_block - 1) / per_block * per_block;
    if (tasks > 0x7fffffffLL) return bfail(b, LGCA_ERR_INVALID, "batch work-list too long");
    w.E.push_back(e);
    w.P.push_back((int)tasks);
    w.nsteps.push_back(n);
    return LGCA_OK;
}

// Block map, device arrays (and a key table of nkeys words, to which the
// entries' key offsets are rebased), and the copy through a pinned slot.
int wl_upload(lgca_batch *b, WorkList &w, int per_block, size_t nkeys)
{
    const int ne = (int)w.E.size();
    if (ne == 0) return LGCA_OK;
    const int nblocks = w.P.back() / per_block;  // every entry's tasks fill whole blocks
    w.Bl.resize(nblocks);
    for (int l = 0; l < ne; ++l)
        for (int blk = w.P[l] / per_block; blk < w.P[l + 1] / per_block; ++blk) w.Bl[blk] = l;
    int st;
    if ((st = grow(b, w.dE, w.capE, (size_t)ne)) != LGCA_OK) return st;
    if ((st = grow(b, w.dP, w.capB, (size_t)ne + 1 + nblocks)) != LGCA_OK) return st;
    if (nkeys) {
        if ((st = grow(b, w.dK, w.capK, nkeys)) != LGCA_OK) return st;
        for (auto &e : w.E) e.keys = w.dK + reinterpret_cast<size_t>(e.keys);
    }
    w.dB = w.dP + ne + 1;
    if (!w.base) BCK(b, cudaMalloc(&w.base, sizeof(int)));
    for (auto &sg : w.stage)
        if (!sg.copied) BCK(b, cudaEventCreateWithFlags(&sg.copied, cudaEventDisableTiming));
    // entries, then prefix and block map (contiguous on the device as on the host)
    auto &sg = w.stage[w.slot];
    w.slot ^= 1;
    BCK(b, cudaEventSynchronize(sg.copied));
    const size_t eb = (ne * sizeof(BatchEntry) + 15) & ~(size_t)15;
    const size_t ib = ((size_t)ne + 1 + nblocks) * sizeof(int);
    if (sg.cap < eb + ib) {
        if (sg.host) cudaFreeHost(sg.host);
        sg.host = nullptr;
        sg.cap = 0;
        BCK(b, cudaHostAlloc(&sg.host, 2 * (eb + ib), cudaHostAllocDefault));
        sg.cap = 2 * (eb + ib);
    }
    char *hp = static_cast<char *>(sg.host);
    memcpy(hp, w.E.data(), ne * sizeof(BatchEntry));
    memcpy(hp + eb, w.P.data(), (ne + 1) * sizeof(int));
    memcpy(hp + eb + (ne + 1) * sizeof(int), w.Bl.data(), nblocks * sizeof(int));
    BCK(b, cudaMemcpyAsync(w.dE, hp, ne * sizeof(BatchEntry), cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaMemcpyAsync(w.dP, hp + eb, ib, cudaMemcpyHostToDevice, b->stream));
    BCK(b, cudaEventRecord(sg.copied, b->stream));
    return LGCA_OK;
}

// The launch sequence of a list: units 0 .. max-1 in segments of constant
// active prefix; enqueue(k, tasks, n, u) queues n units u .. u + n - 1 over
// the first k entries (launches read their unit from *base + local index, and
// advance *base by n).  Segments of at least two graphs' worth of units
// replay a graph of `per_graph` units.
template <class Enqueue>
int wl_run(lgca_batch *b, WorkList &w, int per_graph, Enqueue enqueue)
{
    const int ne = (int)w.E.size();
    const int max_units = ne ? w.nsteps[0] : 0;
    int s0 = 0;
    while (s0 < max_units) {
        int k = 0;
        while (k < ne && w.nsteps[k] > s0) ++k;
        const int s1 = w.nsteps[k - 1], len = s1 - s0, tasks = w.P[k];
        BCK(b, launch_set_base(w.base, s0, b->stream));
        const int G = per_graph > 0 ? std::min(per_graph, len) : 0;
        int done = 0;
        if (G > 1 && len >= 2 * G) {
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
            const int st = enqueue(k, tasks, G, s0);
            cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
            if (st != LGCA_OK) {
                if (graph) cudaGraphDestroy(graph);
                return st;
            }
            BCK(b, e);
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            BCK(b, e);
            for (; done + G <= len; done += G) {
                e = cudaGraphLaunch(exec, b->stream);
                if (e != cudaSuccess) {
                    cudaGraphExecDestroy(exec);
                    return bcuda(b, e, "cudaGraphLaunch");
                }
            }
            cudaGraphExecDestroy(exec);  // released once its queued launches complete
        }
        if (done < len) {
            const int st = enqueue(k, tasks, len - done, s0 + done);
            if (st != LGCA_OK) return st;
        }
        s0 = s1;
    }
    return LGCA_OK;
}

// Device state of the persistent form, at first use.
int persist_state(lgca_batch *b)
{
    if (b->pbar) return LGCA_OK;
    BCK(b, cudaMalloc(&b->pbar, sizeof(unsigned) + sizeof(int)));
    b->perr = reinterpret_cast<int *>(b->pbar + 1);
    BCK(b, cudaMemsetAsync(b->pbar, 0, sizeof(unsigned) + sizeof(int), b->stream));
    BCK(b, cudaHostAlloc(&b->perr_host, sizeof(int), cudaHostAllocDefault));
    *b->perr_host = 0;
    return LGCA_OK;
}

void wl_free(WorkList &w)
{
    cudaFree(w.dE);
    cudaFree(w.dP);  // dB lives in the same allocation
    cudaFree(w.dK);
    cudaFree(w.base);
    for (auto &sg : w.stage) {
        if (sg.host) cudaFreeHost(sg.host);
        if (sg.copied) cudaEventDestroy(sg.copied);
    }
}

// Steps per pass of a member on the register wavefront, or 0: a member
// whose kernel variant is the wavefront and whose depth the wavefront
// supports for its model and width, when the call gives it a whole pass.
int wave_depth(const lgca_lattice *h, int nsteps)
{
    if (h->variant != VARIANT_WAVE || nsteps < h->depth) return 0;
    if (!(h->depth == 2 || h->depth == 4 || h->depth == 8)) return 0;
    return wave_supported(h->model, h->g, h->depth) ? h->depth : 0;
}

}  // namespace

extern "C" {

int lgca_batch_create(lgca_batch_handle *out)
{
    if (!out) return bfail(nullptr, LGCA_ERR_INVALID, "out is NULL");
    *out = nullptr;
    lgca_batch *b = new (std::nothrow) lgca_batch();
    if (!b) return bfail(nullptr, LGCA_ERR_NOMEM, "host allocation failed");
    cudaGetDevice(&b->device);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        int st = bcuda(nullptr, e, "lgca_batch_create");
        lgca_batch_destroy(b);
        return st;
    }
    *out = b;
    return LGCA_OK;
}

int lgca_batch_destroy(lgca_batch_handle b)
{
    if (!b) return LGCA_OK;
    DeviceGuard dg(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (lgca_lattice *m : b->members) {
        // the batch's steps are complete (synchronised above)
        m->batch = nullptr;
        m->batch_done = nullptr;
        m->after_batch = false;
    }
    for (cudaEvent_t e : b->ev) cudaEventDestroy(e);
    wl_free(b->main);
    for (auto &w : b->wave) wl_free(w);
    cudaFree(b->pbar);  // the error flag lives in the same allocation
    if (b->perr_host) cudaFreeHost(b->perr_host);
    if (b->done) cudaEventDestroy(b->done);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return LGCA_OK;
}

int lgca_batch_add(lgca_batch_handle b, lgca_handle h)
{
    if (!b) return bfail(nullptr, LGCA_ERR_INVALID, "invalid batch");
    if (!valid(h)) return bfail(b, LGCA_ERR_INVALID, "invalid lattice handle");
    if (h->device != b->device) return bfail(b, LGCA_ERR_INVALID, "lattice on another device");
    if (h->batch == b) return bfail(b, LGCA_ERR_INVALID, "lattice already in the batch");
    if (h->batch) return bfail(b, LGCA_ERR_INVALID, "lattice already in another batch");
    DeviceGuard dg(b->device);
    cudaEvent_t e;
    BCK(b, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    b->members.push_back(h);
    b->ev.push_back(e);
    h->batch = b;
    h->batch_done = b->done;
    h->after_batch = false;
    h->used = true;  // the first batch call waits for the lattice's queued work
    return LGCA_OK;
}

int lgca_batch_remove(lgca_batch_handle b, lgca_handle h)
{
    if (!b) return bfail(nullptr, LGCA_ERR_INVALID, "invalid batch");
    DeviceGuard dg(b->device);
    for (size_t i = 0; i < b->members.size(); ++i) {
        if (b->members[i] == h) {
            // the lattice's stream waits for its queued batch steps before it
            // leaves (its next work, or the frees of lgca_destroy, follow them)
            const cudaError_t e = h->after_batch ? cudaStreamWaitEvent(h->stream, b->done, 0)
                                                 : cudaSuccess;
            h->after_batch = false;
            h->batch_done = nullptr;
            cudaEventDestroy(b->ev[i]);
            h->batch = nullptr;
            b->members.erase(b->members.begin() + i);
            b->ev.erase(b->ev.begin() + i);
            if (e != cudaSuccess) return bcuda(b, e, "cudaStreamWaitEvent (leaving the batch)");
            return LGCA_OK;
        }
    }
    return bfail(b, LGCA_ERR_INVALID, "lattice not in the batch");
}

int lgca_batch_size(lgca_batch_handle b, int *n)
{
    if (!b || !n) return bfail(b, LGCA_ERR_INVALID, "invalid argument");
    *n = (int)b->members.size();
    return LGCA_OK;
}

int lgca_batch_set_warp_tasks(lgca_batch_handle b, int n)
{
    if (!b || !(n == 0 || n == 1 || n == 2 || n == 4 || n == 8))
        return bfail(b, LGCA_ERR_INVALID, "warp tasks must be 0, 1, 2, 4 or 8");
    b->warp_tasks = n;
    return LGCA_OK;
}

int lgca_batch_set_graph_steps(lgca_batch_handle b, int n)
{
    if (!b || n < 0) return bfail(b, LGCA_ERR_INVALID, "invalid argument");
    b->graph_steps = n;
    return LGCA_OK;
}

int lgca_batch_step_each(lgca_batch_handle b, const int *nsteps)
{
    if (!b) return bfail(nullptr, LGCA_ERR_INVALID, "invalid batch");
    if (!nsteps && !b->members.empty()) return bfail(b, LGCA_ERR_INVALID, "nsteps is NULL");
    DeviceGuard dg(b->device);
    const size_t nm = b->members.size();
    for (size_t i = 0; i < nm; ++i)
        if (nsteps[i] < 0) return bfail(b, LGCA_ERR_INVALID, "negative step count");
    // order after the work queued on a member's own stream since the last
    // call that stepped it; members with none cost no stream call (no host
    // wait either: the work-list copies below queue behind the previous call)
    for (size_t i = 0; i < nm; ++i) {
        lgca_lattice *h = b->members[i];
        if (nsteps[i] == 0 || !h->used) continue;
        BCK(b, cudaEventRecord(b->ev[i], h->stream));
        BCK(b, cudaStreamWaitEvent(b->stream, b->ev[i], 0));
        h->used = false;
    }
    // From here on steps may be queued.  If the call fails part way, the
    // members it covers still order their next use after what it queued
    // (their states are then unspecified, as after any failed call).
    struct OnFailure {
        lgca_batch *b;
        const int *nsteps;
        bool armed = true;
        ~OnFailure()
        {
            if (!armed) return;
            if (cudaEventRecord(b->done, b->stream) != cudaSuccess) cudaStreamSynchronize(b->stream);
            for (size_t i = 0; i < b->members.size(); ++i)
                if (nsteps[i] > 0) b->members[i]->after_batch = true;
        }
    } on_failure{b, nsteps};
    // Members on the register wavefront (kernel variant 2, depth K) run
    // nsteps % K single steps with the others, then nsteps / K passes of K
    // steps; the rest run every step one launch at a time.
    std::vector<int> K(nm, 0);
    for (size_t i = 0; i < nm; ++i) K[i] = nsteps[i] > 0 ? wave_depth(b->members[i], nsteps[i]) : 0;
    auto single_steps = [&](size_t i) { return K[i] ? nsteps[i] % K[i] : nsteps[i]; };
    // lane items per row of a member: word pairs where the width allows
    auto pair_of = [](const lgca_lattice *h) {
        return h->variant != VARIANT_PLAIN && h->wpt == 2 && (h->g.W % 64) == 0;
    };
    // warp tasks per warp: the caller's choice, else 2 once the call's
    // one-step work fills at least four waves of resident warps at 2 tasks per
    // warp (4 blocks of 8 warps per SM), 4 for calls 16 times larger; small
    // calls keep one task per warp for parallelism
    b->call_wt = b->warp_tasks;
    if (b->call_wt == 0) {
        long long all = 0;
        for (size_t i = 0; i < nm; ++i)
            if (single_steps(i) > 0) {
                const lgca_lattice *h = b->members[i];
                all += flat_tasks(h->g.H, pair_of(h) ? (h->g.nw + 1) / 2 : h->g.nw);
            }
        const long long wave = 32LL * sm_count();
        b->call_wt = all >= 128 * wave ? 4 : (all >= 8 * wave ? 2 : 1);
    }
    // kernel code of a member: family x geometry mode x lane path
    auto code_of = [&](const lgca_lattice *h) {
        const int fam = h->model == LGCA_HPP ? 0 : (h->model == LGCA_FHP_I ? 1 : 2);
        const int path = pair_of(h) ? ((h->g.nw & 1) ? 2 : 1) : 0;
        return fam * 9 + geom_mode(h) * 3 + path;
    };
    std::vector<int> code(nm);
    for (size_t i = 0; i < nm; ++i) code[i] = code_of(b->members[i]);
    auto entry_of = [&](size_t i) {
        const lgca_lattice *h = b->members[i];
        BatchEntry e;
        memset(&e, 0, sizeof(e));
        e.a.solid = h->solid;
        e.a.slip = h->slip;
        e.a.chir = h->frozen ? h->chir : nullptr;
        e.a.g = h->g;
        e.a.chunks = (h->g.nw + 31) / 32;
        e.a.force_thr = h->force_thr;
        e.a.fx = h->force_x;
        e.gm = geom_mode(h);
        e.code = code[i];
        e.buf0 = h->buf[h->cur];
        e.buf1 = h->buf[h->cur ^ 1];
        e.seed = h->seed;
        e.t0 = h->t;
        e.nsteps = nsteps[i];  // keys of all its steps in the call
        return e;
    };

    // ---- one-step work-list: members sorted by single steps (descending:
    // a segment's active members are a prefix), then by kernel code, so that
    // the blocks resident at one time mostly run one code path; it holds the
    // key table of every member stepping in the call
    std::vector<int> order(nm);
    for (size_t i = 0; i < nm; ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const int sx = single_steps(x), sy = single_steps(y);
        return sx != sy ? sx > sy : code[x] < code[y];
    });
    WorkList &M = b->main;
    wl_clear(M);
    const int per_block = 8 * b->call_wt;
    size_t nkeys = 0;
    std::vector<size_t> key_off(nm, 0);
    for (int i : order) {
        if (nsteps[i] == 0) continue;
        const lgca_lattice *h = b->members[i];
        BatchEntry e = entry_of(i);
        const bool pair = pair_of(h);
        e.a.wpt = pair ? 2 : 1;
        e.wpt = e.a.wpt;
        e.items = pair ? (h->g.nw + 1) / 2 : h->g.nw;  // lane items per row (last pair may be half)
        e.a.fmagic = flat_magic(h->g.H, e.items);
        key_off[i] = nkeys;
        e.keys = reinterpret_cast<uint64_t *>(nkeys);  // offset; rebased on upload
        nkeys += 2 * (size_t)nsteps[i];
        const int n1 = single_steps(i);
        const int st = wl_add(b, M, e, n1 > 0 ? flat_tasks(h->g.H, e.items) : 0, n1, per_block);
        if (st) return st;
    }
    if (!M.E.empty()) {
        int st = wl_upload(b, M, per_block, nkeys);
        if (st) return st;
        int max_steps = 0;
        for (const auto &e : M.E) max_steps = std::max(max_steps, e.nsteps);
        BCK(b, launch_batch_keys(M.dE, (int)M.E.size(), max_steps, b->stream));
    }
    // ---- wavefront work-lists, one per depth: members sorted by passes
    std::vector<int> worder[3];
    for (int i : order)
        for (int d = 0; d < 3; ++d)
            if (K[i] == WAVE_DEPTHS[d]) worder[d].push_back(i);
    for (int d = 0; d < 3; ++d) {
        WorkList &Wl = b->wave[d];
        wl_clear(Wl);
        const int Kd = WAVE_DEPTHS[d];
        std::stable_sort(worder[d].begin(), worder[d].end(), [&](int x, int y) {
            return nsteps[x] / Kd != nsteps[y] / Kd ? nsteps[x] / Kd > nsteps[y] / Kd : code[x] < code[y];
        });
        for (int i : worder[d]) {
            const lgca_lattice *h = b->members[i];
            BatchEntry e = entry_of(i);
            e.K = Kd;
            e.r = nsteps[i] % Kd;
            e.S = WAVE_SLAB_ROWS;
            e.nstrips = (h->g.nw + 29) / 30;
            e.keys = M.dK + key_off[i];
            const long long own = (long long)e.nstrips * ((h->g.H + e.S - 1) / e.S);
            const int st = wl_add(b, Wl, e, own, nsteps[i] / Kd, WAVE_BLOCK_WARPS);
            if (st) return st;
        }
        const int st = wl_upload(b, Wl, WAVE_BLOCK_WARPS, 0);
        if (st) return st;
    }

    // ---- launches: the single steps of every member, then the passes
    auto gmax_of = [](const WorkList &w, int k) {
        int g = GEOM_NONE;  // the active entries are the first k
        for (int i = 0; i < k; ++i) g = std::max(g, w.E[i].gm);
        return g;
    };
    if (b->persistent) {
        // one cooperative launch per segment, a grid barrier between steps
        if (const int st = persist_state(b)) return st;
        const int st = wl_run(b, M, 0, [&](int k, int tasks, int n, int u) -> int {
            BCK(b, cudaMemsetAsync(b->pbar, 0, sizeof(unsigned), b->stream));
            BCK(b, launch_batch_persist(M.dE, M.dB, tasks, u, n, b->pbar, b->perr, 2000000000ull,
                                        gmax_of(M, k), b->call_wt, b->stream));
            return LGCA_OK;
        });
        if (st) return st;
        BCK(b, cudaMemcpyAsync(b->perr_host, b->perr, sizeof(int), cudaMemcpyDeviceToHost,
                               b->stream));
    } else {
        const int st = wl_run(b, M, b->graph_steps, [&](int k, int tasks, int n, int) -> int {
            const int gmax = gmax_of(M, k);
            for (int s = 0; s < n; ++s)
                BCK(b, launch_batch(M.dE, M.dB, tasks, s, M.base, gmax, b->call_wt, b->stream));
            BCK(b, launch_advance(M.base, n, b->stream));
            return LGCA_OK;
        });
        if (st) return st;
    }
    for (int d = 0; d < 3; ++d) {
        WorkList &Wl = b->wave[d];
        const int Kd = WAVE_DEPTHS[d];
        const int per_graph = b->graph_steps > 0 ? std::max(1, b->graph_steps / Kd) : 0;
        const int st = wl_run(b, Wl, per_graph, [&](int k, int tasks, int n, int) -> int {
            const int gmax = gmax_of(Wl, k);
            for (int j = 0; j < n; ++j)
                BCK(b, launch_batch_wave(Wl.dE, Wl.dB, tasks, j, Wl.base, gmax, Kd, b->stream));
            BCK(b, launch_advance(Wl.base, n, b->stream));
            return LGCA_OK;
        });
        if (st) return st;
    }
    // members continue after the batch: each member's stream waits on `done`
    // at its next use (enter); `done` is recorded again by later calls, which
    // finish later on this stream, so a wait issued then still covers this call
    BCK(b, cudaEventRecord(b->done, b->stream));
    for (size_t i = 0; i < nm; ++i) {
        if (nsteps[i] == 0) continue;
        lgca_lattice *h = b->members[i];
        h->after_batch = true;
        // buffer swaps: one per single step and one per pass
        const int swaps = K[i] ? nsteps[i] % K[i] + nsteps[i] / K[i] : nsteps[i];
        if (swaps & 1) h->cur ^= 1;
        h->t += (uint64_t)nsteps[i];
    }
    on_failure.armed = false;
    return LGCA_OK;
}

int lgca_batch_step(lgca_batch_handle b, int nsteps)
{
    if (!b) return bfail(nullptr, LGCA_ERR_INVALID, "invalid batch");
    std::vector<int> n(b->members.size(), nsteps);
    return lgca_batch_step_each(b, n.data());
}

int lgca_batch_sync(lgca_batch_handle b)
{
    if (!b) return bfail(nullptr, LGCA_ERR_INVALID, "invalid batch");
    DeviceGuard dg(b->device);
    BCK(b, cudaStreamSynchronize(b->stream));
    if (b->perr_host && *b->perr_host) {
        // reported once; the device flag is cleared for the next calls
        *b->perr_host = 0;
        BCK(b, cudaMemsetAsync(b->perr, 0, sizeof(int), b->stream));
        BCK(b, cudaStreamSynchronize(b->stream));
        return bfail(b, LGCA_ERR_TIMEOUT,
                     "a grid barrier of the persistent batch kernel timed out; the members' states "
                     "are unspecified");
    }
    return LGCA_OK;
}

int lgca_batch_set_persistent(lgca_batch_handle b, int on)
{
    if (!b || !(on == 0 || on == 1)) return bfail(b, LGCA_ERR_INVALID, "persistent must be 0 or 1");
    b->persistent = on;
    return LGCA_OK;
}

const char *lgca_batch_last_error(lgca_batch_handle b) { return b ? b->err.c_str() : g_err.c_str(); }

void *lgca_batch_stream(lgca_batch_handle b) { return b ? (void *)b->stream : nullptr; }

}  // extern "C"
