// Allocation-free entry point: the random-cell body force on caller-owned
// device buffers, with its work arrays in a fixed device array of this file.
//
// Who needs it: a host program that keeps many lattices resident and has
// handed the whole device-memory budget to them (the serving loop's
// admission budget, or an embedding application with its own pool) cannot
// let a call take more device memory, and a cudaMalloc/cudaFree in the middle
// of a step sequence also synchronises the device, stalling the other
// lattices' work queued on other streams.  Such a caller passes its own state
// and geometry buffers and gets the reference body force
// (src/omp_lattice.cpp:254-346) without any allocation.
//
// The work arrays (first-occurrence table, per-block gains, running total)
// sit in g_bf_scratch below: LGCA_NOALLOC_MAX_CELLS * 4 bytes + 4 KiB, held
// by every GPU that loads the library until the process exits.  All calls
// share it and it keeps the last call's contents.  The running total starts
// from zero in every call; the table is left all ones by each call that
// completes, which a mark at the end of the array records, and a call that
// finds the mark missing (the first call, a call on a larger lattice than the
// last, or after a call that stopped early) clears the table first.  Calls
// whose work overlaps on the GPU (different streams, or different host
// threads) race on it and must be ordered by the caller.
//
// The device address of the array is looked up once per device and cached;
// it stays valid for the life of that device's CUDA context (a
// cudaDeviceReset ends it).
#include "internal.cuh"
#include "../../include/lgca_gpu.h"
#include "../../include/lgca/rng.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

namespace lgca_gpu {
void record_error(const char *msg);
}

using namespace lgca_gpu;

namespace {

constexpr unsigned long long kMaxCells = LGCA_NOALLOC_MAX_CELLS;
constexpr size_t kScratchBytes = (size_t)kMaxCells * 4 + 4096;
constexpr int kMaxDevices = 64;

// The fixed scratch.  In host code this name is only a stand-in for the
// device array: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_bf_scratch[kScratchBytes];

std::mutex g_mu;
void *g_addr[kMaxDevices] = {nullptr};

int fail(int status, const char *msg)
{
    record_error(msg);
    return status;
}

// Device address of g_bf_scratch on the current device, looked up once per
// device (the first call on a device does it).
int scratch_address(void **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(LGCA_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(LGCA_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_bf_scratch);
        if (e != cudaSuccess || p == nullptr) {
            char buf[256];
            snprintf(buf, sizeof(buf), "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
            return fail(LGCA_ERR_CUDA, buf);
        }
        g_addr[dev] = p;
    }
    *out = g_addr[dev];
    return LGCA_OK;
}

}  // namespace

extern "C" int lgca_apply_body_force_noalloc(int model, int dim_x, int dim_y, uint64_t *planes,
                                             size_t plane_stride, int row_pitch,
                                             const uint64_t *solid, const uint64_t *slip,
                                             uint64_t seed, uint64_t call, int forcing,
                                             int bf_dir, unsigned long long *reverted,
                                             void *stream)
{
    if (model < LGCA_HPP || model > LGCA_FHP_III) return fail(LGCA_ERR_INVALID, "unknown model");
    if (dim_x < 1 || dim_y < 1) return fail(LGCA_ERR_INVALID, "invalid dimensions");
    const unsigned long long ncells = (unsigned long long)dim_x * (unsigned long long)dim_y;
    if (ncells > kMaxCells) {
        char buf[160];
        snprintf(buf, sizeof(buf),
                 "lattice of %llu cells exceeds the allocation-free limit of %llu cells",
                 ncells, kMaxCells);
        return fail(LGCA_ERR_INVALID, buf);
    }
    const int nw = (dim_x + 63) / 64;
    if (!planes) return fail(LGCA_ERR_INVALID, "planes is NULL");
    if (row_pitch < nw) return fail(LGCA_ERR_INVALID, "row_pitch smaller than ceil(dim_x / 64)");
    if (plane_stride < (size_t)dim_y * (size_t)row_pitch)
        return fail(LGCA_ERR_INVALID, "plane_stride smaller than dim_y * row_pitch");
    if (!(bf_dir == 'x' || bf_dir == 'y' || bf_dir == 0))
        return fail(LGCA_ERR_INVALID, "bf_dir must be 'x', 'y' or 0");
    if (body_force_scratch_bytes((size_t)ncells) + 2 * BODY_FORCE_STICKY_BYTES > kScratchBytes)
        return fail(LGCA_ERR_INVALID, "scratch too small for this lattice");

    void *scratch = nullptr;
    int st = scratch_address(&scratch);
    if (st != LGCA_OK) return st;

    PlaneGeom g;
    g.W = dim_x;
    g.H = dim_y;
    g.nw = nw;
    g.pitch = row_pitch;
    g.ps = plane_stride;
    g.L = (dim_x - 1) & 63;
    g.lastmask = (g.L == 63) ? ~0ull : ((1ull << (g.L + 1)) - 1ull);
    // the end of the array: the table's clean mark, then the count when the
    // caller does not want it
    unsigned char *tail = static_cast<unsigned char *>(scratch) + kScratchBytes -
                          2 * BODY_FORCE_STICKY_BYTES;
    unsigned long long *rev =
        reverted ? reverted
                 : reinterpret_cast<unsigned long long *>(tail + BODY_FORCE_STICKY_BYTES);
    const uint64_t key = lgca_rng_key(seed, LGCA_STREAM_FSEQ, call);
    cudaError_t e = launch_body_force(model, g, planes, solid, slip, key, forcing, bf_dir, scratch,
                                      tail, rev, nullptr, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(LGCA_ERR_CUDA, cudaGetErrorString(e));
    return LGCA_OK;
}
