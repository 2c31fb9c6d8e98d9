// Kernels around the step: layout conversion, initialisation, cell-type
// planes, integer block sums, reference-arithmetic post-processing and
// reductions.  All work on the bit-plane layout described in internal.cuh.
#include "internal.cuh"
#include "../../include/lgca/rng.h"

#include <math.h>

// FULL and the block-sum kernels
#include "block_sums.cuh"

namespace lgca_gpu {

static inline unsigned grid_for(long long n, int threads)
{
    return (unsigned)((n + threads - 1) / threads);
}

// 8x8 bit-matrix transpose of a 64-bit word (H. S. Warren, "Hacker's
// Delight", 2nd ed., section 7-3): byte i bit j <-> byte j bit i.  Turns 8
// reference cells (byte = cell, bit = channel) into 8 channel bytes (byte =
// channel, bit = cell) and back.
__device__ __forceinline__ uint64_t transpose8(uint64_t x)
{
    x = (x & 0xAA55AA55AA55AA55ull) | ((x & 0x00AA00AA00AA00AAull) << 7) |
        ((x >> 7) & 0x00AA00AA00AA00AAull);
    x = (x & 0xCCCC3333CCCC3333ull) | ((x & 0x0000CCCC0000CCCCull) << 14) |
        ((x >> 14) & 0x0000CCCC0000CCCCull);
    x = (x & 0xF0F0F0F00F0F0F0Full) | ((x & 0x00000000F0F0F0F0ull) << 28) |
        ((x >> 28) & 0x00000000F0F0F0F0ull);
    return x;
}

// ------------------------------------------------------------------ layout
template <int D>
__global__ void k_aos_to_planes(PlaneGeom g, const uint8_t *__restrict__ aos,
                                uint64_t *__restrict__ planes)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.H * g.nw) return;
    const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
    const int x0 = 64 * w, n = min(64, g.W - x0);
    const uint8_t *row = aos + (size_t)y * g.W + x0;
    uint64_t out[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (n == 64 && ((reinterpret_cast<uintptr_t>(row) & 7) == 0)) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint64_t v = transpose8(*reinterpret_cast<const uint64_t *>(row + 8 * j));
#pragma unroll
            for (int d = 0; d < D; ++d) out[d] |= ((v >> (8 * d)) & 0xffull) << (8 * j);
        }
    } else {
        for (int i = 0; i < n; ++i) {
            const unsigned b = row[i];
#pragma unroll
            for (int d = 0; d < D; ++d) out[d] |= (uint64_t)((b >> d) & 1u) << i;
        }
    }
    const size_t o = (size_t)y * g.pitch + w;
#pragma unroll
    for (int d = 0; d < D; ++d) planes[(size_t)d * g.ps + o] = out[d];
}

template <int D>
__global__ void k_planes_to_aos(PlaneGeom g, const uint64_t *__restrict__ planes,
                                uint8_t *__restrict__ aos)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.H * g.nw) return;
    const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
    const int x0 = 64 * w, n = min(64, g.W - x0);
    uint8_t *row = aos + (size_t)y * g.W + x0;
    const size_t o = (size_t)y * g.pitch + w;
    uint64_t in[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int d = 0; d < D; ++d) in[d] = planes[(size_t)d * g.ps + o];
    if (n == 64 && ((reinterpret_cast<uintptr_t>(row) & 7) == 0)) {
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            uint64_t v = 0;
#pragma unroll
            for (int d = 0; d < D; ++d) v |= ((in[d] >> (8 * j)) & 0xffull) << (8 * d);
            *reinterpret_cast<uint64_t *>(row + 8 * j) = transpose8(v);
        }
    } else {
        for (int i = 0; i < n; ++i) {
            unsigned b = 0;
#pragma unroll
            for (int d = 0; d < D; ++d) b |= (unsigned)((in[d] >> i) & 1ull) << d;
            row[i] = (uint8_t)b;
        }
    }
}

#define LGCA_DISPATCH_D(D, KERNEL, GRID, BLOCK, STREAM, ...)                        \
    switch (D) {                                                                   \
    case 4: KERNEL<4><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;             \
    case 6: KERNEL<6><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;             \
    default: KERNEL<7><<<GRID, BLOCK, 0, STREAM>>>(__VA_ARGS__); break;            \
    }

cudaError_t launch_aos_to_planes(int D, const PlaneGeom &g, const uint8_t *aos, uint64_t *planes,
                                 cudaStream_t s)
{
    const unsigned grid = grid_for((long long)g.H * g.nw, 256);
    LGCA_DISPATCH_D(D, k_aos_to_planes, grid, 256, s, g, aos, planes);
    return cudaGetLastError();
}

cudaError_t launch_planes_to_aos(int D, const PlaneGeom &g, const uint64_t *planes, uint8_t *aos,
                                 cudaStream_t s)
{
    const unsigned grid = grid_for((long long)g.H * g.nw, 256);
    LGCA_DISPATCH_D(D, k_planes_to_aos, grid, 256, s, g, planes, aos);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- geometry
__global__ void k_types_to_planes(PlaneGeom g, const int32_t *__restrict__ types,
                                  uint64_t *__restrict__ solid, uint64_t *__restrict__ slip,
                                  int *bad)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.H * g.nw) return;
    const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
    const int x0 = 64 * w, n = min(64, g.W - x0);
    const int32_t *row = types + (size_t)y * g.W + x0;
    uint64_t so = 0, sl = 0;
    bool invalid = false;
    for (int i = 0; i < n; ++i) {
        const int t = row[i];
        so |= (uint64_t)(t == 1) << i;
        sl |= (uint64_t)(t == 2) << i;
        invalid |= (t < 0 || t > 2);
    }
    if (invalid) atomicOr(bad, 1);
    const size_t o = (size_t)y * g.pitch + w;
    solid[o] = so;
    slip[o] = sl;
}

__global__ void k_planes_to_types(PlaneGeom g, const uint64_t *__restrict__ solid,
                                  const uint64_t *__restrict__ slip, int32_t *__restrict__ types)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.H * g.nw) return;
    const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
    const int x0 = 64 * w, n = min(64, g.W - x0);
    const size_t o = (size_t)y * g.pitch + w;
    const uint64_t so = solid ? solid[o] : 0ull, sl = slip ? slip[o] : 0ull;
    int32_t *row = types + (size_t)y * g.W + x0;
    for (int i = 0; i < n; ++i)
        row[i] = ((so >> i) & 1ull) ? 1 : (((sl >> i) & 1ull) ? 2 : 0);
}

cudaError_t launch_types_to_planes(const PlaneGeom &g, const int32_t *types, uint64_t *solid,
                                   uint64_t *slip, int *bad, cudaStream_t s)
{
    k_types_to_planes<<<grid_for((long long)g.H * g.nw, 256), 256, 0, s>>>(g, types, solid, slip,
                                                                           bad);
    return cudaGetLastError();
}

cudaError_t launch_planes_to_types(const PlaneGeom &g, const uint64_t *solid, const uint64_t *slip,
                                   int32_t *types, cudaStream_t s)
{
    k_planes_to_types<<<grid_for((long long)g.H * g.nw, 256), 256, 0, s>>>(g, solid, slip, types);
    return cudaGetLastError();
}

// Painting: every cell of a shape gets one type, on the device.  The mask of
// a word holds the cells of that word inside the shape; the solid bit is set
// for SOLID_NO_SLIP, the slip bit for SOLID_SLIP, and both are cleared for
// FLUID.  Shapes: rectangle [a, c) x [b, d); disc (x-a)^2 + (y-b)^2 < c^2 in
// 64-bit integers; disc of diameter c with the distance taken as
// float(sqrt(double(dx^2 + dy^2))) and compared with c / 2.0 in double (the
// obstacle test of Lattice::apply_bc_karman_vortex_street, with Real = float).
__device__ __forceinline__ bool paint_in(int shape, long long x, long long y, long long a,
                                         long long b, long long c, long long d)
{
    if (shape == 0) return x >= a && x < c && y >= b && y < d;
    const long long dx = x - a, dy = y - b, r2 = dx * dx + dy * dy;
    if (shape == 1) return r2 < c * c;
    const float dist = (float)sqrt((double)r2);
    return (double)dist < (double)(float)c / 2.0;
}

__global__ void k_paint(PlaneGeom g, uint64_t *__restrict__ solid, uint64_t *__restrict__ slip,
                        int shape, int type, long long a, long long b, long long c, long long d)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.H * g.nw) return;
    const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
    const int x0 = 64 * w, n = min(64, g.W - x0);
    // rows and words that cannot meet the shape: nothing to do
    if (shape == 0) {
        if (y < b || y >= d || x0 + n <= a || x0 >= c) return;
    } else {
        const long long rb = (shape == 1 ? c : c / 2) + 1;  // bound on the radius
        if (y < b - rb || y > b + rb || x0 + n - 1 < a - rb || x0 > a + rb) return;
    }
    uint64_t m = 0;
    for (int i = 0; i < n; ++i)
        m |= (uint64_t)paint_in(shape, x0 + i, y, a, b, c, d) << i;
    if (!m) return;
    const size_t o = (size_t)y * g.pitch + w;
    solid[o] = (type == 1) ? (solid[o] | m) : (solid[o] & ~m);
    slip[o] = (type == 2) ? (slip[o] | m) : (slip[o] & ~m);
}

cudaError_t launch_paint(const PlaneGeom &g, uint64_t *solid, uint64_t *slip, int shape, int type,
                         long long a, long long b, long long c, long long d, cudaStream_t s)
{
    k_paint<<<grid_for((long long)g.H * g.nw, 256), 256, 0, s>>>(g, solid, slip, shape, type, a,
                                                                  b, c, d);
    return cudaGetLastError();
}

__global__ void k_bytes_to_plane(PlaneGeom g, const uint8_t *__restrict__ bytes,
                                 uint64_t *__restrict__ plane)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.H * g.nw) return;
    const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
    const int x0 = 64 * w, n = min(64, g.W - x0);
    const uint8_t *row = bytes + (size_t)y * g.W + x0;
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v |= (uint64_t)(row[i] != 0) << i;
    plane[(size_t)y * g.pitch + w] = v;
}

cudaError_t launch_bytes_to_plane(const PlaneGeom &g, const uint8_t *bytes, uint64_t *plane,
                                  cudaStream_t s)
{
    k_bytes_to_plane<<<grid_for((long long)g.H * g.nw, 256), 256, 0, s>>>(g, bytes, plane);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ init
// Lattice::init_random (src/lattice.cpp:198-217) with the INIT stream:
// channel d of FLUID site (x, y) is occupied iff
// (draw(key(seed, INIT, d), (y << 32) | x) >> 32) < thr_d.
template <int D>
__global__ void k_init_random(PlaneGeom g, const uint64_t *__restrict__ solid,
                              const uint64_t *__restrict__ slip, uint64_t *__restrict__ planes,
                              uint64_t seed, uint64_t thr_move, uint64_t thr_rest)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.H * g.nw) return;
    const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
    const int x0 = 64 * w, n = min(64, g.W - x0);
    const size_t o = (size_t)y * g.pitch + w;
    uint64_t fluid = (w == g.nw - 1) ? g.lastmask : ~0ull;
    if (solid) fluid &= ~solid[o];
    if (slip) fluid &= ~slip[o];
#pragma unroll 1
    for (int d = 0; d < D; ++d) {
        const uint64_t key = lgca_rng_key(seed, LGCA_STREAM_INIT, (uint64_t)d);
        const uint64_t thr = (d == 6) ? thr_rest : thr_move;
        uint64_t v = 0;
        for (int i = 0; i < n; ++i) {
            const uint64_t u =
                lgca_rng_draw(key, lgca_rng_index((uint32_t)y, (uint32_t)(x0 + i))) >> 32;
            v |= (uint64_t)(u < thr) << i;
        }
        planes[(size_t)d * g.ps + o] = v & fluid;
    }
}

cudaError_t launch_init_random(int D, const PlaneGeom &g, const uint64_t *solid,
                               const uint64_t *slip, uint64_t *planes, uint64_t seed,
                               uint64_t thr_move, uint64_t thr_rest, cudaStream_t s)
{
    const unsigned grid = grid_for((long long)g.H * g.nw, 256);
    LGCA_DISPATCH_D(D, k_init_random, grid, 256, s, g, solid, slip, planes, seed, thr_move,
                    thr_rest);
    return cudaGetLastError();
}

template <int MODEL>
static cudaError_t block_sums_model(const PlaneGeom &g, const uint64_t *planes, int B, int32_t *N,
                                    int32_t *Jx2, int32_t *Jy, cudaStream_t s)
{
    const int Wb = (g.W + B - 1) / B, Hb = (g.H + B - 1) / B;
    auto seg_grid = [&](long long warps) { return grid_for(warps * 32, 128); };
    switch (B) {
    case 8:
        k_block_sums_seg<MODEL, 8><<<seg_grid(seg_block_sums_warps<8>(g.nw, Hb)), 128, 0, s>>>(
            g, planes, Wb, Hb, N, Jx2, Jy);
        break;
    case 16:
        k_block_sums_seg<MODEL, 16><<<seg_grid(seg_block_sums_warps<16>(g.nw, Hb)), 128, 0, s>>>(
            g, planes, Wb, Hb, N, Jx2, Jy);
        break;
    case 32:
        k_block_sums_seg<MODEL, 32><<<seg_grid(seg_block_sums_warps<32>(g.nw, Hb)), 128, 0, s>>>(
            g, planes, Wb, Hb, N, Jx2, Jy);
        break;
    case 64:
        k_block_sums_seg<MODEL, 64><<<seg_grid(seg_block_sums_warps<64>(g.nw, Hb)), 128, 0, s>>>(
            g, planes, Wb, Hb, N, Jx2, Jy);
        break;
    default:
        if (B % 64 == 0 && B <= 2048 && ((B / 64) & (B / 64 - 1)) == 0) {
            const int K = B / 64, chunks = (g.nw + 31) / 32;
            const long long tasks = (long long)Hb * chunks;
            k_block_sums_wide<MODEL><<<grid_for(tasks, 4), 128, 0, s>>>(g, planes, K, B, Wb, Hb,
                                                                        chunks, N, Jx2, Jy);
        } else {
            k_block_sums_any<MODEL><<<grid_for((long long)Wb * Hb, 128), 128, 0, s>>>(
                g, planes, B, Wb, Hb, N, Jx2, Jy);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_block_sums(int model, const PlaneGeom &g, const uint64_t *planes, int B,
                              int32_t *N, int32_t *Jx2, int32_t *Jy, cudaStream_t s)
{
    switch (model) {
    case M_HPP: return block_sums_model<M_HPP>(g, planes, B, N, Jx2, Jy, s);
    case M_FHP_I: return block_sums_model<M_FHP_I>(g, planes, B, N, Jx2, Jy, s);
    default: return block_sums_model<M_FHP_II>(g, planes, B, N, Jx2, Jy, s);
    }
}

// ------------------------------------------------------- post-processing
// Per-cell values with the reference's FP32 arithmetic
// (src/omp_lattice.cpp:360-394): the reference sums n_d * e_d in direction
// order; every partial sum is a multiple of 1/2 in x and k*sin60 with |k| <= 2
// in y, all exactly representable, so the sums equal 0.5*k and k*sin60
// computed directly (and are never -0).
template <int MODEL>
__device__ __forceinline__ void cell_values(const uint64_t *v, int i, float &rho, float &mx,
                                            float &my)
{
    constexpr int D = ModelTraits<MODEL>::D;
    int b[7];
#pragma unroll
    for (int d = 0; d < D; ++d) b[d] = (int)((v[d] >> i) & 1ull);
    int n = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) n += b[d];
    rho = (float)n;
    if (MODEL == M_HPP) {
        mx = (float)(b[0] - b[2]);
        my = (float)(b[1] - b[3]);
    } else {
        const float S = 0.866025388240814208984375f;  // (float)sin(pi/3)
        mx = 0.5f * (float)(2 * b[0] + b[1] - b[2] - 2 * b[3] - b[4] + b[5]);
        my = S * (float)(b[1] + b[2] - b[4] - b[5]);
    }
}

template <int MODEL>
__global__ void k_cell_post(PlaneGeom g, const uint64_t *__restrict__ planes,
                            float *__restrict__ density, float *__restrict__ momentum)
{
    constexpr int D = ModelTraits<MODEL>::D;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)g.H * g.nw) return;
    const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
    const int x0 = 64 * w, n = min(64, g.W - x0);
    uint64_t v[7];
    const size_t o = (size_t)y * g.pitch + w;
#pragma unroll
    for (int d = 0; d < D; ++d) v[d] = planes[(size_t)d * g.ps + o];
    const size_t c0 = (size_t)y * g.W + x0;
    for (int i = 0; i < n; ++i) {
        float rho, mx, my;
        cell_values<MODEL>(v, i, rho, mx, my);
        if (density) density[c0 + i] = rho;
        if (momentum) {
            momentum[2 * (c0 + i)] = mx;
            momentum[2 * (c0 + i) + 1] = my;
        }
    }
}

// src/omp_lattice.cpp:397-454: coarse cell c anchored at (2r*cx, 2r*cy); the
// window walks y = 0..2r, x = 0..2r over linear cell indices and keeps a cell
// when the index is inside the lattice and |x_nb - x_anchor| <= r; FP32 sums
// in that order, then division by the count.
template <int MODEL>
__global__ void k_mean_post(PlaneGeom g, const uint64_t *__restrict__ planes, int r, int Wc,
                            int Hc, float *__restrict__ mdens, float *__restrict__ mmom)
{
    constexpr int D = ModelTraits<MODEL>::D;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)Wc * Hc) return;
    const long long ncells = (long long)g.W * g.H;
    const long long cell = (idx % Wc) * (2LL * r) + (idx / Wc) * (2LL * r) * g.W;
    const int px = (int)(cell % g.W);
    float md = 0.0f, mx = 0.0f, my = 0.0f;
    int cnt = 0;
    for (int yy = 0; yy <= 2 * r; ++yy) {
        for (int xx = 0; xx <= 2 * r; ++xx) {
            const long long nb = cell + (long long)yy * g.W + xx;
            if (nb >= ncells) continue;
            const int x = (int)(nb % g.W), y = (int)(nb / g.W);
            if (abs(x - px) > r) continue;
            uint64_t v[7];
            const size_t o = (size_t)y * g.pitch + (x >> 6);
#pragma unroll
            for (int d = 0; d < D; ++d) v[d] = __ldg(planes + (size_t)d * g.ps + o);
            float rho, cx, cy;
            cell_values<MODEL>(v, x & 63, rho, cx, cy);
            cnt++;
            md = __fadd_rn(md, rho);
            mx = __fadd_rn(mx, cx);
            my = __fadd_rn(my, cy);
        }
    }
    const float fc = (float)cnt;
    if (mdens) mdens[idx] = __fdiv_rn(md, fc);
    if (mmom) {
        mmom[2 * idx] = __fdiv_rn(mx, fc);
        mmom[2 * idx + 1] = __fdiv_rn(my, fc);
    }
}

cudaError_t launch_cell_post(int model, const PlaneGeom &g, const uint64_t *planes, float *cd,
                             float *cm, cudaStream_t s)
{
    const unsigned grid = grid_for((long long)g.H * g.nw, 128);
    switch (model) {
    case M_HPP: k_cell_post<M_HPP><<<grid, 128, 0, s>>>(g, planes, cd, cm); break;
    case M_FHP_I: k_cell_post<M_FHP_I><<<grid, 128, 0, s>>>(g, planes, cd, cm); break;
    default: k_cell_post<M_FHP_II><<<grid, 128, 0, s>>>(g, planes, cd, cm); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_mean_post(int model, const PlaneGeom &g, const uint64_t *planes, int r,
                             float *md, float *mm, cudaStream_t s)
{
    const int Wc = g.W / (2 * r), Hc = g.H / (2 * r);
    if (Wc <= 0 || Hc <= 0) return cudaSuccess;
    const unsigned grid = grid_for((long long)Wc * Hc, 128);
    switch (model) {
    case M_HPP: k_mean_post<M_HPP><<<grid, 128, 0, s>>>(g, planes, r, Wc, Hc, md, mm); break;
    case M_FHP_I: k_mean_post<M_FHP_I><<<grid, 128, 0, s>>>(g, planes, r, Wc, Hc, md, mm); break;
    default: k_mean_post<M_FHP_II><<<grid, 128, 0, s>>>(g, planes, r, Wc, Hc, md, mm); break;
    }
    return cudaGetLastError();
}

// -------------------------------------------------------------- reductions
template <int D>
__global__ void k_count(PlaneGeom g, const uint64_t *__restrict__ planes,
                        unsigned long long *out)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long c = 0;
    if (idx < (long long)g.H * g.nw) {
        const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
        const size_t o = (size_t)y * g.pitch + w;
#pragma unroll
        for (int d = 0; d < D; ++d) c += (unsigned long long)__popcll(planes[(size_t)d * g.ps + o]);
    }
    for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(FULL, c, off);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

cudaError_t launch_count(int D, const PlaneGeom &g, const uint64_t *planes,
                         unsigned long long *out, cudaStream_t s)
{
    const unsigned grid = grid_for((long long)g.H * g.nw, 256);
    LGCA_DISPATCH_D(D, k_count, grid, 256, s, g, planes, out);
    return cudaGetLastError();
}

// src/omp_lattice.cpp:508-557: sum over FLUID cells of momentum/density
// (density > 1e-6), in double here; the count of FLUID cells separately.
template <int MODEL>
__global__ void k_mean_velocity(PlaneGeom g, const uint64_t *__restrict__ planes,
                                const uint64_t *__restrict__ solid,
                                const uint64_t *__restrict__ slip, double *dsum,
                                unsigned long long *nfluid)
{
    constexpr int D = ModelTraits<MODEL>::D;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double sx = 0.0, sy = 0.0;
    unsigned long long nf = 0;
    if (idx < (long long)g.H * g.nw) {
        const int y = (int)(idx / g.nw), w = (int)(idx - (long long)y * g.nw);
        const size_t o = (size_t)y * g.pitch + w;
        uint64_t fluid = (w == g.nw - 1) ? g.lastmask : ~0ull;
        if (solid) fluid &= ~solid[o];
        if (slip) fluid &= ~slip[o];
        nf = (unsigned long long)__popcll(fluid);
        uint64_t v[7], any = 0;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            v[d] = planes[(size_t)d * g.ps + o];
            any |= v[d];
        }
        uint64_t m = fluid & any;
        while (m) {
            const int i = __ffsll((long long)m) - 1;
            m &= m - 1;
            float rho, mx, my;
            cell_values<MODEL>(v, i, rho, mx, my);
            sx += (double)__fdiv_rn(mx, rho);
            sy += (double)__fdiv_rn(my, rho);
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        sx += __shfl_xor_sync(FULL, sx, off);
        sy += __shfl_xor_sync(FULL, sy, off);
        nf += __shfl_xor_sync(FULL, nf, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(dsum, sx);
        atomicAdd(dsum + 1, sy);
        atomicAdd(nfluid, nf);
    }
}

cudaError_t launch_mean_velocity(int model, const PlaneGeom &g, const uint64_t *planes,
                                 const uint64_t *solid, const uint64_t *slip, double *dsum,
                                 unsigned long long *nfluid, cudaStream_t s)
{
    const unsigned grid = grid_for((long long)g.H * g.nw, 256);
    switch (model) {
    case M_HPP: k_mean_velocity<M_HPP><<<grid, 256, 0, s>>>(g, planes, solid, slip, dsum, nfluid); break;
    case M_FHP_I: k_mean_velocity<M_FHP_I><<<grid, 256, 0, s>>>(g, planes, solid, slip, dsum, nfluid); break;
    default: k_mean_velocity<M_FHP_II><<<grid, 256, 0, s>>>(g, planes, solid, slip, dsum, nfluid); break;
    }
    return cudaGetLastError();
}

}  // namespace lgca_gpu
