// Integer block-sum kernels (launched from aux.cu): B x B sums of the
// particle count and the two momentum components, by __popc on the
// bit-planes.  Kept apart from the launchers so that the kernel bodies also
// build as host C++ (the CPU emulation in the tests).
#pragma once
#include "internal.cuh"

namespace lgca_gpu {

static constexpr unsigned FULL = 0xffffffffu;

// ------------------------------------------------------------ block sums
// Momentum weights: FHP Jx2 = 2n0 + n1 - n2 - 2n3 - n4 + n5 (units of 1/2,
// lattice vectors src/lgca_models.h:246), Jy = n1 + n2 - n4 - n5 (units of
// sin 60); HPP Jx2 = 2(n0 - n2), Jy = n1 - n3 (src/lgca_models.h:51-52).
template <int MODEL>
__device__ __forceinline__ void accum_counts(const uint64_t *v, uint64_t m, int &N, int &Jx2,
                                             int &Jy)
{
    constexpr int D = ModelTraits<MODEL>::D;
    int c[7];
#pragma unroll
    for (int d = 0; d < D; ++d) c[d] = __popcll(v[d] & m);
    int n = 0;
#pragma unroll
    for (int d = 0; d < D; ++d) n += c[d];
    N += n;
    if (MODEL == M_HPP) {
        Jx2 += 2 * (c[0] - c[2]);
        Jy += c[1] - c[3];
    } else {
        Jx2 += 2 * c[0] + c[1] - c[2] - 2 * c[3] - c[4] + c[5];
        Jy += c[1] + c[2] - c[4] - c[5];
    }
}

// B divides 64 (B >= 8): S = 64/B blocks per word.  A warp takes 32/QG
// consecutive words of one block row; the QG consecutive lanes of a word
// split the block's B rows into groups of 8, and their sums are added by
// shuffles.  Launch: seg_block_sums_warps(...) warps.
template <int B>
__host__ __device__ __forceinline__ long long seg_block_sums_warps(int nw, int Hb)
{
    constexpr int WPW = 32 / (B / 8);  // words per warp
    return (long long)Hb * ((nw + WPW - 1) / WPW);
}
template <int MODEL, int B>
__global__ void k_block_sums_seg(PlaneGeom g, const uint64_t *__restrict__ planes, int Wb, int Hb,
                                 int32_t *__restrict__ N, int32_t *__restrict__ Jx2,
                                 int32_t *__restrict__ Jy)
{
    static_assert(B >= 8 && 64 % B == 0, "B divides 64");
    constexpr int D = ModelTraits<MODEL>::D;
    constexpr int S = 64 / B, QG = B / 8, WPW = 32 / QG;
    const int wchunks = (g.nw + WPW - 1) / WPW;
    const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (wid >= (long long)Hb * wchunks) return;  // whole warp
    const int lane = threadIdx.x & 31;
    const int by = (int)(wid / wchunks), wc = (int)(wid - (long long)by * wchunks);
    const int q = lane % QG, w = wc * WPW + lane / QG;
    int n[S], jx[S], jy[S];
#pragma unroll
    for (int s = 0; s < S; ++s) n[s] = jx[s] = jy[s] = 0;
    if (w < g.nw) {
#pragma unroll 4
        for (int i = 0; i < 8; ++i) {
            const int y = by * B + q * 8 + i;
            if (y >= g.H) break;
            uint64_t v[7];
            const size_t o = (size_t)y * g.pitch + w;
#pragma unroll
            for (int d = 0; d < D; ++d) v[d] = __ldg(planes + (size_t)d * g.ps + o);
#pragma unroll
            for (int s = 0; s < S; ++s) {
                const uint64_t m = (B == 64) ? ~0ull : (((1ull << B) - 1ull) << (s * B));
                accum_counts<MODEL>(v, m, n[s], jx[s], jy[s]);
            }
        }
    }
#pragma unroll
    for (int off = 1; off < QG; off <<= 1) {
#pragma unroll
        for (int s = 0; s < S; ++s) {
            n[s] += __shfl_xor_sync(FULL, n[s], off);
            jx[s] += __shfl_xor_sync(FULL, jx[s], off);
            jy[s] += __shfl_xor_sync(FULL, jy[s], off);
        }
    }
    if (q != 0 || w >= g.nw) return;
#pragma unroll
    for (int s = 0; s < S; ++s) {
        const int bx = w * S + s;
        if (bx < Wb) {
            const size_t o = (size_t)by * Wb + bx;
            N[o] = n[s];
            Jx2[o] = jx[s];
            Jy[o] = jy[s];
        }
    }
}

// B = 64 * K (K | 32): one thread per (block row, word), then a shuffle
// reduction over the K lanes of a block.
template <int MODEL>
__global__ void k_block_sums_wide(PlaneGeom g, const uint64_t *__restrict__ planes, int K, int B,
                                  int Wb, int Hb, int chunks, int32_t *__restrict__ N,
                                  int32_t *__restrict__ Jx2, int32_t *__restrict__ Jy)
{
    constexpr int D = ModelTraits<MODEL>::D;
    const int lane = threadIdx.x & 31;
    const long long task = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (task >= (long long)Hb * chunks) return;
    const int by = (int)(task / chunks), ch = (int)(task - (long long)by * chunks);
    const int w = ch * 32 + lane;
    int n = 0, jx = 0, jy = 0;
    if (w < g.nw) {
        const int y1 = min(g.H, (by + 1) * B);
        for (int y = by * B; y < y1; ++y) {
            uint64_t v[7];
            const size_t o = (size_t)y * g.pitch + w;
#pragma unroll
            for (int d = 0; d < D; ++d) v[d] = __ldg(planes + (size_t)d * g.ps + o);
            accum_counts<MODEL>(v, ~0ull, n, jx, jy);
        }
    }
    for (int off = K >> 1; off > 0; off >>= 1) {
        n += __shfl_xor_sync(FULL, n, off);
        jx += __shfl_xor_sync(FULL, jx, off);
        jy += __shfl_xor_sync(FULL, jy, off);
    }
    if ((lane & (K - 1)) == 0 && w < g.nw) {
        const int bx = w / K;
        const size_t o = (size_t)by * Wb + bx;
        N[o] = n;
        Jx2[o] = jx;
        Jy[o] = jy;
    }
}

// Any B: one thread per block.
template <int MODEL>
__global__ void k_block_sums_any(PlaneGeom g, const uint64_t *__restrict__ planes, int B, int Wb,
                                 int Hb, int32_t *__restrict__ N, int32_t *__restrict__ Jx2,
                                 int32_t *__restrict__ Jy)
{
    constexpr int D = ModelTraits<MODEL>::D;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)Wb * Hb) return;
    const int by = (int)(idx / Wb), bx = (int)(idx - (long long)by * Wb);
    const int x0 = bx * B, x1 = min(g.W, x0 + B);
    const int y1 = min(g.H, (by + 1) * B);
    int n = 0, jx = 0, jy = 0;
    for (int y = by * B; y < y1; ++y) {
        for (int w = x0 >> 6; w <= (x1 - 1) >> 6; ++w) {
            const int lo = max(x0 - 64 * w, 0), hi = min(x1 - 64 * w, 64);
            const uint64_t m = (hi - lo == 64) ? ~0ull : (((1ull << (hi - lo)) - 1ull) << lo);
            uint64_t v[7];
            const size_t o = (size_t)y * g.pitch + w;
#pragma unroll
            for (int d = 0; d < D; ++d) v[d] = __ldg(planes + (size_t)d * g.ps + o);
            accum_counts<MODEL>(v, m, n, jx, jy);
        }
    }
    N[idx] = n;
    Jx2[idx] = jx;
    Jy[idx] = jy;
}

}  // namespace lgca_gpu
