// Register wavefront form of the temporally blocked step (one warp's strip
// and slab): K lattice steps per pass over global memory with no shared
// memory.  Used by the one-lattice kernel k_wave (wave.cu) and the batch
// kernel k_batch_wave (batch_kernels.cuh).
//
// One warp owns a strip of 32 consecutive words (30 output words plus one
// halo word on each side) and a slab of S output rows.  It walks down the
// slab one input row at a time (K halo rows above and below).  Time level L
// keeps, per lane, the two most recent rows of level L that level L+1 still
// needs, so each new row of level L lets level L+1 produce the row above it:
//
//   level L+1, row q   <-   level L rows q-1 (planes 1,2), q (0,3,6), q+1 (4,5)
//
// (FHP; HPP reads row q-1 plane 1, row q planes 0,2, row q+1 plane 3).  x
// neighbours come from the adjacent lanes by shuffle.  After j steps the j
// outermost bits of the two halo lanes are stale (they would need words
// outside the strip), which never reaches the 30 output words for K < 64.
// Rows follow the torus; only lattices whose width is a multiple of 64 take
// this path, so the x seam is a plain word wrap.
#pragma once
#include "internal.cuh"
#include "../../include/lgca/rng.h"

namespace lgca_gpu {

static constexpr unsigned FULLW = 0xffffffffu;

// Keys of the K steps of a pass: from the kernel parameters (one lattice) or
// from a batch's key table (chirality, forcing interleaved per step).
struct ParamKeys {
    const MultiStepArgs &m;
    __device__ __forceinline__ uint64_t chir(int L) const { return m.chir_keys[L]; }
    __device__ __forceinline__ uint64_t force(int L) const { return m.force_keys[L]; }
};
template <int K> struct TableKeys {
    uint64_t c[K], f[K];  // held in registers for the whole pass
    __device__ __forceinline__ explicit TableKeys(const uint64_t *p)  // keys of the pass's first step
    {
#pragma unroll
        for (int L = 0; L < K; ++L) {
            c[L] = __ldg(p + 2 * L);
            f[L] = __ldg(p + 2 * L + 1);
        }
    }
    __device__ __forceinline__ uint64_t chir(int L) const { return c[L]; }
    __device__ __forceinline__ uint64_t force(int L) const { return f[L]; }
};

// One warp's strip sx (30 output words) and slab sy (S output rows) of a
// K-step pass from src to dst; a.src / a.dst are not used.
template <int MODEL, int GM, int K, class Keys>
__device__ __forceinline__ void wave_strip(const StepArgs &a, const uint64_t *__restrict__ src,
                                           uint64_t *__restrict__ dst, const Keys &keys, int S,
                                           int sx, int sy)
{
    constexpr int D = ModelTraits<MODEL>::D;
    constexpr int WEST = (MODEL == M_HPP) ? 2 : 3;
    const PlaneGeom &g = a.g;
    const int lane = threadIdx.x & 31;
    const int w0 = sx * 30;  // first output word; lane i holds word w0 - 1 + i
    const int y0 = sy * S;   // first output row
    const int nw = g.nw, H = g.H;
    int gw = w0 - 1 + lane;
    gw = gw < 0 ? gw + nw : (gw >= nw ? gw % nw : gw);
    const bool store_lane = lane >= 1 && lane <= 30 && (w0 + lane - 1) < nw;
    const unsigned ps = (unsigned)g.ps;
    const bool forcing = a.force_thr != 0;
    const int fb = a.fx & 63;
    const bool flane = forcing && gw == (a.fx >> 6);

    // global row of slab-local input row q (q = 0 is y0 - K)
    auto grow = [&](int q) -> int {
        int y = y0 - K + q;
        if (y < 0) y += H * ((-y + H - 1) / H);
        return y >= H ? y % H : y;
    };
    auto fluid_word = [&](unsigned o) -> uint64_t {
        uint64_t f = ~0ull;
        if (GM >= GEOM_NOSLIP) f &= ~__ldg(a.solid + o);
        if (GM == GEOM_FULL) f &= ~__ldg(a.slip + o);
        return f;
    };
    // forcing of global step (t0 + L) on a row of level L held by this lane
    auto force = [&](uint64_t *v, int gy, int L) {
        if (!flane) return;
        const uint64_t u =
            lgca_rng_draw(keys.force(L), lgca_rng_index((uint32_t)gy, (uint32_t)a.fx)) >> 32;
        if (u >= a.force_thr) return;
        const uint64_t fl = (~v[0] & v[WEST] & fluid_word((unsigned)gy * g.pitch + gw)) &
                            (1ull << fb);
        v[0] |= fl;
        v[WEST] &= ~fl;
    };

    // per level: rows q-1 (prev2) and q (prev1) of that level
    uint64_t p1[K][7], p2[K][7];
#pragma unroll
    for (int L = 0; L < K; ++L)
#pragma unroll
        for (int d = 0; d < 7; ++d) p1[L][d] = p2[L][d] = 0ull;

    const int iters = S + 2 * K;
#pragma unroll 1
    for (int it = 0; it < iters; ++it) {
        // ---- level 0: load input row q = it
        const int gyn = grow(it);
        uint64_t cur[7];
        {
            const unsigned o = (unsigned)gyn * g.pitch + gw;
#pragma unroll
            for (int d = 0; d < D; ++d) cur[d] = __ldcg(src + (d * ps + o));  // L2: see pdl_wait
            force(cur, gyn, 0);
        }
#pragma unroll
        for (int L = 0; L < K; ++L) {
            // level L+1 computes row q = it - L - 1 from level L rows q-1, q, q+1
            uint64_t out[7];
            const bool active = it >= 2 * L + 2;  // warp-uniform
            const int q = it - L - 1;
            int gy = 0;
            if (active) {
                gy = grow(q);
                const bool even = (gy & 1) == 0;
                auto shl = [&](uint64_t v) -> uint64_t {
                    const uint32_t hi = __shfl_up_sync(FULLW, (uint32_t)(v >> 32), 1);
                    return (v << 1) | (lane == 0 ? 0ull : (uint64_t)(hi >> 31));
                };
                auto shr = [&](uint64_t v) -> uint64_t {
                    const uint32_t lo = __shfl_down_sync(FULLW, (uint32_t)v, 1);
                    return (v >> 1) | (lane == 31 ? 0ull : ((uint64_t)(lo & 1u) << 63));
                };
                uint64_t p[7];
                if (MODEL == M_HPP) {
                    p[0] = shl(p1[L][0]);
                    p[1] = p2[L][1];
                    p[2] = shr(p1[L][2]);
                    p[3] = cur[3];
                } else {
                    p[0] = shl(p1[L][0]);
                    p[3] = shr(p1[L][3]);
                    if (even) {
                        p[1] = shl(p2[L][1]);
                        p[2] = p2[L][2];
                        p[4] = cur[4];
                        p[5] = shl(cur[5]);
                    } else {
                        p[1] = p2[L][1];
                        p[2] = shr(p2[L][2]);
                        p[4] = shr(cur[4]);
                        p[5] = cur[5];
                    }
                    if (D == 7) p[6] = p1[L][6];
                }
                uint64_t c[7];
#pragma unroll
                for (int d = 0; d < D; ++d) c[d] = p[d];
                if (MODEL != M_HPP) {
                    const uint64_t chir =
                        a.chir ? __ldg(a.chir + ((unsigned)gy * g.pitch + gw))
                               : lgca_rng_draw(keys.chir(L),
                                               lgca_rng_index((uint32_t)gy, (uint32_t)gw));
                    collide<MODEL>(c, chir);
                } else {
                    collide<MODEL>(c, 0ull);
                }
                if (GM == GEOM_NONE) {
#pragma unroll
                    for (int d = 0; d < D; ++d) out[d] = c[d];
                } else {
                    const unsigned o = (unsigned)gy * g.pitch + gw;
                    const uint64_t solid = __ldg(a.solid + o);
                    const uint64_t slip = (GM == GEOM_FULL) ? __ldg(a.slip + o) : 0ull;
                    const uint64_t fluid = ~(solid | slip);
                    const bool nsrow = (gy == 0) || (gy == H - 1);
                    const uint64_t ew =
                        (gw == 0 ? 1ull : 0ull) | (gw == nw - 1 ? (1ull << 63) : 0ull);
#pragma unroll
                    for (int d = 0; d < D; ++d) {
                        uint64_t o2 = (fluid & c[d]) | (solid & p[Dirs<MODEL>::inv(d)]);
                        if (GM == GEOM_FULL) {
                            const uint64_t sxm = nsrow ? p[Dirs<MODEL>::mirx(d)] : p[d];
                            o2 |= slip & ((ew & p[Dirs<MODEL>::miry(d)]) | (~ew & sxm));
                        }
                        out[d] = o2;
                    }
                }
                if (L + 1 < K) force(out, gy, L + 1);
            } else {
#pragma unroll
                for (int d = 0; d < 7; ++d) out[d] = 0ull;
            }
            // shift level L's window: row q becomes q-1, the new row becomes q
#pragma unroll
            for (int d = 0; d < 7; ++d) {
                p2[L][d] = p1[L][d];
                p1[L][d] = cur[d];
            }
            if (L + 1 == K) {
                // level K row q is final: store the strip's output words
                const int oy = y0 + (q - K);
                if (active && q >= K && q < K + S && oy < H && store_lane) {
                    uint64_t *dp = dst + ((unsigned)oy * g.pitch + (w0 + lane - 1));
#pragma unroll
                    for (int d = 0; d < D; ++d) dp[d * ps] = out[d];
                }
            } else {
#pragma unroll
                for (int d = 0; d < 7; ++d) cur[d] = out[d];
            }
        }
    }
}

}  // namespace lgca_gpu
