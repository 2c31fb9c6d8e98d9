// Temporally blocked step: K lattice steps per pass over global memory.
//
// Each CTA owns an output tile of 32 words (2048 sites) x THO rows.  It loads
// the tile plus a halo of one word on each side and K rows above and below
// into shared memory, advances K steps there (double-buffered), and writes
// only the tile.  A step pulls from the rows y-1, y, y+1 and from the sites
// x-1, x+1 (see step.cu), so after j steps the rows within j of the halo edge
// and the j outermost bits of the two halo words are stale; with K < 64 the
// tile itself is exact.  Forcing of each step is applied to the tile's copy of
// the state before that step's pull, exactly as in the one-step kernel.
//
// Only lattices whose width is a multiple of 64 take this path (the periodic
// x seam is then a plain word wrap); the host falls back to one step per pass
// otherwise.
#include "internal.cuh"
#include "../../include/lgca/rng.h"

namespace lgca_gpu {

static constexpr int TWI = 34;  // words per tile row incl. the two halo words

template <int MODEL, int GM, int K, int THO>
struct Tile {
    static constexpr int D = ModelTraits<MODEL>::D;
    static constexpr int R = THO + 2 * K;
    static constexpr int PLANE = R * TWI;                   // words per plane
    static constexpr int BUF = D * PLANE;                   // words per state buffer
    static constexpr int GEO = (GM == GEOM_FULL ? 2 : (GM == GEOM_NOSLIP ? 1 : 0));
    static constexpr size_t SMEM = (size_t)(2 * BUF + GEO * PLANE) * sizeof(uint64_t);
};

template <int MODEL, int GM, int K, int THO>
__global__ void __launch_bounds__(256) k_multistep(const __grid_constant__ MultiStepArgs m)
{
    pdl_launch_dependents();
    pdl_wait();
    using T = Tile<MODEL, GM, K, THO>;
    constexpr int D = T::D, R = T::R, PL = T::PLANE;
    extern __shared__ uint64_t smem[];
    uint64_t *buf0 = smem, *buf1 = smem + T::BUF;
    uint64_t *s_solid = smem + 2 * T::BUF;
    uint64_t *s_slip = s_solid + PL;

    const StepArgs &a = m.base;
    const PlaneGeom &g = a.g;
    const int nw = g.nw, H = g.H;
    const int w0 = blockIdx.x * 32;   // first output word
    const int y0 = blockIdx.y * THO;  // first output row
    const unsigned ps = (unsigned)g.ps;
    const int nthr = blockDim.x;

    auto grow = [&](int r) -> int {  // global row of tile row r
        int y = y0 - K + r;
        y %= H;
        return y < 0 ? y + H : y;
    };
    auto gword = [&](int i) -> int {  // global word of tile column i
        int w = w0 - 1 + i;
        w %= nw;
        return w < 0 ? w + nw : w;
    };

    // ---- load tile + halo
    for (int it = threadIdx.x; it < R * TWI; it += nthr) {
        const int r = it / TWI, i = it - r * TWI;
        const unsigned o = (unsigned)grow(r) * g.pitch + gword(i);
#pragma unroll
        for (int d = 0; d < D; ++d) buf0[d * PL + it] = __ldcg(a.src + (d * ps + o));  // L2: see pdl_wait
        if (GM >= GEOM_NOSLIP) s_solid[it] = __ldg(a.solid + o);
        if (GM == GEOM_FULL) s_slip[it] = __ldg(a.slip + o);
    }
    __syncthreads();

    constexpr int WEST = (MODEL == M_HPP) ? 2 : 3;
    const bool forcing = a.force_thr != 0;
    const int fw = a.fx >> 6, fb = a.fx & 63;
    // tile columns holding the forcing word (several when nw < TWI and the
    // tile wraps around the lattice)
    uint64_t fmask = 0;
    if (forcing)
        for (int i = 0; i < TWI; ++i)
            if (gword(i) == fw) fmask |= 1ull << i;

#pragma unroll 1
    for (int j = 1; j <= K; ++j) {
        uint64_t *src = (j & 1) ? buf0 : buf1;
        uint64_t *dst = (j & 1) ? buf1 : buf0;
        const uint64_t fkey = m.force_keys[j - 1];
        const uint64_t ckey = m.chir_keys[j - 1];

        // forcing of step j-1 on the rows that feed level j
        if (fmask) {
            for (int r = j - 1 + threadIdx.x; r < R - j + 1; r += nthr) {
                const int gy = grow(r);
                const uint64_t u =
                    lgca_rng_draw(fkey, lgca_rng_index((uint32_t)gy, (uint32_t)a.fx)) >> 32;
                if (u >= a.force_thr) continue;
                for (uint64_t mm = fmask; mm; mm &= mm - 1) {
                    const int idx = r * TWI + (__ffsll((long long)mm) - 1);
                    uint64_t fl = ~src[idx] & src[WEST * PL + idx];
                    if (GM >= GEOM_NOSLIP) fl &= ~s_solid[idx];
                    if (GM == GEOM_FULL) fl &= ~s_slip[idx];
                    fl &= 1ull << fb;
                    src[idx] |= fl;
                    src[WEST * PL + idx] &= ~fl;
                }
            }
            __syncthreads();
        }

        const int rlo = j, rhi = R - j;
        for (int it = threadIdx.x + rlo * TWI; it < rhi * TWI; it += nthr) {
            const int r = it / TWI, i = it - r * TWI;
            const int gy = grow(r);
            const bool even = (gy & 1) == 0;
            const int im = it - TWI, ip = it + TWI;  // same column, rows r-1 / r+1
            // west / east neighbour words (stale zero beyond the halo)
            auto west = [&](int d, int idx) -> uint64_t {
                return i > 0 ? (src[d * PL + idx - 1] >> 63) : 0ull;
            };
            auto east = [&](int d, int idx) -> uint64_t {
                return i < TWI - 1 ? (src[d * PL + idx + 1] & 1ull) : 0ull;
            };
            uint64_t p[7];
            if (MODEL == M_HPP) {
                p[0] = (src[0 * PL + it] << 1) | west(0, it);
                p[1] = src[1 * PL + im];
                p[2] = (src[2 * PL + it] >> 1) | (east(2, it) << 63);
                p[3] = src[3 * PL + ip];
            } else {
                p[0] = (src[0 * PL + it] << 1) | west(0, it);
                p[3] = (src[3 * PL + it] >> 1) | (east(3, it) << 63);
                if (even) {
                    p[1] = (src[1 * PL + im] << 1) | west(1, im);
                    p[2] = src[2 * PL + im];
                    p[4] = src[4 * PL + ip];
                    p[5] = (src[5 * PL + ip] << 1) | west(5, ip);
                } else {
                    p[1] = src[1 * PL + im];
                    p[2] = (src[2 * PL + im] >> 1) | (east(2, im) << 63);
                    p[4] = (src[4 * PL + ip] >> 1) | (east(4, ip) << 63);
                    p[5] = src[5 * PL + ip];
                }
                if (D == 7) p[6] = src[6 * PL + it];
            }
            const int gw = gword(i);
            uint64_t c[7];
#pragma unroll
            for (int d = 0; d < D; ++d) c[d] = p[d];
            if (MODEL != M_HPP) {
                const uint64_t chir =
                    a.chir ? __ldg(a.chir + ((unsigned)gy * g.pitch + gw))
                           : lgca_rng_draw(ckey, lgca_rng_index((uint32_t)gy, (uint32_t)gw));
                collide<MODEL>(c, chir);
            } else {
                collide<MODEL>(c, 0ull);
            }
            uint64_t out[7];
            if (GM == GEOM_NONE) {
#pragma unroll
                for (int d = 0; d < D; ++d) out[d] = c[d];
            } else {
                const uint64_t solid = s_solid[it];
                const uint64_t slip = (GM == GEOM_FULL) ? s_slip[it] : 0ull;
                const uint64_t fluid = ~(solid | slip);
                const bool nsrow = (gy == 0) || (gy == H - 1);
                const uint64_t ew = (gw == 0 ? 1ull : 0ull) | (gw == nw - 1 ? (1ull << 63) : 0ull);
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    uint64_t o = (fluid & c[d]) | (solid & p[Dirs<MODEL>::inv(d)]);
                    if (GM == GEOM_FULL) {
                        const uint64_t sx = nsrow ? p[Dirs<MODEL>::mirx(d)] : p[d];
                        o |= slip & ((ew & p[Dirs<MODEL>::miry(d)]) | (~ew & sx));
                    }
                    out[d] = o;
                }
            }
            if (j < K) {
#pragma unroll
                for (int d = 0; d < D; ++d) dst[d * PL + it] = out[d];
            } else if (i >= 1 && i <= 32 && r >= K && r < K + THO) {
                const int oy = y0 + (r - K), ow = w0 + i - 1;
                if (oy < H && ow < nw) {
                    uint64_t *dp = a.dst + ((unsigned)oy * g.pitch + ow);
#pragma unroll
                    for (int d = 0; d < D; ++d) dp[d * ps] = out[d];
                }
            }
        }
        __syncthreads();
    }
}

template <int MODEL, int GM, int K, int THO>
static cudaError_t launch_tile(const MultiStepArgs &m, cudaStream_t st)
{
    using T = Tile<MODEL, GM, K, THO>;
    auto kern = k_multistep<MODEL, GM, K, THO>;
    // opt in to more than 48 KB of dynamic shared memory (per device context)
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)T::SMEM);
    if (e != cudaSuccess) return e;
    const dim3 grid((unsigned)((m.base.g.nw + 31) / 32), (unsigned)((m.base.g.H + THO - 1) / THO));
    if (grid.y > 65535u) return cudaErrorInvalidConfiguration;
    return launch_pdl(kern, grid, dim3(256), T::SMEM, st, m);
}

// Tile heights per depth: shared memory = (2 * D + geometry planes) * (THO + 2K) * 34 * 8 B.
template <int MODEL, int GM>
static cudaError_t launch_depth(const MultiStepArgs &m, cudaStream_t st)
{
    switch (m.depth) {
    case 2: return launch_tile<MODEL, GM, 2, 16>(m, st);
    case 4: return launch_tile<MODEL, GM, 4, 16>(m, st);
    case 8: return launch_tile<MODEL, GM, 8, 16>(m, st);
    default: return cudaErrorInvalidValue;
    }
}

template <int MODEL>
static cudaError_t launch_geom(int gm, const MultiStepArgs &m, cudaStream_t st)
{
    switch (gm) {
    case GEOM_NONE: return launch_depth<MODEL, GEOM_NONE>(m, st);
    case GEOM_NOSLIP: return launch_depth<MODEL, GEOM_NOSLIP>(m, st);
    default: return launch_depth<MODEL, GEOM_FULL>(m, st);
    }
}

bool multistep_supported(int model, const PlaneGeom &g, int depth)
{
    (void)model;
    return (depth == 2 || depth == 4 || depth == 8) && (g.W % 64) == 0 && g.H >= 2;
}

cudaError_t launch_multistep(int model, int gm, const MultiStepArgs &m, cudaStream_t st)
{
    switch (model) {
    case M_HPP: return launch_geom<M_HPP>(gm, m, st);
    case M_FHP_I: return launch_geom<M_FHP_I>(gm, m, st);
    default: return launch_geom<M_FHP_II>(gm, m, st);
    }
}

}  // namespace lgca_gpu
