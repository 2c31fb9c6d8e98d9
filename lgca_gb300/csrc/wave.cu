// Temporally blocked step, register wavefront form, for one lattice: the
// kernel k_wave (one warp per strip and slab; the warp body and its layout
// are in wave_body.cuh) and its launchers.
#include "wave_body.cuh"

namespace lgca_gpu {

template <int MODEL, int GM, int K>
__global__ void __launch_bounds__(128) k_wave(const __grid_constant__ MultiStepArgs m, int S,
                                              int nstrips)
{
    pdl_launch_dependents();
    pdl_wait();
    const int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int nslabs = (m.base.g.H + S - 1) / S;
    if (warp >= nstrips * nslabs) return;
    wave_strip<MODEL, GM, K>(m.base, m.base.src, m.base.dst, ParamKeys{m}, S, warp % nstrips,
                             warp / nstrips);
}

template <int MODEL, int GM, int K>
static cudaError_t launch_k(const MultiStepArgs &m, cudaStream_t st)
{
    const PlaneGeom &g = m.base.g;
    const int nstrips = (g.nw + 29) / 30;
    // slab height: enough warps to fill the GPU, long enough to amortise the
    // 2K halo rows
    int S = 64;
    while (S > 8 && (long long)nstrips * ((g.H + S - 1) / S) < 4 * 152 * 8) S >>= 1;
    const long long warps = (long long)nstrips * ((g.H + S - 1) / S);
    const long long blocks = (warps + 3) / 4;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    return launch_pdl(k_wave<MODEL, GM, K>, dim3((unsigned)blocks), dim3(128), 0, st, m, S,
                      nstrips);
}

template <int MODEL, int GM>
static cudaError_t launch_wave_depth(const MultiStepArgs &m, cudaStream_t st)
{
    switch (m.depth) {
    case 2: return launch_k<MODEL, GM, 2>(m, st);
    case 4: return launch_k<MODEL, GM, 4>(m, st);
    case 8:
        if constexpr (MODEL == M_HPP) return launch_k<MODEL, GM, 8>(m, st);
        return cudaErrorInvalidValue;
    default: return cudaErrorInvalidValue;
    }
}

template <int MODEL>
static cudaError_t launch_wave_geom(int gm, const MultiStepArgs &m, cudaStream_t st)
{
    switch (gm) {
    case GEOM_NONE: return launch_wave_depth<MODEL, GEOM_NONE>(m, st);
    case GEOM_NOSLIP: return launch_wave_depth<MODEL, GEOM_NOSLIP>(m, st);
    default: return launch_wave_depth<MODEL, GEOM_FULL>(m, st);
    }
}

// FHP keeps 7 words per time level in registers, so depth 8 would spill.
bool wave_supported(int model, const PlaneGeom &g, int depth)
{
    const bool ok_depth = depth == 2 || depth == 4 || (depth == 8 && model == M_HPP);
    return ok_depth && (g.W % 64) == 0 && g.H >= 2;
}

cudaError_t launch_wave(int model, int gm, const MultiStepArgs &m, cudaStream_t st)
{
    switch (model) {
    case M_HPP: return launch_wave_geom<M_HPP>(gm, m, st);
    case M_FHP_I: return launch_wave_geom<M_FHP_I>(gm, m, st);
    default: return launch_wave_geom<M_FHP_II>(gm, m, st);
    }
}

}  // namespace lgca_gpu
