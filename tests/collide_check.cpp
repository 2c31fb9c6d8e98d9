// Host check of the bit-sliced collision rules of the CUDA kernels
// (lgca_gb300/csrc/collide.cuh): prints, for every model, chirality p and
// input state s (bit d = channel d), the output state computed on 64-bit
// words.  tests/test_collide_circuit.py compiles it with g++ and compares
// the table with the reference's (tests/golden/collide_tables.npz).
#include "../lgca_gb300/csrc/collide.cuh"
#include <cstdio>
using namespace lgca_gpu;

template <int M> static void dump()
{
    constexpr int D = ModelTraits<M>::D;
    for (int p = 0; p < 2; ++p)
        for (int s = 0; s < (1 << D); ++s) {
            // the state sits at bit 37 of each word; other bits carry noise
            // that must not leak into bit 37
            uint64_t n[7];
            for (int d = 0; d < 7; ++d)
                n[d] = (((uint64_t)((s >> d) & 1)) << 37) | (0x9E3779B97F4A7C15ULL * (d + 3) & ~(1ULL << 37));
            const uint64_t pw = ((uint64_t)p << 37) | (0xC2B2AE3D27D4EB4FULL & ~(1ULL << 37));
            collide<M>(n, pw);
            int out = 0;
            for (int d = 0; d < D; ++d) out |= (int)((n[d] >> 37) & 1) << d;
            std::printf("%d %d %d %d\n", M, p, s, out);
        }
}

int main()
{
    dump<M_HPP>();
    dump<M_FHP_I>();
    dump<M_FHP_II>();
    dump<M_FHP_III>();
    return 0;
}
