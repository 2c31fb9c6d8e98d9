/*
 * Counter-based random numbers shared by the CUDA kernels, the host code and
 * the CPU oracle.  Every random decision of a lattice-gas run is a pure
 * function of (seed, stream, counter, index), so the same run gives the same
 * bits on the GPU, on the CPU and inside the reference OMP_Lattice harness.
 *
 * The generator is SplitMix64 (G. L. Steele, D. Lea, C. H. Flood, "Fast
 * splittable pseudorandom number generators", OOPSLA 2014): the state advances
 * by the odd constant GAMMA and each output is the state passed through the
 * 64-bit finaliser below (the "mix64variant13" constants published with it).
 * Instead of a sequential state we key one SplitMix64 sequence per
 * (seed, stream, counter) and jump straight to element `index`:
 *
 *   key(seed, stream, t) = mix(mix(seed ^ (stream * STREAM_MUL)) + t * GAMMA)
 *   draw(key, index)     = mix(key + index * GAMMA)
 *
 * Uses on the lattice (W x H sites, x fastest, t = global step number):
 *   chirality  bit (x & 63) of draw(key(seed, CHIR, t), (y << 32) | (x >> 6))
 *              -> one call yields the chirality of 64 consecutive sites;
 *   forcing    u = draw(key(seed, FORCE, t), (y << 32) | x) >> 32,
 *              the site flips when u < thr (thr = floor(p * 2^32));
 *   init       channel d of site (x, y) is occupied when
 *              draw(key(seed, INIT, d), (y << 32) | x) >> 32 < thr_d;
 *   body force the reference's sequential random-cell forcing draws its
 *              k-th candidate of call c as
 *              (draw(key(seed, FSEQ, c), k) >> 33) % num_cells.
 *
 * Plain C99 so that it compiles as C, C++ and CUDA (host and device).
 */
#ifndef LGCA_RNG_H_
#define LGCA_RNG_H_

#include <stdint.h>

#if defined(__CUDACC__)
#define LGCA_HD __host__ __device__ __forceinline__
#else
#define LGCA_HD static inline
#endif

#define LGCA_RNG_GAMMA      0x9e3779b97f4a7c15ULL
#define LGCA_RNG_STREAM_MUL 0xd1b54a32d192ed03ULL

/* Stream identifiers: one independent sequence per kind of random decision. */
enum {
    LGCA_STREAM_CHIR  = 1, /* FHP collision chirality, 64 sites per draw   */
    LGCA_STREAM_FORCE = 2, /* forcing-column Bernoulli flips, one per site */
    LGCA_STREAM_INIT  = 3, /* initial occupation, counter = channel        */
    LGCA_STREAM_FSEQ  = 4  /* random-cell body force candidates            */
};

LGCA_HD uint64_t lgca_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

LGCA_HD uint64_t lgca_rng_key(uint64_t seed, uint32_t stream, uint64_t t)
{
    return lgca_mix64(lgca_mix64(seed ^ ((uint64_t)stream * LGCA_RNG_STREAM_MUL)) +
                      t * LGCA_RNG_GAMMA);
}

LGCA_HD uint64_t lgca_rng_draw(uint64_t key, uint64_t index)
{
    return lgca_mix64(key + index * LGCA_RNG_GAMMA);
}

/* Index of site (x, y) / word (w, y) for lgca_rng_draw. */
LGCA_HD uint64_t lgca_rng_index(uint32_t y, uint32_t x)
{
    return ((uint64_t)y << 32) | (uint64_t)x;
}

/* Threshold for a Bernoulli(p) draw compared against the top 32 bits of a
 * draw: occupied/flipped iff (draw >> 32) < thr.  thr lies in [0, 2^32]. */
static inline uint64_t lgca_prob_threshold(double p)
{
    if (!(p > 0.0)) return 0;
    if (p >= 1.0) return 4294967296ULL;
    return (uint64_t)(p * 4294967296.0);
}

#endif /* LGCA_RNG_H_ */
