/*
 * CPU oracle for the lattice-gas hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference OMP_Lattice algorithm (keva92/lgca,
 * src/omp_lattice.cpp, src/lgca_models.h, src/lattice.cpp) on the reference's
 * own state format: one byte per cell, bit d = occupation of channel d
 * (src/lgca_bitset.h:31-245 with bit index dir + 8*cell, src/lattice.cpp:212).
 *
 * Only the tests, the smoke check and the benchmark's CPU-baseline leg use
 * this library.  The product path (lgca_gb300, liblgca_gpu.so) never links or
 * calls it.  Its results are pinned against the reference itself, compiled
 * with hooks into oracle/_ref (see oracle/ref_harness.cpp) and against the
 * golden fixtures under tests/golden/.
 *
 * Randomness follows include/lgca/rng.h, the generator shared with the GPU
 * code, so chirality, forcing and initial occupation are reproducible.
 */
#ifndef LGCA_ORACLE_H_
#define LGCA_ORACLE_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Models and cell types carry the reference's enum values
 * (src/lgca_common.h:49-60). */
enum { OR_HPP = 0, OR_FHP_I = 1, OR_FHP_II = 2, OR_FHP_III = 3 };
enum { OR_FLUID = 0, OR_SOLID_NO_SLIP = 1, OR_SOLID_SLIP = 2 };

typedef struct {
    int model;            /* OR_HPP .. OR_FHP_III                             */
    int W, H;             /* lattice dimensions (x fastest)                    */
    uint64_t seed;        /* seed of the shared counter-based generator        */
    const uint8_t *chir;  /* NULL: chirality from the generator; else W*H      */
                          /* bytes (0/1) used every step (the reference's      */
                          /* frozen m_rnd_cpu field)                           */
    int force_x;          /* forcing column, -1 for none                       */
    uint64_t force_thr;   /* Bernoulli threshold of a flip (lgca_prob_threshold)*/
} oracle_cfg;

int oracle_num_dir(int model);

/* Collision of one cell: byte in (bit d = channel d), chirality p -> byte out. */
uint8_t oracle_collide(int model, uint8_t in, int p);

/* Forcing column: per-site Bernoulli W->E reversal applied to the state
 * before the pull of step t (same rule as src/omp_lattice.cpp:293-318). */
void oracle_force_column(const oracle_cfg *cfg, const int32_t *types, uint8_t *state,
                         uint64_t t);

/* One pull-stream + collide step (src/omp_lattice.cpp:100-249): reads
 * `state`, writes `next`.  Chirality of step t comes from cfg. */
void oracle_collide_and_propagate(const oracle_cfg *cfg, const int32_t *types,
                                  const uint8_t *state, uint8_t *next, uint64_t t);

/* `nsteps` full steps starting at global step t0 (forcing, then step, then
 * swap).  The result is left in `state`; `tmp` is scratch of the same size. */
void oracle_run(const oracle_cfg *cfg, const int32_t *types, uint8_t *state, uint8_t *tmp,
                uint64_t t0, int nsteps);

/* Bernoulli initial occupation on fluid cells: channel d occupied with
 * probability p_move (moving channels) or p_rest (rest channel 6). */
void oracle_init_bernoulli(int model, int W, int H, const int32_t *types, uint8_t *state,
                           uint64_t seed, double p_move, double p_rest);

/* Exact integer block sums over non-overlapping B x B blocks (edge blocks
 * clipped).  N = particles; Jx2 = x momentum in units of 1/2; Jy = y momentum
 * in units of sin(60 deg) for FHP and of 1 for HPP.  Outputs Hb*Wb int32. */
void oracle_block_sums(int model, int W, int H, const uint8_t *state, int B,
                       int32_t *N, int32_t *Jx2, int32_t *Jy);

/* src/omp_lattice.cpp:360-394: per-cell density and FP32 momentum. */
void oracle_cell_post_process(int model, int W, int H, const uint8_t *state,
                              float *cell_density, float *cell_momentum);

/* src/omp_lattice.cpp:397-454: coarse means over the reference's window. */
void oracle_mean_post_process(int W, int H, int r, const float *cell_density,
                              const float *cell_momentum, float *mean_density,
                              float *mean_momentum);

/* src/lattice.cpp:180-195 */
uint64_t oracle_count_particles(int W, int H, const uint8_t *state);

/* src/omp_lattice.cpp:508-557, summed in cell order in double. */
void oracle_mean_velocity(int W, int H, const int32_t *types, const float *cell_density,
                          const float *cell_momentum, float *ux, float *uy);

/* src/omp_lattice.cpp:254-346 with rand() replaced by the FSEQ stream of
 * call `call`.  bf_dir is 'x', 'y' or 0.  Returns the number of reverted
 * particles. */
unsigned oracle_apply_body_force(int model, int W, int H, const int32_t *types,
                                 uint8_t *state, uint64_t seed, uint64_t call, int forcing,
                                 int bf_dir);

/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int oracle_threads(void);

#ifdef __cplusplus
}
#endif

#endif /* LGCA_ORACLE_H_ */
