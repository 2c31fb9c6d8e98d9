/*
 * Hook harness around the UNMODIFIED reference OMP_Lattice -- TEST
 * INFRASTRUCTURE ONLY.
 *
 * Compiled by oracle/Makefile (target `ref`) directly from the reference sources where
 * they lie (src/lattice.cpp and src/omp_lattice.cpp are #included below, not
 * copied) into oracle/_ref/libref_oracle.so.  The tests use it to pin the C
 * restatement in oracle/lgca_oracle.c and to generate tests/golden/.
 *
 * Hooks (no reference line is edited):
 *  - access: `private`/`protected` are defined to `public` while the two
 *    reference translation units are compiled here, so the harness can size
 *    the lattice to any W x H (the reference derives its dimensions from the
 *    test case, src/lattice.cpp:69-122) and reach the state, the cell-type
 *    map and the chirality field (src/lattice.h:80,88,111);
 *  - chirality: before every step m_rnd_cpu is refilled from the shared
 *    counter-based generator (include/lgca/rng.h), or set once to a given
 *    frozen field (the reference's own semantics, src/omp_lattice.cpp:84,198);
 *  - forcing column: applied to m_node_state_cpu before each step;
 *  - random-cell body force: `rand` is defined to lgca_ref_rand while
 *    src/omp_lattice.cpp is compiled, so the draws of apply_body_force
 *    (src/omp_lattice.cpp:269) come from the generator's FSEQ stream.
 */
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <cassert>
#include <chrono>
#include <fstream>
#include <iostream>
#include <limits>
#include <string>
#include <vector>
#include <unistd.h>
#include <fcntl.h>
#include <omp.h>
#include <tbb/spin_mutex.h>
#include <tbb/blocked_range.h>
#include <tbb/parallel_for.h>
#include "tclap/CmdLine.h"

#include "../include/lgca/rng.h"

static uint64_t g_rand_key = 0;
static uint64_t g_rand_counter = 0;

/* rand() of the reference's body-force loop: 31-bit draws of the FSEQ stream. */
static int lgca_ref_rand()
{
    return (int)(lgca_rng_draw(g_rand_key, g_rand_counter++) >> 33);
}

#define private public
#define protected public
#define rand lgca_ref_rand
#include "lattice.cpp"
#include "omp_lattice.cpp"
#undef rand
#undef protected
#undef private

using namespace lgca;

namespace {

/* Silence the reference constructor's parameter printout (src/lattice.cpp:156). */
struct Quiet {
    int saved;
    Quiet() { fflush(stdout); saved = dup(1); int dn = open("/dev/null", O_WRONLY); dup2(dn, 1); close(dn); }
    ~Quiet() { fflush(stdout); dup2(saved, 1); close(saved); }
};

template <Model M>
OMP_Lattice<M> *make_lattice(int W, int H, int r)
{
    OMP_Lattice<M> *L;
    {
        Quiet q;
        L = new OMP_Lattice<M>("periodic", 64.0f, 0.3f, 1);
    }
    L->m_dim_x = (unsigned)W;
    L->m_dim_y = (unsigned)H;
    L->m_num_cells = (size_t)W * (size_t)H;
    L->m_num_nodes = L->m_num_cells * L->NUM_DIR;
    L->m_coarse_graining_radius = (unsigned)r;
    L->m_coarse_dim_x = (unsigned)(W / (2 * r));
    L->m_coarse_dim_y = (unsigned)(H / (2 * r));
    L->m_num_coarse_cells = (size_t)L->m_coarse_dim_x * L->m_coarse_dim_y;
    L->free_memory();
    L->allocate_memory();
    delete L->m_model;
    L->m_model = new ModelDescriptor<M>((unsigned)W, (unsigned)H);
    for (size_t c = 0; c < L->m_num_cells; ++c) L->m_cell_type_cpu[c] = CellType::FLUID;
    return L;
}

template <Model M>
void load_state(OMP_Lattice<M> *L, const int32_t *types, const uint8_t *state)
{
    for (size_t c = 0; c < L->m_num_cells; ++c) {
        L->m_cell_type_cpu[c] = types ? (CellType)types[c] : CellType::FLUID;
        L->m_node_state_cpu(c) = state[c];
    }
}

template <Model M>
void store_state(OMP_Lattice<M> *L, uint8_t *state)
{
    for (size_t c = 0; c < L->m_num_cells; ++c) state[c] = L->m_node_state_cpu(c);
}

template <Model M>
int run_t(int W, int H, const int32_t *types, uint8_t *state, uint64_t seed, int chir_mode,
          const uint8_t *chir, int force_x, uint64_t force_thr, uint64_t t0, int nsteps)
{
    OMP_Lattice<M> *L = make_lattice<M>(W, H, 1);
    load_state(L, types, state);
    const size_t n = L->m_num_cells;
    if (chir_mode == 1)
        for (size_t c = 0; c < n; ++c) L->m_rnd_cpu[c] = chir[c] != 0;
    const int west_ch = M == Model::HPP ? 2 : 3;
    for (int s = 0; s < nsteps; ++s) {
        const uint64_t t = t0 + (uint64_t)s;
        if (chir_mode == 0) {
            const uint64_t key = lgca_rng_key(seed, LGCA_STREAM_CHIR, t);
            /* m_rnd_cpu packs 8 cells per byte: rows may be split across
               threads only when no byte straddles two rows */
#pragma omp parallel for schedule(static) if (W % 8 == 0)
            for (int y = 0; y < H; ++y) {
                uint64_t w = 0;
                for (int x = 0; x < W; ++x) {
                    if ((x & 63) == 0)
                        w = lgca_rng_draw(key, lgca_rng_index((uint32_t)y, (uint32_t)(x >> 6)));
                    L->m_rnd_cpu[(size_t)y * W + x] = ((w >> (x & 63)) & 1u) != 0;
                }
            }
        }
        if (force_x >= 0 && force_x < W && force_thr > 0) {
            const uint64_t key = lgca_rng_key(seed, LGCA_STREAM_FORCE, t);
            for (int y = 0; y < H; ++y) {
                const size_t cell = (size_t)y * W + force_x;
                if (L->m_cell_type_cpu[cell] != CellType::FLUID) continue;
                uint64_t u = lgca_rng_draw(key, lgca_rng_index((uint32_t)y, (uint32_t)force_x)) >> 32;
                if (u >= force_thr) continue;
                if (!L->m_node_state_cpu[0 + cell * 8] && L->m_node_state_cpu[west_ch + cell * 8]) {
                    L->m_node_state_cpu[0 + cell * 8] = true;
                    L->m_node_state_cpu[west_ch + cell * 8] = false;
                }
            }
        }
        L->collide_and_propagate(false);
    }
    store_state(L, state);
    delete L;
    return 0;
}

template <Model M>
int post_t(int W, int H, int r, const uint8_t *state, float *cd, float *cm, float *md, float *mm)
{
    OMP_Lattice<M> *L = make_lattice<M>(W, H, r);
    load_state(L, nullptr, state);
    L->copy_data_to_output_buffer();
    L->post_process();
    const size_t n = L->m_num_cells, nc = L->m_num_coarse_cells;
    memcpy(cd, L->m_cell_density_cpu, n * sizeof(float));
    memcpy(cm, L->m_cell_momentum_cpu, 2 * n * sizeof(float));
    memcpy(md, L->m_mean_density_cpu, nc * sizeof(float));
    memcpy(mm, L->m_mean_momentum_cpu, 2 * nc * sizeof(float));
    delete L;
    return 0;
}

template <Model M>
unsigned body_force_t(int W, int H, const int32_t *types, uint8_t *state, uint64_t seed,
                      uint64_t call, int forcing, int bf_dir)
{
    OMP_Lattice<M> *L = make_lattice<M>(W, H, 1);
    load_state(L, types, state);
    L->m_bf_dir = (char)bf_dir;
    g_rand_key = lgca_rng_key(seed, LGCA_STREAM_FSEQ, call);
    g_rand_counter = 0;
    L->apply_body_force(forcing);
    store_state(L, state);
    delete L;
    return 0; /* the reference does not report how many particles it reverted */
}

template <Model M>
void mean_velocity_t(int W, int H, const int32_t *types, const uint8_t *state, float *u)
{
    OMP_Lattice<M> *L = make_lattice<M>(W, H, 1);
    load_state(L, types, state);
    L->copy_data_to_output_buffer();
    L->post_process();
    std::vector<Real> v = L->get_mean_velocity();
    u[0] = v[0];
    u[1] = v[1];
    delete L;
}

template <Model M>
uint64_t count_t(int W, int H, const uint8_t *state)
{
    OMP_Lattice<M> *L = make_lattice<M>(W, H, 1);
    load_state(L, nullptr, state);
    uint64_t n = L->get_n_particles();
    delete L;
    return n;
}

template <Model M>
int dims_t(const char *test_case, float Re, float Ma, int r, int *out_i, float *out_f)
{
    OMP_Lattice<M> *L;
    {
        Quiet q;
        L = new OMP_Lattice<M>(test_case, Re, Ma, r);
    }
    out_i[0] = (int)L->dim_x();
    out_i[1] = (int)L->dim_y();
    out_i[2] = (int)L->coarse_dim_x();
    out_i[3] = (int)L->coarse_dim_y();
    out_i[4] = (int)L->get_initial_forcing();
    out_i[5] = (int)L->get_equilibrium_forcing();
    out_i[6] = (int)L->m_bf_dir;
    out_f[0] = L->nu_s();
    out_f[1] = L->c_s();
    out_f[2] = L->u();
    delete L;
    return 0;
}

template <Model M>
int geometry_t(int W, int H, const char *bc, int32_t *types)
{
    OMP_Lattice<M> *L = make_lattice<M>(W, H, 1);
    std::string s(bc);
    if (s == "periodic") L->apply_bc_periodic();
    else if (s == "pipe") L->apply_bc_pipe();
    else if (s == "karman") L->apply_bc_karman_vortex_street();
    else if (s == "reflecting_back") L->apply_bc_reflecting("back");
    else if (s == "reflecting_forward") L->apply_bc_reflecting("forward");
    else { delete L; return -1; }
    for (size_t c = 0; c < L->m_num_cells; ++c) types[c] = (int32_t)L->m_cell_type_cpu[c];
    delete L;
    return 0;
}

template <Model M>
int init_t(int W, int H, const char *what, uint8_t *state)
{
    OMP_Lattice<M> *L = make_lattice<M>(W, H, 1);
    std::string s(what);
    if (s == "single_collision") L->init_single_collision();
    else { delete L; return -1; }
    store_state(L, state);
    delete L;
    return 0;
}

} // namespace

#define DISPATCH(model, fn, args)                                    \
    switch (model) {                                                 \
    case 0: return fn<Model::HPP> args;                              \
    case 1: return fn<Model::FHP_I> args;                            \
    case 2: return fn<Model::FHP_II> args;                           \
    default: return fn<Model::FHP_III> args;                         \
    }

template <Model M> static int collide_t(int in, int p)
{
    unsigned char a[8], b[8];
    for (int d = 0; d < 8; ++d) a[d] = b[d] = (unsigned char)((in >> d) & 1);
    ModelDescriptor<M>::collide(a, b, p != 0);
    int out = 0;
    for (int d = 0; d < (int)ModelDescriptor<M>::NUM_DIR; ++d) out |= (b[d] & 1) << d;
    return out;
}

extern "C" {

int ref_collide(int model, int in, int p) { DISPATCH(model, collide_t, (in, p)) }

int ref_run(int model, int W, int H, const int32_t *types, uint8_t *state, uint64_t seed,
            int chir_mode, const uint8_t *chir, int force_x, uint64_t force_thr, uint64_t t0,
            int nsteps)
{
    DISPATCH(model, run_t, (W, H, types, state, seed, chir_mode, chir, force_x, force_thr, t0, nsteps))
}

int ref_post_process(int model, int W, int H, int r, const uint8_t *state, float *cd, float *cm,
                     float *md, float *mm)
{
    DISPATCH(model, post_t, (W, H, r, state, cd, cm, md, mm))
}

unsigned ref_body_force(int model, int W, int H, const int32_t *types, uint8_t *state,
                        uint64_t seed, uint64_t call, int forcing, int bf_dir)
{
    DISPATCH(model, body_force_t, (W, H, types, state, seed, call, forcing, bf_dir))
}

uint64_t ref_count_particles(int model, int W, int H, const uint8_t *state)
{
    DISPATCH(model, count_t, (W, H, state))
}

void ref_mean_velocity(int model, int W, int H, const int32_t *types, const uint8_t *state,
                       float *u)
{
    switch (model) {
    case 0: mean_velocity_t<Model::HPP>(W, H, types, state, u); break;
    case 1: mean_velocity_t<Model::FHP_I>(W, H, types, state, u); break;
    case 2: mean_velocity_t<Model::FHP_II>(W, H, types, state, u); break;
    default: mean_velocity_t<Model::FHP_III>(W, H, types, state, u); break;
    }
}

int ref_dims(int model, const char *test_case, float Re, float Ma, int r, int *out_i, float *out_f)
{
    DISPATCH(model, dims_t, (test_case, Re, Ma, r, out_i, out_f))
}

int ref_geometry(int model, int W, int H, const char *bc, int32_t *types)
{
    DISPATCH(model, geometry_t, (W, H, bc, types))
}

int ref_init(int model, int W, int H, const char *what, uint8_t *state)
{
    DISPATCH(model, init_t, (W, H, what, state))
}

} // extern "C"
