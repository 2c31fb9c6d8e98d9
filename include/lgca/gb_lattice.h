/*
 * gb_lattice.h -- C++ host class with the interface of the reference's
 * Lattice<Model> (keva92/lgca src/lattice.h:32-238), running on the GB300
 * engine through the C ABI of lgca_gpu.h.
 *
 * Header-only; link with -llgca_gpu.  An application written against the
 * reference class (`Lattice<MODEL>* l = new OMP_Lattice<MODEL>(case, Re, Ma,
 * r)`) uses `GB_Lattice<MODEL>` with the same member functions, argument
 * meanings, printed messages and abort-on-invalid-input behaviour.
 *
 * State authority: the geometry setters and the initialisers work on host
 * arrays, as in the reference; they are uploaded before the next GPU call.
 * Stepping, forcing and reductions run on the GPU.  copy_data_to_output_buffer()
 * downloads the state into the output buffer, which post_process() reads, as
 * the reference's post-processing reads its output buffer
 * (src/omp_lattice.cpp:376).
 *
 * Randomness: initial occupation, chirality and body-force draws come from
 * the counter-based generator of rng.h with the lattice seed (default 0), so
 * runs are reproducible; the reference uses rand() (src/utils.h:119-122).
 */
#ifndef LGCA_GB_LATTICE_H_
#define LGCA_GB_LATTICE_H_

#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../lgca_gpu.h"
#include "gb_device.h"
#include "rng.h"

namespace lgca_gb300 {

typedef float Real;  // src/lgca_common.h:46

enum class Model { HPP = 0, FHP_I = 1, FHP_II = 2, FHP_III = 3 };  // src/lgca_common.h:49-54
enum class CellType { FLUID = 0, SOLID_NO_SLIP = 1, SOLID_SLIP = 2 };  // src/lgca_common.h:56-60

template <Model M> struct ModelInfo;
template <> struct ModelInfo<Model::HPP> { static constexpr unsigned NUM_DIR = 4; static constexpr int INV0 = 2; };
template <> struct ModelInfo<Model::FHP_I> { static constexpr unsigned NUM_DIR = 6; static constexpr int INV0 = 3; };
template <> struct ModelInfo<Model::FHP_II> { static constexpr unsigned NUM_DIR = 7; static constexpr int INV0 = 3; };
template <> struct ModelInfo<Model::FHP_III> { static constexpr unsigned NUM_DIR = 7; static constexpr int INV0 = 3; };

template <Model model_>
class GB_Lattice {
public:
    static constexpr unsigned SPATIAL_DIM = 2;
    static constexpr unsigned NUM_DIR = ModelInfo<model_>::NUM_DIR;

    // Lattice<M>::Lattice (src/lattice.cpp:29-157): dimensions and physical
    // parameters from the test case, then the GPU lattice.
    GB_Lattice(const std::string test_case, const Real Re, const Real Ma_s,
               const int coarse_graining_radius, uint64_t seed = 0)
        : m_seed(seed)
    {
        m_test_case = test_case;
        assert(Re > 1.0e-06);
        m_Re = Re;
        assert(Ma_s > 1.0e-06);
        m_Ma_s = Ma_s;
        m_d = m_rho / NUM_DIR;
        m_nu = 1.0 / 12.0 * 1.0 / (m_d * std::pow((1.0 - m_d), 3.0)) - 1.0 / 8.0;
        m_g = SPATIAL_DIM / (SPATIAL_DIM + 2.0) * (1.0 - 2.0 * m_d) / (1.0 - m_d);
        m_nu_s = m_nu / m_g;
        m_c_s = m_c / std::sqrt(SPATIAL_DIM);
        m_u = m_Ma_s * m_c_s;
        if (test_case == "pipe") {
            m_dim_y = (int)((Re * m_nu_s) / m_u + 0.5);
        } else if (test_case == "karman") {
            Real diameter = (Re * m_nu_s) / m_u;
            m_dim_y = (int)(3.0 * diameter + 0.5);
        } else if (test_case == "collision") {
            m_dim_y = 8;
        } else if (test_case == "diffusion" || test_case == "periodic" || test_case == "box") {
            m_dim_y = (int)Re;
        } else {
            printf("ERROR in Lattice::Lattice(): Invalid test case %s.\n", test_case.c_str());
            abort();
        }
        const int r = coarse_graining_radius;
        m_dim_y += (2 * r) - (m_dim_y % (2 * r));
        if (test_case == "pipe" || test_case == "karman" || test_case == "collision")
            m_dim_x = 2 * m_dim_y;
        else
            m_dim_x = m_dim_y;
        if (test_case == "collision") m_dim_x++;
        m_bf_dir = (test_case == "pipe" || test_case == "karman") ? 'x' : 0;
        init_storage(r);
        print_info();
    }

    // Extension: a lattice of explicit dimensions (the reference derives them
    // from the test case only).
    GB_Lattice(unsigned dim_x, unsigned dim_y, int coarse_graining_radius, uint64_t seed = 0,
               char bf_dir = 0)
        : m_seed(seed)
    {
        m_test_case = "custom";
        m_Re = 1.0f;
        m_Ma_s = 0.3f;
        m_d = m_rho / NUM_DIR;
        m_nu = 1.0 / 12.0 * 1.0 / (m_d * std::pow((1.0 - m_d), 3.0)) - 1.0 / 8.0;
        m_g = SPATIAL_DIM / (SPATIAL_DIM + 2.0) * (1.0 - 2.0 * m_d) / (1.0 - m_d);
        m_nu_s = m_nu / m_g;
        m_c_s = m_c / std::sqrt(SPATIAL_DIM);
        m_u = m_Ma_s * m_c_s;
        m_dim_x = dim_x;
        m_dim_y = dim_y;
        m_bf_dir = bf_dir;
        init_storage(coarse_graining_radius);
    }

    virtual ~GB_Lattice() = default;

    GB_Lattice(const GB_Lattice &) = delete;
    GB_Lattice &operator=(const GB_Lattice &) = delete;

    // ---- geometry (host map), src/lattice.cpp:219-395
    void apply_cell_type_all(const CellType t)
    {
        for (size_t c = 0; c < m_num_cells; ++c) m_cell_type[c] = t;
        m_dev->mark_types_dirty();
    }
    void apply_boundary_cell_type_east(const CellType t)
    {
        for (size_t c = m_dim_x - 1; c < m_num_cells; c += m_dim_x) m_cell_type[c] = t;
        m_dev->mark_types_dirty();
    }
    void apply_boundary_cell_type_north(const CellType t)
    {
        for (size_t c = m_num_cells - m_dim_x; c < m_num_cells; ++c) m_cell_type[c] = t;
        m_dev->mark_types_dirty();
    }
    void apply_boundary_cell_type_west(const CellType t)
    {
        for (size_t c = 0; c < m_num_cells; c += m_dim_x) m_cell_type[c] = t;
        m_dev->mark_types_dirty();
    }
    void apply_boundary_cell_type_south(const CellType t)
    {
        for (size_t c = 0; c < m_dim_x; ++c) m_cell_type[c] = t;
        m_dev->mark_types_dirty();
    }
    void apply_bc_periodic() { apply_cell_type_all(CellType::FLUID); }
    void apply_bc_reflecting(const std::string bounce_type)
    {
        apply_cell_type_all(CellType::FLUID);
        CellType t;
        if (bounce_type == "back") t = CellType::SOLID_NO_SLIP;
        else if (bounce_type == "forward") t = CellType::SOLID_SLIP;
        else {
            printf("ERROR in apply_bc_reflecting(): Invalid bounce type %s.\n", bounce_type.c_str());
            abort();
        }
        apply_boundary_cell_type_east(t);
        apply_boundary_cell_type_north(t);
        apply_boundary_cell_type_west(t);
        apply_boundary_cell_type_south(t);
    }
    void apply_bc_pipe()
    {
        apply_cell_type_all(CellType::FLUID);
        apply_boundary_cell_type_north(CellType::SOLID_NO_SLIP);
        apply_boundary_cell_type_south(CellType::SOLID_NO_SLIP);
    }
    // Disc of diameter dim_y/3 at (dim_x/6, dim_y/2), src/lattice.cpp:252-280.
    void apply_bc_karman_vortex_street()
    {
        apply_bc_pipe();
        const int center_x = m_dim_x / 6;
        const int center_y = m_dim_y / 2 + 1 / 10 * m_dim_y;
        const Real diameter = m_dim_y / 3;
        for (size_t cell = 0; cell < m_num_cells; ++cell) {
            const int pos_x = cell % m_dim_x, pos_y = cell / m_dim_x;
            const Real dist = std::sqrt(std::pow((pos_x - center_x), 2.0) + std::pow((pos_y - center_y), 2.0));
            if (dist < (diameter / 2.0)) m_cell_type[cell] = CellType::SOLID_NO_SLIP;
        }
        m_dev->mark_types_dirty();
    }

    // ---- initialisers (host state), src/lattice.cpp:165-308,463-496
    void init_zero() {}  // the state starts empty (src/lattice.cpp:166-170)
    void init_random() { init_bernoulli_fluid(nullptr); }
    void init_single(const std::vector<size_t> occupied_nodes)
    {
        pull_state();
        init_zero();
        for (size_t n : occupied_nodes) m_node_state[n / 8] |= (uint8_t)(1u << (n % 8));
        m_dev->mark_state_dirty();
    }
    void init_single_collision()
    {
        std::vector<size_t> nodes;
        nodes.push_back((m_dim_x * m_dim_y / 2 + 1) * 8);
        nodes.push_back((m_dim_x * m_dim_y / 2 + 5) * 8 + ModelInfo<model_>::INV0);
        init_single(nodes);
    }
    void init_diffusion()
    {
        const int center_x = m_dim_x / 2, center_y = m_dim_y / 2;
        const Real diameter = m_dim_y / 4;
        std::vector<uint8_t> in_disc(m_num_cells, 0);
        for (size_t cell = 0; cell < m_num_cells; ++cell) {
            const int pos_x = cell % m_dim_x, pos_y = cell / m_dim_x;
            const Real dist = std::sqrt(std::pow((pos_x - center_x), 2.0) + std::pow((pos_y - center_y), 2.0));
            in_disc[cell] = dist < (diameter / 2.0);
        }
        init_bernoulli_fluid(in_disc.data());
    }

    // ---- queries
    unsigned long get_n_particles()
    {
        push();
        m_num_particles = m_dev->count_particles();
        return (unsigned long)m_num_particles;
    }
    // Bitset::print of the state (src/lgca_bitset.h:198-203)
    void print()
    {
        pull_state();
        for (size_t i = 0; i < m_num_cells * 8; ++i) printf("%d ", (m_node_state[i / 8] >> (i % 8)) & 1);
        printf("\n");
    }
    void print_info()
    {
        printf("Parameter for test case \"%s\":\n", m_test_case.c_str());
        printf("\n");
        printf("Reynolds number             Re   = %10.2f\n", m_Re);
        printf("Mach number                 Ma   = %10.2f\n", m_Ma_s);
        printf("Density                     rho  = %10.2f\n", m_rho);
        printf("Velocity                    u    = %10.2f\n", m_u);
        printf("Sound speed                 c    = %10.2f\n", m_c);
        printf("Scaled sound speed          c_s  = %10.2f\n", m_c_s);
        printf("Viscosity                   nu   = %10.2f\n", m_nu);
        printf("Scaled viscosity            nu_s = %10.2f\n", m_nu_s);
        printf("Galilean breaking factor    g    = %10.2f\n", m_g);
        printf("\n");
        printf("Number of cells in x direction: %d\n", m_dim_x);
        printf("Number of cells in y direction: %d\n", m_dim_y);
        printf("\n");
        printf("Number of coarse cells in x direction: %d\n", m_coarse_dim_x);
        printf("Number of coarse cells in y direction: %d\n", m_coarse_dim_y);
        printf("\n");
    }
    size_t get_equilibrium_forcing()  // src/lattice.cpp:455-461
    {
        Real forcing = (8.0 * m_nu_s * m_Ma_s * m_c_s) / std::pow((Real)m_dim_y, 2.0);
        return std::ceil(0.5 * m_num_cells * forcing);
    }
    size_t get_initial_forcing() { return (size_t)(0.01 * m_num_cells); }  // src/lattice.cpp:446-451

    // ---- the backend half (OMP_Lattice<M>, src/omp_lattice.h:27-78)
    void setup_parallel()  // src/omp_lattice.cpp:492-505 prints the thread count
    {
        printf("GB300 configuration parameters: Executing calculation on the current CUDA device.\n\n");
    }
    // src/omp_lattice.cpp:100-249; the argument is ignored as in the reference
    void collide_and_propagate(const bool p = false)
    {
        (void)p;
        push();
        m_dev->step(1);
    }
    // Extension: n steps in one call (the engine may fuse them).
    void collide_and_propagate_n(int nsteps)
    {
        push();
        m_dev->step(nsteps);
    }
    std::vector<Real> get_mean_velocity()  // src/omp_lattice.cpp:508-557
    {
        push();
        return m_dev->mean_velocity();
    }
    void apply_body_force(const int forcing)  // src/omp_lattice.cpp:254-346
    {
        push();
        m_dev->body_force(forcing, m_bf_dir);
    }
    // src/omp_lattice.cpp:349-454, on the output buffer
    void post_process()
    {
        m_dev->post_process(m_node_state_out.data(), (int)m_coarse_graining_radius,
                            m_cell_density.data(), m_cell_momentum.data(), m_mean_density.data(),
                            m_mean_momentum.data());
    }
    void copy_data_to_device()
    {
        m_dev->mark_types_dirty();
        m_dev->mark_state_dirty();
        push();
    }
    void copy_data_from_device() { pull_state(); }
    void copy_data_to_output_buffer()
    {
        pull_state();
        m_node_state_out = m_node_state;
        m_dev->output_taken();
    }

    // ---- getters (src/lattice.h:213-237)
    Real nu_s() const { return m_nu_s; }
    Real c_s() const { return m_c_s; }
    Real u() const { return m_u; }
    unsigned int dim_x() const { return m_dim_x; }
    unsigned int dim_y() const { return m_dim_y; }
    size_t num_cells() const { return m_num_cells; }
    unsigned int coarse_dim_x() const { return m_coarse_dim_x; }
    unsigned int coarse_dim_y() const { return m_coarse_dim_y; }
    size_t num_coarse_cells() const { return m_num_coarse_cells; }
    Real *cell_density() { return m_cell_density.data(); }
    const Real *cell_density() const { return m_cell_density.data(); }
    Real *mean_density() { return m_mean_density.data(); }
    const Real *mean_density() const { return m_mean_density.data(); }
    Real *cell_momentum() { return m_cell_momentum.data(); }
    const Real *cell_momentum() const { return m_cell_momentum.data(); }
    Real *mean_momentum() { return m_mean_momentum.data(); }
    const Real *mean_momentum() const { return m_mean_momentum.data(); }
    Real cell_density(const int x, const int y) { return m_cell_density[y * m_dim_x + x]; }
    Real mean_density(const int x, const int y) { return m_mean_density[y * m_dim_x + x]; }

    // ---- extensions of this engine
    lgca_handle handle() { push(); return m_dev->handle(); }
    uint64_t seed() const { return m_seed; }
    char bf_dir() const { return m_bf_dir; }
    uint64_t last_reverted() const { return m_dev->last_reverted(); }
    const uint8_t *node_state() { pull_state(); return m_node_state.data(); }
    const CellType *cell_types() const { return m_cell_type.data(); }
    void set_forcing_column(int x, double p)
    {
        m_dev->check(lgca_set_forcing_column(m_dev->handle(), x, p), "set_forcing_column");
    }
    void set_temporal_depth(int depth)
    {
        m_dev->check(lgca_set_temporal_depth(m_dev->handle(), depth), "set_temporal_depth");
    }
    // Integer B x B block sums (N, Jx2, Jy), each ceil(H/B) x ceil(W/B).
    void block_sums(int B, std::vector<int32_t> &N, std::vector<int32_t> &Jx2, std::vector<int32_t> &Jy)
    {
        push();
        const size_t nb = (size_t)((m_dim_x + B - 1) / B) * ((m_dim_y + B - 1) / B);
        N.resize(nb);
        Jx2.resize(nb);
        Jy.resize(nb);
        m_dev->check(lgca_block_sums(m_dev->handle(), B, N.data(), Jx2.data(), Jy.data()), "block_sums");
    }

protected:
    void init_storage(int r)
    {
        assert(m_dim_x > 0 && m_dim_y > 0);
        if (model_ != Model::HPP) assert(m_dim_y % 2 == 0);
        m_num_cells = (size_t)m_dim_x * m_dim_y;
        m_num_nodes = m_num_cells * NUM_DIR;
        m_num_particles = 0;
        assert(r > 0);
        m_coarse_graining_radius = r;
        m_coarse_dim_x = m_dim_x / (2 * r);
        m_coarse_dim_y = m_dim_y / (2 * r);
        m_num_coarse_cells = (size_t)m_coarse_dim_x * m_coarse_dim_y;
        m_cell_type.assign(m_num_cells, CellType::FLUID);
        m_node_state.assign(m_num_cells, 0);
        m_node_state_out.assign(m_num_cells, 0);
        m_cell_density.assign(m_num_cells, 0.0f);
        m_cell_momentum.assign(2 * m_num_cells, 0.0f);
        m_mean_density.assign(m_num_coarse_cells, 0.0f);
        m_mean_momentum.assign(2 * m_num_coarse_cells, 0.0f);
        m_dev.reset(new DeviceLattice((int)model_, m_dim_x, m_dim_y, m_seed));
        m_dev->handle();  // the GPU lattice exists from construction on
    }
    // Bernoulli(1/NUM_DIR) per channel of FLUID cells (src/lattice.cpp:198-217,
    // :465-496) from the INIT stream, as lgca_init_random draws it; other
    // cells keep their state, as in the reference.
    void init_bernoulli_fluid(const uint8_t *mask)
    {
        pull_state();
        const uint64_t thr = lgca_prob_threshold(1.0 / NUM_DIR);
        uint64_t keys[8];
        for (unsigned d = 0; d < NUM_DIR; ++d) keys[d] = lgca_rng_key(m_seed, LGCA_STREAM_INIT, d);
        for (size_t cell = 0; cell < m_num_cells; ++cell) {
            if (m_cell_type[cell] != CellType::FLUID || (mask && !mask[cell])) continue;
            const uint32_t x = cell % m_dim_x, y = cell / m_dim_x;
            uint8_t s = m_node_state[cell];
            for (unsigned d = 0; d < NUM_DIR; ++d) {
                const bool on = (lgca_rng_draw(keys[d], lgca_rng_index(y, x)) >> 32) < thr;
                s = on ? (uint8_t)(s | (1u << d)) : (uint8_t)(s & ~(1u << d));
            }
            m_node_state[cell] = s;
        }
        m_dev->mark_state_dirty();
    }
    // host -> device when the host arrays changed
    void push() { m_dev->push(m_cell_type.data(), m_node_state.data()); }
    // device -> host when the device state moved on
    void pull_state()
    {
        push();
        m_dev->pull(m_node_state.data());
    }
    unsigned int m_dim_x = 0, m_dim_y = 0;
    size_t m_num_cells = 0, m_num_nodes = 0, m_num_particles = 0;
    unsigned int m_coarse_graining_radius = 1, m_coarse_dim_x = 0, m_coarse_dim_y = 0;
    size_t m_num_coarse_cells = 0;
    std::string m_test_case;
    const Real m_rho = 1.0, m_c = 1.0;
    Real m_Re = 0, m_Ma_s = 0, m_d = 0, m_nu = 0, m_g = 0, m_nu_s = 0, m_c_s = 0, m_u = 0;
    char m_bf_dir = 0;
    uint64_t m_seed = 0;

    std::vector<CellType> m_cell_type;
    std::vector<uint8_t> m_node_state, m_node_state_out;  // one byte per cell, bit d = channel d
    std::vector<Real> m_cell_density, m_mean_density, m_cell_momentum, m_mean_momentum;

    std::unique_ptr<DeviceLattice> m_dev;  // the GPU lattice and its upload state
};

}  // namespace lgca_gb300

#endif /* LGCA_GB_LATTICE_H_ */
