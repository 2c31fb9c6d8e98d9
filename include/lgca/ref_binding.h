/*
 * ref_binding.h -- lgca::GB_Lattice<Model>, a backend of the reference's own
 * abstract class lgca::Lattice<Model> (keva92/lgca src/lattice.h:32-238) that
 * runs on the GB300 engine through the C ABI of lgca_gpu.h.
 *
 * The reference's apps hold a Lattice<MODEL>* and create the backend in one
 * line (apps/pipe/pipe_viewer.cpp:46: `new OMP_Lattice<MODEL>("pipe", m_Re,
 * m_Ma, CG_RADIUS)`).  With the reference's src/ and lib/ on the include path
 * (plus its TBB headers), and this repository's include/ directory:
 *
 *     #include "lgca/ref_binding.h"
 *     m_lattice = new GB_Lattice<MODEL>("pipe", m_Re, m_Ma, CG_RADIUS);
 *
 * and the app links src/lattice.cpp as before plus -llgca_gpu.
 *
 * What stays the reference's: the constructor's dimensions and physical
 * parameters, the geometry setters, the initialisers, get_n_particles, print
 * and the forcing amounts are the base class's own non-virtual members
 * (src/lattice.cpp), working on the host arrays.  This class allocates those
 * arrays as OMP_Lattice::allocate_memory does (src/omp_lattice.cpp:457-471),
 * frees them as free_memory does (src/omp_lattice.cpp:474-489), and
 * implements the pure virtual backend members (src/lattice.h:187-211) on
 * the GPU:
 *
 *   collide_and_propagate   lgca_collide_and_propagate (src/omp_lattice.cpp:100-249)
 *   apply_body_force        lgca_apply_body_force      (src/omp_lattice.cpp:254-346)
 *   get_mean_velocity       lgca_mean_velocity         (src/omp_lattice.cpp:508-557)
 *   post_process            lgca_post_process on the output buffer (src/omp_lattice.cpp:349-454)
 *   copy_data_*             uploads / downloads of the host arrays (src/lattice.cpp:422-441)
 *
 * The host arrays are uploaded at the first GPU call.  The base class's
 * setters and initialisers cannot tell this class that they ran, so a caller
 * that changes the host arrays after the first GPU call calls
 * copy_data_to_device() (the reference's own member for that) or
 * mark_host_dirty().  The state returns to the host in
 * copy_data_to_output_buffer(), which every reference app calls once per
 * frame, and in copy_data_from_device(); get_n_particles() counts the host
 * state as in the reference, so it is current after either.
 *
 * Randomness: chirality and the body-force cell draws come from the
 * counter-based generator (rng.h) with the lattice seed; the reference uses
 * rand() (src/omp_lattice.cpp:84,269).  To step with the reference's frozen
 * per-cell chirality field m_rnd_cpu (src/omp_lattice.cpp:84,198), call
 * use_frozen_chirality() after construction.
 *
 * The device half is shared with the stand-alone class of gb_lattice.h
 * (gb_device.h), whose app loops the GPU tests compare with the oracle.
 */
#ifndef LGCA_REF_BINDING_H_
#define LGCA_REF_BINDING_H_

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "lattice.h"  // the reference's class (src/lattice.h)

#include "../lgca_gpu.h"
#include "gb_device.h"

namespace lgca {

template <Model model_>
class GB_Lattice : public Lattice<model_> {
public:
    GB_Lattice(const string test_case, const Real Re, const Real Ma_s,
               const int coarse_graining_radius, uint64_t seed = 0)
        : Lattice<model_>(test_case, Re, Ma_s, coarse_graining_radius),
          m_dev((int)model_, this->m_dim_x, this->m_dim_y, seed)
    {
        // host arrays as OMP_Lattice::allocate_memory (src/omp_lattice.cpp:457-471)
        this->m_cell_type_cpu = (CellType *)malloc(this->m_num_cells * sizeof(CellType));
        this->m_cell_density_cpu = (Real *)malloc(this->m_num_cells * sizeof(Real));
        this->m_mean_density_cpu = (Real *)malloc(this->m_num_coarse_cells * sizeof(Real));
        this->m_cell_momentum_cpu = (Real *)malloc(this->SPATIAL_DIM * this->m_num_cells * sizeof(Real));
        this->m_mean_momentum_cpu =
            (Real *)malloc(this->SPATIAL_DIM * this->m_num_coarse_cells * sizeof(Real));
        this->m_node_state_cpu.resize(this->m_num_cells * 8);
        this->m_node_state_out_cpu.resize(this->m_num_cells * 8);
        this->m_rnd_cpu.resize(this->m_num_cells);
        this->m_rnd_cpu.fill_random();  // the reference's frozen field, src/omp_lattice.cpp:84
        for (size_t c = 0; c < this->m_num_cells; ++c) this->m_cell_type_cpu[c] = CellType::FLUID;
    }

    ~GB_Lattice() override
    {
        // src/omp_lattice.cpp:474-489
        free(this->m_cell_type_cpu);
        free(this->m_cell_density_cpu);
        free(this->m_mean_density_cpu);
        free(this->m_cell_momentum_cpu);
        free(this->m_mean_momentum_cpu);
        this->m_cell_type_cpu = nullptr;
        this->m_cell_density_cpu = nullptr;
        this->m_mean_density_cpu = nullptr;
        this->m_cell_momentum_cpu = nullptr;
        this->m_mean_momentum_cpu = nullptr;
    }

    // src/omp_lattice.cpp:492-505 prints the thread configuration
    void setup_parallel() override
    {
        printf("GB300 configuration parameters: Executing calculation on the current CUDA device.\n\n");
    }

    // The argument is ignored, as in the reference (src/omp_lattice.cpp:101,198).
    void collide_and_propagate(const bool p = false) override
    {
        (void)p;
        push();
        m_dev.step(1);
    }

    std::vector<Real> get_mean_velocity() override
    {
        push();
        const std::vector<float> u = m_dev.mean_velocity();
        return std::vector<Real>{u[0], u[1]};
    }

    void apply_body_force(const int forcing) override
    {
        push();
        m_dev.body_force(forcing, this->m_bf_dir);
    }

    // On the output buffer, as the reference (src/omp_lattice.cpp:376).
    void post_process() override
    {
        m_dev.post_process(this->m_node_state_out_cpu.ptr(), (int)this->m_coarse_graining_radius,
                           this->m_cell_density_cpu, this->m_cell_momentum_cpu,
                           this->m_mean_density_cpu, this->m_mean_momentum_cpu);
    }

    void copy_data_to_device() override
    {
        mark_host_dirty();
        push();
    }

    void copy_data_from_device() override { pull(); }

    void copy_data_to_output_buffer() override
    {
        pull();
        this->m_node_state_out_cpu.copy(this->m_node_state_cpu);
        m_dev.output_taken();
    }

    // ---- extensions of this backend
    // The host arrays changed after the first GPU call.
    void mark_host_dirty()
    {
        m_dev.mark_types_dirty();
        m_dev.mark_state_dirty();
    }
    // Step with the frozen per-cell field m_rnd_cpu (one bit per cell), the
    // reference's own chirality model, instead of the per-step draws.
    void use_frozen_chirality()
    {
        std::vector<uint8_t> f(this->m_num_cells);
        for (size_t c = 0; c < f.size(); ++c) f[c] = this->m_rnd_cpu[c] ? 1 : 0;
        m_dev.check(lgca_set_chirality(m_dev.handle(), f.data()), "use_frozen_chirality");
    }
    // The engine's handle, for its other entry points (block sums, batches...).
    lgca_handle handle()
    {
        push();
        return m_dev.handle();
    }
    uint64_t last_reverted() const { return m_dev.last_reverted(); }

private:
    void push() { m_dev.push(this->m_cell_type_cpu, this->m_node_state_cpu.ptr()); }
    void pull()
    {
        push();
        m_dev.pull(this->m_node_state_cpu.ptr());
    }

    lgca_gb300::DeviceLattice m_dev;
};

}  // namespace lgca

#endif /* LGCA_REF_BINDING_H_ */
