// Check of include/lgca/ref_binding.h against the reference's own class.
//
// Compiled by tests/test_ref_binding.py with the reference's src/ and lib/ on
// the include path and its src/lattice.cpp linked in (from where they lie),
// so GB_Lattice<M> derives from the real lgca::Lattice<M> (src/lattice.h:32-238).
// Instantiating `new GB_Lattice<M>(...)` as the apps' one-line switch does
// (apps/pipe/pipe_viewer.cpp:46) only compiles if every pure virtual member
// is overridden.
//
//   ref_binding_check host CASE MODEL   an app's set-up through the binding on
//                                       the host only (the reference
//                                       constructor, apply_bc_*, init_random,
//                                       get_n_particles) -- no GPU needed
//   ref_binding_check gpu CASE MODEL    also four frames of the pipe viewer's
//                                       loop (controller, body force, steps,
//                                       post-processing) on the GPU
#include "lgca/ref_binding.h"

#include <cstring>
#include <string>
#include <type_traits>

using namespace lgca;

static_assert(!std::is_abstract<GB_Lattice<Model::HPP>>::value, "HPP backend is abstract");
static_assert(!std::is_abstract<GB_Lattice<Model::FHP_I>>::value, "FHP-I backend is abstract");
static_assert(!std::is_abstract<GB_Lattice<Model::FHP_II>>::value, "FHP-II backend is abstract");
static_assert(!std::is_abstract<GB_Lattice<Model::FHP_III>>::value, "FHP-III backend is abstract");
static_assert(std::is_base_of<Lattice<Model::FHP_III>, GB_Lattice<Model::FHP_III>>::value,
              "GB_Lattice derives from the reference's Lattice");

template <Model M> static int run(const std::string &tc, Real Re, Real Ma, int r, bool gpu)
{
    // the apps' declared type is the reference base class
    Lattice<M> *lattice = new GB_Lattice<M>(tc, Re, Ma, r);
    if (tc == "pipe") lattice->apply_bc_pipe();
    else if (tc == "karman") lattice->apply_bc_karman_vortex_street();
    else if (tc == "box") lattice->apply_bc_reflecting("back");
    else lattice->apply_bc_periodic();
    lattice->init_random();
    const unsigned long n0 = lattice->get_n_particles();
    unsigned long n1 = n0;
    float u0 = 0.0f;
    if (gpu) {
        lattice->setup_parallel();
        int forcing = (int)lattice->get_initial_forcing();
        for (int frame = 0; frame < 4; ++frame) {  // apps/pipe/pipe_viewer.cpp:107-136
            std::vector<Real> u = lattice->get_mean_velocity();
            if (u[0] < lattice->u()) {
                if (u[0] > 0.9 * lattice->u()) forcing = (int)lattice->get_equilibrium_forcing();
                lattice->apply_body_force(forcing);
            }
            for (int s = 0; s < 5; ++s) lattice->collide_and_propagate(false);
            lattice->copy_data_to_output_buffer();
            lattice->post_process();
        }
        n1 = lattice->get_n_particles();
        u0 = lattice->get_mean_velocity()[0];
    }
    printf("{\"dims\": [%u, %u], \"coarse\": [%u, %u], \"particles\": %lu, \"particles_end\": %lu, "
           "\"initial_forcing\": %zu, \"equilibrium_forcing\": %zu, \"u0\": %g}\n",
           lattice->dim_x(), lattice->dim_y(), lattice->coarse_dim_x(), lattice->coarse_dim_y(), n0,
           n1, lattice->get_initial_forcing(), lattice->get_equilibrium_forcing(), u0);
    delete lattice;
    return n1 == n0 ? 0 : 1;
}

int main(int argc, char **argv)
{
    const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
    const std::string tc = argc > 2 ? argv[2] : "pipe";
    const int model = argc > 3 ? std::atoi(argv[3]) : 3;
    const Real Re = 80.0f, Ma = 0.3f;
    const int r = tc == "karman" ? 20 : 10;
    switch (model) {
    case 0: return run<Model::HPP>(tc, Re, Ma, r, gpu);
    case 1: return run<Model::FHP_I>(tc, Re, Ma, r, gpu);
    case 2: return run<Model::FHP_II>(tc, Re, Ma, r, gpu);
    default: return run<Model::FHP_III>(tc, Re, Ma, r, gpu);
    }
}
