/*
 * gb_device.h -- the device half shared by the two C++ lattice classes of this
 * repository: gb_lattice.h (a stand-alone class with the reference's
 * Lattice<Model> interface) and ref_binding.h (a backend subclass of the
 * reference's own lgca::Lattice<Model>, src/lattice.h:32-238).
 *
 * Both keep the reference's host arrays -- the cell-type map
 * (src/lattice.h:80) and the state, one byte per cell with bit d = channel d
 * (src/lattice.h:88, src/lgca_bitset.h:35) -- authoritative until the first
 * GPU call, as the reference's non-virtual setters and initialisers write
 * them on the host.  DeviceLattice owns the GPU lattice behind them: it is
 * created on first use, receives the host arrays when they are marked dirty,
 * and runs the backend members of OMP_Lattice<M> (src/omp_lattice.h:27-78)
 * through the C ABI of lgca_gpu.h.  Errors print the reference's message form
 * and abort, the reference's error behaviour (src/lattice.cpp:94-95).
 */
#ifndef LGCA_GB_DEVICE_H_
#define LGCA_GB_DEVICE_H_

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../lgca_gpu.h"

namespace lgca_gb300 {

class DeviceLattice {
public:
    DeviceLattice(int model, unsigned dim_x, unsigned dim_y, uint64_t seed)
        : m_model(model), m_dim_x(dim_x), m_dim_y(dim_y), m_seed(seed)
    {
    }
    ~DeviceLattice()
    {
        if (m_snap) lgca_destroy(m_snap);
        if (m_h) lgca_destroy(m_h);
    }
    DeviceLattice(const DeviceLattice &) = delete;
    DeviceLattice &operator=(const DeviceLattice &) = delete;

    size_t num_cells() const { return (size_t)m_dim_x * m_dim_y; }
    uint64_t seed() const { return m_seed; }
    uint64_t last_reverted() const { return m_last_reverted; }

    // The GPU lattice, created at the first call.
    lgca_handle handle()
    {
        if (!m_h && lgca_create(m_model, (int)m_dim_x, (int)m_dim_y, m_seed, &m_h) != LGCA_OK) {
            printf("ERROR in GB_Lattice: %s\n", lgca_last_error(nullptr));
            abort();
        }
        return m_h;
    }

    // The host map or state changed (a setter or initialiser ran on the host).
    void mark_types_dirty() { m_types_dirty = true; }
    void mark_state_dirty() { m_state_dirty = true; }

    // host -> device of what is marked dirty; `types` holds num_cells values
    // of a cell-type enum (0 fluid, 1 no-slip, 2 slip), `state` num_cells bytes
    template <class CellT> void push(const CellT *types, const uint8_t *state)
    {
        lgca_handle h = handle();
        if (m_types_dirty) {
            std::vector<int32_t> t(num_cells());
            for (size_t c = 0; c < t.size(); ++c) t[c] = (int32_t)types[c];
            check(lgca_set_cell_types(h, t.data()), "set_cell_types");
            m_types_dirty = false;
        }
        if (m_state_dirty) {
            check(lgca_upload_state(h, state), "upload_state");
            m_state_dirty = false;
            m_state_stale = false;
            ++m_version;
        }
    }

    // device -> host state when the device state moved on since the last pull
    void pull(uint8_t *state)
    {
        if (m_state_stale) {
            check(lgca_download_state(handle(), state), "download_state");
            m_state_stale = false;
        }
    }

    // src/omp_lattice.cpp:100-249, nsteps times
    void step(int nsteps)
    {
        check(lgca_collide_and_propagate(handle(), nsteps), "collide_and_propagate");
        m_state_stale = true;
        ++m_version;
    }

    // src/omp_lattice.cpp:254-346
    void body_force(int forcing, char bf_dir)
    {
        uint64_t n = 0;
        check(lgca_apply_body_force(handle(), forcing, bf_dir, &n), "apply_body_force");
        m_last_reverted = n;
        m_state_stale = true;
        ++m_version;
    }

    // src/omp_lattice.cpp:508-557
    std::vector<float> mean_velocity()
    {
        float ux = 0, uy = 0;
        check(lgca_mean_velocity(handle(), &ux, &uy), "get_mean_velocity");
        return std::vector<float>{ux, uy};
    }

    uint64_t count_particles()
    {
        uint64_t n = 0;
        check(lgca_count_particles(handle(), &n), "get_n_particles");
        return n;
    }

    // The output buffer was refreshed from the device state.
    void output_taken() { m_out_version = m_version; }

    // src/omp_lattice.cpp:349-454 on the output buffer `out` (num_cells
    // bytes): the device state itself when the buffer still holds it, else a
    // second GPU lattice loaded with the buffer.
    void post_process(const uint8_t *out, int r, float *cell_density, float *cell_momentum,
                      float *mean_density, float *mean_momentum)
    {
        lgca_handle src = handle();
        if (m_out_version != m_version || m_state_dirty) {
            if (!m_snap)
                check(lgca_create(m_model, (int)m_dim_x, (int)m_dim_y, m_seed, &m_snap), "post_process");
            check(lgca_upload_state(m_snap, out), "post_process");
            src = m_snap;
        }
        check(lgca_post_process(src, r, cell_density, cell_momentum, mean_density, mean_momentum),
              "post_process");
    }

    void check(int status, const char *what)
    {
        if (status != LGCA_OK) {
            printf("ERROR in GB_Lattice::%s(): %s\n", what, lgca_last_error(m_h));
            abort();
        }
    }

private:
    int m_model;
    unsigned m_dim_x, m_dim_y;
    uint64_t m_seed, m_last_reverted = 0;
    lgca_handle m_h = nullptr, m_snap = nullptr;
    bool m_types_dirty = true, m_state_dirty = true, m_state_stale = false;
    uint64_t m_version = 0, m_out_version = ~0ull;
};

}  // namespace lgca_gb300

#endif /* LGCA_GB_DEVICE_H_ */
