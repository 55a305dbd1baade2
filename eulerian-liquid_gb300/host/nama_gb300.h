// nama_gb300.h -- C++ host interface mirroring the reference's hot-path API on top of the
// C ABI (include/eulerian_liquid_gb300.h).
//
// The reference's types (include/nama/common/grid.h, staggered_grid.h) are std::vector-backed,
// i-fastest grids; the minimal Grid3 / StaggeredGrid3 here have the same layout and accessors,
// so a reference Grid3f's data() can be handed over unchanged.  Names and argument meaning follow
//   src/project/3d/fluid/advection.cpp:9-27      advect_collocated_grid, advect_staggered_grid
//   src/project/3d/fluid/boundary.cpp:6-34       compute_staggered_grid_weight
//   src/project/3d/fluid/projection.cpp:14-134   assign_indices, update_velocity_using_pressure
//   src/project/3d/eulerian_liquid/simulator.cpp Simulator step methods
// and errors are the reference's: std::runtime_error("No fluid") when there is no fluid cell,
// std::runtime_error with the library's message for any other failure.
#pragma once

#include <cstddef>
#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "eulerian_liquid_gb300.h"

namespace nama_gb300 {

template <typename T>
class Grid3 {
   public:
    Grid3() = default;
    Grid3(int ni, int nj, int nk, float dx, T value = T{}) { create(ni, nj, nk, dx, value); }
    void create(int ni, int nj, int nk, float dx, T value = T{}) {
        m_ni = ni;
        m_nj = nj;
        m_nk = nk;
        m_dx = dx;
        m_data.assign((size_t)ni * nj * nk, value);
    }
    int ni() const { return m_ni; }
    int nj() const { return m_nj; }
    int nk() const { return m_nk; }
    float dx() const { return m_dx; }
    size_t size() const { return m_data.size(); }
    T* data() { return m_data.data(); }
    const T* data() const { return m_data.data(); }
    // ArrayBase::calc_index (include/nama/common/array.h:281-286)
    T& operator()(int i, int j, int k) { return m_data[i + (size_t)m_ni * (j + (size_t)m_nj * k)]; }
    const T& operator()(int i, int j, int k) const { return m_data[i + (size_t)m_ni * (j + (size_t)m_nj * k)]; }
    T& operator[](size_t q) { return m_data[q]; }
    const T& operator[](size_t q) const { return m_data[q]; }

   private:
    int m_ni = 0, m_nj = 0, m_nk = 0;
    float m_dx = 0;
    std::vector<T> m_data;
};

using Grid3f = Grid3<float>;
using Grid3i = Grid3<int>;
using Grid3c = Grid3<char>;

// MAC grid: u (ni+1,nj,nk), v (ni,nj+1,nk), w (ni,nj,nk+1) (staggered_grid.h:100-112)
template <typename T>
class StaggeredGrid3 {
   public:
    static constexpr int dim = 3;
    StaggeredGrid3() = default;
    void create(int ni, int nj, int nk, float dx, T value = T{}) {
        m_ni = ni;
        m_nj = nj;
        m_nk = nk;
        m_dx = dx;
        m_data[0].create(ni + 1, nj, nk, dx, value);
        m_data[1].create(ni, nj + 1, nk, dx, value);
        m_data[2].create(ni, nj, nk + 1, dx, value);
    }
    Grid3<T>& operator[](int d) { return m_data[d]; }
    const Grid3<T>& operator[](int d) const { return m_data[d]; }
    Grid3<T>& u() { return m_data[0]; }
    Grid3<T>& v() { return m_data[1]; }
    Grid3<T>& w() { return m_data[2]; }
    const Grid3<T>& u() const { return m_data[0]; }
    const Grid3<T>& v() const { return m_data[1]; }
    const Grid3<T>& w() const { return m_data[2]; }
    int ni() const { return m_ni; }
    int nj() const { return m_nj; }
    int nk() const { return m_nk; }
    float dx() const { return m_dx; }

   private:
    int m_ni = 0, m_nj = 0, m_nk = 0;
    float m_dx = 0;
    Grid3<T> m_data[3];
};

using StaggeredGrid3f = StaggeredGrid3<float>;
using StaggeredGrid3c = StaggeredGrid3<char>;

namespace fluid {

// advection.cpp:9-16: grid(x) = grid_temp(trace_rk2(x, -dt, velocity)), trilinear sample
void advect_collocated_grid(Grid3f& grid, const Grid3f& grid_temp, const StaggeredGrid3f& velocity, float dt,
                            int trace = EL_TRACE_RK2, int sample = EL_SAMPLE_TRILINEAR);
// advection.cpp:18-27
void advect_staggered_grid(StaggeredGrid3f& grid, const StaggeredGrid3f& grid_temp,
                           const StaggeredGrid3f& velocity, float dt, int trace = EL_TRACE_RK2,
                           int sample = EL_SAMPLE_TRILINEAR);
// boundary.cpp:6-34
void compute_staggered_grid_weight(StaggeredGrid3f& weight, const Grid3f& nodal_solid_level_set);
// projection.cpp:14-28 (throws std::runtime_error("No fluid"))
int assign_indices(Grid3i& indices, const Grid3f& level_set, const StaggeredGrid3f& velocity_weight);
// projection.cpp:93-134
void update_velocity_using_pressure(StaggeredGrid3f& velocity, const Grid3f& pressure, const Grid3f& level_set,
                                    float dt);

}  // namespace fluid

namespace eulerian_liquid {

struct SimulationParams {
    float cfl = 2.0f;  // simulation_params.h:9
};

// Simulator (include/nama/project/3d/eulerian_liquid/simulator.h:18-75): the state lives on the
// GPU; the public host grids are refreshed by sync_to_host() and pushed by sync_to_device().
class Simulator {
   public:
    Simulator() = default;
    ~Simulator();
    Simulator(const Simulator&) = delete;
    Simulator& operator=(const Simulator&) = delete;

    void update(std::function<void(Simulator&, float)> f, float dt_frame, bool use_cfl);
    void set_params(const SimulationParams& params) { m_params = params; }

    void create_grid(float width, int ni, int nj, int nk);

    // scene (levelset_emitter.cpp): liquid target 0, nodal solid target 1
    void clear_level_sets();
    void add_liquid_sphere(float cx, float cy, float cz, float r);
    void add_liquid_pool(float height);
    void add_liquid_box(const double lo[3], const double hi[3]);
    void add_solid_room();
    void add_solid_box(const double lo[3], const double hi[3]);
    void init_scene();  // simulator.cpp:72-76 (after the emitters above)

    void advect_velocity(float dt);
    void advect_level_set(float dt);
    void add_gravity(float dt);
    void solve_pressure(float dt);
    void extrapolate_level_set();
    void extrapolate_velocity();
    void find_valid_velocity();
    void find_valid_level_set();
    void set_invalid_velocity_zero();
    void compute_weights();
    void calc_cell_centered_solid_phi();

    // the reference's whole second-order step without reinitialisation, in one call
    void step_hot_path(float dt);

    void sync_to_host();
    void sync_to_device();

    // solver choice and tolerance (the reference: Eigen IC-PCG, tol 1e-4, 1000 iterations)
    el_solve_params solve_params{EL_SOLVER_MIXED, 1e-4, 1000, 4, 8, 1e-4};
    el_solve_stats last_solve{};
    float gravity = 9.80665f;

    SimulationParams m_params;
    float m_dx = 0;
    int m_ni = 0, m_nj = 0, m_nk = 0;
    StaggeredGrid3f m_velocity, m_velocity_weight;
    StaggeredGrid3c m_velocity_valid;
    Grid3f m_level_set, m_pressure, m_nodal_solid_phi, m_cell_centered_solid_level_set;
    Grid3c m_level_set_valid;

   private:
    void check(int status) const;
    el_ctx* m_ctx = nullptr;
};

}  // namespace eulerian_liquid
}  // namespace nama_gb300
