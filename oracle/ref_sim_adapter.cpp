// ref_sim_adapter.cpp -- C entry points over the reference simulator's own sources, compiled
// unchanged from the reference tree against the Eigen-interface subset in oracle/eigen_min:
//
//   src/project/3d/fluid/projection.cpp      assign_indices, build_matrix,
//                                            build_grid_from_vector,
//                                            update_velocity_using_pressure
//   src/project/3d/fluid/boundary.cpp        compute_staggered_grid_weight
//   src/project/3d/fluid/extrapolation.cpp   extrapolate, extrapolate_const
//   src/project/3d/fluid/time_stepping.cpp   calc_time_step
//   src/project/3d/fluid/advection.cpp       advect_collocated_grid, advect_staggered_grid
//   src/project/3d/fluid/levelset_emitter.cpp, src/project/3d/eulerian_liquid/scene.cpp
//   src/project/3d/eulerian_liquid/simulator.cpp   the Simulator step methods
//   src/common/meshing.cpp, src/common/mesh.cpp    marching cubes and OBJ output
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py into oracle/_ref/ (git-ignored), and
// only where the reference tree is present.  The product never loads it; tests/ use it to
// pin the CPU restatement (oracle/oracle.cpp) and tests/golden/make_golden.py to record
// fixtures.  The one substitution is the linear solver inside Simulator::solve_pressure
// (Eigen's ConjugateGradient + IncompleteCholesky, not installed here): see
// oracle/eigen_min/Eigen/IterativeLinearSolvers.
//
// Arrays are the reference's i-fastest layout (include/nama/common/array.h:281-286), passed
// as raw pointers; grids are built with the reference's own shapes and origins
// (staggered_grid.h:100-112, simulator.cpp:52-70).

#include <nama/common/meshing.h>
#include <nama/project/3d/eulerian_liquid/simulator.h>
#include <nama/project/3d/fluid/advection.h>
#include <nama/project/3d/fluid/boundary.h>
#include <nama/project/3d/fluid/extrapolation.h>
#include <nama/project/3d/fluid/levelset_emitter.h>
#include <nama/project/3d/fluid/projection.h>
#include <nama/project/3d/fluid/time_stepping.h>
#include <nama/utils/logger.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>

using nama::Grid3c;
using nama::Grid3f;
using nama::Grid3i;
using nama::StaggeredGrid3c;
using nama::StaggeredGrid3f;
namespace fluid = nama::_3d::fluid;
namespace el = nama::_3d::eulerian_liquid;

namespace {

constexpr int kUnknown = std::numeric_limits<int>::max();

void log_to_null() {
    static std::once_flag once;
    std::call_once(once, [] {
        nama::utils::Logger::set_output_file("/dev/null");
        nama::utils::Logger::create_output_file();
    });
}

template <typename G, typename T>
void fill(G& g, const T* src) {
    std::memcpy(g.data(), src, g.size() * sizeof(T));
}

template <typename G, typename T>
void dump(const G& g, T* dst) {
    std::memcpy(dst, g.data(), g.size() * sizeof(T));
}

// A scene's grids with the shapes Simulator::create_grid gives them (simulator.cpp:52-70).
struct Fields {
    float dx;
    Grid3f phi, nodal_solid;
    StaggeredGrid3f vel, weight;
    Fields(int ni, int nj, int nk, float dx_) : dx(dx_) {
        const Eigen::Vector3f o(0, 0, 0);
        phi.create(ni, nj, nk, dx, o);
        nodal_solid.create(ni + 1, nj + 1, nk + 1, dx, Eigen::Vector3f(-dx * 0.5, -dx * 0.5, -dx * 0.5));
        vel.create(ni, nj, nk, dx, o);
        weight.create(ni, nj, nk, dx, o);
    }
};

}  // namespace

#define REF_EXPORT extern "C" __attribute__((visibility("default")))

// boundary.cpp:6-34
REF_EXPORT void refsim_compute_weights(int ni, int nj, int nk, double dx, const float* solid,
                                       float* wu, float* wv, float* ww) {
    Fields f(ni, nj, nk, (float)dx);
    fill(f.nodal_solid, solid);
    fluid::compute_staggered_grid_weight(f.weight, f.nodal_solid);
    dump(f.weight.u(), wu);
    dump(f.weight.v(), wv);
    dump(f.weight.w(), ww);
}

// projection.cpp:14-28; returns the matrix size, -1 for the reference's "No fluid"
REF_EXPORT int refsim_assign_indices(int ni, int nj, int nk, double dx, const float* phi,
                                     const float* wu, const float* wv, const float* ww, int* indices) {
    Fields f(ni, nj, nk, (float)dx);
    fill(f.phi, phi);
    fill(f.weight.u(), wu);
    fill(f.weight.v(), wv);
    fill(f.weight.w(), ww);
    Grid3i idx;
    idx.create(ni, nj, nk, (float)dx, Eigen::Vector3f(0, 0, 0));
    int n;
    try {
        n = fluid::assign_indices(idx, f.phi, f.weight);
    } catch (const std::runtime_error&) {
        return -1;
    }
    dump(idx, indices);
    return n;
}

// projection.cpp:30-83, the matrix and right-hand side laid out on the grid: diag(c) = A(c,c),
// offx(c) = A(c, c+x) etc. for liquid cells, 0 elsewhere; rhs(c) = b(c).  Returns the number
// of stored entries that are neither a diagonal nor a coupling with a -+x/y/z neighbour, or
// that break the symmetry A(c,n) = A(n,c) (0 for a well-posed scene), -1 for "No fluid".
REF_EXPORT int refsim_build_matrix(int ni, int nj, int nk, double dx, const float* phi,
                                   const float* u, const float* v, const float* w, const float* wu,
                                   const float* wv, const float* ww, double dt, double* diag,
                                   double* offx, double* offy, double* offz, double* rhs,
                                   long long* nnz) {
    Fields f(ni, nj, nk, (float)dx);
    fill(f.phi, phi);
    fill(f.vel.u(), u);
    fill(f.vel.v(), v);
    fill(f.vel.w(), w);
    fill(f.weight.u(), wu);
    fill(f.weight.v(), wv);
    fill(f.weight.w(), ww);
    Grid3i idx;
    idx.create(ni, nj, nk, (float)dx, Eigen::Vector3f(0, 0, 0));
    int n;
    try {
        n = fluid::assign_indices(idx, f.phi, f.weight);
    } catch (const std::runtime_error&) {
        return -1;
    }
    Eigen::SparseMatrix<double, Eigen::RowMajor> A;
    Eigen::VectorXd b;
    fluid::build_matrix(A, b, n, idx, f.phi, f.vel, f.weight, (float)dt);
    *nnz = A.nonZeros();
    const long long N = (long long)ni * nj * nk;
    std::fill(diag, diag + N, 0.0);
    std::fill(offx, offx + N, 0.0);
    std::fill(offy, offy + N, 0.0);
    std::fill(offz, offz + N, 0.0);
    std::fill(rhs, rhs + N, 0.0);
    const int* outer = A.outerIndexPtr();
    const int* inner = A.innerIndexPtr();
    const double* val = A.valuePtr();
    int odd = 0;
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                const int r = idx(i, j, k);
                if (r == kUnknown) continue;
                const long long c = i + (long long)ni * (j + (long long)nj * k);
                rhs[c] = b(r);
                auto id = [&](int x, int y, int z) {
                    if (x < 0 || y < 0 || z < 0 || x >= ni || y >= nj || z >= nk) return -1;
                    const int q = idx(x, y, z);
                    return q == kUnknown ? -1 : q;
                };
                const int px = id(i + 1, j, k), py = id(i, j + 1, k), pz = id(i, j, k + 1);
                const int mx = id(i - 1, j, k), my = id(i, j - 1, k), mz = id(i, j, k - 1);
                for (int q = outer[r]; q < outer[r + 1]; ++q) {
                    const int col = inner[q];
                    if (col == r) diag[c] = val[q];
                    else if (col == px) offx[c] = val[q];
                    else if (col == py) offy[c] = val[q];
                    else if (col == pz) offz[c] = val[q];
                    else if (col == mx || col == my || col == mz) {
                        if (val[q] != A.coeff(col, r)) ++odd;
                    } else ++odd;
                }
            }
    return odd;
}

// projection.cpp:85-91
REF_EXPORT void refsim_build_grid_from_vector(int ni, int nj, int nk, double dx, const double* vec,
                                              int n, const int* indices, double background,
                                              float* out) {
    Grid3f g;
    g.create(ni, nj, nk, (float)dx, Eigen::Vector3f(0, 0, 0));
    Grid3i idx;
    idx.create(ni, nj, nk, (float)dx, Eigen::Vector3f(0, 0, 0));
    fill(idx, indices);
    Eigen::VectorXd x(n);
    for (int q = 0; q < n; ++q) x(q) = vec[q];
    fluid::build_grid_from_vector(g, x, idx, (float)background);
    dump(g, out);
}

// projection.cpp:93-134 (u, v, w updated in place)
REF_EXPORT void refsim_update_velocity(int ni, int nj, int nk, double dx, float* u, float* v,
                                       float* w, const float* p, const float* phi, double dt) {
    Fields f(ni, nj, nk, (float)dx);
    fill(f.phi, phi);
    fill(f.vel.u(), u);
    fill(f.vel.v(), v);
    fill(f.vel.w(), w);
    Grid3f pressure;
    pressure.create(ni, nj, nk, (float)dx, Eigen::Vector3f(0, 0, 0));
    fill(pressure, p);
    fluid::update_velocity_using_pressure(f.vel, pressure, f.phi, (float)dt);
    dump(f.vel.u(), u);
    dump(f.vel.v(), v);
    dump(f.vel.w(), w);
}

// extrapolation.cpp:5-46 (grid and valid updated in place; valid as 0/1 bytes)
REF_EXPORT void refsim_extrapolate(float* grid, unsigned char* valid, int n0, int n1, int n2,
                                   int layers, int keep_valid) {
    nama::Array3f g(n0, n1, n2);
    nama::Array3c m(n0, n1, n2);
    std::memcpy(g.data(), grid, g.size() * sizeof(float));
    std::memcpy(m.data(), valid, m.size());
    if (keep_valid)
        fluid::extrapolate_const(g, m, layers);  // extrapolation.cpp:48-51
    else
        fluid::extrapolate(g, m, layers);
    std::memcpy(grid, g.data(), g.size() * sizeof(float));
    std::memcpy(valid, m.data(), m.size());
}

// time_stepping.cpp:5-7 with staggered_grid.h:230-248
REF_EXPORT float refsim_calc_time_step(int ni, int nj, int nk, double dx, const float* u,
                                       const float* v, const float* w, double cfl) {
    Fields f(ni, nj, nk, (float)dx);
    fill(f.vel.u(), u);
    fill(f.vel.v(), v);
    fill(f.vel.w(), w);
    return fluid::calc_time_step((float)cfl, f.vel);
}

// advection.cpp:9-27 (RK2 trace + trilinear sampling, FP32)
REF_EXPORT void refsim_advect_collocated(int ni, int nj, int nk, double dx, float* out,
                                         const float* phi, const float* u, const float* v,
                                         const float* w, double dt) {
    Fields f(ni, nj, nk, (float)dx);
    fill(f.phi, phi);
    fill(f.vel.u(), u);
    fill(f.vel.v(), v);
    fill(f.vel.w(), w);
    Grid3f result = f.phi;
    fluid::advect_collocated_grid(result, f.phi, f.vel, (float)dt);
    dump(result, out);
}

REF_EXPORT void refsim_advect_staggered(int ni, int nj, int nk, double dx, float* ou, float* ov,
                                        float* ow, const float* u, const float* v, const float* w,
                                        double dt) {
    Fields f(ni, nj, nk, (float)dx);
    fill(f.vel.u(), u);
    fill(f.vel.v(), v);
    fill(f.vel.w(), w);
    StaggeredGrid3f result = f.vel;
    fluid::advect_staggered_grid(result, f.vel, f.vel, (float)dt);
    dump(result.u(), ou);
    dump(result.v(), ov);
    dump(result.w(), ow);
}

// ---------------------------------------------------------------------------------------
// The reference's Simulator (simulator.cpp), driven field by field.

struct RefSim {
    el::Simulator sim;
    el::Scene scene;
};

REF_EXPORT void* refsim_new(int ni, int nj, int nk, double cfl) {
    log_to_null();
    auto* s = new RefSim;
    s->sim.create_grid(1, ni, nj, nk);
    el::SimulationParams p;
    p.cfl = (float)cfl;
    s->sim.set_params(p);
    return s;
}

REF_EXPORT void refsim_free(void* h) { delete static_cast<RefSim*>(h); }

REF_EXPORT double refsim_dx(void* h) { return static_cast<RefSim*>(h)->sim.m_dx; }

// emitters of levelset_emitter.cpp:10-32 added to the scene (liquid = 1, solid = 0)
REF_EXPORT void refsim_add_sphere(void* h, int liquid, double cx, double cy, double cz, double r) {
    auto* s = static_cast<RefSim*>(h);
    auto e = std::make_shared<fluid::LevelSetEmitterFunction>(
        nama::_3d::function::sphere(Eigen::Vector3f((float)cx, (float)cy, (float)cz), (float)r));
    if (liquid)
        s->scene.add_liquid_emitter(std::move(e));
    else
        s->scene.add_solid_emitter(std::move(e));
}

REF_EXPORT void refsim_add_pool(void* h, double height) {
    auto* s = static_cast<RefSim*>(h);
    s->scene.add_liquid_emitter(
        std::make_shared<fluid::LevelSetEmitterFunction>(nama::_3d::function::pool((float)height)));
}

REF_EXPORT void refsim_add_room(void* h) {
    auto* s = static_cast<RefSim*>(h);
    const auto& g = s->sim.m_nodal_solid_phi;
    s->scene.add_solid_emitter(std::make_shared<fluid::LevelSetEmitterGrid>(
        nama::_3d::function::room(g.ni(), g.nj(), g.nk())));
}

// Simulator::set_scene + init_scene (simulator.cpp:72-76)
REF_EXPORT void refsim_init_scene(void* h) {
    auto* s = static_cast<RefSim*>(h);
    s->sim.set_scene(s->scene);
    s->sim.init_scene();
}

// Field access: pointer and element count of a named field.
REF_EXPORT void* refsim_field(void* h, const char* name, long long* count, int* elem) {
    auto& m = static_cast<RefSim*>(h)->sim;
    const std::string n(name);
    auto ret = [&](auto& g) -> void* {
        *count = (long long)g.size();
        *elem = (int)sizeof(*g.data());
        return (void*)g.data();
    };
    if (n == "phi") return ret(m.m_level_set);
    if (n == "phi_valid") return ret(m.m_level_set_valid);
    if (n == "u") return ret(m.m_velocity.u());
    if (n == "v") return ret(m.m_velocity.v());
    if (n == "w") return ret(m.m_velocity.w());
    if (n == "weight_u") return ret(m.m_velocity_weight.u());
    if (n == "weight_v") return ret(m.m_velocity_weight.v());
    if (n == "weight_w") return ret(m.m_velocity_weight.w());
    if (n == "valid_u") return ret(m.m_velocity_valid.u());
    if (n == "valid_v") return ret(m.m_velocity_valid.v());
    if (n == "valid_w") return ret(m.m_velocity_valid.w());
    if (n == "pressure") return ret(m.m_pressure);
    if (n == "indices") return ret(m.m_indices);
    if (n == "solid_nodal") return ret(m.m_nodal_solid_phi);
    if (n == "solid_cell") return ret(m.m_cell_centered_solid_level_set);
    *count = 0;
    *elem = 0;
    return nullptr;
}

// The step recipe update_second_order (apps/eulerian_liquid_3d.cpp:106-120), with or without
// its reinitialize() call; the app defines it, so it is restated here as the same calls.
static void second_order(el::Simulator& sim, float dt, bool reinit) {
    sim.extrapolate_velocity();
    sim.extrapolate_level_set();
    sim.advect_level_set(dt);
    sim.advect_velocity(dt);
    if (reinit) sim.reinitialize();
    sim.add_gravity(dt);
    sim.find_valid_velocity();
    sim.set_invalid_velocity_zero();
    sim.solve_pressure(dt);
}

// Runs one Simulator method.  Returns 0, or -1 for the reference's "No fluid" exception,
// -2 for an unknown name.
REF_EXPORT int refsim_call(void* h, const char* method, double dt) {
    auto& m = static_cast<RefSim*>(h)->sim;
    const std::string n(method);
    const float t = (float)dt;
    try {
        if (n == "compute_weights") m.compute_weights();
        else if (n == "find_valid_level_set") m.find_valid_level_set();
        else if (n == "calc_cell_centered_solid_phi") m.calc_cell_centered_solid_phi();
        else if (n == "extrapolate_velocity") m.extrapolate_velocity();
        else if (n == "extrapolate_level_set") m.extrapolate_level_set();
        else if (n == "advect_level_set") m.advect_level_set(t);
        else if (n == "advect_velocity") m.advect_velocity(t);
        else if (n == "reinitialize") m.reinitialize();
        else if (n == "add_gravity") m.add_gravity(t);
        else if (n == "find_valid_velocity") m.find_valid_velocity();
        else if (n == "set_invalid_velocity_zero") m.set_invalid_velocity_zero();
        else if (n == "solve_pressure") m.solve_pressure(t);
        else if (n == "second_order") second_order(m, t, true);
        else if (n == "second_order_no_reinit") second_order(m, t, false);
        // Simulator::update (simulator.cpp:23-42): CFL sub-steps of the recipe over one frame dt
        else if (n == "update_frame") m.update([](el::Simulator& s, float d) { second_order(s, d, true); }, t, true);
        else if (n == "update_frame_no_reinit")
            m.update([](el::Simulator& s, float d) { second_order(s, d, false); }, t, true);
        else return -2;
    } catch (const std::runtime_error&) {
        return -1;
    }
    return 0;
}

// Marching cubes (method 0) or dual marching cubes (method 1) of a cell-centred grid
// (meshing.cpp:11-128), written as OBJ by Mesh::save (mesh.cpp:53).  counts = {vertices,
// faces, indices per face}.  Returns 0, or -1 when the file cannot be written.
REF_EXPORT int refsim_mesh_obj(const float* phi, int ni, int nj, int nk, double dx, double ox,
                               double oy, double oz, double isolevel, int method, const char* path,
                               long long* counts) {
    Grid3f g;
    g.create(ni, nj, nk, (float)dx, Eigen::Vector3f((float)ox, (float)oy, (float)oz));
    fill(g, phi);
    nama::Mesh3f mesh = nama::get_mesh(
        g, (float)isolevel,
        method ? nama::MeshingMethod::DUAL_MARCHING_CUBES : nama::MeshingMethod::MARCHING_CUBES);
    const long long per = static_cast<long long>(mesh.get_type());
    counts[0] = (long long)mesh.vertices().size();
    counts[1] = per ? (long long)mesh.indices().size() / per : 0;
    counts[2] = per;
    try {
        if (path && *path) mesh.save(path);
    } catch (const std::exception&) {
        return -1;
    }
    return 0;
}
