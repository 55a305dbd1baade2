// C++ check of the host interface (eulerian-liquid_gb300/host/nama_gb300.h) driven the way the
// reference's app drives its Simulator: update(update_second_order, 1/60, use_cfl) with the
// reference's step order (apps/eulerian_liquid_3d.cpp:106-120), reinitialisation left out.
// Prints "ok" and exits 0 when every check holds.  Given a directory, it also writes the state
// before one more step of a fixed dt and the fields after it, as raw little-endian arrays, for a
// comparison of the host interface's numbers with the oracle (tests/test_gpu_cpp_shim.py).
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "nama_gb300.h"

using namespace nama_gb300;
using eulerian_liquid::Simulator;

static int failures = 0;
#define CHECK(cond)                                                  \
    do {                                                             \
        if (!(cond)) {                                               \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond); \
            ++failures;                                              \
        }                                                            \
    } while (0)

static void update_second_order(Simulator& sim, float dt) {
    sim.extrapolate_velocity();
    sim.extrapolate_level_set();
    sim.advect_level_set(dt);
    sim.advect_velocity(dt);
    sim.add_gravity(dt);
    sim.find_valid_velocity();
    sim.set_invalid_velocity_zero();
    sim.solve_pressure(dt);
}

template <typename G>
static bool dump(const std::string& dir, const char* name, const G& g) {
    FILE* f = std::fopen((dir + "/" + name).c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(g.data(), sizeof(g[0]), g.size(), f) == g.size();
    return std::fclose(f) == 0 && ok;
}

int main(int argc, char** argv) {
    const int n = 32;
    Simulator sim;
    sim.create_grid(1.0f, n, n, n);
    sim.set_params(eulerian_liquid::SimulationParams{1.0f});
    // the reference's water_drop scene (apps/eulerian_liquid_3d.cpp:49-68)
    sim.clear_level_sets();
    sim.add_liquid_sphere(0.25f, 0.6f, 0.25f, 0.16f);
    sim.add_liquid_sphere(0.5f, 0.5f, 0.5f, 0.16f);
    sim.add_liquid_sphere(0.75f, 0.7f, 0.75f, 0.16f);
    sim.add_liquid_pool(0.25f);
    sim.add_solid_room();
    sim.init_scene();
    sim.compute_weights();
    sim.find_valid_level_set();

    for (int frame = 0; frame < 3; ++frame) sim.update(update_second_order, 1.0f / 60.0f, true);
    CHECK(sim.last_solve.status == EL_OK);
    CHECK(sim.last_solve.fluid_cells > 1000);
    sim.sync_to_host();
    bool finite = true;
    for (int d = 0; d < 3; ++d)
        for (size_t q = 0; q < sim.m_velocity[d].size(); ++q) finite = finite && std::isfinite(sim.m_velocity[d][q]);
    CHECK(finite);
    // the domain's outermost faces are zeroed by set_invalid_velocity_zero and never touched by
    // update_velocity_using_pressure (interior faces only, projection.cpp:93-134); faces between
    // fluid and solid cells may carry velocity until the next step zeroes them, as in the reference
    bool walls = true;
    for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j) {
            walls = walls && sim.m_velocity.u()(0, j, k) == 0.0f && sim.m_velocity.u()(n, j, k) == 0.0f;
            walls = walls && sim.m_velocity.v()(j, 0, k) == 0.0f && sim.m_velocity.v()(j, n, k) == 0.0f;
            walls = walls && sim.m_velocity.w()(j, k, 0) == 0.0f && sim.m_velocity.w()(j, k, n) == 0.0f;
        }
    CHECK(walls);
    // liquid falls: the mean vertical velocity of valid faces is negative after three frames
    double vsum = 0;
    int vcount = 0;
    for (size_t q = 0; q < sim.m_velocity.v().size(); ++q)
        if (sim.m_velocity_valid.v()[q]) {
            vsum += sim.m_velocity.v()[q];
            ++vcount;
        }
    CHECK(vcount > 0 && vsum / vcount < 0);

    // free functions on host grids
    Grid3f phi = sim.m_level_set, out(n, n, n, sim.m_dx);
    StaggeredGrid3f zero;
    zero.create(n, n, n, sim.m_dx);
    fluid::advect_collocated_grid(out, phi, zero, 0.01f);
    bool same = true;
    for (size_t q = 0; q < phi.size(); ++q) same = same && out[q] == phi[q];
    CHECK(same);  // zero velocity and dx = 1/32: the foot point is the sample point
    StaggeredGrid3f wts;
    wts.create(n, n, n, sim.m_dx);
    fluid::compute_staggered_grid_weight(wts, sim.m_nodal_solid_phi);
    bool weights_same = true;
    for (int d = 0; d < 3; ++d)
        for (size_t q = 0; q < wts[d].size(); ++q) weights_same = weights_same && wts[d][q] == sim.m_velocity_weight[d][q];
    CHECK(weights_same);
    Grid3i idx(n, n, n, sim.m_dx);
    const int m = fluid::assign_indices(idx, sim.m_level_set, sim.m_velocity_weight);
    CHECK(m > 1000 && m == sim.last_solve.fluid_cells);
    StaggeredGrid3f adv;
    adv.create(n, n, n, sim.m_dx);
    fluid::advect_staggered_grid(adv, sim.m_velocity, sim.m_velocity, 0.005f);
    CHECK(std::isfinite(adv.u()[n / 2]));

    // the reference's failure path: std::runtime_error("No fluid")
    Grid3f air(n, n, n, sim.m_dx, 1.0f);
    bool threw = false;
    try {
        fluid::assign_indices(idx, air, sim.m_velocity_weight);
    } catch (const std::runtime_error& e) {
        threw = std::string(e.what()) == "No fluid";
    }
    CHECK(threw);

    if (argc > 1) {
        // one more step of a fixed dt: its input state, and the fields it leaves
        const std::string dir = argv[1];
        sim.sync_to_host();
        bool ok = dump(dir, "in_phi", sim.m_level_set) && dump(dir, "in_valid_phi", sim.m_level_set_valid);
        const char* comp[3] = {"u", "v", "w"};
        for (int d = 0; d < 3; ++d) {
            ok = ok && dump(dir, (std::string("in_") + comp[d]).c_str(), sim.m_velocity[d]);
            ok = ok && dump(dir, (std::string("in_valid_") + comp[d]).c_str(), sim.m_velocity_valid[d]);
            ok = ok && dump(dir, (std::string("weight_") + comp[d]).c_str(), sim.m_velocity_weight[d]);
        }
        sim.solve_params.tol = 1e-6;
        update_second_order(sim, 1.0f / 240.0f);
        CHECK(sim.last_solve.status == EL_OK);
        sim.sync_to_host();
        ok = ok && dump(dir, "out_phi", sim.m_level_set) && dump(dir, "out_pressure", sim.m_pressure);
        for (int d = 0; d < 3; ++d) ok = ok && dump(dir, (std::string("out_") + comp[d]).c_str(), sim.m_velocity[d]);
        CHECK(ok);
    }

    if (failures == 0) std::printf("ok\n");
    return failures == 0 ? 0 : 1;
}
