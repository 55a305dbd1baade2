// shim.cpp -- the C++ host mirror of the reference's hot-path API over the C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "nama_gb300.h"

namespace nama_gb300 {

namespace {

[[noreturn]] void raise(int status, const std::string& msg) {
    if (status == EL_ERR_NO_FLUID) throw std::runtime_error("No fluid");
    throw std::runtime_error(msg + ": " + el_status_string(status));
}

void check_ctx(el_ctx* ctx, int status) {
    if (status == EL_OK) return;
    raise(status, ctx ? el_ctx_last_error(ctx) : "eulerian_liquid_gb300");
}

// The free functions' device context: one per thread, kept between calls and made again only
// when the grid's shape or spacing or the caller's current device changes, so a call pays for
// its copies and kernels, not for a context's allocations.  Each call copies up every input it
// reads and copies down its outputs, like the reference's by-reference grids, so nothing a call
// leaves on the device is read by the next one.  The context lives on the caller's current
// device (the library gives that device back as current on return).
struct Cached {
    el_ctx* ctx = nullptr;
    int ni = 0, nj = 0, nk = 0, device = -1;
    float dx = 0;
    void* faces[9] = {};   // advect_staggered_grid: device copies of three MAC grids
    ~Cached() { release(); }
    void release() {
        for (void*& p : faces) {
            if (p) cudaFree(p);
            p = nullptr;
        }
        if (ctx) el_ctx_destroy(ctx);
        ctx = nullptr;
    }
};

struct Scoped {
    el_ctx* ctx = nullptr;
    Cached* cache = nullptr;
    Scoped(int ni, int nj, int nk, float dx) {
        static thread_local Cached cached;
        int device = 0;
        if (cudaGetDevice(&device) != cudaSuccess) raise(EL_ERR_CUDA, "cudaGetDevice");
        if (!cached.ctx || cached.ni != ni || cached.nj != nj || cached.nk != nk || cached.dx != dx ||
            cached.device != device) {
            cached.release();
            check_ctx(nullptr, el_ctx_create(ni, nj, nk, dx, EL_F32, device, &cached.ctx));
            cached.ni = ni;
            cached.nj = nj;
            cached.nk = nk;
            cached.dx = dx;
            cached.device = device;
        }
        ctx = cached.ctx;
        cache = &cached;
    }
    template <typename G>
    void up(int field, const G& g) {
        check_ctx(ctx, el_upload(ctx, field, g.data(), g.size() * sizeof(g[0])));
    }
    template <typename G>
    void down(int field, G& g) {
        check_ctx(ctx, el_download(ctx, field, g.data(), g.size() * sizeof(g[0])));
    }
};

}  // namespace

namespace fluid {

void advect_collocated_grid(Grid3f& grid, const Grid3f& grid_temp, const StaggeredGrid3f& velocity, float dt,
                            int trace, int sample) {
    Scoped s(grid.ni(), grid.nj(), grid.nk(), grid_temp.dx());
    s.up(EL_FIELD_PHI, grid_temp);
    s.up(EL_FIELD_U, velocity.u());
    s.up(EL_FIELD_V, velocity.v());
    s.up(EL_FIELD_W, velocity.w());
    check_ctx(s.ctx, el_advect_level_set(s.ctx, dt, trace, sample));
    s.down(EL_FIELD_PHI, grid);
}

void advect_staggered_grid(StaggeredGrid3f& grid, const StaggeredGrid3f& grid_temp, const StaggeredGrid3f& velocity,
                           float dt, int trace, int sample) {
    const int ni = grid.ni(), nj = grid.nj(), nk = grid.nk();
    Scoped s(ni, nj, nk, grid_temp.dx());
    const el_grid g{ni, nj, nk, grid_temp.dx()};
    // device copies of the three grids the kernels read and the three they write, kept with the
    // cached context
    void** d = s.cache->faces;
    const Grid3f* src[6] = {&grid_temp.u(), &grid_temp.v(), &grid_temp.w(), &velocity.u(), &velocity.v(),
                            &velocity.w()};
    for (int q = 0; q < 9; ++q) {
        const size_t bytes = src[q % 3]->size() * sizeof(float);
        if (!d[q] && cudaMalloc(&d[q], bytes) != cudaSuccess) {
            d[q] = nullptr;
            raise(EL_ERR_OUT_OF_MEMORY, "advect_staggered_grid");
        }
        if (q < 6 && cudaMemcpy(d[q], src[q]->data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess)
            raise(EL_ERR_CUDA, "advect_staggered_grid: copy to the device");
    }
    int st = el_advect_staggered_grid(&g, EL_F32, d[6], d[7], d[8], d[0], d[1], d[2], d[3], d[4], d[5], dt, trace,
                                      sample, nullptr);
    if (st == EL_OK && cudaDeviceSynchronize() != cudaSuccess) st = EL_ERR_CUDA;
    Grid3f* dst[3] = {&grid.u(), &grid.v(), &grid.w()};
    for (int q = 0; q < 3 && st == EL_OK; ++q)
        if (cudaMemcpy(dst[q]->data(), d[6 + q], dst[q]->size() * sizeof(float), cudaMemcpyDeviceToHost) !=
            cudaSuccess)
            st = EL_ERR_CUDA;
    if (st != EL_OK) raise(st, "advect_staggered_grid");
}

void compute_staggered_grid_weight(StaggeredGrid3f& weight, const Grid3f& nodal_solid_level_set) {
    Scoped s(weight.ni(), weight.nj(), weight.nk(), weight.dx());
    s.up(EL_FIELD_SOLID_NODAL, nodal_solid_level_set);
    check_ctx(s.ctx, el_compute_weights(s.ctx));
    s.down(EL_FIELD_WEIGHT_U, weight.u());
    s.down(EL_FIELD_WEIGHT_V, weight.v());
    s.down(EL_FIELD_WEIGHT_W, weight.w());
}

int assign_indices(Grid3i& indices, const Grid3f& level_set, const StaggeredGrid3f& velocity_weight) {
    Scoped s(level_set.ni(), level_set.nj(), level_set.nk(), level_set.dx());
    s.up(EL_FIELD_PHI, level_set);
    s.up(EL_FIELD_WEIGHT_U, velocity_weight.u());
    s.up(EL_FIELD_WEIGHT_V, velocity_weight.v());
    s.up(EL_FIELD_WEIGHT_W, velocity_weight.w());
    int n = 0;
    check_ctx(s.ctx, el_assign_indices(s.ctx, &n));
    s.down(EL_FIELD_INDICES, indices);
    return n;
}

void update_velocity_using_pressure(StaggeredGrid3f& velocity, const Grid3f& pressure, const Grid3f& level_set,
                                    float dt) {
    Scoped s(level_set.ni(), level_set.nj(), level_set.nk(), level_set.dx());
    s.up(EL_FIELD_PHI, level_set);
    s.up(EL_FIELD_PRESSURE, pressure);
    s.up(EL_FIELD_U, velocity.u());
    s.up(EL_FIELD_V, velocity.v());
    s.up(EL_FIELD_W, velocity.w());
    check_ctx(s.ctx, el_update_velocity_using_pressure(s.ctx, dt));
    s.down(EL_FIELD_U, velocity.u());
    s.down(EL_FIELD_V, velocity.v());
    s.down(EL_FIELD_W, velocity.w());
}

}  // namespace fluid

namespace eulerian_liquid {

Simulator::~Simulator() {
    if (m_ctx) el_ctx_destroy(m_ctx);
}

void Simulator::check(int status) const { check_ctx(m_ctx, status); }

// simulator.cpp:52-70
void Simulator::create_grid(float width, int ni, int nj, int nk) {
    m_ni = ni;
    m_nj = nj;
    m_nk = nk;
    m_dx = width / ni;
    if (m_ctx) el_ctx_destroy(m_ctx);
    m_ctx = nullptr;
    // the scene lives on the caller's current device
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) raise(EL_ERR_CUDA, "cudaGetDevice");
    check(el_ctx_create(ni, nj, nk, m_dx, EL_F32, device, &m_ctx));
    m_velocity.create(ni, nj, nk, m_dx);
    m_velocity_weight.create(ni, nj, nk, m_dx);
    m_velocity_valid.create(ni, nj, nk, m_dx, 1);
    m_level_set.create(ni, nj, nk, m_dx);
    m_level_set_valid.create(ni, nj, nk, m_dx, 1);
    m_pressure.create(ni, nj, nk, m_dx);
    m_nodal_solid_phi.create(ni + 1, nj + 1, nk + 1, m_dx);
    m_cell_centered_solid_level_set.create(ni, nj, nk, m_dx);
}

void Simulator::clear_level_sets() {
    check(el_emit_clear(m_ctx, 0));
    check(el_emit_clear(m_ctx, 1));
}
void Simulator::add_liquid_sphere(float cx, float cy, float cz, float r) { check(el_emit_sphere(m_ctx, 0, cx, cy, cz, r)); }
void Simulator::add_liquid_pool(float h) { check(el_emit_pool(m_ctx, 0, h)); }
void Simulator::add_liquid_box(const double lo[3], const double hi[3]) { check(el_emit_box(m_ctx, 0, lo, hi)); }
void Simulator::add_solid_room() { check(el_emit_room(m_ctx, 1)); }
void Simulator::add_solid_box(const double lo[3], const double hi[3]) { check(el_emit_box(m_ctx, 1, lo, hi)); }
void Simulator::init_scene() { calc_cell_centered_solid_phi(); }

// simulator.cpp:23-42: substeps of the CFL step clamped to the frame
void Simulator::update(std::function<void(Simulator&, float)> f, float dt_frame, bool use_cfl) {
    if (!use_cfl) {
        f(*this, dt_frame);
        return;
    }
    float dt_total = 0;
    while (dt_total < dt_frame) {
        double dt_cfl = 0;
        check(el_calc_time_step(m_ctx, m_params.cfl, &dt_cfl));
        float dt_sub = (float)dt_cfl;
        if (dt_total + dt_sub > dt_frame) dt_sub = dt_frame - dt_total;
        f(*this, dt_sub);
        dt_total += dt_sub;
    }
}

void Simulator::advect_velocity(float dt) { check(el_advect_velocity(m_ctx, dt, EL_TRACE_RK2, EL_SAMPLE_TRILINEAR)); }
void Simulator::advect_level_set(float dt) { check(el_advect_level_set(m_ctx, dt, EL_TRACE_RK2, EL_SAMPLE_TRILINEAR)); }
void Simulator::add_gravity(float dt) { check(el_add_gravity(m_ctx, dt, gravity)); }
void Simulator::solve_pressure(float dt) {
    const int st = el_solve_pressure(m_ctx, dt, &solve_params, &last_solve);
    // like the reference, a solve that stops at the iteration cap is not an error
    if (st != EL_OK && st != EL_ERR_NOT_CONVERGED) check(st);
}
void Simulator::extrapolate_level_set() { check(el_extrapolate_level_set(m_ctx, 10)); }
void Simulator::extrapolate_velocity() { check(el_extrapolate_velocity(m_ctx, 10)); }
void Simulator::find_valid_velocity() { check(el_find_valid_velocity(m_ctx)); }
void Simulator::find_valid_level_set() { check(el_find_valid_level_set(m_ctx)); }
void Simulator::set_invalid_velocity_zero() { check(el_set_invalid_velocity_zero(m_ctx)); }
void Simulator::compute_weights() { check(el_compute_weights(m_ctx)); }
void Simulator::calc_cell_centered_solid_phi() { check(el_calc_cell_centered_solid_phi(m_ctx)); }

void Simulator::step_hot_path(float dt) {
    el_step_params p{EL_TRACE_RK2, EL_SAMPLE_TRILINEAR, EL_TRACE_RK2, EL_SAMPLE_TRILINEAR, gravity, 10, solve_params};
    el_step_stats st{};
    const int rc = el_step(m_ctx, dt, &p, &st);
    last_solve = st.solve;
    if (rc != EL_OK && rc != EL_ERR_NOT_CONVERGED) check(rc);
}

void Simulator::sync_to_host() {
    auto down = [&](int f, auto& g) { check(el_download(m_ctx, f, g.data(), g.size() * sizeof(g[0]))); };
    down(EL_FIELD_PHI, m_level_set);
    down(EL_FIELD_U, m_velocity.u());
    down(EL_FIELD_V, m_velocity.v());
    down(EL_FIELD_W, m_velocity.w());
    down(EL_FIELD_PRESSURE, m_pressure);
    down(EL_FIELD_SOLID_NODAL, m_nodal_solid_phi);
    down(EL_FIELD_SOLID_CELL, m_cell_centered_solid_level_set);
    down(EL_FIELD_WEIGHT_U, m_velocity_weight.u());
    down(EL_FIELD_WEIGHT_V, m_velocity_weight.v());
    down(EL_FIELD_WEIGHT_W, m_velocity_weight.w());
    down(EL_FIELD_VALID_U, m_velocity_valid.u());
    down(EL_FIELD_VALID_V, m_velocity_valid.v());
    down(EL_FIELD_VALID_W, m_velocity_valid.w());
    down(EL_FIELD_VALID_PHI, m_level_set_valid);
}

void Simulator::sync_to_device() {
    auto up = [&](int f, const auto& g) { check(el_upload(m_ctx, f, g.data(), g.size() * sizeof(g[0]))); };
    up(EL_FIELD_PHI, m_level_set);
    up(EL_FIELD_U, m_velocity.u());
    up(EL_FIELD_V, m_velocity.v());
    up(EL_FIELD_W, m_velocity.w());
    up(EL_FIELD_SOLID_NODAL, m_nodal_solid_phi);
    up(EL_FIELD_VALID_U, m_velocity_valid.u());
    up(EL_FIELD_VALID_V, m_velocity_valid.v());
    up(EL_FIELD_VALID_W, m_velocity_valid.w());
    up(EL_FIELD_VALID_PHI, m_level_set_valid);
}

}  // namespace eulerian_liquid
}  // namespace nama_gb300
