// ref_adapter.cpp -- instantiates the reference's own Eigen-free header templates
// (include/nama/math/interpolation.h, include/nama/math/ode.h) through a small duck-typed
// grid and 3-vector, and exports them over a C ABI so the oracle restatement can be checked
// against the reference bit for bit.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/build.py into oracle/_ref/ (git-ignored) and only
// when the reference tree is present; nothing in the product uses it.
//
// Interfaces the templates require (interpolation.h:35-72, 139-202; ode.h:7-35):
//   Grid: dim, value_type, coordinate_type, dx(), origin()[a], extrapolate(i,j,k)
//   StaggeredGrid: dim, operator[](d) -> Grid
//   TV: operator[], TV + TV, scalar * TV

#include <nama/math/interpolation.h>
#include <nama/math/ode.h>

#include <algorithm>

namespace refadapt {

template <typename T>
struct V3 {
    T c[3];
    T& operator[](int a) { return c[a]; }
    const T& operator[](int a) const { return c[a]; }
    V3 operator+(const V3& o) const { return {{c[0] + o.c[0], c[1] + o.c[1], c[2] + o.c[2]}}; }
    friend V3 operator*(T s, const V3& v) { return {{s * v.c[0], s * v.c[1], s * v.c[2]}}; }
};

template <typename T>
struct Grid {
    static constexpr int dim = 3;
    using value_type = T;
    using coordinate_type = T;
    const T* data;
    int n0, n1, n2;
    T h;
    V3<T> o;
    T dx() const { return h; }
    V3<T> origin() const { return o; }
    const T& extrapolate(int i, int j, int k) const {
        i = std::clamp(i, 0, n0 - 1);
        j = std::clamp(j, 0, n1 - 1);
        k = std::clamp(k, 0, n2 - 1);
        return data[i + (long long)n0 * (j + (long long)n1 * k)];
    }
    // GridBase::pos, written as the reference's grid.h:355-367 evaluates it
    V3<T> pos(int i, int j, int k) const {
        V3<T> r{{(i + static_cast<T>(0.5)) * h, (j + static_cast<T>(0.5)) * h,
                 (k + static_cast<T>(0.5)) * h}};
        return {{r[0] + o[0], r[1] + o[1], r[2] + o[2]}};
    }
};

template <typename T>
struct Staggered {
    static constexpr int dim = 3;
    Grid<T> g[3];
    const Grid<T>& operator[](int d) const { return g[d]; }
};

template <typename T>
Staggered<T> make_mac(int ni, int nj, int nk, T h, const T* u, const T* v, const T* w) {
    // staggered_grid.h:100-112: origin - (0.5,0,0)*dx etc.
    Staggered<T> s;
    s.g[0] = Grid<T>{u, ni + 1, nj, nk, h, {{T(0) - T(0.5) * h, T(0) - T(0) * h, T(0) - T(0) * h}}};
    s.g[1] = Grid<T>{v, ni, nj + 1, nk, h, {{T(0) - T(0) * h, T(0) - T(0.5) * h, T(0) - T(0) * h}}};
    s.g[2] = Grid<T>{w, ni, nj, nk + 1, h, {{T(0) - T(0) * h, T(0) - T(0) * h, T(0) - T(0.5) * h}}};
    return s;
}

template <typename T>
void advect(T* out, const Grid<T>& src, const Staggered<T>& mac, T dt, int weno) {
    nama::StaggeredGridField<Staggered<T>, V3<T>> field(mac);
    for (int k = 0; k < src.n2; ++k)
        for (int j = 0; j < src.n1; ++j)
            for (int i = 0; i < src.n0; ++i) {
                V3<T> foot = nama::math::trace_rk2(src.pos(i, j, k), -dt, field);
                out[i + (long long)src.n0 * (j + (long long)src.n1 * k)] =
                    weno ? nama::math::weno6_interp(foot, src) : nama::math::lerp(foot, src);
            }
}

}  // namespace refadapt

using namespace refadapt;

extern "C" {

#define REF_DEFINE(SUF, T)                                                                         \
    __attribute__((visibility("default"))) void ref_index_fraction_##SUF(double pos, double origin, \
                                                                         double dx, int* idx,      \
                                                                         T* frac) {                \
        auto [i, f] = nama::math::calc_index_and_fraction<T>((T)pos, (T)origin, (T)dx);            \
        *idx = i;                                                                                   \
        *frac = f;                                                                                  \
    }                                                                                               \
    __attribute__((visibility("default"))) T ref_weno6_1d_##SUF(const T* v, double f) {            \
        T ff[1] = {(T)f};                                                                           \
        return nama::math::weno6_interp_1d<T, T>(v, ff);                                            \
    }                                                                                               \
    __attribute__((visibility("default"))) T ref_sample_##SUF(const T* d, int n0, int n1, int n2,  \
                                                              double ox, double oy, double oz,     \
                                                              double dx, double x, double y,       \
                                                              double z, int weno) {                \
        Grid<T> g{d, n0, n1, n2, (T)dx, {{(T)ox, (T)oy, (T)oz}}};                                   \
        V3<T> p{{(T)x, (T)y, (T)z}};                                                                \
        return weno ? nama::math::weno6_interp(p, g) : nama::math::lerp(p, g);                      \
    }                                                                                               \
    __attribute__((visibility("default"))) void ref_trace_rk2_##SUF(                               \
        int ni, int nj, int nk, double dx, const T* u, const T* v, const T* w, double x, double y,  \
        double z, double dt, T* out3) {                                                             \
        auto mac = make_mac<T>(ni, nj, nk, (T)dx, u, v, w);                                         \
        nama::StaggeredGridField<Staggered<T>, V3<T>> field(mac);                                   \
        V3<T> r = nama::math::trace_rk2(V3<T>{{(T)x, (T)y, (T)z}}, (T)dt, field);                   \
        out3[0] = r[0];                                                                             \
        out3[1] = r[1];                                                                             \
        out3[2] = r[2];                                                                             \
    }                                                                                               \
    /* advect_collocated_grid / advect_staggered_grid loop bodies (advection.cpp:9-27) */          \
    __attribute__((visibility("default"))) void ref_advect_collocated_##SUF(                       \
        int ni, int nj, int nk, double dx, T* out, const T* phi, const T* u, const T* v,            \
        const T* w, double dt, int weno) {                                                          \
        auto mac = make_mac<T>(ni, nj, nk, (T)dx, u, v, w);                                         \
        Grid<T> src{phi, ni, nj, nk, (T)dx, {{T(0), T(0), T(0)}}};                                  \
        advect(out, src, mac, (T)dt, weno);                                                         \
    }                                                                                               \
    __attribute__((visibility("default"))) void ref_advect_staggered_##SUF(                        \
        int ni, int nj, int nk, double dx, T* ou, T* ov, T* ow, const T* u, const T* v,             \
        const T* w, double dt, int weno) {                                                          \
        auto mac = make_mac<T>(ni, nj, nk, (T)dx, u, v, w);                                         \
        advect(ou, mac.g[0], mac, (T)dt, weno);                                                     \
        advect(ov, mac.g[1], mac, (T)dt, weno);                                                     \
        advect(ow, mac.g[2], mac, (T)dt, weno);                                                     \
    }

REF_DEFINE(f32, float)
REF_DEFINE(f64, double)

}  // extern "C"
