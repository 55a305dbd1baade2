// oracle.cpp -- CPU restatement of daichi-nama/eulerian-liquid's per-step grid hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker: tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / --impl reference leg are the only users.  The product
// (eulerian-liquid_gb300/) never links, loads or calls it.
//
// Every routine is instantiated for T = float (the reference's own field type, with the
// reference's float->double promotions reproduced where its double literals cause them)
// and T = double (the FP64 restatement the GPU FP64 path is checked against to 1e-12).
// Compile with -ffp-contract=off so x86_64 and aarch64 give identical bits.
//
// Pinning: the interpolation / RK-trace part is pinned bit-for-bit against the reference's
// own header templates (include/nama/math/interpolation.h, include/nama/math/ode.h),
// compiled from the reference tree into oracle/_ref by oracle/build_ref.py, and against the
// known answers in test/math/interpolation.cpp:13-42 and test/common/grid.cpp:32-39.
// Projection, weights, extrapolation and masks need Eigen, which is absent, so they are
// restated here and checked by properties (symmetry, SPD, scipy direct solves); the
// Eigen ConjugateGradient/IncompleteCholesky call (simulator.cpp:102-109) is restated as
// standard PCG with Bridson's MIC(0) (or IC(0)/Jacobi) preconditioner: parity for the
// pressure is "to the solve tolerance", never bitwise.
//
// Layout: every array is i-fastest, index i + n0*(j + n1*k)   (include/nama/common/array.h:281-286)
//   phi, pressure: (ni, nj, nk), origin (0,0,0)
//   u / v / w and their face weights: (ni+1,nj,nk) / (ni,nj+1,nk) / (ni,nj,nk+1), origin shifted
//   by -dx/2 along the face normal (include/nama/common/staggered_grid.h:100-112)
//   nodal solid phi: (ni+1, nj+1, nk+1), origin (-dx/2,-dx/2,-dx/2)  (simulator.cpp:67-68)

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace orc {

using idx_t = long long;

template <typename T>
struct View {
    const T* d;
    int n0, n1, n2;
    T ox, oy, oz, dx;
    inline T at(int i, int j, int k) const { return d[i + (idx_t)n0 * (j + (idx_t)n1 * k)]; }
    // GridBase::extrapolate: clamp-to-edge read (include/nama/common/grid.h:369-377)
    inline T clamped(int i, int j, int k) const {
        i = std::clamp(i, 0, n0 - 1);
        j = std::clamp(j, 0, n1 - 1);
        k = std::clamp(k, 0, n2 - 1);
        return at(i, j, k);
    }
};

template <typename T>
struct Vec3 {
    T x, y, z;
};

// Shapes and origins of the scene's grids (staggered_grid.h:100-112, simulator.cpp:58-69).
// comp: 0 = cell centred (phi), 1/2/3 = u/v/w faces.
template <typename T>
inline View<T> make_view(const T* d, int ni, int nj, int nk, T dx, int comp) {
    View<T> g{d, ni, nj, nk, T(0), T(0), T(0), dx};
    const T half = T(0.5) * dx;
    if (comp == 1) { g.n0 = ni + 1; g.ox = T(0) - half; }
    if (comp == 2) { g.n1 = nj + 1; g.oy = T(0) - half; }
    if (comp == 3) { g.n2 = nk + 1; g.oz = T(0) - half; }
    return g;
}

// GridBase::pos (grid.h:355-367): (idx + 0.5) * dx + origin, per axis.
template <typename T>
inline Vec3<T> grid_pos(const View<T>& g, int i, int j, int k) {
    return {(i + T(0.5)) * g.dx + g.ox, (j + T(0.5)) * g.dx + g.oy, (k + T(0.5)) * g.dx + g.oz};
}

// calc_index_and_fraction (include/nama/math/interpolation.h:10-15)
template <typename T>
inline void index_fraction(T pos, T origin, T dx, int& idx, T& frac) {
    T t = (pos - origin - T(0.5) * dx) / dx;
    idx = (int)std::floor(t);
    frac = t - (T)idx;
}

template <typename T>
inline T lerp1(T a, T b, T f) {  // interpolation.h:17-21
    return (1 - f) * a + f * b;
}

// lerp(x, grid) for a 3-D grid: clamped 8-point gather, x then y then z (interpolation.h:35-72)
template <typename T>
inline T sample_trilinear(const View<T>& g, const Vec3<T>& p) {
    int i, j, k;
    T fx, fy, fz;
    index_fraction(p.x, g.ox, g.dx, i, fx);
    index_fraction(p.y, g.oy, g.dx, j, fy);
    index_fraction(p.z, g.oz, g.dx, k, fz);
    T c000 = g.clamped(i, j, k), c100 = g.clamped(i + 1, j, k);
    T c010 = g.clamped(i, j + 1, k), c110 = g.clamped(i + 1, j + 1, k);
    T c001 = g.clamped(i, j, k + 1), c101 = g.clamped(i + 1, j, k + 1);
    T c011 = g.clamped(i, j + 1, k + 1), c111 = g.clamped(i + 1, j + 1, k + 1);
    T lo = lerp1(lerp1(c000, c100, fx), lerp1(c010, c110, fx), fy);
    T hi = lerp1(lerp1(c001, c101, fx), lerp1(c011, c111, fx), fy);
    return lerp1(lo, hi, fz);
}

// Six-point WENO interpolation on nodes -2..3 with the interpolation point in [0, 1)
// (interpolation.h:74-111).  The three cubic candidates are written in Newton form; the
// smoothness indicators are the published quadratic forms (coefficients /180).  For T=float
// the reference's double literals (0.5, 6.0, 10.0, 20.0, 180.0) promote those
// sub-expressions to double before the result is stored back as float; that is reproduced
// with explicit double temporaries.
template <typename T>
inline T weno6_1d(const T v[6], T f) {
    const T eps = T(1e-6);
    T node[6];
    for (int n = 0; n < 6; ++n) node[n] = T(-2.0 + n);
    const T x = node[2] + f;
    T cand[3];
    for (int s = 0; s < 3; ++s) {
        const T e0 = x - node[s], e1 = x - node[s + 1], e2 = x - node[s + 2];
        const T first = v[s + 1] - v[s];
        const T second = v[s + 2] - 2 * v[s + 1] + v[s];
        const T third = v[s + 3] - 3 * v[s + 2] + 3 * v[s + 1] - v[s];
        const T linear = v[s] + first * e0;
        const double quad = (double)second * 0.5 * e0 * e1;
        const double cubic = (double)third / 6.0 * e0 * e1 * e2;
        cand[s] = (T)((double)linear + quad + cubic);
    }
    T gamma[3];
    gamma[0] = (T)((double)((node[4] - x) * (node[5] - x)) / 20.0);
    gamma[1] = (T)((double)((node[5] - x) * (x - node[0])) / 10.0);
    gamma[2] = (T)((double)((x - node[0]) * (x - node[1])) / 20.0);
    T beta[3];
    beta[0] = (T)((double)(814 * v[3] * v[3] + 4326 * v[2] * v[2] + 2976 * v[1] * v[1]
                           + 244 * v[0] * v[0] - 3579 * v[2] * v[3] - 6927 * v[2] * v[1]
                           + 1854 * v[2] * v[0] + 2634 * v[3] * v[1] - 683 * v[3] * v[0]
                           - 1659 * v[1] * v[0])
                  / 180.0);
    beta[1] = (T)((double)(1986 * v[3] * v[3] + 1986 * v[2] * v[2] + 244 * v[1] * v[1]
                           + 244 * v[4] * v[4] + 1074 * v[2] * v[4] - 3777 * v[2] * v[3]
                           - 1269 * v[2] * v[1] + 1074 * v[3] * v[1] - 1269 * v[4] * v[3]
                           - 293 * v[4] * v[1])
                  / 180.0);
    beta[2] = (T)((double)(814 * v[2] * v[2] + 4326 * v[3] * v[3] + 2976 * v[4] * v[4]
                           + 244 * v[5] * v[5] - 683 * v[2] * v[5] + 2634 * v[2] * v[4]
                           - 3579 * v[2] * v[3] - 6927 * v[3] * v[4] + 1854 * v[3] * v[5]
                           - 1659 * v[4] * v[5])
                  / 180.0);
    for (int s = 0; s < 3; ++s) gamma[s] /= (eps + beta[s]) * (eps + beta[s]);
    T wt[3];
    for (int s = 0; s < 3; ++s) wt[s] = gamma[s] / (gamma[0] + gamma[1] + gamma[2]);
    return wt[0] * cand[0] + wt[1] * cand[1] + wt[2] * cand[2];
}

// weno6_interp(x, grid) in 3-D: 6^3 clamped gather at offsets -2..3, 36 x-passes, 6 y-passes,
// 1 z-pass (interpolation.h:124-137, 166-183).
template <typename T>
inline T sample_weno6(const View<T>& g, const Vec3<T>& p) {
    int i, j, k;
    T fx, fy, fz;
    index_fraction(p.x, g.ox, g.dx, i, fx);
    index_fraction(p.y, g.oy, g.dx, j, fy);
    index_fraction(p.z, g.oz, g.dx, k, fz);
    T zline[6];
    for (int dk = 0; dk < 6; ++dk) {
        T yline[6];
        for (int dj = 0; dj < 6; ++dj) {
            T xline[6];
            for (int di = 0; di < 6; ++di) xline[di] = g.clamped(i + di - 2, j + dj - 2, k + dk - 2);
            yline[dj] = weno6_1d(xline, fx);
        }
        zline[dk] = weno6_1d(yline, fy);
    }
    return weno6_1d(zline, fz);
}

// StaggeredGridField: trilinear velocity of the MAC grid at a point (include/nama/math/ode.h:7-18)
template <typename T>
struct Velocity {
    View<T> u, v, w;
    inline Vec3<T> operator()(const Vec3<T>& p) const {
        return {sample_trilinear(u, p), sample_trilinear(v, p), sample_trilinear(w, p)};
    }
};

enum { TRACE_RK2 = 0, TRACE_RK3 = 1 };
enum { SAMPLE_TRILINEAR = 0, SAMPLE_WENO6 = 1 };

// trace_rk2, midpoint rule (ode.h:30-35).  dt is the signed step (the caller passes -dt).
template <typename T>
inline Vec3<T> trace_rk2(const Vec3<T>& p, T dt, const Velocity<T>& vel) {
    Vec3<T> k1 = vel(p);
    const T h = T(0.5) * dt;
    Vec3<T> k2 = vel({p.x + h * k1.x, p.y + h * k1.y, p.z + h * k1.z});
    return {p.x + dt * k2.x, p.y + dt * k2.y, p.z + dt * k2.z};
}

// RK3 backtrace: Ralston's third-order tableau (c = 0, 1/2, 3/4; b = 2/9, 1/3, 4/9).  The
// reference has no RK3 (ode.h:24-35 has RK1/RK2 only); this is the project's definition.
template <typename T>
inline Vec3<T> trace_rk3(const Vec3<T>& p, T dt, const Velocity<T>& vel) {
    Vec3<T> k1 = vel(p);
    const T h2 = T(0.5) * dt;
    Vec3<T> k2 = vel({p.x + h2 * k1.x, p.y + h2 * k1.y, p.z + h2 * k1.z});
    const T h3 = T(0.75) * dt;
    Vec3<T> k3 = vel({p.x + h3 * k2.x, p.y + h3 * k2.y, p.z + h3 * k2.z});
    const T b1 = dt * (T(2) / T(9)), b2 = dt * (T(1) / T(3)), b3 = dt * (T(4) / T(9));
    return {p.x + b1 * k1.x + b2 * k2.x + b3 * k3.x, p.y + b1 * k1.y + b2 * k2.y + b3 * k3.y,
            p.z + b1 * k1.z + b2 * k2.z + b3 * k3.z};
}

template <typename T>
inline Vec3<T> trace(const Vec3<T>& p, T dt, const Velocity<T>& vel, int scheme_trace) {
    return scheme_trace == TRACE_RK3 ? trace_rk3(p, dt, vel) : trace_rk2(p, dt, vel);
}

template <typename T>
inline T sample(const View<T>& g, const Vec3<T>& p, int scheme_sample) {
    return scheme_sample == SAMPLE_WENO6 ? sample_weno6(g, p) : sample_trilinear(g, p);
}

// Advect one grid (cell-centred or one face component) through the old MAC velocity:
// out(x) = src(trace(x, -dt, vel))  (src/project/3d/fluid/advection.cpp:9-27).
template <typename T>
void advect_grid(T* out, const View<T>& src, const Velocity<T>& vel, T dt, int scheme_trace,
                 int scheme_sample) {
    const T mdt = -dt;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < src.n2; ++k)
        for (int j = 0; j < src.n1; ++j)
            for (int i = 0; i < src.n0; ++i) {
                Vec3<T> foot = trace(grid_pos(src, i, j, k), mdt, vel, scheme_trace);
                out[i + (idx_t)src.n0 * (j + (idx_t)src.n1 * k)] = sample(src, foot, scheme_sample);
            }
}

// fraction_inside(phi_left, phi_right): liquid fraction of a segment (include/nama/math/level_set.h:68-80)
template <typename T>
inline T fraction_inside(T a, T b) {
    if (a < T(0) && b < T(0)) return T(1);
    if (a < T(0) && b >= T(0)) return a / (a - b);
    if (a >= T(0) && b < T(0)) return b / (b - a);
    return T(0);
}

// fraction_inside(bl, br, tl, tr): inside area fraction of a square from its corner values
// (level_set.h:82-163, after Batty's Fluid3D).  Corners are walked in the cyclic order
// bl, br, tr, tl.  The reference's 0.5 / 0.25 literals are double; for T=float the
// products are formed in double and rounded on return, reproduced here.
template <typename T>
inline T fraction_inside4(T bl, T br, T tl, T tr) {
    const int inside = (bl < T(0)) + (tl < T(0)) + (br < T(0)) + (tr < T(0));
    T c[4] = {bl, br, tr, tl};
    auto rotate = [&c]() {
        T t = c[0];
        c[0] = c[1];
        c[1] = c[2];
        c[2] = c[3];
        c[3] = t;
    };
    if (inside == 4) return T(1);
    if (inside == 3) {
        while (c[0] < 0) rotate();
        T s0 = 1 - fraction_inside(c[0], c[3]);
        T s1 = 1 - fraction_inside(c[0], c[1]);
        return (T)(1 - 0.5 * s0 * s1);
    }
    if (inside == 2) {
        while (c[0] >= 0 || !(c[1] < 0 || c[2] < 0)) rotate();
        if (c[1] < 0) {
            T left = fraction_inside(c[0], c[3]);
            T right = fraction_inside(c[1], c[2]);
            return (T)(0.5 * (left + right));
        }
        T centre = (T)(0.25 * (c[0] + c[1] + c[2] + c[3]));
        if (centre < 0) {
            T area = 0;
            T s1 = 1 - fraction_inside(c[0], c[3]);
            T s3 = 1 - fraction_inside(c[2], c[3]);
            area = (T)(area + 0.5 * s1 * s3);
            T s2 = 1 - fraction_inside(c[2], c[1]);
            T s0 = 1 - fraction_inside(c[0], c[1]);
            area = (T)(area + 0.5 * s0 * s2);
            return 1 - area;
        }
        T area = 0;
        T s0 = fraction_inside(c[0], c[1]);
        T s1 = fraction_inside(c[0], c[3]);
        area = (T)(area + 0.5 * s0 * s1);
        T s2 = fraction_inside(c[2], c[1]);
        T s3 = fraction_inside(c[2], c[3]);
        area = (T)(area + 0.5 * s2 * s3);
        return area;
    }
    if (inside == 1) {
        while (c[0] >= 0) rotate();
        T s0 = fraction_inside(c[0], c[3]);
        T s1 = fraction_inside(c[0], c[1]);
        return (T)(0.5 * s0 * s1);
    }
    return T(0);
}

// compute_staggered_grid_weight: open fraction of each face from the nodal solid level set,
// clamped to [0,1] (src/project/3d/fluid/boundary.cpp:6-34).
template <typename T>
void compute_weights(int ni, int nj, int nk, const T* solid, T* wu, T* wv, T* ww) {
    const int s0 = ni + 1, s1 = nj + 1;
    auto S = [&](int i, int j, int k) { return solid[i + (idx_t)s0 * (j + (idx_t)s1 * k)]; };
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni + 1; ++i) {
                T f = 1 - fraction_inside4(S(i, j, k), S(i, j + 1, k), S(i, j, k + 1), S(i, j + 1, k + 1));
                wu[i + (idx_t)(ni + 1) * (j + (idx_t)nj * k)] = std::clamp(f, T(0), T(1));
            }
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj + 1; ++j)
            for (int i = 0; i < ni; ++i) {
                T f = 1 - fraction_inside4(S(i, j, k), S(i, j, k + 1), S(i + 1, j, k), S(i + 1, j, k + 1));
                wv[i + (idx_t)ni * (j + (idx_t)(nj + 1) * k)] = std::clamp(f, T(0), T(1));
            }
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nk + 1; ++k)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                T f = 1 - fraction_inside4(S(i, j, k), S(i, j + 1, k), S(i + 1, j, k), S(i + 1, j + 1, k));
                ww[i + (idx_t)ni * (j + (idx_t)nj * k)] = std::clamp(f, T(0), T(1));
            }
}

template <typename T>
struct Faces {
    int ni, nj, nk;
    const T *u, *v, *w;
    inline T U(int i, int j, int k) const { return u[i + (idx_t)(ni + 1) * (j + (idx_t)nj * k)]; }
    inline T V(int i, int j, int k) const { return v[i + (idx_t)ni * (j + (idx_t)(nj + 1) * k)]; }
    inline T W(int i, int j, int k) const { return w[i + (idx_t)ni * (j + (idx_t)nj * k)]; }
};

// is_pressure_valid: any of the cell's six face weights is positive (projection.cpp:8-12).
// Cells outside the grid are not valid (the reference reads out of range there; every scene
// it builds has zero-weight walls so the case never arises).
template <typename T>
inline bool pressure_valid(const Faces<T>& wt, int i, int j, int k) {
    if (i < 0 || j < 0 || k < 0 || i >= wt.ni || j >= wt.nj || k >= wt.nk) return false;
    return wt.U(i, j, k) > 0 || wt.U(i + 1, j, k) > 0 || wt.V(i, j, k) > 0 || wt.V(i, j + 1, k) > 0
           || wt.W(i, j, k) > 0 || wt.W(i, j, k + 1) > 0;
}

static constexpr int UNKNOWN_INDEX = std::numeric_limits<int>::max();

// assign_indices: serial k-j-i numbering of liquid, pressure-valid cells (projection.cpp:14-28).
// Returns the count; 0 means the reference's "No fluid" exception.
template <typename T>
int assign_indices(int ni, int nj, int nk, const T* phi, const Faces<T>& wt, int* indices) {
    int n = 0;
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                idx_t c = i + (idx_t)ni * (j + (idx_t)nj * k);
                indices[c] = (pressure_valid(wt, i, j, k) && phi[c] < 0) ? n++ : UNKNOWN_INDEX;
            }
    return n;
}

// build_matrix, grid-shaped (projection.cpp:30-83).  For each liquid cell, neighbours are
// visited -x, +x, -y, +y, -z, +z; a valid liquid neighbour adds w to the diagonal and -w
// off-diagonal, a valid air neighbour adds w / max(theta, 0.01) (ghost fluid), a solid one
// adds nothing; the right-hand side always gets -/+ w * u_face; finally b *= dx / dt.
// off_x[c] holds A(c, c+x) (and by symmetry A(c+x, c)); likewise off_y, off_z.
template <typename T>
void build_matrix(int ni, int nj, int nk, const T* phi, const Faces<T>& vel, const Faces<T>& wt,
                  T dt, T dx, double* diag, double* offx, double* offy, double* offz, double* rhs) {
    const idx_t N = (idx_t)ni * nj * nk;
    auto P = [&](int i, int j, int k) { return phi[i + (idx_t)ni * (j + (idx_t)nj * k)]; };
    const T scale = dx / dt;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                const idx_t c = i + (idx_t)ni * (j + (idx_t)nj * k);
                diag[c] = offx[c] = offy[c] = offz[c] = rhs[c] = 0.0;
                if (!(pressure_valid(wt, i, j, k) && P(i, j, k) < 0)) continue;
                double d = 0.0, b = 0.0;
                const T pc = P(i, j, k);
                auto visit = [&](int x, int y, int z, T face_vel, T weight, bool forward, double* off) {
                    if (pressure_valid(wt, x, y, z)) {
                        if (P(x, y, z) < 0) {
                            d += weight;
                            if (off) *off = -(double)weight;
                        } else {
                            T theta = fraction_inside(pc, P(x, y, z));
                            theta = std::max(theta, T(0.01));
                            d += weight / theta;
                        }
                    }
                    if (forward)
                        b -= weight * face_vel;
                    else
                        b += weight * face_vel;
                };
                visit(i - 1, j, k, vel.U(i, j, k), wt.U(i, j, k), false, nullptr);
                visit(i + 1, j, k, vel.U(i + 1, j, k), wt.U(i + 1, j, k), true, &offx[c]);
                visit(i, j - 1, k, vel.V(i, j, k), wt.V(i, j, k), false, nullptr);
                visit(i, j + 1, k, vel.V(i, j + 1, k), wt.V(i, j + 1, k), true, &offy[c]);
                visit(i, j, k - 1, vel.W(i, j, k), wt.W(i, j, k), false, nullptr);
                visit(i, j, k + 1, vel.W(i, j, k + 1), wt.W(i, j, k + 1), true, &offz[c]);
                diag[c] = d;
                rhs[c] = b * (double)scale;
            }
    (void)N;
}

// update_velocity_using_pressure (projection.cpp:93-134): interior faces only, with the
// reference's loop ranges [1, n-1) on the tangential axes.
template <typename T>
void update_velocity(int ni, int nj, int nk, T* u, T* v, T* w, const T* p, const T* phi, T dt, T dx) {
    auto C = [&](int i, int j, int k) { return (idx_t)i + (idx_t)ni * (j + (idx_t)nj * k); };
    auto face = [&](T* f, idx_t fi, idx_t a, idx_t b) {
        if (phi[b] < 0 || phi[a] < 0) {
            T theta = 1;
            if (phi[b] >= 0 || phi[a] >= 0) theta = fraction_inside(phi[a], phi[b]);
            theta = std::max(theta, T(0.01));
            f[fi] -= dt * (p[b] - p[a]) / (dx * theta);
        }
    };
#pragma omp parallel for collapse(2)
    for (int k = 1; k < nk - 1; ++k)
        for (int j = 1; j < nj - 1; ++j)
            for (int i = 1; i < ni; ++i) face(u, i + (idx_t)(ni + 1) * (j + (idx_t)nj * k), C(i - 1, j, k), C(i, j, k));
#pragma omp parallel for collapse(2)
    for (int k = 1; k < nk - 1; ++k)
        for (int j = 1; j < nj; ++j)
            for (int i = 1; i < ni - 1; ++i) face(v, i + (idx_t)ni * (j + (idx_t)(nj + 1) * k), C(i, j - 1, k), C(i, j, k));
#pragma omp parallel for collapse(2)
    for (int k = 1; k < nk; ++k)
        for (int j = 1; j < nj - 1; ++j)
            for (int i = 1; i < ni - 1; ++i) face(w, i + (idx_t)ni * (j + (idx_t)nj * k), C(i, j, k - 1), C(i, j, k));
}

// extrapolate: Jacobi layers; each invalid cell with valid 26-neighbours takes their mean
// (z, y, x loop order) and becomes valid; stops early when no cell was invalid
// (src/project/3d/fluid/extrapolation.cpp:5-46).
template <typename T>
void extrapolate(T* grid, uint8_t* valid, int n0, int n1, int n2, int layers) {
    const idx_t N = (idx_t)n0 * n1 * n2;
    std::vector<T> tmp(grid, grid + N);
    std::vector<uint8_t> old(N);
    for (int l = 0; l < layers; ++l) {
        std::memcpy(old.data(), valid, N);
        int any_invalid = 0;
#pragma omp parallel for collapse(2) reduction(| : any_invalid)
        for (int k = 0; k < n2; ++k)
            for (int j = 0; j < n1; ++j)
                for (int i = 0; i < n0; ++i) {
                    const idx_t c = i + (idx_t)n0 * (j + (idx_t)n1 * k);
                    if (old[c]) continue;
                    any_invalid = 1;
                    T sum = 0;
                    int count = 0;
                    for (int dk = -1; dk <= 1; ++dk)
                        for (int dj = -1; dj <= 1; ++dj)
                            for (int di = -1; di <= 1; ++di) {
                                int x = i + di, y = j + dj, z = k + dk;
                                if (x < 0 || x >= n0 || y < 0 || y >= n1 || z < 0 || z >= n2) continue;
                                idx_t q = x + (idx_t)n0 * (y + (idx_t)n1 * z);
                                if (old[q]) {
                                    sum += grid[q];
                                    ++count;
                                }
                            }
                    if (count > 0) {
                        tmp[c] = sum / static_cast<T>(count);
                        valid[c] = 1;
                    }
                }
        if (!any_invalid) return;
        std::memcpy(grid, tmp.data(), N * sizeof(T));
    }
}

// find_valid_velocity (simulator.cpp:125-158)
template <typename T>
void find_valid_velocity(int ni, int nj, int nk, const T* phi, const Faces<T>& wt, uint8_t* vu,
                         uint8_t* vv, uint8_t* vw) {
    const idx_t Nu = (idx_t)(ni + 1) * nj * nk, Nv = (idx_t)ni * (nj + 1) * nk, Nw = (idx_t)ni * nj * (nk + 1);
    for (idx_t q = 0; q < Nu; ++q) vu[q] = wt.u[q] == 0 ? 0 : 1;
    for (idx_t q = 0; q < Nv; ++q) vv[q] = wt.v[q] == 0 ? 0 : 1;
    for (idx_t q = 0; q < Nw; ++q) vw[q] = wt.w[q] == 0 ? 0 : 1;
    auto P = [&](int i, int j, int k) { return phi[i + (idx_t)ni * (j + (idx_t)nj * k)]; };
    for (int k = 1; k < nk - 1; ++k)
        for (int j = 1; j < nj - 1; ++j)
            for (int i = 1; i < ni; ++i)
                if (P(i - 1, j, k) >= 0 && P(i, j, k) >= 0) vu[i + (idx_t)(ni + 1) * (j + (idx_t)nj * k)] = 0;
    for (int k = 1; k < nk - 1; ++k)
        for (int j = 1; j < nj; ++j)
            for (int i = 1; i < ni - 1; ++i)
                if (P(i, j - 1, k) >= 0 && P(i, j, k) >= 0) vv[i + (idx_t)ni * (j + (idx_t)(nj + 1) * k)] = 0;
    for (int k = 1; k < nk; ++k)
        for (int j = 1; j < nj - 1; ++j)
            for (int i = 1; i < ni - 1; ++i)
                if (P(i, j, k - 1) >= 0 && P(i, j, k) >= 0) vw[i + (idx_t)ni * (j + (idx_t)nj * k)] = 0;
}

// ---------------------------------------------------------------------------------------
// Conjugate gradients on the grid-shaped matrix (the Eigen ConjugateGradient call in
// simulator.cpp:102-109): x0 = 0, stop when |r|^2 < tol^2 |b|^2 on the recursively
// updated residual, at most maxit iterations.  Active rows are those with diag > 0.
enum { PRE_NONE = 0, PRE_JACOBI = 1, PRE_IC0 = 2, PRE_MIC0 = 3 };

struct GridMatrix {
    int n0, n1, n2;
    const double *diag, *ox, *oy, *oz;
    idx_t N() const { return (idx_t)n0 * n1 * n2; }
};

static void spmv(const GridMatrix& A, const double* p, double* out) {
    const int n0 = A.n0, n1 = A.n1, n2 = A.n2;
    const idx_t sx = 1, sy = n0, sz = (idx_t)n0 * n1;
#pragma omp parallel for collapse(2)
    for (int k = 0; k < n2; ++k)
        for (int j = 0; j < n1; ++j)
            for (int i = 0; i < n0; ++i) {
                const idx_t c = i + sy * j + sz * k;
                if (A.diag[c] == 0.0) {
                    out[c] = 0.0;
                    continue;
                }
                double s = A.diag[c] * p[c];
                if (i > 0) s += A.ox[c - sx] * p[c - sx];
                if (i < n0 - 1) s += A.ox[c] * p[c + sx];
                if (j > 0) s += A.oy[c - sy] * p[c - sy];
                if (j < n1 - 1) s += A.oy[c] * p[c + sy];
                if (k > 0) s += A.oz[c - sz] * p[c - sz];
                if (k < n2 - 1) s += A.oz[c] * p[c + sz];
                out[c] = s;
            }
}

static double dot(const double* a, const double* b, idx_t n) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s)
    for (idx_t q = 0; q < n; ++q) s += a[q] * b[q];
    return s;
}

// Incomplete Cholesky on the 7-point pattern in natural (i-fastest) order, in Bridson's
// formulation ("Fluid Simulation for Computer Graphics", 2nd ed., sec. 5.4): tau = 0 gives
// IC(0), tau = 0.97 gives MIC(0); sigma = 0.25 is the safety fallback to the plain diagonal.
static void factor_ic(const GridMatrix& A, double tau, double sigma, double* precon) {
    const int n0 = A.n0, n1 = A.n1, n2 = A.n2;
    const idx_t sy = n0, sz = (idx_t)n0 * n1;
    for (int k = 0; k < n2; ++k)
        for (int j = 0; j < n1; ++j)
            for (int i = 0; i < n0; ++i) {
                const idx_t c = i + sy * j + sz * k;
                precon[c] = 0.0;
                if (A.diag[c] == 0.0) continue;
                double e = A.diag[c];
                if (i > 0) {
                    const idx_t q = c - 1;
                    const double a = A.ox[q] * precon[q];
                    e -= a * a + tau * A.ox[q] * (A.oy[q] + A.oz[q]) * precon[q] * precon[q];
                }
                if (j > 0) {
                    const idx_t q = c - sy;
                    const double a = A.oy[q] * precon[q];
                    e -= a * a + tau * A.oy[q] * (A.ox[q] + A.oz[q]) * precon[q] * precon[q];
                }
                if (k > 0) {
                    const idx_t q = c - sz;
                    const double a = A.oz[q] * precon[q];
                    e -= a * a + tau * A.oz[q] * (A.ox[q] + A.oy[q]) * precon[q] * precon[q];
                }
                if (e < sigma * A.diag[c]) e = A.diag[c];
                precon[c] = 1.0 / std::sqrt(e);
            }
}

static void apply_ic(const GridMatrix& A, const double* precon, const double* r, double* q, double* z) {
    const int n0 = A.n0, n1 = A.n1, n2 = A.n2;
    const idx_t sy = n0, sz = (idx_t)n0 * n1;
    for (int k = 0; k < n2; ++k)
        for (int j = 0; j < n1; ++j)
            for (int i = 0; i < n0; ++i) {
                const idx_t c = i + sy * j + sz * k;
                if (A.diag[c] == 0.0) {
                    q[c] = 0.0;
                    continue;
                }
                double t = r[c];
                if (i > 0) t -= A.ox[c - 1] * precon[c - 1] * q[c - 1];
                if (j > 0) t -= A.oy[c - sy] * precon[c - sy] * q[c - sy];
                if (k > 0) t -= A.oz[c - sz] * precon[c - sz] * q[c - sz];
                q[c] = t * precon[c];
            }
    for (int k = n2 - 1; k >= 0; --k)
        for (int j = n1 - 1; j >= 0; --j)
            for (int i = n0 - 1; i >= 0; --i) {
                const idx_t c = i + sy * j + sz * k;
                if (A.diag[c] == 0.0) {
                    z[c] = 0.0;
                    continue;
                }
                double t = q[c];
                if (i < n0 - 1) t -= A.ox[c] * precon[c] * z[c + 1];
                if (j < n1 - 1) t -= A.oy[c] * precon[c] * z[c + sy];
                if (k < n2 - 1) t -= A.oz[c] * precon[c] * z[c + sz];
                z[c] = t * precon[c];
            }
}

static int pcg(const GridMatrix& A, const double* b, double* x, int precond, double tol, int maxit,
               int* iters_out, double* relres_out) {
    const idx_t N = A.N();
    std::vector<double> r(b, b + N), z(N), p(N), Ap(N), precon, qtmp;
    std::fill(x, x + N, 0.0);
    const double bb = dot(b, b, N);
    *iters_out = 0;
    *relres_out = 0.0;
    if (bb == 0.0) return 0;
    if (precond == PRE_IC0 || precond == PRE_MIC0) {
        precon.resize(N);
        qtmp.resize(N);
        factor_ic(A, precond == PRE_MIC0 ? 0.97 : 0.0, 0.25, precon.data());
    }
    auto apply_pre = [&](const double* in, double* out) {
        if (precond == PRE_JACOBI) {
#pragma omp parallel for
            for (idx_t q = 0; q < N; ++q) out[q] = A.diag[q] > 0.0 ? in[q] / A.diag[q] : 0.0;
        } else if (precond == PRE_IC0 || precond == PRE_MIC0) {
            apply_ic(A, precon.data(), in, qtmp.data(), out);
        } else {
            std::memcpy(out, in, N * sizeof(double));
        }
    };
    const double threshold = tol * tol * bb;
    double rr = bb;
    if (rr < threshold) {
        *relres_out = std::sqrt(rr / bb);
        return 0;
    }
    apply_pre(r.data(), p.data());
    double rz = dot(r.data(), p.data(), N);
    int it = 0;
    while (it < maxit) {
        spmv(A, p.data(), Ap.data());
        const double alpha = rz / dot(p.data(), Ap.data(), N);
#pragma omp parallel for
        for (idx_t q = 0; q < N; ++q) {
            x[q] += alpha * p[q];
            r[q] -= alpha * Ap[q];
        }
        rr = dot(r.data(), r.data(), N);
        ++it;
        if (rr < threshold) break;
        apply_pre(r.data(), z.data());
        const double rz_new = dot(r.data(), z.data(), N);
        const double beta = rz_new / rz;
        rz = rz_new;
#pragma omp parallel for
        for (idx_t q = 0; q < N; ++q) p[q] = z[q] + beta * p[q];
    }
    *iters_out = it;
    *relres_out = std::sqrt(rr / bb);
    return rr < threshold ? 0 : 1;
}

// ---------------------------------------------------------------------------------------
// Level-set emitters (src/project/3d/fluid/levelset_emitter.cpp:10-79): each writes
// min(grid, f(x)) at its grid's sample positions; the list starts from FLT_MAX.
// sphere: (x - c).norm() - r with Eigen::Vector3f, whose unrolled three-term reduction sums
// x^2 + (y^2 + z^2) (pinned against the reference's levelset_emitter.cpp:10-12 compiled here)
template <typename T>
inline T sphere_sdf(const Vec3<T>& p, T cx, T cy, T cz, T r) {
    T dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
    return std::sqrt(dx * dx + (dy * dy + dz * dz)) - r;
}

// Exact signed distance to an axis-aligned box [lo, hi] (new: the reference has no box).
// Axes whose extent is given as infinite are ignored (a slab / quarter space).
template <typename T>
inline T box_sdf(const Vec3<T>& p, const T lo[3], const T hi[3]) {
    const T pc[3] = {p.x, p.y, p.z};
    T outside2 = 0, inside = -std::numeric_limits<T>::max();
    for (int a = 0; a < 3; ++a) {
        T q = std::max(lo[a] - pc[a], pc[a] - hi[a]);
        if (q > 0) outside2 += q * q;
        inside = std::max(inside, q);
    }
    return outside2 > 0 ? std::sqrt(outside2) : inside;
}

}  // namespace orc

using namespace orc;

// =========================================================================================
// C entry points (ctypes).  _f32 / _f64 suffix = field type T.
extern "C" {

#define OR_EXPORT __attribute__((visibility("default")))

#define DEFINE_ADVECT(SUF, T)                                                                      \
    OR_EXPORT void or_advect_collocated_##SUF(int ni, int nj, int nk, double dx, T* out,             \
                                              const T* phi, const T* u, const T* v, const T* w,      \
                                              double dt, int scheme_trace, int scheme_sample) {      \
        const T tdx = (T)dx;                                                                        \
        Velocity<T> vel{make_view(u, ni, nj, nk, tdx, 1), make_view(v, ni, nj, nk, tdx, 2),         \
                        make_view(w, ni, nj, nk, tdx, 3)};                                           \
        advect_grid(out, make_view(phi, ni, nj, nk, tdx, 0), vel, (T)dt, scheme_trace, scheme_sample); \
    }                                                                                               \
    OR_EXPORT void or_advect_staggered_##SUF(int ni, int nj, int nk, double dx, T* out_u, T* out_v,  \
                                             T* out_w, const T* u, const T* v, const T* w,           \
                                             double dt, int scheme_trace, int scheme_sample) {       \
        const T tdx = (T)dx;                                                                        \
        Velocity<T> vel{make_view(u, ni, nj, nk, tdx, 1), make_view(v, ni, nj, nk, tdx, 2),         \
                        make_view(w, ni, nj, nk, tdx, 3)};                                           \
        advect_grid(out_u, vel.u, vel, (T)dt, scheme_trace, scheme_sample);                         \
        advect_grid(out_v, vel.v, vel, (T)dt, scheme_trace, scheme_sample);                         \
        advect_grid(out_w, vel.w, vel, (T)dt, scheme_trace, scheme_sample);                         \
    }                                                                                               \
    OR_EXPORT T or_sample_trilinear_##SUF(const T* d, int n0, int n1, int n2, double ox, double oy,  \
                                          double oz, double dx, double x, double y, double z) {     \
        View<T> g{d, n0, n1, n2, (T)ox, (T)oy, (T)oz, (T)dx};                                       \
        return sample_trilinear(g, Vec3<T>{(T)x, (T)y, (T)z});                                      \
    }                                                                                               \
    OR_EXPORT T or_sample_weno6_##SUF(const T* d, int n0, int n1, int n2, double ox, double oy,      \
                                      double oz, double dx, double x, double y, double z) {         \
        View<T> g{d, n0, n1, n2, (T)ox, (T)oy, (T)oz, (T)dx};                                       \
        return sample_weno6(g, Vec3<T>{(T)x, (T)y, (T)z});                                          \
    }                                                                                               \
    OR_EXPORT void or_index_fraction_##SUF(double pos, double origin, double dx, int* idx, T* frac) { \
        index_fraction((T)pos, (T)origin, (T)dx, *idx, *frac);                                      \
    }                                                                                               \
    OR_EXPORT void or_trace_##SUF(int ni, int nj, int nk, double dx, const T* u, const T* v,         \
                                  const T* w, double x, double y, double z, double dt, int scheme,  \
                                  T* out3) {                                                        \
        const T tdx = (T)dx;                                                                        \
        Velocity<T> vel{make_view(u, ni, nj, nk, tdx, 1), make_view(v, ni, nj, nk, tdx, 2),         \
                        make_view(w, ni, nj, nk, tdx, 3)};                                           \
        Vec3<T> r = trace(Vec3<T>{(T)x, (T)y, (T)z}, (T)dt, vel, scheme);                           \
        out3[0] = r.x;                                                                              \
        out3[1] = r.y;                                                                              \
        out3[2] = r.z;                                                                              \
    }                                                                                               \
    OR_EXPORT T or_fraction_inside_##SUF(T a, T b) { return fraction_inside(a, b); }                 \
    OR_EXPORT T or_fraction_inside4_##SUF(T bl, T br, T tl, T tr) { return fraction_inside4(bl, br, tl, tr); } \
    OR_EXPORT void or_compute_weights_##SUF(int ni, int nj, int nk, const T* solid, T* wu, T* wv,     \
                                            T* ww) {                                                \
        compute_weights(ni, nj, nk, solid, wu, wv, ww);                                             \
    }                                                                                               \
    OR_EXPORT int or_assign_indices_##SUF(int ni, int nj, int nk, const T* phi, const T* wu,        \
                                          const T* wv, const T* ww, int* indices) {                 \
        Faces<T> wt{ni, nj, nk, wu, wv, ww};                                                        \
        return assign_indices(ni, nj, nk, phi, wt, indices);                                        \
    }                                                                                               \
    OR_EXPORT void or_build_matrix_##SUF(int ni, int nj, int nk, double dx, const T* phi,           \
                                         const T* u, const T* v, const T* w, const T* wu,           \
                                         const T* wv, const T* ww, double dt, double* diag,         \
                                         double* offx, double* offy, double* offz, double* rhs) {   \
        Faces<T> vel{ni, nj, nk, u, v, w}, wt{ni, nj, nk, wu, wv, ww};                              \
        build_matrix(ni, nj, nk, phi, vel, wt, (T)dt, (T)dx, diag, offx, offy, offz, rhs);         \
    }                                                                                               \
    OR_EXPORT void or_update_velocity_##SUF(int ni, int nj, int nk, double dx, T* u, T* v, T* w,     \
                                            const T* p, const T* phi, double dt) {                  \
        update_velocity(ni, nj, nk, u, v, w, p, phi, (T)dt, (T)dx);                                 \
    }                                                                                               \
    OR_EXPORT void or_extrapolate_##SUF(T* grid, uint8_t* valid, int n0, int n1, int n2, int layers) { \
        extrapolate(grid, valid, n0, n1, n2, layers);                                               \
    }                                                                                               \
    OR_EXPORT void or_find_valid_velocity_##SUF(int ni, int nj, int nk, const T* phi, const T* wu,  \
                                                const T* wv, const T* ww, uint8_t* vu, uint8_t* vv, \
                                                uint8_t* vw) {                                      \
        Faces<T> wt{ni, nj, nk, wu, wv, ww};                                                        \
        find_valid_velocity(ni, nj, nk, phi, wt, vu, vv, vw);                                       \
    }                                                                                               \
    /* calc_cell_centered_solid_phi (simulator.cpp:191-200): mean of 8 nodal values */              \
    OR_EXPORT void or_cell_solid_phi_##SUF(int ni, int nj, int nk, const T* solid, T* out) {         \
        const int s0 = ni + 1, s1 = nj + 1;                                                         \
        auto S = [&](int i, int j, int k) { return solid[i + (idx_t)s0 * (j + (idx_t)s1 * k)]; };   \
        for (int k = 0; k < nk; ++k)                                                                \
            for (int j = 0; j < nj; ++j)                                                            \
                for (int i = 0; i < ni; ++i)                                                        \
                    out[i + (idx_t)ni * (j + (idx_t)nj * k)] =                                      \
                        (T)((S(i, j, k) + S(i + 1, j, k) + S(i, j + 1, k) + S(i + 1, j + 1, k)      \
                             + S(i, j, k + 1) + S(i + 1, j, k + 1) + S(i, j + 1, k + 1)             \
                             + S(i + 1, j + 1, k + 1)) * 0.125);                                    \
    }                                                                                               \
    /* max_absolute_value over u, v, w (staggered_grid.h:230-248) */                                \
    OR_EXPORT T or_max_abs_##SUF(const T* a, long long n) {                                         \
        T m = 0;                                                                                    \
        for (long long q = 0; q < n; ++q) m = std::max(m, (T)std::fabs(a[q]));                      \
        return m;                                                                                   \
    }                                                                                               \
    /* emitters: min(grid, sdf) at grid positions of a (n0,n1,n2) grid with the given origin */    \
    OR_EXPORT void or_emit_sphere_##SUF(T* g, int n0, int n1, int n2, double ox, double oy,          \
                                        double oz, double dx, double cx, double cy, double cz,      \
                                        double r) {                                                 \
        View<T> v{g, n0, n1, n2, (T)ox, (T)oy, (T)oz, (T)dx};                                       \
        for (int k = 0; k < n2; ++k)                                                                \
            for (int j = 0; j < n1; ++j)                                                            \
                for (int i = 0; i < n0; ++i) {                                                      \
                    T& e = g[i + (idx_t)n0 * (j + (idx_t)n1 * k)];                                  \
                    e = std::min(e, sphere_sdf(grid_pos(v, i, j, k), (T)cx, (T)cy, (T)cz, (T)r));   \
                }                                                                                   \
    }                                                                                               \
    OR_EXPORT void or_emit_pool_##SUF(T* g, int n0, int n1, int n2, double ox, double oy, double oz, \
                                      double dx, double height) {                                   \
        View<T> v{g, n0, n1, n2, (T)ox, (T)oy, (T)oz, (T)dx};                                       \
        for (int k = 0; k < n2; ++k)                                                                \
            for (int j = 0; j < n1; ++j)                                                            \
                for (int i = 0; i < n0; ++i) {                                                      \
                    T& e = g[i + (idx_t)n0 * (j + (idx_t)n1 * k)];                                  \
                    e = std::min(e, grid_pos(v, i, j, k).y - (T)height);                            \
                }                                                                                   \
    }                                                                                               \
    OR_EXPORT void or_emit_box_##SUF(T* g, int n0, int n1, int n2, double ox, double oy, double oz,  \
                                     double dx, const double* lo, const double* hi) {               \
        View<T> v{g, n0, n1, n2, (T)ox, (T)oy, (T)oz, (T)dx};                                       \
        const T tlo[3] = {(T)lo[0], (T)lo[1], (T)lo[2]}, thi[3] = {(T)hi[0], (T)hi[1], (T)hi[2]};   \
        for (int k = 0; k < n2; ++k)                                                                \
            for (int j = 0; j < n1; ++j)                                                            \
                for (int i = 0; i < n0; ++i) {                                                      \
                    T& e = g[i + (idx_t)n0 * (j + (idx_t)n1 * k)];                                  \
                    e = std::min(e, box_sdf(grid_pos(v, i, j, k), tlo, thi));                       \
                }                                                                                   \
    }                                                                                               \
    /* room (levelset_emitter.cpp:18-32): -1 on the outer layer, -0.01 on the next, +1 inside */  \
    OR_EXPORT void or_emit_room_##SUF(T* g, int n0, int n1, int n2) {                               \
        for (int k = 0; k < n2; ++k)                                                                \
            for (int j = 0; j < n1; ++j)                                                            \
                for (int i = 0; i < n0; ++i) {                                                      \
                    T val;                                                                          \
                    if (i == 0 || i == n0 - 1 || j == 0 || j == n1 - 1 || k == 0 || k == n2 - 1)   \
                        val = (T)-1.0;                                                              \
                    else if (i == 1 || i == n0 - 2 || j == 1 || j == n1 - 2 || k == 1 || k == n2 - 2) \
                        val = (T)-0.01;                                                             \
                    else                                                                            \
                        val = (T)1.0;                                                               \
                    T& e = g[i + (idx_t)n0 * (j + (idx_t)n1 * k)];                                  \
                    e = std::min(e, val);                                                           \
                }                                                                                   \
    }

DEFINE_ADVECT(f32, float)
DEFINE_ADVECT(f64, double)

OR_EXPORT int or_pcg(int n0, int n1, int n2, const double* diag, const double* offx,
                     const double* offy, const double* offz, const double* rhs, double* x,
                     int precond, double tol, int maxit, int* iters, double* relres) {
    GridMatrix A{n0, n1, n2, diag, offx, offy, offz};
    return pcg(A, rhs, x, precond, tol, maxit, iters, relres);
}

OR_EXPORT void or_spmv(int n0, int n1, int n2, const double* diag, const double* offx,
                       const double* offy, const double* offz, const double* p, double* out) {
    GridMatrix A{n0, n1, n2, diag, offx, offy, offz};
    spmv(A, p, out);
}

}  // extern "C"
