// el_advect.cu -- semi-Lagrangian advection of the level set and the MAC velocity.
//
// Reference: src/project/3d/fluid/advection.cpp:9-27 (loop drivers), include/nama/math/ode.h
// (StaggeredGridField, trace_rk2), include/nama/math/interpolation.h (lerp, weno6_interp).
// Per output sample: sample position -> backtrace through the old velocity (trilinear MAC
// interpolation at every RK stage) -> trilinear or WENO6 sample of the old field at the foot
// point.  Two forms: advect_kernel, one thread per sample reading global memory (the stateless
// operators; any dt), and the tiled kernels below, which stage what a tile of samples reads
// (the velocity boxes; for WENO6 the level-set box and its x-pass smoothness terms) in shared
// memory once -- under the CFL limit the foot point moves at most about one cell -- and fall
// back to the global reads for a sample whose stencil leaves the box.  The boxes arrive by TMA
// box copies (cp.async.bulk.tensor) wherever the array's row pitch is a multiple of 16 bytes;
// the parts of a box outside the grid are then filled in from the clamped entries in shared
// memory, so that a box holds the clamped grid either way.
#include <cstring>
#include <limits>

#include "el_internal.cuh"
#include "el_tma.cuh"

namespace el {

template <typename T>
struct Mac {
    GridView<T> u, v, w;
};

struct DtArg {
    const Scalars* s;  // device scalars holding dt, or null
    double v;          // dt by value when s is null
};

__device__ __forceinline__ double dt_value(const DtArg& a) { return a.s ? a.s->dt : a.v; }

// Set when a tile's wait for its box copies gave up (the tile's outputs are then NaN, so that
// the step's solve fails on them); read and cleared by advect_fault_take().
__device__ unsigned advect_wait_fault;

// a box copy of one array (on = 0: the array is staged by plain loads)
struct BoxMap {
    CUtensorMap m;
    int on;
};
struct MacMaps {
    BoxMap c[3];
};

// floor(t) and t - floor(t), the same values as index_fraction.  FP32: t + 1.5 * 2^23 rounded
// toward -inf holds floor(t) in its low mantissa bits (exact for |t| < 2^22); outside that range
// (and for NaN) the index lands millions of cells away, i.e. outside every staged box, and the
// sample takes the exact global path.
template <typename T>
__device__ __forceinline__ void floor_index(T t, int& idx, T& frac) {
    if constexpr (sizeof(T) == 4) {
        const float big = 12582912.0f;  // 1.5 * 2^23, bit pattern 0x4B400000
        const float r = __fadd_rd(t, big);
        idx = (int)((unsigned)__float_as_int(r) - 0x4B400000u);
        frac = t - (r - big);
    } else {
        const T fl = floor(t);
        idx = (int)fl;
        frac = t - fl;
    }
}

// one axis of a trilinear read: index_fraction's floor index and fraction (floor_index: the
// same values)
template <typename T>
__device__ __forceinline__ void axis_index(T pos, T origin, T dx, T inv_dx, int& idx, T& frac) {
    T t;
    if constexpr (sizeof(T) == 8)
        t = (pos - origin - T(0.5) * dx) / dx;
    else
        t = (pos - origin - T(0.5) * dx) * inv_dx;
    floor_index(t, idx, frac);
}

// axis_index of one coordinate against two origins; FP32 in packed float2 arithmetic, the same
// operations as axis_index and floor_index lane by lane
template <typename T>
__device__ __forceinline__ void axis_index_pair(T pos, T o1, T o2, T dx, T inv_dx, int& i1, T& f1, int& i2, T& f2) {
    if constexpr (sizeof(T) == 4) {
        const float h = 0.5f * dx;
        const float2 t = __fmul2_rn(__fadd2_rn(__fadd2_rn(make_float2(pos, pos), make_float2(-o1, -o2)),
                                               make_float2(-h, -h)),
                                    make_float2(inv_dx, inv_dx));
        const float big = 12582912.0f;  // 1.5 * 2^23, as floor_index
        const float2 r = __fadd2_rd(t, make_float2(big, big));
        const float2 fl = __fadd2_rn(r, make_float2(-big, -big));
        const float2 f = __fadd2_rn(t, make_float2(-fl.x, -fl.y));
        i1 = (int)((unsigned)__float_as_int(r.x) - 0x4B400000u);
        i2 = (int)((unsigned)__float_as_int(r.y) - 0x4B400000u);
        f1 = f.x;
        f2 = f.y;
    } else {
        axis_index(pos, o1, dx, inv_dx, i1, f1);
        axis_index(pos, o2, dx, inv_dx, i2, f2);
    }
}

// the 8 points of a trilinear read at floor indices (i, j, k) are inside the grid (then clamping
// changes none of them)
template <typename T>
__device__ __forceinline__ bool tri_inside(const GridView<T>& g, int i, int j, int k) {
    return (unsigned)i < (unsigned)(g.n0 - 1) && (unsigned)j < (unsigned)(g.n1 - 1) && (unsigned)k < (unsigned)(g.n2 - 1);
}

// the 8 values of an inside read: one base address and fixed strides
template <typename T>
struct Tri8 {
    T c[8];
};
template <typename T>
__device__ __forceinline__ Tri8<T> tri_load(const GridView<T>& g, int i, int j, int k) {
    const long long sy = g.n0, sz = (long long)g.n0 * g.n1;
    const T* p = g.d + (i + sy * j + sz * k);
    return Tri8<T>{{__ldg(p), __ldg(p + 1), __ldg(p + sy), __ldg(p + sy + 1), __ldg(p + sz), __ldg(p + sz + 1),
                    __ldg(p + sz + sy), __ldg(p + sz + sy + 1)}};
}
// the trilinear combination of 8 loaded points: x, then y, then z lerps; FP32 with the z = 0 and
// z = 1 halves side by side in packed float2 arithmetic (each lane rounded as its scalar lerp)
template <typename T>
__device__ __forceinline__ T tri_mix(const Tri8<T>& v, T fx, T fy, T fz) {
    if constexpr (sizeof(T) == 4) {
        auto lerp2 = [](float2 a, float2 b, float f) {
            const float g = 1.f - f;
            return __ffma2_rn(make_float2(f, f), b, __fmul2_rn(make_float2(g, g), a));
        };
        const float2 x0 = lerp2(make_float2(v.c[0], v.c[4]), make_float2(v.c[1], v.c[5]), fx);
        const float2 x1 = lerp2(make_float2(v.c[2], v.c[6]), make_float2(v.c[3], v.c[7]), fx);
        const float2 y = lerp2(x0, x1, fy);
        return lerp1(y.x, y.y, fz);
    } else {
        TriIdx<T> t;
        t.fx = fx;
        t.fy = fy;
        t.fz = fz;
        return tri_combine(t, v.c[0], v.c[1], v.c[2], v.c[3], v.c[4], v.c[5], v.c[6], v.c[7]);
    }
}

// u, v, w at one position from global memory: the three components share six axis coordinates
// (u at a face in x, cells in y and z; v and w likewise).  When all three reads are inside the
// grid (the common case) their 24 loads go out together from fixed offsets; otherwise each
// takes the clamped gather -- the values of three sample_trilinear calls either way
template <typename T>
__device__ __forceinline__ void velocity_at(const Mac<T>& m, T x, T y, T z, T dx, T inv, T& vx, T& vy,
                                            T& vz) {
    int ixf, ixc, jyf, jyc, kzf, kzc;
    T fxf, fxc, fyf, fyc, fzf, fzc;
    axis_index_pair(x, m.u.ox, m.v.ox, dx, inv, ixf, fxf, ixc, fxc);
    axis_index_pair(y, m.v.oy, m.u.oy, dx, inv, jyf, fyf, jyc, fyc);
    axis_index_pair(z, m.w.oz, m.u.oz, dx, inv, kzf, fzf, kzc, fzc);
    if (tri_inside(m.u, ixf, jyc, kzc) && tri_inside(m.v, ixc, jyf, kzc) && tri_inside(m.w, ixc, jyc, kzf)) {
        const Tri8<T> a = tri_load(m.u, ixf, jyc, kzc), b = tri_load(m.v, ixc, jyf, kzc),
                      c = tri_load(m.w, ixc, jyc, kzf);
        vx = tri_mix(a, fxf, fyc, fzc);
        vy = tri_mix(b, fxc, fyf, fzc);
        vz = tri_mix(c, fxc, fyc, fzf);
    } else {
        vx = sample_trilinear(m.u, x, y, z, dx, inv);
        vy = sample_trilinear(m.v, x, y, z, dx, inv);
        vz = sample_trilinear(m.w, x, y, z, dx, inv);
    }
}

// trace_rk2 (ode.h:30-35) or Ralston RK3 (c = 0, 1/2, 3/4; b = 2/9, 1/3, 4/9); h is the
// signed step (-dt for a backtrace).
template <typename T, int TRACE>
__device__ __forceinline__ void backtrace_from(const Mac<T>& m, T ax, T ay, T az, T& x, T& y, T& z, T h, T dx, T inv) {
    const T h2 = T(0.5) * h;
    T bx, by, bz;
    velocity_at(m, x + h2 * ax, y + h2 * ay, z + h2 * az, dx, inv, bx, by, bz);
    if constexpr (TRACE == EL_TRACE_RK2) {
        x = x + h * bx;
        y = y + h * by;
        z = z + h * bz;
    } else {
        const T h3 = T(0.75) * h;
        T cx, cy, cz;
        velocity_at(m, x + h3 * bx, y + h3 * by, z + h3 * bz, dx, inv, cx, cy, cz);
        const T w1 = h * (T(2) / T(9)), w2 = h * (T(1) / T(3)), w3 = h * (T(4) / T(9));
        x = x + w1 * ax + w2 * bx + w3 * cx;
        y = y + w1 * ay + w2 * by + w3 * cy;
        z = z + w1 * az + w2 * bz + w3 * cz;
    }
}

template <typename T, int TRACE>
__device__ __forceinline__ void backtrace(const Mac<T>& m, T& x, T& y, T& z, T h, T dx, T inv) {
    T ax, ay, az;
    velocity_at(m, x, y, z, dx, inv, ax, ay, az);
    backtrace_from<T, TRACE>(m, ax, ay, az, x, y, z, h, dx, inv);
}

// The velocity at the centre of cell (i, j, k), the first stage of a level-set backtrace: the
// trilinear read there has fractions 1/2 along a component's own axis and 0 along the others,
// so each component is the mean of its two faces (a zero fraction leaves its first value).
// Exact fractions where index_fraction of the rounded cell position may carry a rounding error
// of an ulp or so.  The faces of a cell are inside every grid (no clamping).
template <typename T>
__device__ __forceinline__ void cell_velocity(const Mac<T>& m, int i, int j, int k, T& vx, T& vy, T& vz) {
    const long long cu = lin3(i, j, k, m.u.n0, m.u.n1), cv = lin3(i, j, k, m.v.n0, m.v.n1);
    const long long cw = lin3(i, j, k, m.w.n0, m.w.n1);
    vx = lerp1(__ldg(m.u.d + cu), __ldg(m.u.d + cu + 1), T(0.5));
    vy = lerp1(__ldg(m.v.d + cv), __ldg(m.v.d + cv + m.v.n0), T(0.5));
    vz = lerp1(__ldg(m.w.d + cw), __ldg(m.w.d + cw + (long long)m.w.n0 * m.w.n1), T(0.5));
}

// out(x) = src(trace(x, -dt)) for every sample of src's grid (cell centres or one face
// component); positions are GridBase::pos = (idx + 0.5) * dx + origin (grid.h:355-367).
template <typename T, int TRACE, int SAMPLE>
__global__ void __launch_bounds__(256) advect_kernel(GridView<T> src, T* __restrict__ out, Mac<T> mac,
                                                     DtArg dt, T dx, T inv_dx) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= src.n0 || j >= src.n1) return;
    const T h = -(T)dt_value(dt);
    T x = (i + T(0.5)) * dx + src.ox;
    T y = (j + T(0.5)) * dx + src.oy;
    T z = (k + T(0.5)) * dx + src.oz;
    backtrace<T, TRACE>(mac, x, y, z, h, dx, inv_dx);
    T r;
    if constexpr (SAMPLE == EL_SAMPLE_WENO6)
        r = sample_weno6(src, x, y, z, dx, inv_dx);
    else
        r = sample_trilinear(src, x, y, z, dx, inv_dx);
    const long long oc = lin3(i, j, k, src.n0, src.n1);
    if (EL_IN(oc, (long long)src.n0 * src.n1 * src.n2, 1)) out[oc] = r;
}

// ---------------------------------------------------------------------------------------
// Tiled variants.  Under the CFL limit (cfl <= 1) the foot point and every RK stage lie within
// one cell of the sample, so every trilinear velocity sample of a 32 x 8 x 8 tile of outputs
// reads indices within [tile - 2, tile + 1] of each MAC grid: a CTA stages those boxes of u, v
// and w (40 x 12 x 12 values each) in shared memory once and samples them there.  A sample
// whose 8 points are not all in the box (a larger dt) reads global memory instead, with the
// same arithmetic, so the results do not depend on which path a sample took.  The velocity
// advection computes u, v and w of a tile in one CTA (when the advected field is the advecting
// velocity, as in advect_velocity), sharing the staged boxes; the level set samples phi from
// global memory at the foot point.
//
// The box holds the clamped grid (entry p = value at clamp(box origin + p)), so a sample reads
// its 8 points at the unclamped indices i, i+1 (j, k likewise) with no clamping and gets exactly
// the values of the clamped gather lerp() makes; the 8 reads sit at fixed offsets from one
// address.  The floor of the cell coordinate is taken without conversions (floor_index), and
// the three components at one position share their cell-centred and face coordinates.  Along
// x a box starts four entries left of the tile (a box copy starts on a 16-byte boundary) and
// holds 40 entries; along y and z the halo is two.
constexpr int kTileX = 32, kTileY = 8, kTileZ = 8, kHalo = 2, kHaloX = 4;
constexpr int kBoxX = kTileX + 2 * kHaloX, kBoxY = kTileY + 2 * kHalo, kBoxZ = kTileZ + 2 * kHalo;
constexpr int kBoxN = kBoxX * kBoxY * kBoxZ;

// the cell coordinate of index_fraction: (pos - origin - dx / 2) / dx
template <typename T>
__device__ __forceinline__ T cell_coord(T pos, T origin, T dx, T inv_dx) {
    if constexpr (sizeof(T) == 8)
        return (pos - origin - T(0.5) * dx) / dx;
    else
        return (pos - origin - T(0.5) * dx) * inv_dx;
}

// one axis of a position: box-relative floor index and fraction
template <typename T>
struct AxisPos {
    int a;
    T f;
};

template <typename T>
__device__ __forceinline__ AxisPos<T> axis_pos(T pos, T origin, int box0, T dx, T inv_dx) {
    AxisPos<T> p;
    int idx;
    floor_index(cell_coord(pos, origin, dx, inv_dx), idx, p.f);
    p.a = (int)((unsigned)idx - (unsigned)box0);
    return p;
}

template <typename T>
__device__ __forceinline__ T lerp_combine(T fx, T fy, T fz, T c000, T c100, T c010, T c110, T c001, T c101, T c011,
                                          T c111) {
    if constexpr (sizeof(T) == 4) {
        // FP32: the z = 0 and z = 1 halves side by side in packed float2 arithmetic (the same
        // lerps, x then y, each lane rounded as its scalar operations), then the z lerp
        auto lerp2 = [](float2 a, float2 b, float f) {
            const float g = 1.f - f;
            return __ffma2_rn(make_float2(f, f), b, __fmul2_rn(make_float2(g, g), a));
        };
        const float2 x0 = lerp2(make_float2(c000, c001), make_float2(c100, c101), fx);
        const float2 x1 = lerp2(make_float2(c010, c011), make_float2(c110, c111), fx);
        const float2 y = lerp2(x0, x1, fy);
        return lerp1(y.x, y.y, fz);
    } else {
        const T lo = lerp1(lerp1(c000, c100, fx), lerp1(c010, c110, fx), fy);
        const T hi = lerp1(lerp1(c001, c101, fx), lerp1(c011, c111, fx), fy);
        return lerp1(lo, hi, fz);
    }
}

// axis_pos of one coordinate against two origins (FP32: in packed float2 arithmetic, the same
// operations as cell_coord and floor_index lane by lane)
template <typename T>
__device__ __forceinline__ void axis_pos_pair(T pos, T o1, T o2, int box0, T dx, T inv_dx, AxisPos<T>& p1,
                                              AxisPos<T>& p2) {
    int i1, i2;
    axis_index_pair(pos, o1, o2, dx, inv_dx, i1, p1.f, i2, p2.f);
    p1.a = (int)((unsigned)i1 - (unsigned)box0);
    p2.a = (int)((unsigned)i2 - (unsigned)box0);
}

// trilinear sample from a staged box at box-relative (x, y, z); false when the 8 points are not
// all inside the box.  CHECK = false: the caller knows they are (see advect_velocity_tiled_kernel)
template <typename T, bool CHECK = true>
__device__ __forceinline__ bool staged_lerp(const T* box, const AxisPos<T>& x, const AxisPos<T>& y,
                                            const AxisPos<T>& z, T& out) {
    if (CHECK && ((unsigned)x.a >= (unsigned)(kBoxX - 1) || (unsigned)y.a >= (unsigned)(kBoxY - 1) ||
                  (unsigned)z.a >= (unsigned)(kBoxZ - 1)))
        return false;
    const T* p = box + (z.a * kBoxY + y.a) * kBoxX + x.a;
    constexpr int SY = kBoxX, SZ = kBoxX * kBoxY;
    out = lerp_combine(x.f, y.f, z.f, p[0], p[1], p[SY], p[SY + 1], p[SZ], p[SZ + 1], p[SZ + SY], p[SZ + SY + 1]);
    return true;
}

template <typename T>
struct Staged {
    const T* box;         // shared memory, [z][y][x] over the box
    int bx0, by0, bz0;    // grid index of the box's first entry
};

template <typename T, bool CHECK = true>
__device__ __forceinline__ T sample_staged(const GridView<T>& g, const Staged<T>& b, T x, T y, T z, T dx, T inv) {
    T r;
    if (staged_lerp<T, CHECK>(b.box, axis_pos(x, g.ox, b.bx0, dx, inv), axis_pos(y, g.oy, b.by0, dx, inv),
                              axis_pos(z, g.oz, b.bz0, dx, inv), r) ||
        !CHECK)
        return r;
    return sample_trilinear(g, x, y, z, dx, inv);
}

template <typename T>
struct StagedMac {
    Staged<T> u, v, w;
};

// u at (face x, cell y, cell z), v at (cell, face, cell), w at (cell, cell, face): six axis
// positions serve all three (the cell origins are those of the other components' grids)
template <typename T, bool CHECK = true>
__device__ __forceinline__ void velocity_at_staged(const Mac<T>& m, const StagedMac<T>& s, T x, T y, T z, T dx, T inv,
                                                   T& vx, T& vy, T& vz) {
    AxisPos<T> xf, xc, yf, yc, zf, zc;
    axis_pos_pair(x, m.u.ox, m.v.ox, s.u.bx0, dx, inv, xf, xc);
    axis_pos_pair(y, m.v.oy, m.u.oy, s.u.by0, dx, inv, yf, yc);
    axis_pos_pair(z, m.w.oz, m.u.oz, s.u.bz0, dx, inv, zf, zc);
    if (!staged_lerp<T, CHECK>(s.u.box, xf, yc, zc, vx) && CHECK) vx = sample_trilinear(m.u, x, y, z, dx, inv);
    if (!staged_lerp<T, CHECK>(s.v.box, xc, yf, zc, vy) && CHECK) vy = sample_trilinear(m.v, x, y, z, dx, inv);
    if (!staged_lerp<T, CHECK>(s.w.box, xc, yc, zf, vz) && CHECK) vz = sample_trilinear(m.w, x, y, z, dx, inv);
}

// backtrace with the staged velocity: the same stages and arithmetic as backtrace(), from the
// first stage's velocity (ax, ay, az) at (x, y, z)
template <typename T, int TRACE, bool CHECK = true>
__device__ __forceinline__ void backtrace_staged_from(const Mac<T>& m, const StagedMac<T>& sm, T ax, T ay, T az, T& x,
                                                      T& y, T& z, T h, T dx, T inv) {
    const T h2 = T(0.5) * h;
    T bx, by, bz;
    velocity_at_staged<T, CHECK>(m, sm, x + h2 * ax, y + h2 * ay, z + h2 * az, dx, inv, bx, by, bz);
    if constexpr (TRACE == EL_TRACE_RK2) {
        x = x + h * bx;
        y = y + h * by;
        z = z + h * bz;
    } else {
        const T h3 = T(0.75) * h;
        T cx, cy, cz;
        velocity_at_staged<T, CHECK>(m, sm, x + h3 * bx, y + h3 * by, z + h3 * bz, dx, inv, cx, cy, cz);
        const T w1 = h * (T(2) / T(9)), w2 = h * (T(1) / T(3)), w3 = h * (T(4) / T(9));
        x = x + w1 * ax + w2 * bx + w3 * cx;
        y = y + w1 * ay + w2 * by + w3 * cy;
        z = z + w1 * az + w2 * bz + w3 * cz;
    }
}

template <typename T, int TRACE, bool CHECK = true>
__device__ __forceinline__ void backtrace_staged(const Mac<T>& m, const StagedMac<T>& sm, T& x, T& y, T& z, T h, T dx,
                                                 T inv) {
    T ax, ay, az;
    velocity_at_staged<T, CHECK>(m, sm, x, y, z, dx, inv, ax, ay, az);
    backtrace_staged_from<T, TRACE, CHECK>(m, sm, ax, ay, az, x, y, z, h, dx, inv);
}

// The velocity at the centre of a face of component c, the first stage of its backtrace: the
// trilinear read there has fractions 0 and 1/2 only, so it is the face's own value and the
// four-point means of the two other components, in the trilinear read's order (x, then y, then
// z; a zero fraction leaves its first value).  Exact fractions where index_fraction of the
// rounded face position may carry a rounding error of an ulp or so.  Every point lies in the
// staged boxes (their halos are at least one entry), which hold the clamped grid.
template <typename T>
__device__ __forceinline__ T box_at(const Staged<T>& b, int I, int J, int K) {
    return b.box[(K * kBoxY + J) * kBoxX + I];
}

template <typename T>
__device__ __forceinline__ T mid4(T a, T b, T c, T d) {
    return lerp1(lerp1(a, b, T(0.5)), lerp1(c, d, T(0.5)), T(0.5));
}

template <typename T>
__device__ __forceinline__ void face_velocity(const StagedMac<T>& s, int c, int i, int j, int k, T& vx, T& vy, T& vz) {
    const int I = i - s.u.bx0, J = j - s.u.by0, K = k - s.u.bz0;
    if (c == 0) {
        vx = box_at(s.u, I, J, K);
        vy = mid4(box_at(s.v, I - 1, J, K), box_at(s.v, I, J, K), box_at(s.v, I - 1, J + 1, K), box_at(s.v, I, J + 1, K));
        vz = mid4(box_at(s.w, I - 1, J, K), box_at(s.w, I, J, K), box_at(s.w, I - 1, J, K + 1), box_at(s.w, I, J, K + 1));
    } else if (c == 1) {
        vx = mid4(box_at(s.u, I, J - 1, K), box_at(s.u, I + 1, J - 1, K), box_at(s.u, I, J, K), box_at(s.u, I + 1, J, K));
        vy = box_at(s.v, I, J, K);
        vz = mid4(box_at(s.w, I, J - 1, K), box_at(s.w, I, J, K), box_at(s.w, I, J - 1, K + 1), box_at(s.w, I, J, K + 1));
    } else {
        vx = mid4(box_at(s.u, I, J, K - 1), box_at(s.u, I + 1, J, K - 1), box_at(s.u, I, J, K), box_at(s.u, I + 1, J, K));
        vy = mid4(box_at(s.v, I, J, K - 1), box_at(s.v, I, J + 1, K - 1), box_at(s.v, I, J, K), box_at(s.v, I, J + 1, K));
        vz = box_at(s.w, I, J, K);
    }
}

// max(|a|, |b|) that is NaN when either is (fmax would drop a NaN)
template <typename T>
__device__ __forceinline__ T fmax_nan(T m, T v) {
    const T a = v < T(0) ? -v : v;
    return (a > m || a != a) ? a : m;
}

// A box that arrived by a box copy, made the clamped box: an entry outside the grid takes the
// value of its clamped entry (inside the grid, so the copy filled it), one warp per row; with
// MAX, vmax gathers the largest |value| of the entries inside the grid (the values the clamped
// box holds).  A box that lies inside the grid is only scanned for vmax, in 16-byte reads.
template <typename T, int BX, int BY, int BZ, bool MAX>
__device__ __forceinline__ void finish_box(T* box, const GridView<T>& g, int bx0, int by0, int bz0, T& vmax) {
    const int tid = threadIdx.x + blockDim.x * threadIdx.y, nthr = blockDim.x * blockDim.y;
    const bool edge = bx0 < 0 || by0 < 0 || bz0 < 0 || bx0 + BX > g.n0 || by0 + BY > g.n1 || bz0 + BZ > g.n2;
    if (!edge) {
        if constexpr (MAX) {
            static_assert((BX * BY * BZ * sizeof(T)) % 16 == 0, "whole 16-byte reads");
            constexpr int nv = BX * BY * BZ * (int)sizeof(T) / 16;
            for (int e = tid; e < nv; e += nthr) {
                if constexpr (sizeof(T) == 4) {
                    const float4 q = reinterpret_cast<const float4*>(box)[e];
                    vmax = fmax_nan(fmax_nan(fmax_nan(fmax_nan(vmax, q.x), q.y), q.z), q.w);
                } else {
                    const double2 q = reinterpret_cast<const double2*>(box)[e];
                    vmax = fmax_nan(fmax_nan(vmax, q.x), q.y);
                }
            }
        }
        return;
    }
    const int lane = tid & 31, warp = tid >> 5, nwarps = nthr >> 5;
    for (int row = warp; row < BY * BZ; row += nwarps) {
        const int bz = row / BY, by = row - bz * BY;
        const int cy = clampi(by0 + by, 0, g.n1 - 1) - by0, cz = clampi(bz0 + bz, 0, g.n2 - 1) - bz0;
        const bool row_in = cy == by && cz == bz;
        const T* src = box + (cz * BY + cy) * BX;
        T* dst = box + row * BX;
        for (int x = lane; x < BX; x += 32) {
            const int cx = clampi(bx0 + x, 0, g.n0 - 1) - bx0;
            if (row_in && cx == x) {
                if (MAX) vmax = fmax_nan(vmax, dst[x]);
            } else {
                dst[x] = src[cx];
            }
        }
    }
}

// Issues the box copies of a tile (one thread; the mbarrier is the CTA's own), `bytes` in all.
__device__ __forceinline__ void copy_boxes_begin(uint64_t* bar, unsigned bytes) {
    mbar_init(bar, 1);
    mbar_init_fence();
    mbar_expect_tx(bar, bytes);
}

// Every thread waits (bounded) for the CTA's box copies; true, the same in every thread, when a
// wait gave up.  Then the fault is recorded and one thread waits once more (bounded) so that no
// copy is still landing when the CTA ends.  Call after a barrier that follows the mbarrier's
// initialisation.
__device__ __forceinline__ bool copy_boxes_failed(uint64_t* bar) {
    const bool ok = mbar_wait(bar, 0);
    if (!__syncthreads_or(!ok)) return false;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        atomicOr(&advect_wait_fault, 1u);
        mbar_wait(bar, 0);
    }
    __syncthreads();
    return true;
}

// NaN into a thread's outputs of a tile whose boxes did not arrive (rows j, planes z0 .. z0+nz-1)
template <typename T>
__device__ __forceinline__ void nan_column(const GridView<T>& g, T* __restrict__ o, int i, int j, int z0, int nz) {
    if (i >= g.n0 || j >= g.n1) return;
    for (int kk = 0; kk < nz && z0 + kk < g.n2; ++kk) {
        const long long oc = lin3(i, j, z0 + kk, g.n0, g.n1);
        if (EL_IN(oc, (long long)g.n0 * g.n1 * g.n2, 4)) o[oc] = std::numeric_limits<T>::quiet_NaN();
    }
}

// Stages the clamped boxes of u, v, w around tile (x0, y0, z0): a component with a box map by a
// box copy (then finish_box), the others by plain loads, rows of kBoxX along x, one warp per row.
// vmax gathers the largest |value| this thread staged or scanned (NaN if it met one).  `failed`:
// the box copies did not arrive (the same in every thread).
template <typename T>
__device__ __forceinline__ StagedMac<T> stage_mac(const Mac<T>& m, const MacMaps& maps, T* smem, uint64_t* bar,
                                                  int x0, int y0, int z0, T& vmax, bool& failed) {
    const int bx0 = x0 - kHaloX, by0 = y0 - kHalo, bz0 = z0 - kHalo;
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    const int lane = tid & 31, warp = tid >> 5, nwarps = (blockDim.x * blockDim.y) >> 5;
    // the flags in registers (a parameter indexed at run time would be copied to local memory)
    const bool on0 = maps.c[0].on != 0, on1 = maps.c[1].on != 0, on2 = maps.c[2].on != 0;
    const int ncopy = (int)on0 + (int)on1 + (int)on2;
    if (ncopy && tid == 0) {
        copy_boxes_begin(bar, (unsigned)(ncopy * kBoxN * sizeof(T)));
        if (on0) tma_load_3d(smem, &maps.c[0].m, bar, bx0, by0, bz0);
        if (on1) tma_load_3d(smem + kBoxN, &maps.c[1].m, bar, bx0, by0, bz0);
        if (on2) tma_load_3d(smem + 2 * kBoxN, &maps.c[2].m, bar, bx0, by0, bz0);
    }
    for (int row = warp; row < 3 * kBoxY * kBoxZ; row += nwarps) {
        const int comp = row / (kBoxY * kBoxZ), r = row - comp * (kBoxY * kBoxZ);
        if (comp == 0 ? on0 : (comp == 1 ? on1 : on2)) continue;
        const int bz = r / kBoxY, by = r - bz * kBoxY;
        const GridView<T>& g = comp == 0 ? m.u : (comp == 1 ? m.v : m.w);
        T* dst = smem + comp * kBoxN + (bz * kBoxY + by) * kBoxX;
        const int gy = clampi(by0 + by, 0, g.n1 - 1), gz = clampi(bz0 + bz, 0, g.n2 - 1);
        const T* src = g.d + (long long)g.n0 * (gy + (long long)g.n1 * gz);
        const T va = __ldg(src + clampi(bx0 + lane, 0, g.n0 - 1));
        dst[lane] = va;
        vmax = fmax_nan(vmax, va);
        if (lane < kBoxX - 32) {
            const T vb = __ldg(src + clampi(bx0 + 32 + lane, 0, g.n0 - 1));
            dst[32 + lane] = vb;
            vmax = fmax_nan(vmax, vb);
        }
    }
    failed = false;
    if (ncopy) {
        __syncthreads();  // the mbarrier's initialisation is seen by every thread
        failed = copy_boxes_failed(bar);
        if (!failed) {
            if (on0) finish_box<T, kBoxX, kBoxY, kBoxZ, true>(smem, m.u, bx0, by0, bz0, vmax);
            if (on1) finish_box<T, kBoxX, kBoxY, kBoxZ, true>(smem + kBoxN, m.v, bx0, by0, bz0, vmax);
            if (on2) finish_box<T, kBoxX, kBoxY, kBoxZ, true>(smem + 2 * kBoxN, m.w, bx0, by0, bz0, vmax);
        }
    }
    return StagedMac<T>{{smem, bx0, by0, bz0}, {smem + kBoxN, bx0, by0, bz0}, {smem + 2 * kBoxN, bx0, by0, bz0}};
}

// The largest |velocity| the CTA staged (NaN if it staged a NaN), as the same value in every
// thread.  Call after the staging, in place of the __syncthreads that ends it.
template <typename T>
__device__ __forceinline__ T box_max(T vmax) {
    __shared__ T wmax[kTileX * kTileY / 32];
    for (int o = 16; o > 0; o >>= 1) vmax = fmax_nan(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    const int tid = threadIdx.x + blockDim.x * threadIdx.y;
    if ((tid & 31) == 0) wmax[tid >> 5] = vmax;
    __syncthreads();
    T m = T(0);
#pragma unroll
    for (int q = 0; q < kTileX * kTileY / 32; ++q) m = fmax_nan(m, wmax[q]);
    return m;
}

// A step moves no sample more than one cell when |v| |dt| / dx < 1 over the staged boxes (every
// RK stage and the foot point are convex combinations of velocities read inside the boxes, by
// induction): then all of a tile's staged reads fall inside its boxes (the halo is two cells)
// and the reads need no check.  False for a NaN or infinite velocity or dt.
template <typename T>
__device__ __forceinline__ bool within_one_cell(T vmax, T h, T inv_dx) {
    const T reach = vmax * (h < T(0) ? -h : h) * inv_dx;
    return reach <= T(0.999);
}

// the u, v, w samples of a tile (CHECK: each staged read is checked and falls back to the
// global read outside the box)
template <typename T, int TRACE, bool CHECK>
__device__ __forceinline__ void velocity_tile(const Mac<T>& mac, const StagedMac<T>& sm, T* __restrict__ ou,
                                              T* __restrict__ ov, T* __restrict__ ow, T h, T dx, T inv_dx, int x0,
                                              int y0, int z0) {
    const int i = x0 + threadIdx.x, j = y0 + threadIdx.y;
#pragma unroll 1
    for (int kk = 0; kk < kTileZ; ++kk) {
        const int k = z0 + kk;
#pragma unroll 1
        for (int c = 0; c < 3; ++c) {
            // the component's grid, box and output, picked by value (no local arrays)
            GridView<T> g = mac.u;
            Staged<T> b = sm.u;
            T* o = ou;
            if (c == 1) {
                g = mac.v;
                b = sm.v;
                o = ov;
            } else if (c == 2) {
                g = mac.w;
                b = sm.w;
                o = ow;
            }
            if (i >= g.n0 || j >= g.n1 || k >= g.n2) continue;
            T x = (i + T(0.5)) * dx + g.ox;
            T y = (j + T(0.5)) * dx + g.oy;
            T z = (k + T(0.5)) * dx + g.oz;
            T ax, ay, az;
            face_velocity(sm, c, i, j, k, ax, ay, az);
            backtrace_staged_from<T, TRACE, CHECK>(mac, sm, ax, ay, az, x, y, z, h, dx, inv_dx);
            const long long oc = lin3(i, j, k, g.n0, g.n1);
            const T r = sample_staged<T, CHECK>(g, b, x, y, z, dx, inv_dx);
            if (EL_IN(oc, (long long)g.n0 * g.n1 * g.n2, 2)) o[oc] = r;
        }
    }
}

// u, v, w of a tile, each advected through the (old) velocity itself
template <typename T, int TRACE>
__global__ void __launch_bounds__(kTileX * kTileY, 3) advect_velocity_tiled_kernel(
    Mac<T> mac, T* __restrict__ ou, T* __restrict__ ov, T* __restrict__ ow, DtArg dt, T dx, T inv_dx,
    const __grid_constant__ MacMaps maps) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* smem = reinterpret_cast<T*>(align128(smem_raw));
    __shared__ uint64_t bar;
    const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * kTileY, z0 = blockIdx.z * kTileZ;
    T vmax = T(0);
    bool failed;
    const StagedMac<T> sm = stage_mac(mac, maps, smem, &bar, x0, y0, z0, vmax, failed);
    if (failed) {
        const int i = x0 + threadIdx.x, j = y0 + threadIdx.y;
        nan_column(mac.u, ou, i, j, z0, kTileZ);
        nan_column(mac.v, ov, i, j, z0, kTileZ);
        nan_column(mac.w, ow, i, j, z0, kTileZ);
        return;
    }
    const T bm = box_max(vmax);  // ends the staging (a barrier)
    const T h = -(T)dt_value(dt);
    if (within_one_cell(bm, h, inv_dx))
        velocity_tile<T, TRACE, false>(mac, sm, ou, ov, ow, h, dx, inv_dx, x0, y0, z0);
    else
        velocity_tile<T, TRACE, true>(mac, sm, ou, ov, ow, h, dx, inv_dx, x0, y0, z0);
}

// the level set (cells) through the staged velocity; phi itself from global memory
template <typename T, int TRACE, int SAMPLE>
__global__ void __launch_bounds__(kTileX * kTileY) advect_phi_tiled_kernel(GridView<T> src, T* __restrict__ out,
                                                                           Mac<T> mac, DtArg dt, T dx, T inv_dx,
                                                                           const __grid_constant__ MacMaps maps) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* smem = reinterpret_cast<T*>(align128(smem_raw));
    __shared__ uint64_t bar;
    const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * kTileY, z0 = blockIdx.z * kTileZ;
    T vmax = T(0);
    bool failed;
    const StagedMac<T> sm = stage_mac(mac, maps, smem, &bar, x0, y0, z0, vmax, failed);
    if (failed) {
        nan_column(src, out, x0 + threadIdx.x, y0 + threadIdx.y, z0, kTileZ);
        return;
    }
    const bool inside = within_one_cell(box_max(vmax), -(T)dt_value(dt), inv_dx);  // ends the staging
    const T h = -(T)dt_value(dt);
    const int i = x0 + threadIdx.x, j = y0 + threadIdx.y;
    if (i >= src.n0 || j >= src.n1) return;
#pragma unroll 1
    for (int kk = 0; kk < kTileZ; ++kk) {
        const int k = z0 + kk;
        if (k >= src.n2) break;
        T x = (i + T(0.5)) * dx + src.ox;
        T y = (j + T(0.5)) * dx + src.oy;
        T z = (k + T(0.5)) * dx + src.oz;
        T ax, ay, az;
        cell_velocity(mac, i, j, k, ax, ay, az);
        if (inside)
            backtrace_staged_from<T, TRACE, false>(mac, sm, ax, ay, az, x, y, z, h, dx, inv_dx);
        else
            backtrace_staged_from<T, TRACE, true>(mac, sm, ax, ay, az, x, y, z, h, dx, inv_dx);
        T r;
        if constexpr (SAMPLE == EL_SAMPLE_WENO6)
            r = sample_weno6(src, x, y, z, dx, inv_dx);
        else
            r = sample_trilinear(src, x, y, z, dx, inv_dx);
        const long long oc = lin3(i, j, k, src.n0, src.n1);
        if (EL_IN(oc, (long long)src.n0 * src.n1 * src.n2, 3)) out[oc] = r;
    }
}

// ---------------------------------------------------------------------------------------
// WENO6 level set, tiled.  Under the CFL limit the foot point of a cell lies within one cell
// of it, so the 6^3 stencils of a 32 x 8 x 4 tile of cells read phi within [tile - 3, tile + 4]:
// the CTA stages that clamped box (39 x 15 x 11 nodes) once.  The smoothness indicators of an x-pass
// depend only on the six values it reads, not on the sample's fraction, so they are formed once
// per (row, floor index) of the box -- (eps + IS_s)^2, in FP32 its reciprocal, for the 34 floor
// indices of each of the 165 rows -- and shared by every sample whose stencil uses that row
// segment, instead of being recomputed by all 36 x-passes of every sample.  The y- and z-passes
// combine per-sample values and are evaluated in full.  The backtrace reads the velocity from
// global memory (L1-served).  A foot point outside the box (a larger dt) takes the global
// sample_weno6 path, with the same arithmetic.  The box arrives by one box copy where the cell
// grid's row pitch allows it; along x it then starts four cells left of the tile (a 16-byte
// boundary) and holds 40 entries, of which the first is never read.
constexpr int kWX = 32, kWY = 8, kWZ = 4;
constexpr int kWBX = kWX + 8, kWBY = kWY + 7, kWBZ = kWZ + 7;  // nodes [tile - 4, tile + 4] x [tile - 3, tile + 4]^2
constexpr int kWRows = kWBY * kWBZ;
constexpr int kWBases = kWX + 2;                 // floor indices [tile - 1, tile + 32]
constexpr int kWBoxN = kWBX * kWRows;            // phi box (a multiple of 16 bytes)
constexpr int kWQ = kWRows * kWBases;            // one indicator plane

template <typename T, int TRACE>
__global__ void __launch_bounds__(kWX * kWY, sizeof(T) == 4 ? 2 : 1)
    advect_phi_weno_tiled_kernel(GridView<T> src, T* __restrict__ out, Mac<T> mac, DtArg dt, T dx, T inv_dx,
                                 const __grid_constant__ BoxMap pmap) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* pbox = reinterpret_cast<T*>(align128(smem_raw));  // [z][y][x]
    // [s][row][floor index]; in FP32 s = 0, 1 interleaved ({qa, qb} pairs), then the s = 2 plane
    T* qbox = pbox + kWBoxN;
    const T* pb = pbox + 1;  // the box from node tile - 3 along x
    __shared__ uint64_t bar;
    const int x0 = blockIdx.x * kWX, y0 = blockIdx.y * kWY, z0 = blockIdx.z * kWZ;
    const int bx0 = x0 - 4, by0 = y0 - 3, bz0 = z0 - 3;
    const int tid = threadIdx.x + kWX * threadIdx.y;
    const int lane = tid & 31, warp = tid >> 5;
    if (pmap.on) {
        if (tid == 0) {
            copy_boxes_begin(&bar, (unsigned)(kWBoxN * sizeof(T)));
            tma_load_3d(pbox, &pmap.m, &bar, bx0, by0, bz0);
        }
        __syncthreads();  // the mbarrier's initialisation is seen by every thread
        if (copy_boxes_failed(&bar)) {
            nan_column(src, out, x0 + threadIdx.x, y0 + threadIdx.y, z0, kWZ);
            return;
        }
        T unused = T(0);
        finish_box<T, kWBX, kWBY, kWBZ, false>(pbox, src, bx0, by0, bz0, unused);
    } else {
        for (int row = warp; row < kWRows; row += (kWX * kWY) / 32) {
            const int bz = row / kWBY, by = row - bz * kWBY;
            const int gy = clampi(by0 + by, 0, src.n1 - 1), gz = clampi(bz0 + bz, 0, src.n2 - 1);
            const T* s = src.d + (long long)src.n0 * (gy + (long long)src.n1 * gz);
            T* d = pbox + row * kWBX;
            d[lane] = __ldg(s + clampi(bx0 + lane, 0, src.n0 - 1));
            if (lane < kWBX - 32) d[32 + lane] = __ldg(s + clampi(bx0 + 32 + lane, 0, src.n0 - 1));
        }
    }
    __syncthreads();
    if constexpr (sizeof(T) == 4) {
        // two (row, floor index) entries a thread per pass in packed float2 arithmetic
        constexpr int kStep = kWX * kWY;
        for (int e0 = tid; e0 < kWQ; e0 += 2 * kStep) {
            const int e1 = e0 + kStep < kWQ ? e0 + kStep : e0;  // the tail repeats its first entry
            const int r0 = e0 / kWBases, r1 = e1 / kWBases;
            const float* va = pb + r0 * kWBX + (e0 - r0 * kWBases);
            const float* vb = pb + r1 * kWBX + (e1 - r1 * kWBases);
            float2 v[6];
#pragma unroll
            for (int m = 0; m < 6; ++m) v[m] = make_float2(va[m], vb[m]);
            float2 qa, qb, qc;
            weno6_sq2(v, qa, qb, qc);
            reinterpret_cast<float2*>(qbox)[e0] = make_float2(qa.x, qb.x);  // one 8-byte load for both
            qbox[2 * kWQ + e0] = qc.x;
            if (e1 != e0) {
                reinterpret_cast<float2*>(qbox)[e1] = make_float2(qa.y, qb.y);
                qbox[2 * kWQ + e1] = qc.y;
            }
        }
    } else {
        for (int e = tid; e < kWQ; e += kWX * kWY) {
            const int row = e / kWBases, b = e - row * kWBases;
            const T* v = pb + row * kWBX + b;
            T qa, qb, qc;
            weno6_sq(v[0], v[1], v[2], v[3], v[4], v[5], qa, qb, qc);
            qbox[e] = qa;
            qbox[kWQ + e] = qb;
            qbox[2 * kWQ + e] = qc;
        }
    }
    __syncthreads();
    const int i = x0 + threadIdx.x, j = y0 + threadIdx.y;
    if (i >= src.n0 || j >= src.n1) return;
    const T h = -(T)dt_value(dt);
#pragma unroll 1
    for (int kk = 0; kk < kWZ; ++kk) {
        const int k = z0 + kk;
        if (k >= src.n2) break;
        T x = (i + T(0.5)) * dx + src.ox;
        T y = (j + T(0.5)) * dx + src.oy;
        T z = (k + T(0.5)) * dx + src.oz;
        T ax, ay, az;
        cell_velocity(mac, i, j, k, ax, ay, az);
        backtrace_from<T, TRACE>(mac, ax, ay, az, x, y, z, h, dx, inv_dx);
        // stencil origin (floor - 2) relative to the box, per axis
        const AxisPos<T> px = axis_pos(x, src.ox, x0 - 1, dx, inv_dx);
        const AxisPos<T> py = axis_pos(y, src.oy, y0 - 1, dx, inv_dx);
        const AxisPos<T> pz = axis_pos(z, src.oz, z0 - 1, dx, inv_dx);
        T r;
        if ((unsigned)px.a < (unsigned)kWBases && (unsigned)py.a < (unsigned)(kWY + 2) &&
            (unsigned)pz.a < (unsigned)(kWZ + 2)) {
            const WenoAxis<T> wx = weno_axis(px.f);
            const WenoAxis<T> wy = weno_axis(py.f);
            T zl[6];
            if constexpr (sizeof(T) == 4) {
                // FP32: packed float2 arithmetic (two lanes per instruction, each rounded as its
                // scalar operation): the x-passes of rows dj and dj + 1, and the y-passes of
                // planes dk and dk + 1, together; the expressions of weno6_combine / weno6_eval
#pragma unroll
                for (int dk = 0; dk < 6; dk += 2) {
                    float2 yl2[6];  // .x: plane dk, .y: plane dk + 1
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int row0 = (pz.a + dk + h) * kWBY + py.a;
#pragma unroll
                        for (int dj = 0; dj < 6; dj += 2) {
                            const int row = row0 + dj;
                            const float* va = pb + row * kWBX + px.a;
                            const float* vb = va + kWBX;
                            const float2 qa2 = reinterpret_cast<const float2*>(qbox)[row * kWBases + px.a];
                            const float2 qb2 = reinterpret_cast<const float2*>(qbox)[(row + 1) * kWBases + px.a];
                            const float* qc = qbox + 2 * kWQ + row * kWBases + px.a;
                            float2 v[6];
#pragma unroll
                            for (int m = 0; m < 6; ++m) v[m] = make_float2(va[m], vb[m]);
                            const float2 rr = weno6_combine2(wx, v, make_float2(qa2.x, qb2.x),
                                                             make_float2(qa2.y, qb2.y), make_float2(qc[0], qc[kWBases]));
                            if (h == 0) {
                                yl2[dj].x = rr.x;
                                yl2[dj + 1].x = rr.y;
                            } else {
                                yl2[dj].y = rr.x;
                                yl2[dj + 1].y = rr.y;
                            }
                        }
                    }
                    const float2 zv = weno6_eval2(wy, yl2);
                    zl[dk] = zv.x;
                    zl[dk + 1] = zv.y;
                }
            } else {
#pragma unroll
            for (int dk = 0; dk < 6; ++dk) {
                const int row0 = (pz.a + dk) * kWBY + py.a;
                T yl[6];
#pragma unroll
                for (int dj = 0; dj < 6; ++dj) {
                    const int row = row0 + dj;
                    const T* v = pb + row * kWBX + px.a;
                    const T* q = qbox + row * kWBases + px.a;
                    yl[dj] = weno6_combine(wx, v[0], v[1], v[2], v[3], v[4], v[5], q[0], q[kWQ], q[2 * kWQ]);
                }
                const T zv = weno6_eval(wy, yl[0], yl[1], yl[2], yl[3], yl[4], yl[5]);
                zl[0] = dk == 0 ? zv : zl[0];
                zl[1] = dk == 1 ? zv : zl[1];
                zl[2] = dk == 2 ? zv : zl[2];
                zl[3] = dk == 3 ? zv : zl[3];
                zl[4] = dk == 4 ? zv : zl[4];
                zl[5] = dk == 5 ? zv : zl[5];
            }
            }
            r = weno6_eval(weno_axis(pz.f), zl[0], zl[1], zl[2], zl[3], zl[4], zl[5]);
        } else {
            r = sample_weno6(src, x, y, z, dx, inv_dx);
        }
        const long long oc = lin3(i, j, k, src.n0, src.n1);
        if (EL_IN(oc, (long long)src.n0 * src.n1 * src.n2, 3)) out[oc] = r;
    }
}

// Grid views of the scene's grids (staggered_grid.h:100-112): comp 0 = cells, 1/2/3 = u/v/w.
template <typename T>
GridView<T> make_view(const void* d, int ni, int nj, int nk, T dx, int comp) {
    GridView<T> g{static_cast<const T*>(d), ni, nj, nk, T(0), T(0), T(0)};
    const T half = T(0.5) * dx;
    if (comp == 1) { g.n0 = ni + 1; g.ox = T(0) - half; }
    if (comp == 2) { g.n1 = nj + 1; g.oy = T(0) - half; }
    if (comp == 3) { g.n2 = nk + 1; g.oz = T(0) - half; }
    return g;
}

template <typename T, int TRACE, int SAMPLE>
static void launch_one(const GridView<T>& src, void* out, const Mac<T>& mac, DtArg dt, T dx, int rows,
                       cudaStream_t s) {
    dim3 block(32, rows, 1);
    dim3 grid((src.n0 + 31) / 32, (src.n1 + rows - 1) / rows, src.n2);
    advect_kernel<T, TRACE, SAMPLE><<<grid, block, 0, s>>>(src, static_cast<T*>(out), mac, dt, dx,
                                                           T(1) / dx);
}

template <typename T>
static void launch_dispatch(const GridView<T>& src, void* out, const Mac<T>& mac, DtArg dt, T dx,
                            int trace, int sample, int rows, cudaStream_t s) {
    if (trace == EL_TRACE_RK2 && sample == EL_SAMPLE_TRILINEAR)
        launch_one<T, EL_TRACE_RK2, EL_SAMPLE_TRILINEAR>(src, out, mac, dt, dx, rows, s);
    else if (trace == EL_TRACE_RK2 && sample == EL_SAMPLE_WENO6)
        launch_one<T, EL_TRACE_RK2, EL_SAMPLE_WENO6>(src, out, mac, dt, dx, rows, s);
    else if (trace == EL_TRACE_RK3 && sample == EL_SAMPLE_TRILINEAR)
        launch_one<T, EL_TRACE_RK3, EL_SAMPLE_TRILINEAR>(src, out, mac, dt, dx, rows, s);
    else
        launch_one<T, EL_TRACE_RK3, EL_SAMPLE_WENO6>(src, out, mac, dt, dx, rows, s);
}

// Launch the advection of `which` (0 = cell-centred grid `in`, 1..3 = face component) into out.
// Returns the number of kernels launched.
template <typename T>
static int advect_launch(int ni, int nj, int nk, double dx_d, int comp, void* out, const void* in,
                         const void* vu, const void* vv, const void* vw, DtArg dt, int trace,
                         int sample, int rows, cudaStream_t s) {
    const T dx = (T)dx_d;
    Mac<T> mac{make_view<T>(vu, ni, nj, nk, dx, 1), make_view<T>(vv, ni, nj, nk, dx, 2),
               make_view<T>(vw, ni, nj, nk, dx, 3)};
    GridView<T> src = make_view<T>(in, ni, nj, nk, dx, comp);
    launch_dispatch<T>(src, out, mac, dt, dx, trace, sample, rows, s);
    return 1;
}

// The box map of one array for boxes of bx x by x bz (on = 0 when copies are off or the
// array's pitch or address does not allow them: the kernel then stages it by plain loads).
template <typename T>
static BoxMap box_map(const GridView<T>& g, bool copy, unsigned bx, unsigned by, unsigned bz) {
    BoxMap b;
    std::memset(&b, 0, sizeof(b));
    b.on = copy && tma_encode_3d(&b.m, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64,
                                 (int)sizeof(T), g.d, g.n0, g.n1, g.n2, g.n0, bx, by, bz);
    return b;
}

template <typename T>
static MacMaps mac_maps(const Mac<T>& mac, bool copy) {
    MacMaps m;
    m.c[0] = box_map(mac.u, copy, kBoxX, kBoxY, kBoxZ);
    m.c[1] = box_map(mac.v, copy, kBoxX, kBoxY, kBoxZ);
    m.c[2] = box_map(mac.w, copy, kBoxX, kBoxY, kBoxZ);
    return m;
}

// the tiled kernels: the level set (any scheme), and the velocity advecting itself (trilinear);
// dynamic shared memory holds the boxes plus 128 bytes to align them
template <typename T, int TRACE, int SAMPLE>
static int launch_phi_tiled(const GridView<T>& src, void* out, const Mac<T>& mac, DtArg dt, T dx, bool copy,
                            cudaStream_t s) {
    const int smem = 3 * kBoxN * (int)sizeof(T) + 128;
    if (cudaFuncSetAttribute(advect_phi_tiled_kernel<T, TRACE, SAMPLE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess)
        return -1;
    const dim3 grid((src.n0 + kTileX - 1) / kTileX, (src.n1 + kTileY - 1) / kTileY, (src.n2 + kTileZ - 1) / kTileZ);
    advect_phi_tiled_kernel<T, TRACE, SAMPLE><<<grid, dim3(kTileX, kTileY, 1), smem, s>>>(
        src, static_cast<T*>(out), mac, dt, dx, T(1) / dx, mac_maps(mac, copy));
    return 1;
}

template <typename T, int TRACE>
static int launch_phi_weno_tiled(const GridView<T>& src, void* out, const Mac<T>& mac, DtArg dt, T dx, bool copy,
                                 cudaStream_t s) {
    const int smem = (kWBoxN + 3 * kWQ) * (int)sizeof(T) + 128;
    if (cudaFuncSetAttribute(advect_phi_weno_tiled_kernel<T, TRACE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess)
        return -1;
    const dim3 grid((src.n0 + kWX - 1) / kWX, (src.n1 + kWY - 1) / kWY, (src.n2 + kWZ - 1) / kWZ);
    advect_phi_weno_tiled_kernel<T, TRACE><<<grid, dim3(kWX, kWY, 1), smem, s>>>(
        src, static_cast<T*>(out), mac, dt, dx, T(1) / dx, box_map(src, copy, kWBX, kWBY, kWBZ));
    return 1;
}

template <typename T, int TRACE>
static int launch_velocity_tiled(const Mac<T>& mac, void* ou, void* ov, void* ow, DtArg dt, T dx, bool copy,
                                 cudaStream_t s) {
    const int smem = 3 * kBoxN * (int)sizeof(T) + 128;
    if (cudaFuncSetAttribute(advect_velocity_tiled_kernel<T, TRACE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem) != cudaSuccess)
        return -1;
    // tiles over the largest extent of the three face grids
    const dim3 grid((mac.u.n0 + kTileX - 1) / kTileX, (mac.v.n1 + kTileY - 1) / kTileY,
                    (mac.w.n2 + kTileZ - 1) / kTileZ);
    advect_velocity_tiled_kernel<T, TRACE><<<grid, dim3(kTileX, kTileY, 1), smem, s>>>(
        mac, static_cast<T*>(ou), static_cast<T*>(ov), static_cast<T*>(ow), dt, dx, T(1) / dx, mac_maps(mac, copy));
    return 1;
}

template <typename T>
static int advect_phi_tiled_t(int ni, int nj, int nk, double dx_d, void* out, const void* in, const void* vu,
                              const void* vv, const void* vw, DtArg dt, int trace, int sample, bool copy,
                              cudaStream_t s) {
    const T dx = (T)dx_d;
    Mac<T> mac{make_view<T>(vu, ni, nj, nk, dx, 1), make_view<T>(vv, ni, nj, nk, dx, 2),
               make_view<T>(vw, ni, nj, nk, dx, 3)};
    GridView<T> src = make_view<T>(in, ni, nj, nk, dx, 0);
    if (sample == EL_SAMPLE_WENO6)
        return trace == EL_TRACE_RK2 ? launch_phi_weno_tiled<T, EL_TRACE_RK2>(src, out, mac, dt, dx, copy, s)
                                     : launch_phi_weno_tiled<T, EL_TRACE_RK3>(src, out, mac, dt, dx, copy, s);
    if (trace == EL_TRACE_RK2)
        return launch_phi_tiled<T, EL_TRACE_RK2, EL_SAMPLE_TRILINEAR>(src, out, mac, dt, dx, copy, s);
    return launch_phi_tiled<T, EL_TRACE_RK3, EL_SAMPLE_TRILINEAR>(src, out, mac, dt, dx, copy, s);
}

template <typename T>
static int advect_velocity_tiled_t(int ni, int nj, int nk, double dx_d, void* ou, void* ov, void* ow, const void* vu,
                                   const void* vv, const void* vw, DtArg dt, int trace, bool copy, cudaStream_t s) {
    const T dx = (T)dx_d;
    Mac<T> mac{make_view<T>(vu, ni, nj, nk, dx, 1), make_view<T>(vv, ni, nj, nk, dx, 2),
               make_view<T>(vw, ni, nj, nk, dx, 3)};
    if (trace == EL_TRACE_RK2) return launch_velocity_tiled<T, EL_TRACE_RK2>(mac, ou, ov, ow, dt, dx, copy, s);
    return launch_velocity_tiled<T, EL_TRACE_RK3>(mac, ou, ov, ow, dt, dx, copy, s);
}

// Level set through the tiled kernel; returns kernels launched, -1 on a launch set-up failure.
// copy: stage the boxes by box copies where the arrays allow it (else plain loads throughout).
int advect_phi_tiled(int dtype, int ni, int nj, int nk, double dx, void* out, const void* in, const void* vu,
                     const void* vv, const void* vw, const Scalars* dts, double dtv, int trace, int sample, bool copy,
                     cudaStream_t s) {
    DtArg dt{dts, dtv};
    if (dtype == EL_F64)
        return advect_phi_tiled_t<double>(ni, nj, nk, dx, out, in, vu, vv, vw, dt, trace, sample, copy, s);
    return advect_phi_tiled_t<float>(ni, nj, nk, dx, out, in, vu, vv, vw, dt, trace, sample, copy, s);
}

// u, v, w advected through themselves with trilinear sampling, one tiled launch
int advect_velocity_tiled(int dtype, int ni, int nj, int nk, double dx, void* ou, void* ov, void* ow, const void* vu,
                          const void* vv, const void* vw, const Scalars* dts, double dtv, int trace, bool copy,
                          cudaStream_t s) {
    DtArg dt{dts, dtv};
    if (dtype == EL_F64)
        return advect_velocity_tiled_t<double>(ni, nj, nk, dx, ou, ov, ow, vu, vv, vw, dt, trace, copy, s);
    return advect_velocity_tiled_t<float>(ni, nj, nk, dx, ou, ov, ow, vu, vv, vw, dt, trace, copy, s);
}

// the box-copy wait fault word, read and cleared (synchronises the device)
bool advect_fault_take() {
    unsigned v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, advect_wait_fault, sizeof(v)) != cudaSuccess) return false;
    if (v) cudaMemcpyToSymbol(advect_wait_fault, &z, sizeof(z));
    return v != 0;
}

int advect_any(int dtype, int ni, int nj, int nk, double dx, int comp, void* out, const void* in,
               const void* vu, const void* vv, const void* vw, const Scalars* dts, double dtv,
               int trace, int sample, cudaStream_t s, int rows) {
    DtArg dt{dts, dtv};
    rows = (rows == 1 || rows == 2 || rows == 8) ? rows : 4;
    if (dtype == EL_F64)
        return advect_launch<double>(ni, nj, nk, dx, comp, out, in, vu, vv, vw, dt, trace, sample, rows, s);
    return advect_launch<float>(ni, nj, nk, dx, comp, out, in, vu, vv, vw, dt, trace, sample, rows, s);
}

EL_CHECK_EXPORT(advect)

}  // namespace el
