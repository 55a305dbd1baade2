// el_advect.cu -- semi-Lagrangian advection of the level set and the MAC velocity.
//
// Reference: src/project/3d/fluid/advection.cpp:9-27 (loop drivers), include/nama/math/ode.h
// (StaggeredGridField, trace_rk2), include/nama/math/interpolation.h (lerp, weno6_interp).
// One thread per output sample: sample position -> backtrace through the old velocity
// (trilinear MAC interpolation at every RK stage) -> trilinear or WENO6 sample of the old
// field at the foot point.  Reads go through the read-only path; the foot point moves at most
// about one cell per step under the CFL limit, so neighbouring threads gather overlapping
// stencils and the L1/L2 serve most of them.
#include "el_internal.cuh"

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

template <typename T>
__device__ __forceinline__ void velocity_at(const Mac<T>& m, T x, T y, T z, T dx, T inv, T& vx, T& vy,
                                            T& vz) {
    vx = sample_trilinear(m.u, x, y, z, dx, inv);
    vy = sample_trilinear(m.v, x, y, z, dx, inv);
    vz = sample_trilinear(m.w, x, y, z, dx, inv);
}

// trace_rk2 (ode.h:30-35) or Ralston RK3 (c = 0, 1/2, 3/4; b = 2/9, 1/3, 4/9); h is the
// signed step (-dt for a backtrace).
template <typename T, int TRACE>
__device__ __forceinline__ void backtrace(const Mac<T>& m, T& x, T& y, T& z, T h, T dx, T inv) {
    T ax, ay, az;
    velocity_at(m, x, y, z, dx, inv, ax, ay, az);
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
    out[lin3(i, j, k, src.n0, src.n1)] = r;
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

int advect_any(int dtype, int ni, int nj, int nk, double dx, int comp, void* out, const void* in,
               const void* vu, const void* vv, const void* vw, const Scalars* dts, double dtv,
               int trace, int sample, cudaStream_t s, int rows) {
    DtArg dt{dts, dtv};
    rows = (rows == 1 || rows == 2 || rows == 8) ? rows : 4;
    if (dtype == EL_F64)
        return advect_launch<double>(ni, nj, nk, dx, comp, out, in, vu, vv, vw, dt, trace, sample, rows, s);
    return advect_launch<float>(ni, nj, nk, dx, comp, out, in, vu, vv, vw, dt, trace, sample, rows, s);
}

}  // namespace el
