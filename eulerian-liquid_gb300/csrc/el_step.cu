// el_step.cu -- the step pieces around advection and projection, on the device.
//
// Reference: src/project/3d/fluid/extrapolation.cpp:5-51 (extrapolate),
// src/project/3d/eulerian_liquid/simulator.cpp:90-178 (add_gravity, find_valid_velocity,
// set_invalid_velocity_zero), src/project/3d/fluid/time_stepping.cpp:5-7 (calc_time_step),
// src/project/3d/fluid/levelset_emitter.cpp:10-79 (emitters).
#include <type_traits>

#include "el_internal.cuh"

namespace el {

__device__ __forceinline__ float mul_rn2(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn2(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn2(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn2(double a, double b) { return __dadd_rn(a, b); }

// ---------------------------------------------------------------------------------------
// add_gravity + find_valid_velocity + set_invalid_velocity_zero, fused per face
// (simulator.cpp:90-93, 125-158, 169-178).  The phi test applies on faces with index in
// [1, n) along the normal and [1, n-1) along the tangential axes, as the reference's loops.
// The three components in one launch: a thread takes the faces u, v and w at (i, j, k) down a
// column, so that the level set is read once for all three (its values for the neighbouring
// faces come from L1).
// One face after its loads: gravity, the mask (weight nonzero and, on the faces the phi test
// covers, not both cells outside the liquid), the invalid value zeroed.
template <typename T>
__device__ __forceinline__ void mask_face(T val, T wt, bool tested, T pa, T pb, long long fi, T* __restrict__ f,
                                          uint8_t* __restrict__ valid, bool gravity, T gdt, bool zero_invalid) {
    if (gravity) val = val - gdt;
    bool ok = wt != T(0);
    if (ok && tested && pa >= T(0) && pb >= T(0)) ok = false;
    valid[fi] = ok ? 1 : 0;
    if (zero_invalid && !ok) val = T(0);
    if (gravity || (zero_invalid && !ok)) f[fi] = val;
}

template <typename T>
__global__ void masks3_kernel(int ni, int nj, int nk, T* __restrict__ u, T* __restrict__ v, T* __restrict__ w,
                              const T* __restrict__ wu, const T* __restrict__ wv, const T* __restrict__ ww,
                              const T* __restrict__ phi, uint8_t* __restrict__ mu, uint8_t* __restrict__ mv,
                              uint8_t* __restrict__ mw, int apply_gravity, T gravity, const Scalars* s,
                              double dt_value, int zero_invalid, int kz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    if (i > ni || j > nj) return;
    const T dt = apply_gravity ? (T)(s ? s->dt : dt_value) : T(0);
    const T gdt = mul_rn2(gravity, dt);  // the product each face subtracts (one rounding)
    const bool zero = zero_invalid != 0;
    const long long plane = (long long)ni * nj;
#pragma unroll
    for (int kk = 0; kk < kz; ++kk) {
        const int k = blockIdx.z * kz + kk;
        if (k > nk) break;
        // the faces u, v, w at (i, j, k) that exist, and which of them the phi test covers
        // (index in [1, n) along the normal, [1, n - 1) along the tangential axes)
        const bool hu = j < nj && k < nk, hv = i < ni && k < nk, hw = i < ni && j < nj;
        const bool low = i >= 1 && j >= 1 && k >= 1;
        const bool tu = low && i < ni && j < nj - 1 && k < nk - 1;
        const bool tv = low && i < ni - 1 && j < nj && k < nk - 1;
        const bool tw = low && i < ni - 1 && j < nj - 1 && k < nk;
        const long long fu = lin3(i, j, k, ni + 1, nj), fv = lin3(i, j, k, ni, nj + 1), fw = lin3(i, j, k, ni, nj);
        const long long b = fw;  // the cell (i, j, k), inside the grid wherever a test reads it
        // every load first
        const T u0 = hu ? u[fu] : T(0), v0 = hv ? v[fv] : T(0), w0 = hw ? w[fw] : T(0);
        const T wu0 = hu ? __ldg(wu + fu) : T(0), wv0 = hv ? __ldg(wv + fv) : T(0), ww0 = hw ? __ldg(ww + fw) : T(0);
        const T pc = (tu || tv || tw) ? __ldg(phi + b) : T(0);
        const T pxm = tu ? __ldg(phi + b - 1) : T(0), pym = tv ? __ldg(phi + b - ni) : T(0);
        const T pzm = tw ? __ldg(phi + b - plane) : T(0);
        if (hu) mask_face(u0, wu0, tu, pxm, pc, fu, u, mu, false, gdt, zero);
        if (hv) mask_face(v0, wv0, tv, pym, pc, fv, v, mv, apply_gravity != 0, gdt, zero);
        if (hw) mask_face(w0, ww0, tw, pzm, pc, fw, w, mw, false, gdt, zero);
    }
}

template <typename T>
__global__ void gravity_kernel(long long n, T* __restrict__ v, T gravity, const Scalars* s, double dt_value) {
    const T dt = (T)(s ? s->dt : dt_value);
    const T dv = mul_rn2(gravity, dt);
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        v[c] = v[c] - dv;
}

template <typename T>
__global__ void zero_invalid_kernel(long long n, T* __restrict__ f, const uint8_t* __restrict__ valid) {
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        if (!valid[c]) f[c] = T(0);
}

// max |u| over the MAC grid (staggered_grid.h:230-248): |x| as unsigned bits orders like x.
__device__ __forceinline__ void atomic_max_abs(unsigned long long* m, double v) {
    atomicMax(m, (unsigned long long)__double_as_longlong(fabs(v)));
}

// max |a| over one array, in the field type (a maximum of magnitudes is exact in any type, and
// fmax ignores NaN in both), 16-byte loads for the bulk
template <typename T>
__device__ __forceinline__ T maxabs_run(const T* __restrict__ a, long long n, long long t0, long long stride, T m) {
    using V2 = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    constexpr int per = (int)(sizeof(V2) / sizeof(T));
    const long long nv = n / per;
    const V2* av = reinterpret_cast<const V2*>(a);
    for (long long c = t0; c < nv; c += stride) {
        const V2 x = __ldg(av + c);
        if constexpr (sizeof(T) == 4)
            m = fmaxf(fmaxf(fmaxf(m, fabsf(x.x)), fmaxf(fabsf(x.y), fabsf(x.z))), fabsf(x.w));
        else
            m = fmax(m, fmax(fabs(x.x), fabs(x.y)));
    }
    for (long long c = nv * per + t0; c < n; c += stride) m = (T)fmax(m, fabs(a[c]));
    return m;
}

// max(|u|, |v|, |w|) over the three face grids, one launch (the fields are 256-byte aligned)
template <typename T>
__global__ void maxabs3_kernel(const T* __restrict__ u, long long nu, const T* __restrict__ v, long long nv,
                               const T* __restrict__ w, long long nw, unsigned long long* out) {
    const long long t0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    T m = T(0);
    m = maxabs_run(u, nu, t0, stride, m);
    m = maxabs_run(v, nv, t0, stride, m);
    m = maxabs_run(w, nw, t0, stride, m);
    double md = (double)m;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) md = fmax(md, __shfl_down_sync(0xffffffffu, md, o));
    if ((threadIdx.x & 31) == 0) atomic_max_abs(out, md);
}

// dt = cfl * dx / max(max|u|, 1e-4) in the field type (time_stepping.cpp:5-7)
template <typename T>
__global__ void time_step_kernel(const unsigned long long* m, T cfl, T dx, Scalars* s) {
    const T mx = (T)__longlong_as_double((long long)*m);
    const T den = mx > T(1e-4) ? mx : T(1e-4);
    const T dt = mul_rn2(cfl, dx) / den;
    s->maxabs = (double)mx;
    s->dt = (double)dt;
}

__global__ void set_dt_kernel(Scalars* s, double dt) { s->dt = dt; }

// One sub-step of Simulator::update with use_cfl (simulator.cpp:28-36): dt_sub = calc_time_step
// in the field type, cut so that the frame ends exactly: if (t + dt_sub > dt_frame) dt_sub =
// dt_frame - t, with t the time already taken in this frame (kept by the batch record).
template <typename T>
__global__ void substep_kernel(const unsigned long long* m, T cfl, T dx, T dt_frame, const BatchRecord* r,
                               Scalars* s) {
    const T mx = (T)__longlong_as_double((long long)*m);
    const T den = mx > T(1e-4) ? mx : T(1e-4);
    T dt = mul_rn2(cfl, dx) / den;
    if (dt_frame > T(0)) {
        const T t = (T)r->frame_t;
        if (t + dt > dt_frame) dt = dt_frame - t;
    }
    s->maxabs = (double)mx;
    s->dt = (double)dt;
}

// ---------------------------------------------------------------------------------------
// emitters (levelset_emitter.cpp:10-79): min(field, f(x)) at the grid's sample positions.
enum { EMIT_CLEAR = 0, EMIT_SPHERE = 1, EMIT_POOL = 2, EMIT_BOX = 3, EMIT_ROOM = 4 };

struct EmitArgs {
    int kind;
    double a[8];
};

template <typename T>
__global__ void emit_kernel(int n0, int n1, int n2, T* __restrict__ g, T ox, T dx, EmitArgs e) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y * blockDim.y + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n0 || j >= n1) return;
    const long long c = lin3(i, j, k, n0, n1);
    if (e.kind == EMIT_CLEAR) {
        g[c] = (T)3.402823466e+38;  // FLT_MAX, as LevelSetEmitterList::apply
        return;
    }
    // GridBase::pos (grid.h:355-367): (idx + 0.5) * dx + origin
    const T px = add_rn2(mul_rn2(i + T(0.5), dx), ox);
    const T py = add_rn2(mul_rn2(j + T(0.5), dx), ox);
    const T pz = add_rn2(mul_rn2(k + T(0.5), dx), ox);
    T val;
    if (e.kind == EMIT_SPHERE) {
        const T qx = px - (T)e.a[0], qy = py - (T)e.a[1], qz = pz - (T)e.a[2];
        // (x - c).norm() of an Eigen::Vector3f: x^2 + (y^2 + z^2)  (levelset_emitter.cpp:10-12)
        const T ss = add_rn2(mul_rn2(qx, qx), add_rn2(mul_rn2(qy, qy), mul_rn2(qz, qz)));
        val = sqrt(ss) - (T)e.a[3];
    } else if (e.kind == EMIT_POOL) {
        val = py - (T)e.a[0];
    } else if (e.kind == EMIT_BOX) {
        const T p[3] = {px, py, pz};
        T outside2 = T(0), inside = -(T)3.402823466e+38;
        for (int ax = 0; ax < 3; ++ax) {
            const T lo = (T)e.a[ax], hi = (T)e.a[3 + ax];
            const T q = fmax(lo - p[ax], p[ax] - hi);
            if (q > T(0)) outside2 = add_rn2(outside2, mul_rn2(q, q));
            inside = fmax(inside, q);
        }
        val = outside2 > T(0) ? sqrt(outside2) : inside;
    } else {  // room: nodal wall layers (levelset_emitter.cpp:18-32)
        if (i == 0 || i == n0 - 1 || j == 0 || j == n1 - 1 || k == 0 || k == n2 - 1)
            val = (T)-1.0;
        else if (i == 1 || i == n0 - 2 || j == 1 || j == n1 - 2 || k == 1 || k == n2 - 2)
            val = (T)-0.01;
        else
            val = (T)1.0;
    }
    const T old = g[c];
    g[c] = val < old ? val : old;
}

// ---------------------------------------------------------------------------------------
// launchers

static dim3 pgrid(int n0, int n1, int n2, dim3 b) { return dim3((n0 + b.x - 1) / b.x, (n1 + b.y - 1) / b.y, n2); }

static int g1(el_ctx* ctx, long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)ctx->num_sms * ctx->stencil_per_sm));
}

void field_dims(const el_ctx* ctx, int field, int& n0, int& n1, int& n2) {
    n0 = ctx->ni;
    n1 = ctx->nj;
    n2 = ctx->nk;
    if (field == EL_FIELD_U || field == EL_FIELD_WEIGHT_U || field == EL_FIELD_VALID_U) n0++;
    if (field == EL_FIELD_V || field == EL_FIELD_WEIGHT_V || field == EL_FIELD_VALID_V) n1++;
    if (field == EL_FIELD_W || field == EL_FIELD_WEIGHT_W || field == EL_FIELD_VALID_W) n2++;
    if (field == EL_FIELD_SOLID_NODAL) {
        n0++;
        n1++;
        n2++;
    }
}

template <typename T>
static int launch_masks_t(el_ctx* ctx, bool gravity, double g, const Scalars* s, double dtv, bool zero) {
    dim3 block(32, 8, 1);
    constexpr int kz = 8;
    T* f[3];
    const T* wt[3];
    uint8_t* m[3];
    for (int c = 0; c < 3; ++c) {
        f[c] = (T*)ctx->field[EL_FIELD_U + c];
        wt[c] = (const T*)ctx->field[EL_FIELD_WEIGHT_U + c];
        m[c] = (uint8_t*)ctx->field[EL_FIELD_VALID_U + c];
    }
    masks3_kernel<T><<<pgrid(ctx->ni + 1, ctx->nj + 1, (ctx->nk + 1 + kz - 1) / kz, block), block, 0, ctx->stream>>>(
        ctx->ni, ctx->nj, ctx->nk, f[0], f[1], f[2], wt[0], wt[1], wt[2], (const T*)ctx->field[EL_FIELD_PHI], m[0], m[1],
        m[2], gravity ? 1 : 0, (T)g, s, dtv, zero ? 1 : 0, kz);
    return 1;
}

int launch_masks(el_ctx* ctx, bool gravity, double g, const Scalars* s, double dtv, bool zero) {
    return ctx->dtype == EL_F64 ? launch_masks_t<double>(ctx, gravity, g, s, dtv, zero)
                                : launch_masks_t<float>(ctx, gravity, g, s, dtv, zero);
}

int launch_gravity(el_ctx* ctx, double g, const Scalars* s, double dtv) {
    const long long n = (long long)ctx->ni * (ctx->nj + 1) * ctx->nk;
    if (ctx->dtype == EL_F64)
        gravity_kernel<double><<<g1(ctx, n), 256, 0, ctx->stream>>>(n, (double*)ctx->field[EL_FIELD_V], g, s, dtv);
    else
        gravity_kernel<float><<<g1(ctx, n), 256, 0, ctx->stream>>>(n, (float*)ctx->field[EL_FIELD_V], (float)g, s, dtv);
    return 1;
}

int launch_zero_invalid(el_ctx* ctx) {
    for (int comp = 0; comp < 3; ++comp) {
        int n0, n1, n2;
        field_dims(ctx, EL_FIELD_U + comp, n0, n1, n2);
        const long long n = (long long)n0 * n1 * n2;
        const uint8_t* valid = (const uint8_t*)ctx->field[EL_FIELD_VALID_U + comp];
        if (ctx->dtype == EL_F64)
            zero_invalid_kernel<double><<<g1(ctx, n), 256, 0, ctx->stream>>>(n, (double*)ctx->field[EL_FIELD_U + comp], valid);
        else
            zero_invalid_kernel<float><<<g1(ctx, n), 256, 0, ctx->stream>>>(n, (float*)ctx->field[EL_FIELD_U + comp], valid);
    }
    return 3;
}

// Computes dt into ctx->dscal[0].dt on the device.
// max |u|, |v|, |w| into scratch_max (as the bits of a non-negative double)
static void launch_maxabs(el_ctx* ctx, unsigned long long* scratch_max) {
    cudaMemsetAsync(scratch_max, 0, sizeof(unsigned long long), ctx->stream);
    long long n[3];
    for (int comp = 0; comp < 3; ++comp) {
        int n0, n1, n2;
        field_dims(ctx, EL_FIELD_U + comp, n0, n1, n2);
        n[comp] = (long long)n0 * n1 * n2;
    }
    const int per = ctx->dtype == EL_F64 ? 2 : 4;
    const int grid = g1(ctx, n[0] / per);
    if (ctx->dtype == EL_F64)
        maxabs3_kernel<double><<<grid, 256, 0, ctx->stream>>>(
            (const double*)ctx->field[EL_FIELD_U], n[0], (const double*)ctx->field[EL_FIELD_V], n[1],
            (const double*)ctx->field[EL_FIELD_W], n[2], scratch_max);
    else
        maxabs3_kernel<float><<<grid, 256, 0, ctx->stream>>>(
            (const float*)ctx->field[EL_FIELD_U], n[0], (const float*)ctx->field[EL_FIELD_V], n[1],
            (const float*)ctx->field[EL_FIELD_W], n[2], scratch_max);
}

int launch_time_step(el_ctx* ctx, double cfl, unsigned long long* scratch_max) {
    launch_maxabs(ctx, scratch_max);
    if (ctx->dtype == EL_F64)
        time_step_kernel<double><<<1, 1, 0, ctx->stream>>>(scratch_max, cfl, ctx->dx, ctx->dscal);
    else
        time_step_kernel<float><<<1, 1, 0, ctx->stream>>>(scratch_max, (float)cfl, (float)ctx->dx, ctx->dscal);
    return 2;
}

// dt of a batch sub-step into ctx->dscal[0].dt on the device (no host involvement).
int launch_substep(el_ctx* ctx, double cfl, double dt_frame, const BatchRecord* rec, unsigned long long* scratch_max) {
    launch_maxabs(ctx, scratch_max);
    if (ctx->dtype == EL_F64)
        substep_kernel<double><<<1, 1, 0, ctx->stream>>>(scratch_max, cfl, ctx->dx, dt_frame, rec, ctx->dscal);
    else
        substep_kernel<float><<<1, 1, 0, ctx->stream>>>(scratch_max, (float)cfl, (float)ctx->dx, (float)dt_frame, rec,
                                                        ctx->dscal);
    return 2;
}

int launch_set_dt(el_ctx* ctx, double dt) {
    set_dt_kernel<<<1, 1, 0, ctx->stream>>>(ctx->dscal, dt);
    return 1;
}

int launch_emit(el_ctx* ctx, int target, int kind, const double* a, int na) {
    const int field = target == 0 ? EL_FIELD_PHI : EL_FIELD_SOLID_NODAL;
    int n0, n1, n2;
    field_dims(ctx, field, n0, n1, n2);
    EmitArgs e;
    e.kind = kind;
    for (int q = 0; q < 8; ++q) e.a[q] = q < na ? a[q] : 0.0;
    dim3 block(32, 4, 1);
    dim3 grid = pgrid(n0, n1, n2, block);
    if (ctx->dtype == EL_F64) {
        const double dx = ctx->dx;
        const double ox = target == 0 ? 0.0 : -(dx * 0.5);
        emit_kernel<double><<<grid, block, 0, ctx->stream>>>(n0, n1, n2, (double*)ctx->field[field], ox, dx, e);
    } else {
        const float dx = (float)ctx->dx;
        const float ox = target == 0 ? 0.0f : -(dx * 0.5f);
        emit_kernel<float><<<grid, block, 0, ctx->stream>>>(n0, n1, n2, (float*)ctx->field[field], ox, dx, e);
    }
    return 1;
}

}  // namespace el
