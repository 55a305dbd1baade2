// el_warm.cu -- the scene side of the learned warm start: network inputs (and training targets)
// from a context's pressure system, and the network's prediction written back as the initial
// guess of el_solve_pressure.  No counterpart in the reference.
//
// Scaling makes the network see the same numbers whatever dt, dx and flow strength: with
// A = a * A^ (a = mean diagonal / 6, so A^ has unit couplings) and b = rms(b) * b^, the solution
// is p = (rms(b) / a) * A^-1 b^; the network is trained to predict p^ = p * a / rms(b).
#include <cuda_bf16.h>

#include "el_internal.cuh"

namespace el {
int ensure_projection(el_ctx* ctx);
int launch_flags_build(el_ctx* ctx, bool inner32, bool build);
int launch_set_dt(el_ctx* ctx, double dt);
int set_error(el_ctx* ctx, int code, const std::string& msg);
int check_launch(el_ctx* ctx, const char* what);
}  // namespace el

using namespace el;

namespace {

constexpr int kFeat = 16;  // channels of the network input (3 used)

// sums over fluid cells (diagonal > 0): b^2, diagonal, count, p.b -> s
template <typename T>
__global__ void warm_sums_kernel(long long n, const double* __restrict__ diag, const double* __restrict__ b,
                                 const T* __restrict__ pressure, Scalars* s, double* partials, unsigned* counter) {
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const double d = diag[c];
        if (d > 0.0) {
            acc[0] += b[c] * b[c];
            acc[1] += d;
            acc[2] += 1.0;
            acc[3] += (double)pressure[c] * b[c];
        }
    }
    double tot[4];
    if (grid_sum<4>(acc, partials, counter, tot)) {
        const double cnt = tot[2];
        s->rr = (cnt > 0.0 && tot[0] > 0.0) ? sqrt(tot[0] / cnt) : 1.0;  // rms(b)
        s->alpha = (cnt > 0.0 && tot[1] > 0.0) ? tot[1] / (6.0 * cnt) : 1.0;  // a
        s->aux = cnt;
        // energy of the scaled solution, p^ . A^ p^ = p^ . b^ = (a / rms^2) p . b
        s->norm = tot[3] * s->alpha / (s->rr * s->rr);
    }
}

template <typename T>
__global__ void warm_features_kernel(long long n, int ni, int nj, const T* __restrict__ phi, const T* __restrict__ solid,
                                     const double* __restrict__ diag, const T* __restrict__ ox,
                                     const T* __restrict__ oy, const T* __restrict__ oz, const double* __restrict__ b,
                                     const T* __restrict__ pressure, double inv3dx, const Scalars* s,
                                     __nv_bfloat16* __restrict__ feat, __nv_bfloat16* __restrict__ coup,
                                     float* __restrict__ target, uint8_t* __restrict__ fluid) {
    const double rms = s->rr, a = s->alpha;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
        const bool f = diag[c] > 0.0;
        const float ph = fminf(1.f, fmaxf(-1.f, (float)((double)phi[c] * inv3dx)));
        const float bn = f ? (float)(b[c] / rms) : 0.f;
        const float so = solid[c] < T(0) ? 1.f : 0.f;
        uint4 v0, v1 = make_uint4(0u, 0u, 0u, 0u);
        __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&v0);
        h[0] = __floats2bfloat162_rn(ph, bn);
        h[1] = __floats2bfloat162_rn(so, 0.f);
        h[2] = h[3] = __floats2bfloat162_rn(0.f, 0.f);
        uint4* out = reinterpret_cast<uint4*>(feat + c * kFeat);
        out[0] = v0;
        out[1] = v1;
        if (target) target[c] = f ? (float)((double)pressure[c] * a / rms) : 0.f;
        if (coup) {
            // the scaled operator A^ = A / a in Laplacian form: face weights w = -A(c, c+e) >= 0
            // with the +x, +y, +z neighbours and the diagonal's excess over the fluid faces,
            // delta = A(c,c) - sum of the six w (the ghost-fluid terms, >= 0), so that
            // e . A^ e = sum_faces w (e_c - e_n)^2 + sum delta e^2 stays exact under rounding
            const double ia = 1.0 / a;
            float dl = 0.f, wx = 0.f, wy = 0.f, wz = 0.f;
            if (f) {
                const int i = (int)(c % ni), j = (int)((c / ni) % nj), k = (int)(c / ((long long)ni * nj));
                double sw = -(double)ox[c] - (double)oy[c] - (double)oz[c];
                if (i > 0) sw -= (double)ox[c - 1];
                if (j > 0) sw -= (double)oy[c - ni];
                if (k > 0) sw -= (double)oz[c - (long long)ni * nj];
                dl = (float)(fmax(0.0, diag[c] - sw) * ia);
                wx = (float)(-(double)ox[c] * ia);
                wy = (float)(-(double)oy[c] * ia);
                wz = (float)(-(double)oz[c] * ia);
            }
            uint2 q;
            __nv_bfloat162* h2 = reinterpret_cast<__nv_bfloat162*>(&q);
            h2[0] = __floats2bfloat162_rn(dl, wx);
            h2[1] = __floats2bfloat162_rn(wy, wz);
            *reinterpret_cast<uint2*>(coup + c * 4) = q;
        }
        if (fluid) fluid[c] = f ? 1 : 0;
    }
}

template <typename T>
__global__ void warm_guess_kernel(long long n, const float* __restrict__ pred, const double* __restrict__ diag,
                                  const Scalars* s, T* __restrict__ pressure) {
    const double scale = s->rr / s->alpha;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x)
        pressure[c] = diag[c] > 0.0 ? (T)((double)pred[c] * scale) : T(0);
}

int blocks_for(el_ctx* ctx, long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, (long long)ctx->num_sms * 8));
}

// a grid reduction of nv values needs nblocks * nv partials: stay within the context's buffer
int reduce_blocks(el_ctx* ctx, long long n, int nv) {
    return std::max(1, std::min(blocks_for(ctx, n), (int)(ctx->max_partials / nv)));
}

}  // namespace

#define EL_API extern "C" __attribute__((visibility("default")))

EL_API int el_warmstart_features(el_ctx* ctx, int build, double dt, void* features, void* couplings, float* target,
                                 uint8_t* fluid, double* scales) {
    if (!ctx || !features) return EL_ERR_INVALID_ARGUMENT;
    DeviceGuard guard(ctx->device);
    if (guard.err != cudaSuccess) return EL_ERR_CUDA;
    if (build) {
        if (!(dt > 0)) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "warmstart_features: dt must be > 0");
        int rc = ensure_projection(ctx);
        if (rc != EL_OK) return rc;
        ctx->launches += launch_set_dt(ctx, dt);
        ctx->launches += launch_flags_build(ctx, false, true);
    } else if (!ctx->diag64) {
        return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "warmstart_features: no system built yet");
    }
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    Scalars* s2 = ctx->dscal + 2;
    const double inv3dx = 1.0 / (3.0 * ctx->dx);
    __nv_bfloat16* feat = static_cast<__nv_bfloat16*>(features);
    __nv_bfloat16* coup = static_cast<__nv_bfloat16*>(couplings);
    if (ctx->dtype == EL_F64) {
        const double* p = (const double*)ctx->field[EL_FIELD_PRESSURE];
        warm_sums_kernel<double><<<reduce_blocks(ctx, n, 4), 256, 0, ctx->stream>>>(n, ctx->diag64, ctx->rhs64, p, s2,
                                                                              ctx->partials, ctx->counter);
        warm_features_kernel<double><<<blocks_for(ctx, n), 256, 0, ctx->stream>>>(
            n, ctx->ni, ctx->nj, (const double*)ctx->field[EL_FIELD_PHI], (const double*)ctx->field[EL_FIELD_SOLID_CELL], ctx->diag64,
            (const double*)ctx->off[0], (const double*)ctx->off[1], (const double*)ctx->off[2], ctx->rhs64, p, inv3dx,
            s2, feat, coup, target, fluid);
    } else {
        const float* p = (const float*)ctx->field[EL_FIELD_PRESSURE];
        warm_sums_kernel<float><<<reduce_blocks(ctx, n, 4), 256, 0, ctx->stream>>>(n, ctx->diag64, ctx->rhs64, p, s2,
                                                                             ctx->partials, ctx->counter);
        warm_features_kernel<float><<<blocks_for(ctx, n), 256, 0, ctx->stream>>>(
            n, ctx->ni, ctx->nj, (const float*)ctx->field[EL_FIELD_PHI], (const float*)ctx->field[EL_FIELD_SOLID_CELL], ctx->diag64,
            (const float*)ctx->off[0], (const float*)ctx->off[1], (const float*)ctx->off[2], ctx->rhs64, p, inv3dx,
            s2, feat, coup, target, fluid);
    }
    ctx->launches += 2;
    int rc = check_launch(ctx, "warmstart_features");
    if (rc != EL_OK || !scales) return rc;
    Scalars h;
    EL_CUDA_TRY(ctx, cudaMemcpyAsync(&h, s2, sizeof(Scalars), cudaMemcpyDeviceToHost, ctx->stream));
    EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    scales[0] = h.rr;
    scales[1] = h.alpha;
    scales[2] = h.norm;
    return EL_OK;
}

EL_API int el_warmstart_set_guess(el_ctx* ctx, const float* pred) {
    if (!ctx || !pred) return EL_ERR_INVALID_ARGUMENT;
    DeviceGuard guard(ctx->device);
    if (guard.err != cudaSuccess) return EL_ERR_CUDA;
    if (!ctx->diag64) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "warmstart_set_guess: no system built yet");
    const long long n = (long long)ctx->ni * ctx->nj * ctx->nk;
    if (ctx->dtype == EL_F64)
        warm_guess_kernel<double><<<blocks_for(ctx, n), 256, 0, ctx->stream>>>(
            n, pred, ctx->diag64, ctx->dscal + 2, (double*)ctx->field[EL_FIELD_PRESSURE]);
    else
        warm_guess_kernel<float><<<blocks_for(ctx, n), 256, 0, ctx->stream>>>(
            n, pred, ctx->diag64, ctx->dscal + 2, (float*)ctx->field[EL_FIELD_PRESSURE]);
    ctx->launches += 1;
    return check_launch(ctx, "warmstart_set_guess");
}
