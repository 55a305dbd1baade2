// el_extrap.cu -- extrapolation (src/project/3d/fluid/extrapolation.cpp:5-51) ordered by
// distance instead of by sweeps.
//
// extrapolate() runs `layers` Jacobi layers: in layer l every cell that is not valid yet and
// has a valid cell among its 26 neighbours (valid when the layer began) takes the mean of those
// neighbours (summed in z, y, x order) and becomes valid.  By induction a cell becomes valid in
// layer l exactly when its Chebyshev (L-infinity) distance d to the initially valid cells is
// l + 1 (the grid is a box, so king-move paths stay inside it), and the neighbours it averages
// are exactly those with a smaller d.  So the result is fixed by d alone:
//
//   1. d of every cell, capped at layers + 1, by three separable passes (a cube is separable):
//      along x from the valid mask (warp ballots, bit scans), then along y and z,
//      d_xy(c) = min_t max(|t|, d_x(c + t e_y)) with |t| <= layers (four cells per 32-bit word:
//      vmaxu4 / vminu4), the z pass counting the cells of each distance;
//   2. the cells of each distance 1..layers listed (a scan of the counts, block-aggregated
//      scatter);
//   3. one launch per layer over that layer's list: the mean of the neighbours with a smaller d,
//      in the reference's z, y, x order, written in place (no cell of the layer reads another).
//
// The results are those of the reference loop bit for bit (same sums in the same order, same
// division); only cells the layers reach are touched.  Up to four fields go through each
// launch (velocity u, v, w and the level set of a step), each with its own scratch slot.
#include "el_internal.cuh"

namespace el {

namespace {

constexpr int kExMaxFields = 4;
constexpr int kDistThreads = 256;

struct ExField {
    void* g;              // the field (float or double), i-fastest n0 x n1 x n2
    uint8_t* valid;       // its valid mask (written back when write_back)
    uint8_t* da;          // distance scratch, rows padded to `pitch` bytes
    uint8_t* db;
    int* list;            // the cells of distance 1..layers, grouped by distance
    int n0, n1, n2, pitch;
    int write_back;
};

struct ExArgs {
    ExField f[kExMaxFields];
    int nf;
    int layers;
    int* counts;   // [kExMaxFields][256] cells per distance
    int* offsets;  // [kExMaxFields][256] first list entry of each distance
    int* cursors;  // [kExMaxFields][256] scatter cursors
};

__device__ __forceinline__ unsigned splat4(unsigned b) { return b * 0x01010101u; }

// ---- 1a. distance along x: one warp per row, three 32-cell chunks of ballot bits in registers
// (the window reaches 32 cells either side, enough for layers <= 31)
__global__ void __launch_bounds__(kDistThreads) ex_dist_x_kernel(const ExArgs a) {
    const ExField& F = a.f[blockIdx.y];
    const int lane = threadIdx.x & 31;
    const int row = blockIdx.x * (kDistThreads / 32) + (threadIdx.x >> 5);
    const int rows = F.n1 * F.n2;
    if (row >= rows) return;
    const uint8_t* v = F.valid + (long long)row * F.n0;
    uint8_t* out = F.da + (long long)row * F.pitch;
    const unsigned cap = (unsigned)a.layers + 1u;
    const int nch = (F.pitch + 31) / 32;  // chunks over the padded row (padding comes out capped)
    auto ballot = [&](int ch) -> unsigned {
        const int i = ch * 32 + lane;
        const bool on = ch >= 0 && i < F.n0 && v[i] != 0;
        return __ballot_sync(0xffffffffu, on);
    };
    unsigned prev = 0u, cur = ballot(0);
    for (int ch = 0; ch < nch; ++ch) {
        const unsigned next = ch + 1 < nch ? ballot(ch + 1) : 0u;
        // left: bits 0..32+lane of prev|cur (cell at 32 + lane); right: cur|next from the cell up
        const unsigned long long lo = ((unsigned long long)cur << 32) | prev;
        const unsigned long long lmask = lane == 31 ? ~0ull : ((2ull << (32 + lane)) - 1ull);
        const unsigned long long lm = lo & lmask;
        unsigned d = cap;
        if (lm) d = min(d, (unsigned)(32 + lane - (63 - __clzll((long long)lm))));
        const unsigned long long hi = (((unsigned long long)next << 32) | cur) >> lane;
        if (hi) d = min(d, (unsigned)(__ffsll((long long)hi) - 1));
        const int i = ch * 32 + lane;
        if (i < F.pitch) out[i] = (uint8_t)d;
        prev = cur;
        cur = next;
    }
}

// the same for layers > 31: each cell scans its row outwards
__global__ void __launch_bounds__(kDistThreads) ex_dist_x_scan_kernel(const ExArgs a) {
    const ExField& F = a.f[blockIdx.y];
    const long long n = (long long)F.pitch * F.n1 * F.n2;
    const int cap = a.layers + 1;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
         q += (long long)gridDim.x * blockDim.x) {
        const long long row = q / F.pitch;
        const int i = (int)(q - row * F.pitch);
        const uint8_t* v = F.valid + row * F.n0;
        int d = cap;
        for (int t = 0; t < cap; ++t) {
            if ((i - t >= 0 && i - t < F.n0 && v[i - t]) || (i + t < F.n0 && v[i + t])) {
                d = t;
                break;
            }
        }
        F.da[q] = (uint8_t)d;
    }
}

// ---- 1b. one separable pass along y (AXIS 1) or z (AXIS 2): out = min_t max(|t|, in(c + t e))
// over |t| <= layers, four cells per word.  The z pass also counts the cells of each distance.
template <int AXIS>
__global__ void __launch_bounds__(kDistThreads) ex_dist_pass_kernel(const ExArgs a) {
    const ExField& F = a.f[blockIdx.y];
    __shared__ int hist[256];
    if (AXIS == 2) {
        for (int q = threadIdx.x; q < 256; q += blockDim.x) hist[q] = 0;
        __syncthreads();
    }
    const int words = F.pitch / 4;
    const long long nw = (long long)words * F.n1 * F.n2;
    const int m_extent = AXIS == 1 ? F.n1 : F.n2;
    const long long stride = AXIS == 1 ? words : (long long)words * F.n1;  // in words
    const unsigned* in = reinterpret_cast<const unsigned*>(AXIS == 1 ? F.da : F.db);
    unsigned* out = reinterpret_cast<unsigned*>(AXIS == 1 ? F.db : F.da);
    const int L = a.layers;
    const unsigned cap4 = splat4((unsigned)L + 1u);
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nw;
         q += (long long)gridDim.x * blockDim.x) {
        const long long line = q / words;  // (j, k) of the word
        const int m = AXIS == 1 ? (int)(line % F.n1) : (int)(line / F.n1);
        unsigned best = in[q];
        for (int t = 1; t <= L; ++t) {
            const unsigned tt = splat4((unsigned)t);
            if (m - t >= 0) best = __vminu4(best, __vmaxu4(in[q - t * stride], tt));
            if (m + t < m_extent) best = __vminu4(best, __vmaxu4(in[q + t * stride], tt));
        }
        best = __vminu4(best, cap4);
        out[q] = best;
        if (AXIS == 2) {
            const int i0 = (int)(q - line * words) * 4;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const unsigned d = (best >> (8 * b)) & 0xffu;
                if (i0 + b < F.n0 && d >= 1u && (int)d <= L) atomicAdd(&hist[d], 1);
            }
        }
    }
    if (AXIS == 2) {
        __syncthreads();
        for (int q = threadIdx.x; q <= L && q < 256; q += blockDim.x)
            if (hist[q]) atomicAdd(&a.counts[blockIdx.y * 256 + q], hist[q]);
    }
}

// The same pass for layers <= kTileMaxLayers through shared memory: a CTA takes 32 words (128
// cells along x) by kTileRows positions along the pass axis at one position of the third axis,
// stages its input with the halo of `layers` positions either side once, and reads the
// candidates there (each input word is read from memory (kTileRows + 2 layers) / kTileRows
// times instead of 2 layers + 1).  A tile whose input is all at the cap writes the cap.
constexpr int kTileRows = 64;
constexpr int kTileMaxLayers = 31;

// two 16-bit lanes: max / min (native on this GPU, unlike the byte forms), and the byte word
// of four distances split into two such pairs and joined back
__device__ __forceinline__ unsigned max_u16x2(unsigned a, unsigned b) {
    unsigned r;
    asm("max.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}
__device__ __forceinline__ unsigned min_u16x2(unsigned a, unsigned b) {
    unsigned r;
    asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}

template <int AXIS>
__global__ void __launch_bounds__(kDistThreads) ex_dist_tile_kernel(const ExArgs a, int max_other) {
    extern __shared__ uint2 tile[];  // [kTileRows + 2 L][32]: cells {0, 1} and {2, 3} of a word
    __shared__ int hist[kTileMaxLayers + 2];
    const int f = blockIdx.z / max_other, o = blockIdx.z - f * max_other;
    if (f >= a.nf) return;
    const ExField& F = a.f[f];
    const int words = F.pitch / 4;
    const int extent = AXIS == 1 ? F.n1 : F.n2;
    const int other = AXIS == 1 ? F.n2 : F.n1;
    const int w0 = blockIdx.x * 32, m0 = blockIdx.y * kTileRows;
    if (o >= other || w0 >= words || m0 >= extent) return;  // uniform over the CTA
    const int L = a.layers;
    const unsigned cap4 = splat4((unsigned)L + 1u);
    const unsigned cap2 = ((unsigned)L + 1u) * 0x00010001u;
    // word (w, m) of this field: AXIS 1 (y): m = j, o = k; AXIS 2 (z): m = k, o = j
    auto at = [&](int w, int m) -> long long {
        return AXIS == 1 ? ((long long)o * F.n1 + m) * words + w : ((long long)m * F.n1 + o) * words + w;
    };
    const unsigned* in = reinterpret_cast<const unsigned*>(AXIS == 1 ? F.da : F.db);
    unsigned* out = reinterpret_cast<unsigned*>(AXIS == 1 ? F.db : F.da);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int rows = kTileRows + 2 * L;
    int below = 0;
    for (int r = warp; r < rows; r += kDistThreads / 32) {
        const int m = m0 - L + r, w = w0 + lane;
        const unsigned v = (m >= 0 && m < extent && w < words) ? in[at(w, m)] : cap4;
        tile[r * 32 + lane] = make_uint2(__byte_perm(v, 0u, 0x4140), __byte_perm(v, 0u, 0x4342));
        below |= v != cap4;
    }
    if (AXIS == 2)
        for (int q = threadIdx.x; q <= L; q += blockDim.x) hist[q] = 0;
    const bool any = __syncthreads_or(below) != 0;
    const int w = w0 + lane;
    for (int r = warp; r < kTileRows; r += kDistThreads / 32) {
        const int m = m0 + r;
        if (m >= extent || w >= words) continue;
        unsigned best = cap4;
        if (any) {
            uint2 b = tile[(r + L) * 32 + lane];
            for (int t = 1; t <= L; ++t) {
                const unsigned tt = (unsigned)t * 0x00010001u;
                const uint2 lo = tile[(r + L - t) * 32 + lane], hi = tile[(r + L + t) * 32 + lane];
                b.x = min_u16x2(b.x, max_u16x2(min_u16x2(lo.x, hi.x), tt));
                b.y = min_u16x2(b.y, max_u16x2(min_u16x2(lo.y, hi.y), tt));
            }
            b.x = min_u16x2(b.x, cap2);
            b.y = min_u16x2(b.y, cap2);
            best = __byte_perm(b.x, b.y, 0x6420);
        }
        out[at(w, m)] = best;
        if (AXIS == 2 && any) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const unsigned d = (best >> (8 * q)) & 0xffu;
                if (w * 4 + q < F.n0 && d >= 1u && (int)d <= L) atomicAdd(&hist[d], 1);
            }
        }
    }
    if (AXIS == 2) {
        __syncthreads();
        for (int q = threadIdx.x; q <= L; q += blockDim.x)
            if (q >= 1 && hist[q]) atomicAdd(&a.counts[f * 256 + q], hist[q]);
    }
}

// ---- 2. list offsets per field and distance (one block)
__global__ void ex_offsets_kernel(const ExArgs a) {
    if (threadIdx.x != 0) return;
    for (int f = 0; f < a.nf; ++f) {
        int run = 0;
        for (int d = 1; d <= a.layers; ++d) {
            a.offsets[f * 256 + d] = run;
            a.cursors[f * 256 + d] = run;
            run += a.counts[f * 256 + d];
        }
    }
}

// block-aggregated scatter of the cells of distance 1..layers into their distance's range: a
// round takes kScatterWords words per thread; words with no cell in 1..layers (the valid region,
// and the cells beyond reach) only cost their load
constexpr int kScatterWords = 4;

__global__ void __launch_bounds__(kDistThreads) ex_scatter_kernel(const ExArgs a) {
    const ExField& F = a.f[blockIdx.y];
    __shared__ int bcount[256], bbase[256];
    const int L = a.layers;
    const int words = F.pitch / 4;
    const long long nw = (long long)words * F.n1 * F.n2;
    const unsigned* dist = reinterpret_cast<const unsigned*>(F.da);
    const long long per_round = (long long)blockDim.x * kScatterWords;
    // the block's threads share `base`, so the barriers below are uniform within the block
    for (long long base = (long long)blockIdx.x * per_round; base < nw; base += (long long)gridDim.x * per_round) {
        for (int q = threadIdx.x; q <= L; q += blockDim.x) bcount[q] = 0;
        __syncthreads();
        unsigned wv[kScatterWords];
        unsigned short rank[kScatterWords][4];
#pragma unroll
        for (int u = 0; u < kScatterWords; ++u) {
            const long long q = base + threadIdx.x + (long long)u * blockDim.x;
            wv[u] = 0u;  // distance 0 everywhere: nothing to list
            if (q < nw) {
                wv[u] = dist[q];
                const int i0 = (int)(q % words) * 4;
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    const int d = (int)((wv[u] >> (8 * b)) & 0xffu);
                    rank[u][b] = 0;
                    if (i0 + b < F.n0 && d >= 1 && d <= L) rank[u][b] = (unsigned short)atomicAdd(&bcount[d], 1);
                }
            }
        }
        __syncthreads();
        for (int d = threadIdx.x; d <= L; d += blockDim.x)
            if (d >= 1 && bcount[d]) bbase[d] = atomicAdd(&a.cursors[blockIdx.y * 256 + d], bcount[d]);
        __syncthreads();
#pragma unroll
        for (int u = 0; u < kScatterWords; ++u) {
            const long long q = base + threadIdx.x + (long long)u * blockDim.x;
            if (q >= nw) continue;
            const long long line = q / words;
            const int i0 = (int)(q - line * words) * 4;
            const long long cell0 = line * F.n0 + i0;  // (j, k) row start + i
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int d = (int)((wv[u] >> (8 * b)) & 0xffu);
                if (i0 + b < F.n0 && d >= 1 && d <= L &&
                    EL_IN(bbase[d] + rank[u][b], (long long)F.n0 * F.n1 * F.n2, 20))
                    F.list[bbase[d] + rank[u][b]] = (int)(cell0 + b);
            }
        }
        __syncthreads();
    }
}

// ---- 3. one layer: every cell of distance `dist` takes the mean of its neighbours of smaller
// distance, summed in z, y, x order (extrapolation.cpp:24-33)
__device__ __forceinline__ float ex_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double ex_add(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
__global__ void __launch_bounds__(kDistThreads) ex_layer_kernel(const ExArgs a, int dist) {
    int total = 0;
    int start[kExMaxFields + 1];
    for (int f = 0; f < a.nf; ++f) {
        start[f] = total;
        total += a.counts[f * 256 + dist];
    }
    start[a.nf] = total;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
        int f = 0;
        while (f + 1 < a.nf && q >= start[f + 1]) ++f;
        const ExField& F = a.f[f];
        const int li = a.offsets[f * 256 + dist] + (q - start[f]);
        if (!EL_IN(li, (long long)F.n0 * F.n1 * F.n2, 21)) continue;
        const int c = F.list[li];
        if (!EL_IN(c, (long long)F.n0 * F.n1 * F.n2, 22)) continue;
        const int i = c % F.n0, r = c / F.n0;
        const int j = r % F.n1, k = r / F.n1;
        T* g = static_cast<T*>(F.g);
        T sum = T(0);
        int count = 0;
#pragma unroll
        for (int dk = -1; dk <= 1; ++dk) {
            const int z = k + dk;
            if (z < 0 || z >= F.n2) continue;
#pragma unroll
            for (int dj = -1; dj <= 1; ++dj) {
                const int y = j + dj;
                if (y < 0 || y >= F.n1) continue;
                const uint8_t* drow = F.da + ((long long)z * F.n1 + y) * F.pitch;
                const T* grow = g + ((long long)z * F.n1 + y) * F.n0;
#pragma unroll
                for (int di = -1; di <= 1; ++di) {
                    const int x = i + di;
                    if (x < 0 || x >= F.n0) continue;
                    if ((int)drow[x] < dist) {
                        sum = ex_add(sum, grow[x]);
                        ++count;
                    }
                }
            }
        }
        g[c] = sum / (T)count;  // count >= 1: a neighbour has distance dist - 1
        if (F.write_back) F.valid[c] = 1;
    }
}

}  // namespace

// Scratch of one field slot: two distance buffers with padded rows and the distance lists.
static int ensure_ex_slot(el_ctx* ctx, int slot) {
    if (ctx->ex_da[slot]) return EL_OK;
    ctx->ex_da[slot] = (uint8_t*)ctx_alloc(ctx, ctx->ex_dist_bytes);
    ctx->ex_db[slot] = (uint8_t*)ctx_alloc(ctx, ctx->ex_dist_bytes);
    ctx->ex_list[slot] = (int*)ctx_alloc(ctx, ctx->ex_list_bytes);
    if (!ctx->ex_da[slot] || !ctx->ex_db[slot] || !ctx->ex_list[slot])
        return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "extrapolation scratch");
    return EL_OK;
}

// Allocates the scratch of `nfields` slots (outside any stream capture).
int ensure_extrapolation(el_ctx* ctx, int nfields) {
    if (!ctx->ex_counts) {
        ctx->ex_counts = (int*)ctx_alloc(ctx, 3 * kExMaxFields * 256 * sizeof(int));
        if (!ctx->ex_counts) return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "extrapolation counts");
    }
    for (int q = 0; q < nfields && q < kExMaxFields; ++q) {
        const int rc = ensure_ex_slot(ctx, q);
        if (rc != EL_OK) return rc;
    }
    return EL_OK;
}

// Extrapolates up to four fields together; fields[q] is a field id, valid[q] its mask and
// write_back[q] whether the mask is updated (extrapolate) or left alone (extrapolate_const).
// Returns the kernels launched.
int launch_extrapolate_fields(el_ctx* ctx, int nf, const int* fields, uint8_t* const* valid, const bool* write_back,
                              int layers) {
    if (nf < 1 || layers < 1) return 0;
    ExArgs a{};
    a.nf = nf;
    a.layers = std::min(layers, 254);  // distances are bytes; layers + 1 is the cap
    a.counts = ctx->ex_counts;
    a.offsets = ctx->ex_counts + kExMaxFields * 256;
    a.cursors = ctx->ex_counts + 2 * kExMaxFields * 256;
    long long max_words = 0, max_rows = 0;
    for (int q = 0; q < nf; ++q) {
        ExField& F = a.f[q];
        int n0, n1, n2;
        field_dims(ctx, fields[q], n0, n1, n2);
        F.g = ctx->field[fields[q]];
        F.valid = valid[q];
        F.da = ctx->ex_da[q];
        F.db = ctx->ex_db[q];
        F.list = ctx->ex_list[q];
        F.n0 = n0;
        F.n1 = n1;
        F.n2 = n2;
        F.pitch = (n0 + 15) & ~15;
        F.write_back = write_back[q] ? 1 : 0;
        max_words = std::max(max_words, (long long)(F.pitch / 4) * n1 * n2);
        max_rows = std::max(max_rows, (long long)n1 * n2);
    }
    int n = 0;
    cudaMemsetAsync(ctx->ex_counts, 0, kExMaxFields * 256 * sizeof(int), ctx->stream);
    const int wide = ctx->num_sms * 8;  // resident 256-thread blocks of the streaming passes
    if (a.layers <= 31) {
        const dim3 grid((unsigned)((max_rows + kDistThreads / 32 - 1) / (kDistThreads / 32)), nf);
        ex_dist_x_kernel<<<grid, kDistThreads, 0, ctx->stream>>>(a);
    } else {
        ex_dist_x_scan_kernel<<<dim3(wide, nf), kDistThreads, 0, ctx->stream>>>(a);
    }
    const unsigned pass_blocks = (unsigned)std::min<long long>(wide, (max_words + kDistThreads - 1) / kDistThreads);
    if (a.layers <= kTileMaxLayers) {
        int max_words_row = 0, max_n1 = 0, max_n2 = 0;
        for (int q = 0; q < nf; ++q) {
            max_words_row = std::max(max_words_row, a.f[q].pitch / 4);
            max_n1 = std::max(max_n1, a.f[q].n1);
            max_n2 = std::max(max_n2, a.f[q].n2);
        }
        const int smem = (kTileRows + 2 * a.layers) * 32 * (int)sizeof(uint2);
        const unsigned gx = (unsigned)((max_words_row + 31) / 32);
        // y: tiles along j at each k; z: tiles along k at each j
        ex_dist_tile_kernel<1><<<dim3(gx, (max_n1 + kTileRows - 1) / kTileRows, (unsigned)(nf * max_n2)),
                                 kDistThreads, smem, ctx->stream>>>(a, max_n2);
        ex_dist_tile_kernel<2><<<dim3(gx, (max_n2 + kTileRows - 1) / kTileRows, (unsigned)(nf * max_n1)),
                                 kDistThreads, smem, ctx->stream>>>(a, max_n1);
    } else {
        ex_dist_pass_kernel<1><<<dim3(pass_blocks, nf), kDistThreads, 0, ctx->stream>>>(a);
        ex_dist_pass_kernel<2><<<dim3(pass_blocks, nf), kDistThreads, 0, ctx->stream>>>(a);
    }
    ex_offsets_kernel<<<1, 32, 0, ctx->stream>>>(a);
    const unsigned scatter_blocks =
        (unsigned)std::min<long long>(wide, (max_words + kDistThreads * kScatterWords - 1) / (kDistThreads * kScatterWords));
    ex_scatter_kernel<<<dim3(scatter_blocks, nf), kDistThreads, 0, ctx->stream>>>(a);
    n += 5;
    const int layer_blocks = ctx->num_sms * std::max(1, ctx->extrap_per_sm);
    for (int d = 1; d <= a.layers; ++d) {
        if (ctx->dtype == EL_F64)
            ex_layer_kernel<double><<<layer_blocks, kDistThreads, 0, ctx->stream>>>(a, d);
        else
            ex_layer_kernel<float><<<layer_blocks, kDistThreads, 0, ctx->stream>>>(a, d);
        ++n;
    }
    return n;
}

EL_CHECK_EXPORT(extrap)

}  // namespace el
