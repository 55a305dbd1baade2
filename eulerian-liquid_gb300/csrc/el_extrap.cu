// el_extrap.cu -- extrapolation (src/project/3d/fluid/extrapolation.cpp:5-51): the reference's
// layer loop over a bitmask of the valid cells.
//
// extrapolate() runs `layers` Jacobi layers: in layer l every cell that is not valid yet and
// has a valid cell among its 26 neighbours (valid when the layer began) takes the mean of those
// neighbours (summed in z, y, x order) and becomes valid.  Here the valid set S of a field is a
// bitmask, one bit per cell and 32 cells of a row per word, with a zero word before and after
// every row and zero rows and planes around the grid, so that a neighbour outside the grid is a
// zero bit and needs no bounds test.  Per layer:
//   1. ex_dilate_kernel: S' = S dilated by the 3 x 3 x 3 cube -- an OR over z, then over y,
//      through shared memory, then along x by shifts that take the neighbouring words' edge
//      bits -- is written to the other buffer, and the cells of S' \ S (this layer's) are listed
//      per field (block-aggregated).  A tile with no set bit around it, or with every cell set,
//      has none and is copied.
//   2. ex_average_kernel: every listed cell takes the mean of its neighbours in S (the bits of
//      the layer before), summed in z, y, x order, and is marked valid (extrapolate) or not
//      (extrapolate_const).  No listed cell reads another.
// The results are those of the reference loop bit for bit: the same cells, the same sums in the
// same order and the same division.  Up to four fields go through each launch (velocity u, v,
// w and the level set of a step), each with its own scratch slot.
#include "el_internal.cuh"

namespace el {

namespace {

constexpr int kExMaxFields = 4;
constexpr int kExThreads = 256;
// the dilation tile: 8 words (256 cells) of a row x 32 rows x 8 planes, and its one-word /
// one-row / one-plane halo
constexpr int kTW = 8, kTY = 32, kTZ = 8;
constexpr int kHW = kTW + 2, kHY = kTY + 2, kHZ = kTZ + 2;
constexpr int kTileWords = kTW * kTY * kTZ;
constexpr int kPerThread = kTileWords / kExThreads;
constexpr int kHaloWords = kHW * kHY * kHZ;
constexpr int kHaloLoads = (kHaloWords + kExThreads - 1) / kExThreads;
static_assert(kTileWords % kExThreads == 0, "whole outputs per thread");

// what S holds on a dilation tile
enum : uint8_t { kTileZero = 0, kTileMixed = 1, kTileFull = 2 };

struct ExField {
    void* g;            // the field (float or double), i-fastest n0 x n1 x n2
    uint8_t* valid;     // its valid mask (written for the layers' cells when write_back)
    unsigned* s;        // the valid set before the layer: padded bitmask
    unsigned* s_next;   // and after it
    int* list;          // the layer's cells (linear indices)
    const uint8_t* st;  // per dilation tile: S before the layer (kTile*)
    uint8_t* st_next;   // and after it
    const uint8_t* ch;  // per dilation tile: the layer before changed S there
    uint8_t* ch_next;   // this layer does
    int n0, n1, n2;
    int rw;             // words per row, ceil(n0 / 32); a padded row holds rw + 2
    int ntx, nty, ntz;  // dilation tiles along x, y, z
    int write_back;
};

struct ExArgs {
    ExField f[kExMaxFields];
    int nf;
    int* counts;       // this layer's cells per field
    int* counts_next;  // the next layer's, cleared by ex_average_kernel
};

// word (wp, yp, zp) of a padded bitmask: wp = word + 1, yp = y + 1, zp = z + 1
__device__ __forceinline__ long long pad_at(const ExField& F, int wp, int yp, int zp) {
    return wp + (long long)(F.rw + 2) * (yp + (long long)(F.n1 + 2) * zp);
}

// the bits of word w of a row that are cells of the grid
__device__ __forceinline__ unsigned row_mask(int n0, int w) {
    const int rem = n0 - 32 * w;
    return rem >= 32 ? 0xffffffffu : ((1u << rem) - 1u);
}

// ---- the valid masks as bitmasks, in two passes over all fields: the mask's bytes as a flat
// bit stream (32 cells per word, 16-byte loads), then that stream cut into the padded rows.
// The flat words go to the field's list buffer, which the first layer overwrites later.

// bit q of the result: byte q of x is not zero
__device__ __forceinline__ unsigned nonzero_bytes(unsigned x) {
    const unsigned h = (((x & 0x7f7f7f7fu) + 0x7f7f7f7fu) | x) & 0x80808080u;
    return ((h >> 7) & 1u) | ((h >> 14) & 2u) | ((h >> 21) & 4u) | ((h >> 28) & 8u);
}

__global__ void __launch_bounds__(kExThreads) ex_flat_kernel(const ExArgs a) {
    const ExField& F = a.f[blockIdx.y];
    const long long n = (long long)F.n0 * F.n1 * F.n2;
    const long long words = (n + 31) / 32;
    unsigned* flat = reinterpret_cast<unsigned*>(F.list);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < words;
         t += (long long)gridDim.x * blockDim.x) {
        unsigned word = 0u;
        if (32 * t + 32 <= n) {
            const uint4* v4 = reinterpret_cast<const uint4*>(F.valid) + 2 * t;
            const uint4 p = v4[0], q = v4[1];
            word = nonzero_bytes(p.x) | (nonzero_bytes(p.y) << 4) | (nonzero_bytes(p.z) << 8) |
                   (nonzero_bytes(p.w) << 12) | (nonzero_bytes(q.x) << 16) | (nonzero_bytes(q.y) << 20) |
                   (nonzero_bytes(q.z) << 24) | (nonzero_bytes(q.w) << 28);
        } else {
            for (int b = 0; 32 * t + b < n; ++b) word |= (F.valid[32 * t + b] != 0 ? 1u : 0u) << b;
        }
        flat[t] = word;
    }
}

// every word of the first buffer (the padding as zeros), and the padding of the second, so that
// a slot that held another field's layout before is fully defined
__global__ void __launch_bounds__(kExThreads) ex_rows_kernel(const ExArgs a) {
    const ExField& F = a.f[blockIdx.y];
    const int pw = F.rw + 2;
    const long long total = (long long)pw * (F.n1 + 2) * (F.n2 + 2);
    const long long n = (long long)F.n0 * F.n1 * F.n2;
    const long long words = (n + 31) / 32;
    const unsigned* flat = reinterpret_cast<const unsigned*>(F.list);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int wp = (int)(t % pw);
        const long long r = t / pw;
        const int yp = (int)(r % (F.n1 + 2)), zp = (int)(r / (F.n1 + 2));
        if (wp < 1 || wp > F.rw || yp < 1 || yp > F.n1 || zp < 1 || zp > F.n2) {
            F.s[t] = 0u;
            F.s_next[t] = 0u;
            continue;
        }
        // cells 32 (wp - 1) .. + 31 of row (yp - 1, zp - 1) in the flat stream
        const long long c0 = 32ll * (wp - 1) + (long long)F.n0 * ((yp - 1) + (long long)F.n1 * (zp - 1));
        const long long lo = c0 >> 5;
        const unsigned sh = (unsigned)(c0 & 31);
        const unsigned a0 = flat[lo], a1 = lo + 1 < words ? flat[lo + 1] : 0u;
        F.s[t] = __funnelshift_r(a0, a1, sh) & row_mask(F.n0, wp - 1);
    }
}

// ---- 1. one layer's dilation over a tile of one field, and the list of the layer's cells
__global__ void __launch_bounds__(kExThreads, 4) ex_dilate_kernel(const ExArgs a, int ztiles) {
    __shared__ unsigned sm[kHZ][kHY][kHW];  // S over the tile and its halo
    __shared__ unsigned zo[kTZ][kHY][kHW];  // OR over z
    __shared__ unsigned yo[kTZ][kTY][kHW];  // then over y
    __shared__ int wtot[kExThreads / 32];
    __shared__ int base;
    const int f = blockIdx.z / ztiles, zt = blockIdx.z - f * ztiles;
    if (f >= a.nf) return;
    const ExField& F = a.f[f];
    const int w0 = blockIdx.x * kTW, y0 = blockIdx.y * kTY, z0 = zt * kTZ;
    if (w0 >= F.rw || y0 >= F.n1 || z0 >= F.n2) return;  // uniform over the CTA
    const int tid = threadIdx.x;
    const int tile = blockIdx.x + F.ntx * (blockIdx.y + F.nty * zt);
    // output m of the thread: word (w0 + tw, y0 + ty, z0 + tz) of the field
    auto out_at = [&](int m, int& tw, int& ty, int& tz) -> bool {
        const int e = tid + kExThreads * m;
        tw = e % kTW;
        ty = (e / kTW) % kTY;
        tz = e / (kTW * kTY);
        return w0 + tw < F.rw && y0 + ty < F.n1 && z0 + tz < F.n2;
    };
    // a tile that S fills, or that S leaves empty with its neighbour tiles, has no cell of this
    // layer and is not staged: S' = S there, and the buffer S' goes to holds S of two layers
    // back, so its words are copied only if the layer before changed them
    const uint8_t own = F.st[tile];
    int busy = 0;
    if (tid < 27) {
        const int nx = (int)blockIdx.x + tid % 3 - 1, ny = (int)blockIdx.y + (tid / 3) % 3 - 1, nz = zt + tid / 9 - 1;
        if (nx >= 0 && nx < F.ntx && ny >= 0 && ny < F.nty && nz >= 0 && nz < F.ntz)
            busy = F.st[nx + F.ntx * (ny + F.nty * nz)] != kTileZero;
    }
    if (own == kTileFull || !__syncthreads_or(busy)) {
        if (F.ch[tile]) {
#pragma unroll
            for (int m = 0; m < kPerThread; ++m) {
                int tw, ty, tz;
                if (out_at(m, tw, ty, tz)) {
                    const long long q = pad_at(F, w0 + tw + 1, y0 + ty + 1, z0 + tz + 1);
                    F.s_next[q] = F.s[q];
                }
            }
        }
        if (tid == 0) {
            F.st_next[tile] = own;
            F.ch_next[tile] = 0;
        }
        return;
    }
    const int pw = F.rw + 2, py = F.n1 + 2, pz = F.n2 + 2;
    // padded coordinates of halo entry (hw, hy, hz): (w0 + hw, y0 + hy, z0 + hz); the entry's
    // place in sm is its index e.  Every load of the thread is issued before the first store.
    unsigned hv[kHaloLoads];
#pragma unroll
    for (int u = 0; u < kHaloLoads; ++u) {
        const int e = tid + kExThreads * u;
        const int hw = e % kHW, r = e / kHW, hy = r % kHY, hz = r / kHY;
        const int wp = w0 + hw, yp = y0 + hy, zp = z0 + hz;
        hv[u] = 0u;
        if (e < kHaloWords && wp < pw && yp < py && zp < pz) hv[u] = F.s[pad_at(F, wp, yp, zp)];
    }
    unsigned* smf = &sm[0][0][0];
    int any = 0;
#pragma unroll
    for (int u = 0; u < kHaloLoads; ++u) {
        const int e = tid + kExThreads * u;
        if (e < kHaloWords) {
            smf[e] = hv[u];
            any |= hv[u] != 0u;
        }
    }
    // a tile with no set bit around it, or with every cell set, has no cell of this layer: S' = S
    bool skip = !__syncthreads_or(any);
    int full = 1;
#pragma unroll
    for (int m = 0; m < kPerThread; ++m) {
        int tw, ty, tz;
        if (out_at(m, tw, ty, tz) && sm[tz + 1][ty + 1][tw + 1] != row_mask(F.n0, w0 + tw)) full = 0;
    }
    const bool tile_full = __syncthreads_and(full) != 0;
    if (skip || tile_full) {
        int zero = 1;
#pragma unroll
        for (int m = 0; m < kPerThread; ++m) {
            int tw, ty, tz;
            if (out_at(m, tw, ty, tz)) {
                const unsigned v = sm[tz + 1][ty + 1][tw + 1];
                F.s_next[pad_at(F, w0 + tw + 1, y0 + ty + 1, z0 + tz + 1)] = v;
                zero &= v == 0u;
            }
        }
        const bool tile_zero = __syncthreads_and(zero) != 0;
        if (tid == 0) {
            F.st_next[tile] = tile_full ? kTileFull : (tile_zero ? kTileZero : kTileMixed);
            F.ch_next[tile] = 0;
        }
        return;
    }
    for (int e = tid; e < kTZ * kHY * kHW; e += kExThreads) {
        const int hw = e % kHW, r = e / kHW, hy = r % kHY, tz = r / kHY;
        zo[tz][hy][hw] = sm[tz][hy][hw] | sm[tz + 1][hy][hw] | sm[tz + 2][hy][hw];
    }
    __syncthreads();
    for (int e = tid; e < kTZ * kTY * kHW; e += kExThreads) {
        const int hw = e % kHW, r = e / kHW, ty = r % kTY, tz = r / kTY;
        yo[tz][ty][hw] = zo[tz][ty][hw] | zo[tz][ty + 1][hw] | zo[tz][ty + 2][hw];
    }
    __syncthreads();
    // the layer's cells of output m: the dilation along x (a cell's left and right neighbours,
    // across the word's edges), less S, inside the row
    auto new_bits = [&](int tw, int ty, int tz) -> unsigned {
        const unsigned c0 = yo[tz][ty][tw + 1], cm = yo[tz][ty][tw], cp = yo[tz][ty][tw + 2];
        const unsigned dil = c0 | (c0 << 1) | (cm >> 31) | (c0 >> 1) | (cp << 31);
        return dil & ~sm[tz + 1][ty + 1][tw + 1] & row_mask(F.n0, w0 + tw);
    };
    int cnt = 0, zero = 1;
    full = 1;
#pragma unroll
    for (int m = 0; m < kPerThread; ++m) {
        int tw, ty, tz;
        if (!out_at(m, tw, ty, tz)) continue;
        const unsigned nw = new_bits(tw, ty, tz);
        const unsigned sn = sm[tz + 1][ty + 1][tw + 1] | nw;
        F.s_next[pad_at(F, w0 + tw + 1, y0 + ty + 1, z0 + tz + 1)] = sn;
        cnt += __popc(nw);
        zero &= sn == 0u;
        full &= sn == row_mask(F.n0, w0 + tw);
    }
    // the CTA's cells go to one range of the field's list: a scan of the threads' counts
    const int lane = tid & 31, warp = tid >> 5;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wtot[warp] = incl;
    const bool next_zero = __syncthreads_and(zero) != 0;
    const bool next_full = __syncthreads_and(full) != 0;
    if (tid == 0) {
        int run = 0;
        for (int q = 0; q < kExThreads / 32; ++q) {
            const int t = wtot[q];
            wtot[q] = run;
            run += t;
        }
        base = run ? atomicAdd(&a.counts[f], run) : 0;
        F.st_next[tile] = next_full ? kTileFull : (next_zero ? kTileZero : kTileMixed);
        F.ch_next[tile] = run ? 1 : 0;
    }
    __syncthreads();
    int off = base + wtot[warp] + incl - cnt;
    const long long ncell = (long long)F.n0 * F.n1 * F.n2;
    (void)ncell;  // read by the index checks of the debug build
#pragma unroll
    for (int m = 0; m < kPerThread; ++m) {
        int tw, ty, tz;
        if (!out_at(m, tw, ty, tz)) continue;
        unsigned bits = new_bits(tw, ty, tz);
        const long long row0 = (long long)F.n0 * ((y0 + ty) + (long long)F.n1 * (z0 + tz)) + 32 * (w0 + tw);
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1;
            if (EL_IN(off, ncell, 20)) F.list[off] = (int)(row0 + b);
            ++off;
        }
    }
}

// ---- 2. the layer's cells: the mean of the neighbours in S, summed in z, y, x order
// (extrapolation.cpp:24-33)
__device__ __forceinline__ float ex_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double ex_add(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
__global__ void __launch_bounds__(kExThreads) ex_average_kernel(const ExArgs a) {
    int total = 0;
    int start[kExMaxFields + 1];
    for (int f = 0; f < a.nf; ++f) {
        start[f] = total;
        total += a.counts[f];
    }
    start[a.nf] = total;
    // the next layer's counts start from zero (its dilation runs after this kernel)
    if (blockIdx.x == 0 && threadIdx.x < kExMaxFields) a.counts_next[threadIdx.x] = 0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
        int f = 0;
        while (f + 1 < a.nf && q >= start[f + 1]) ++f;
        const ExField& F = a.f[f];
        const long long ncell = (long long)F.n0 * F.n1 * F.n2;
        (void)ncell;
        const int li = q - start[f];
        if (!EL_IN(li, ncell, 21)) continue;
        const int c = F.list[li];
        if (!EL_IN(c, ncell, 22)) continue;
        const int x = c % F.n0, r = c / F.n0;
        const int y = r % F.n1, z = r / F.n1;
        // cells x - 1, x, x + 1 of a padded row: bits 0..2 of the window from the word holding
        // cell x - 1 (padded word (x - 1 + 32) / 32)
        const int lo = (x + 31) >> 5, sh = (x + 31) & 31;
        T* g = static_cast<T*>(F.g);
        T sum = T(0);
        int count = 0;
#pragma unroll
        for (int dz = -1; dz <= 1; ++dz) {
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy) {
                const unsigned* row = F.s + pad_at(F, 0, y + 1 + dy, z + 1 + dz);
                unsigned win = row[lo] >> sh;
                if (sh > 29) win |= row[lo + 1] << (32 - sh);  // the cells straddle two words
                if (!(win & 7u)) continue;
                const T* grow = g + (long long)F.n0 * ((y + dy) + (long long)F.n1 * (z + dz));
#pragma unroll
                for (int dx = -1; dx <= 1; ++dx) {
                    if (win & (1u << (dx + 1))) {
                        sum = ex_add(sum, grow[x + dx]);
                        ++count;
                    }
                }
            }
        }
        g[c] = sum / (T)count;  // count >= 1: the cell has a neighbour in S
        if (F.write_back) F.valid[c] = 1;
    }
}

}  // namespace

// bytes of one padded bitmask of an n0 x n1 x n2 field
size_t extrapolation_bits_bytes(int n0, int n1, int n2) {
    return (size_t)((n0 + 31) / 32 + 2) * (size_t)(n1 + 2) * (size_t)(n2 + 2) * sizeof(unsigned);
}

// dilation tiles over an n0 x n1 x n2 field
size_t extrapolation_tiles(int n0, int n1, int n2) {
    return (size_t)(((n0 + 31) / 32 + kTW - 1) / kTW) * (size_t)((n1 + kTY - 1) / kTY) *
           (size_t)((n2 + kTZ - 1) / kTZ);
}

// Scratch of one field slot: two padded bitmasks, the list of a layer's cells and four arrays
// of tile states (S on each tile after an even / odd layer, and whether that layer changed it).
static int ensure_ex_slot(el_ctx* ctx, int slot) {
    if (ctx->ex_bits[slot][0]) return EL_OK;
    ctx->ex_bits[slot][0] = (unsigned*)ctx_alloc(ctx, ctx->ex_bits_bytes);
    ctx->ex_bits[slot][1] = (unsigned*)ctx_alloc(ctx, ctx->ex_bits_bytes);
    ctx->ex_list[slot] = (int*)ctx_alloc(ctx, ctx->ex_list_bytes);
    ctx->ex_tiles[slot] = (uint8_t*)ctx_alloc(ctx, 4 * ctx->ex_tile_count);
    if (!ctx->ex_bits[slot][0] || !ctx->ex_bits[slot][1] || !ctx->ex_list[slot] || !ctx->ex_tiles[slot])
        return set_error(ctx, EL_ERR_OUT_OF_MEMORY, "extrapolation scratch");
    return EL_OK;
}

// Allocates the scratch of `nfields` slots (outside any stream capture).
int ensure_extrapolation(el_ctx* ctx, int nfields) {
    if (!ctx->ex_counts) {
        ctx->ex_counts = (int*)ctx_alloc(ctx, 2 * kExMaxFields * sizeof(int));
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
    int max_rw = 0, max_n1 = 0, max_n2 = 0;
    long long max_cells = 0, max_padded = 0;
    for (int q = 0; q < nf; ++q) {
        ExField& F = a.f[q];
        int n0, n1, n2;
        field_dims(ctx, fields[q], n0, n1, n2);
        F.g = ctx->field[fields[q]];
        F.valid = valid[q];
        F.list = ctx->ex_list[q];
        F.n0 = n0;
        F.n1 = n1;
        F.n2 = n2;
        F.rw = (n0 + 31) / 32;
        F.ntx = (F.rw + kTW - 1) / kTW;
        F.nty = (n1 + kTY - 1) / kTY;
        F.ntz = (n2 + kTZ - 1) / kTZ;
        F.write_back = write_back[q] ? 1 : 0;
        // the tile states of S_0: unknown (mixed) and changed, so that the first layer stages
        // every tile
        cudaMemsetAsync(ctx->ex_tiles[q], 1, 4 * ctx->ex_tile_count, ctx->stream);
        max_rw = std::max(max_rw, F.rw);
        max_n1 = std::max(max_n1, n1);
        max_n2 = std::max(max_n2, n2);
        max_cells = std::max(max_cells, (long long)n0 * n1 * n2);
        max_padded = std::max(max_padded, (long long)(F.rw + 2) * (n1 + 2) * (n2 + 2));
    }
    auto set_layer = [&](int k) {  // layer k reads buffer (k - 1) & 1 and writes buffer k & 1
        const size_t nt = ctx->ex_tile_count;
        for (int q = 0; q < nf; ++q) {
            ExField& F = a.f[q];
            const int r = (k - 1) & 1, w = k & 1;
            F.s = ctx->ex_bits[q][r];
            F.s_next = ctx->ex_bits[q][w];
            F.st = ctx->ex_tiles[q] + r * nt;
            F.st_next = ctx->ex_tiles[q] + w * nt;
            F.ch = ctx->ex_tiles[q] + (2 + r) * nt;
            F.ch_next = ctx->ex_tiles[q] + (2 + w) * nt;
        }
        a.counts = ctx->ex_counts + (k & 1) * kExMaxFields;
        a.counts_next = ctx->ex_counts + ((k + 1) & 1) * kExMaxFields;
    };
    set_layer(1);
    cudaMemsetAsync(a.counts, 0, kExMaxFields * sizeof(int), ctx->stream);
    const int wide = ctx->num_sms * 8;  // resident 256-thread blocks of the streaming passes
    ex_flat_kernel<<<dim3((unsigned)std::min<long long>(wide, (max_cells / 32 + kExThreads) / kExThreads), nf),
                     kExThreads, 0, ctx->stream>>>(a);
    ex_rows_kernel<<<dim3((unsigned)std::min<long long>(wide, (max_padded + kExThreads - 1) / kExThreads), nf),
                     kExThreads, 0, ctx->stream>>>(a);
    int n = 2;
    const int ztiles = (max_n2 + kTZ - 1) / kTZ;
    const dim3 dgrid((unsigned)((max_rw + kTW - 1) / kTW), (unsigned)((max_n1 + kTY - 1) / kTY),
                     (unsigned)(nf * ztiles));
    const int avg_blocks = ctx->num_sms * std::max(1, ctx->extrap_per_sm);
    for (int k = 1; k <= layers; ++k) {
        set_layer(k);
        ex_dilate_kernel<<<dgrid, kExThreads, 0, ctx->stream>>>(a, ztiles);
        if (ctx->dtype == EL_F64)
            ex_average_kernel<double><<<avg_blocks, kExThreads, 0, ctx->stream>>>(a);
        else
            ex_average_kernel<float><<<avg_blocks, kExThreads, 0, ctx->stream>>>(a);
        n += 2;
    }
    return n;
}

EL_CHECK_EXPORT(extrap)

}  // namespace el
