// el_state.cu -- state dump / restore of a context: a small header and the raw fields, so a run
// can be restarted exactly (parity restarts, recorded training scenes).  No counterpart in the
// reference, whose only dumps are OBJ meshes and text slices of 2D grids.
//
// File layout (little-endian, packed):
//   header, 64 bytes:  char magic[8] = "ELGBSTAT"; uint32 version = 1; uint32 dtype (EL_F32 /
//                      EL_F64); int32 ni, nj, nk; uint32 nfields; double dx; double time;
//                      uint8 reserved[16] = 0
//   nfields records:   uint32 field (enum el_field); uint32 element bytes; uint64 byte count;
//                      the field's bytes in the layout of el_upload
#include <cstdio>
#include <cstring>
#include <vector>

#include "el_internal.cuh"

namespace el {
int set_error(el_ctx* ctx, int code, const std::string& msg);
}  // namespace el

using namespace el;

namespace {

#pragma pack(push, 1)
struct StateHeader {
    char magic[8];
    uint32_t version;
    uint32_t dtype;
    int32_t ni, nj, nk;
    uint32_t nfields;
    double dx;
    double time;
    uint8_t reserved[16];
};
struct FieldRecord {
    uint32_t field;
    uint32_t elem;
    uint64_t bytes;
};
#pragma pack(pop)
static_assert(sizeof(StateHeader) == 64, "header is 64 bytes");
static_assert(sizeof(FieldRecord) == 16, "record header is 16 bytes");

constexpr char kMagic[8] = {'E', 'L', 'G', 'B', 'S', 'T', 'A', 'T'};

// every field but the derived fluid numbering
bool saved_field(int f) { return f >= 0 && f < EL_FIELD_COUNT && f != EL_FIELD_INDICES; }

uint32_t elem_bytes(const el_ctx* c, int f) {
    if (f >= EL_FIELD_VALID_U && f <= EL_FIELD_VALID_PHI) return 1;
    return (uint32_t)c->esz;
}

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

}  // namespace

#define EL_API extern "C" __attribute__((visibility("default")))

EL_API int el_state_save(el_ctx* ctx, const char* path, double time) {
    if (!ctx || !path) return EL_ERR_INVALID_ARGUMENT;
    DeviceGuard guard(ctx->device);
    if (guard.err != cudaSuccess) return EL_ERR_CUDA;
    File out;
    out.f = fopen(path, "wb");
    if (!out.f) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    StateHeader h;
    std::memset(&h, 0, sizeof(h));
    std::memcpy(h.magic, kMagic, 8);
    h.version = 1;
    h.dtype = (uint32_t)ctx->dtype;
    h.ni = ctx->ni;
    h.nj = ctx->nj;
    h.nk = ctx->nk;
    h.dx = ctx->dx;
    h.time = time;
    for (int f = 0; f < EL_FIELD_COUNT; ++f) h.nfields += saved_field(f) ? 1 : 0;
    if (fwrite(&h, sizeof(h), 1, out.f) != 1) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "write failed");
    std::vector<unsigned char> buf;
    for (int f = 0; f < EL_FIELD_COUNT; ++f) {
        if (!saved_field(f)) continue;
        const size_t bytes = ctx->field_bytes[f];
        buf.resize(bytes);
        EL_CUDA_TRY(ctx, cudaMemcpyAsync(buf.data(), ctx->field[f], bytes, cudaMemcpyDeviceToHost, ctx->stream));
        EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        const FieldRecord r{(uint32_t)f, elem_bytes(ctx, f), (uint64_t)bytes};
        if (fwrite(&r, sizeof(r), 1, out.f) != 1 || fwrite(buf.data(), 1, bytes, out.f) != bytes)
            return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "write failed");
    }
    if (fflush(out.f) != 0) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "write failed");
    return EL_OK;
}

EL_API int el_state_load(el_ctx* ctx, const char* path, double* time) {
    if (!ctx || !path) return EL_ERR_INVALID_ARGUMENT;
    DeviceGuard guard(ctx->device);
    if (guard.err != cudaSuccess) return EL_ERR_CUDA;
    File in;
    in.f = fopen(path, "rb");
    if (!in.f) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
    StateHeader h;
    if (fread(&h, sizeof(h), 1, in.f) != 1 || std::memcmp(h.magic, kMagic, 8) != 0 || h.version != 1)
        return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "not a state file (magic or version)");
    if (h.ni != ctx->ni || h.nj != ctx->nj || h.nk != ctx->nk || (int)h.dtype != ctx->dtype)
        return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "state file grid or field type differs from the context");
    if (h.nfields > (uint32_t)EL_FIELD_COUNT) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "bad field count");
    // read every record first, so that a damaged file changes nothing
    std::vector<std::pair<int, std::vector<unsigned char>>> fields;
    for (uint32_t q = 0; q < h.nfields; ++q) {
        FieldRecord r;
        if (fread(&r, sizeof(r), 1, in.f) != 1) return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "truncated state file");
        const int f = (int)r.field;
        if (!saved_field(f) || r.elem != elem_bytes(ctx, f) || r.bytes != ctx->field_bytes[f])
            return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "bad field record " + std::to_string(f));
        std::vector<unsigned char> buf(r.bytes);
        if (fread(buf.data(), 1, r.bytes, in.f) != r.bytes)
            return set_error(ctx, EL_ERR_INVALID_ARGUMENT, "truncated state file");
        fields.emplace_back(f, std::move(buf));
    }
    for (auto& fb : fields) {
        EL_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->field[fb.first], fb.second.data(), fb.second.size(),
                                         cudaMemcpyHostToDevice, ctx->stream));
        EL_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    if (time) *time = h.time;
    return EL_OK;
}
