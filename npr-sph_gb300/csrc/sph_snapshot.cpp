// sph_snapshot.cpp -- snapshot and trajectory files (no counterpart in the
// reference, whose state lives only in the GL buffer and is re-created by 'r').
//
// A snapshot holds what resumes a run bit for bit: the particle records in the
// caller's order (as sph_download_aos returns them), the uniforms of every
// scene, the scene particle counts and the step count. A trajectory is the
// same header followed by frames appended during a run. All integers and
// floats are little-endian; records are the 64-byte sph_particle.
//
//   offset  bytes  field
//   0       8      magic "NPRSPHS1" (snapshot) or "NPRSPHT1" (trajectory)
//   8       4      format version (1)
//   12      4      header bytes (64)
//   16      8      particles n
//   24      4      scenes
//   28      4      flags: bit 0 = snapshot carries the slot order
//   32      8      step count (snapshot) / 0 (trajectory)
//   40      8      seed: a caller tag kept with the data
//   48      8      checksum of the payload (snapshot: everything after the
//                  header; trajectory: the scene table only)
//   56      8      reserved (0)
//   64             scene table: scenes x sph_params (96 B), scenes x u32 counts,
//                  zero padding to a multiple of 64 bytes
//   then           snapshot: n x 64 B records, then (flag bit 0) n x u32: the
//                  record index at each slot of the state, i.e. the within-cell
//                  order that the next neighbour sort keeps; restoring it makes
//                  the resumed run repeat the original bit for bit
//                  trajectory: frames of {u64 step, u64 n, u64 checksum of the
//                  records, u64 0, n x 64 B records}
// Checksum: FNV-1a 64 over the little-endian 64-bit words of the bytes (a
// final partial word is zero-padded).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "sph_ctx.h"
#include "sph_gb300.h"

namespace {

constexpr char kMagicSnap[9] = "NPRSPHS1";
constexpr char kMagicTraj[9] = "NPRSPHT1";
constexpr uint32_t kVersion = 1;
constexpr uint32_t kHeader = 64;
static_assert(sizeof(sph_params) == 96 && sizeof(sph_particle) == 64, "record sizes are part of the format");

struct Header {
    char magic[8];
    uint32_t version, header_bytes;
    uint64_t n;
    uint32_t scenes, flags;
    uint64_t steps, seed, checksum, reserved1;
};
static_assert(sizeof(Header) == 64, "header layout");

uint64_t fnv_words(const void* data, size_t bytes, uint64_t h = 0xcbf29ce484222325ull) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    size_t i = 0;
    for (; i + 8 <= bytes; i += 8) {
        uint64_t w;
        std::memcpy(&w, p + i, 8);
        h = (h ^ w) * 0x100000001b3ull;
    }
    if (i < bytes) {
        uint64_t w = 0;
        std::memcpy(&w, p + i, bytes - i);
        h = (h ^ w) * 0x100000001b3ull;
    }
    return h;
}

size_t table_bytes(uint32_t scenes) {
    const size_t raw = (size_t)scenes * (sizeof(sph_params) + 4);
    return (raw + 63) / 64 * 64;
}

std::vector<unsigned char> scene_table(const sph_ctx* ctx) {
    const uint32_t s = (uint32_t)ctx->params.size();
    std::vector<unsigned char> t(table_bytes(s), 0);
    std::memcpy(t.data(), ctx->params.data(), s * sizeof(sph_params));
    std::memcpy(t.data() + s * sizeof(sph_params), ctx->counts.data(), s * 4);
    return t;
}

struct File {
    FILE* f = nullptr;
    File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

sph_status fail(sph_ctx* ctx, sph_status code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

// Reads and checks a header and the scene table that follows it.
sph_status read_head(FILE* f, const char* magic, Header& h, std::vector<sph_params>& params,
                     std::vector<uint32_t>& counts, std::vector<unsigned char>& table) {
    if (std::fread(&h, sizeof(h), 1, f) != 1) return SPH_ERR_INVALID_ARG;
    if (std::memcmp(h.magic, magic, 8) != 0 || h.version != kVersion || h.header_bytes != kHeader)
        return SPH_ERR_INVALID_ARG;
    if (h.scenes == 0 || h.scenes > (1u << 20) || h.n > (1ull << 30) || (h.flags & ~1u)) return SPH_ERR_INVALID_ARG;
    table.assign(table_bytes(h.scenes), 0);
    if (std::fread(table.data(), 1, table.size(), f) != table.size()) return SPH_ERR_INVALID_ARG;
    params.resize(h.scenes);
    counts.resize(h.scenes);
    std::memcpy(params.data(), table.data(), h.scenes * sizeof(sph_params));
    std::memcpy(counts.data(), table.data() + h.scenes * sizeof(sph_params), h.scenes * 4);
    uint64_t tot = 0;
    for (uint32_t c : counts) tot += c;
    if (tot != h.n) return SPH_ERR_INVALID_ARG;
    return SPH_OK;
}

}  // namespace

struct sph_trajectory {
    FILE* f = nullptr;
    uint64_t n = 0;
    uint64_t frames = 0;
    std::vector<sph_particle> buf;
};

extern "C" {

sph_status sph_snapshot_save(sph_ctx* ctx, const char* path, uint64_t seed) {
    if (!ctx || !path) return SPH_ERR_INVALID_ARG;
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    try {
        const uint64_t n = (uint64_t)ctx->b.n;
        std::vector<sph_particle> recs(n);
        sph_status st = sph_download_aos(ctx, recs.data(), (uint32_t)n);
        if (st) return st;
        std::vector<uint32_t> order(n);
        st = sphgb::engine::slot_order(ctx, order.data());
        if (st) return st;
        const std::vector<unsigned char> table = scene_table(ctx);
        uint64_t sum = fnv_words(table.data(), table.size());
        sum = fnv_words(recs.data(), n * sizeof(sph_particle), sum);
        sum = fnv_words(order.data(), n * 4, sum);
        Header h{};
        std::memcpy(h.magic, kMagicSnap, 8);
        h.version = kVersion;
        h.header_bytes = kHeader;
        h.n = n;
        h.scenes = (uint32_t)ctx->params.size();
        h.flags = 1;
        h.steps = ctx->steps;
        h.seed = seed;
        h.checksum = sum;
        File out(path, "wb");
        if (!out.f) return fail(ctx, SPH_ERR_INVALID_ARG, std::string("cannot open ") + path + " for writing");
        if (std::fwrite(&h, sizeof(h), 1, out.f) != 1 ||
            std::fwrite(table.data(), 1, table.size(), out.f) != table.size() ||
            std::fwrite(recs.data(), sizeof(sph_particle), n, out.f) != n ||
            std::fwrite(order.data(), 4, n, out.f) != n)
            return fail(ctx, SPH_ERR_INVALID_ARG, std::string("short write to ") + path);
        return SPH_OK;
    } catch (const std::bad_alloc&) {
        return fail(ctx, SPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
}

sph_status sph_snapshot_info(const char* path, uint64_t* n, uint32_t* n_scene, uint64_t* steps, uint64_t* seed) {
    if (!path) return SPH_ERR_INVALID_ARG;
    try {
        File in(path, "rb");
        if (!in.f) return SPH_ERR_INVALID_ARG;
        Header h{};
        std::vector<sph_params> params;
        std::vector<uint32_t> counts;
        std::vector<unsigned char> table;
        const sph_status st = read_head(in.f, kMagicSnap, h, params, counts, table);
        if (st) return st;
        if (n) *n = h.n;
        if (n_scene) *n_scene = h.scenes;
        if (steps) *steps = h.steps;
        if (seed) *seed = h.seed;
        return SPH_OK;
    } catch (const std::bad_alloc&) {
        return SPH_ERR_OUT_OF_MEMORY;
    }
}

sph_status sph_snapshot_verify(const char* path) {
    if (!path) return SPH_ERR_INVALID_ARG;
    try {
        File in(path, "rb");
        if (!in.f) return SPH_ERR_INVALID_ARG;
        Header h{};
        std::vector<sph_params> params;
        std::vector<uint32_t> counts;
        std::vector<unsigned char> table;
        sph_status st = read_head(in.f, kMagicSnap, h, params, counts, table);
        if (st) return st;
        uint64_t sum = fnv_words(table.data(), table.size());
        std::vector<sph_particle> recs(h.n);
        if (std::fread(recs.data(), sizeof(sph_particle), h.n, in.f) != h.n) return SPH_ERR_INVALID_ARG;
        sum = fnv_words(recs.data(), h.n * sizeof(sph_particle), sum);
        if (h.flags & 1u) {
            std::vector<uint32_t> order(h.n);
            if (std::fread(order.data(), 4, h.n, in.f) != h.n) return SPH_ERR_INVALID_ARG;
            sum = fnv_words(order.data(), h.n * 4, sum);
        }
        return sum == h.checksum ? SPH_OK : SPH_ERR_INVALID_ARG;
    } catch (const std::bad_alloc&) {
        return SPH_ERR_OUT_OF_MEMORY;
    }
}

sph_status sph_snapshot_load(const char* path, void* stream, sph_ctx** out) {
    if (!path || !out) return SPH_ERR_INVALID_ARG;
    *out = nullptr;
    try {
        File in(path, "rb");
        if (!in.f) return SPH_ERR_INVALID_ARG;
        Header h{};
        std::vector<sph_params> params;
        std::vector<uint32_t> counts;
        std::vector<unsigned char> table;
        sph_status st = read_head(in.f, kMagicSnap, h, params, counts, table);
        if (st) return st;
        std::vector<sph_particle> recs(h.n);
        if (std::fread(recs.data(), sizeof(sph_particle), h.n, in.f) != h.n) return SPH_ERR_INVALID_ARG;
        uint64_t sum = fnv_words(table.data(), table.size());
        sum = fnv_words(recs.data(), h.n * sizeof(sph_particle), sum);
        std::vector<uint32_t> order;
        if (h.flags & 1u) {
            order.resize(h.n);
            if (std::fread(order.data(), 4, h.n, in.f) != h.n) return SPH_ERR_INVALID_ARG;
            sum = fnv_words(order.data(), h.n * 4, sum);
        }
        if (sum != h.checksum) return SPH_ERR_INVALID_ARG;
        sph_ctx* ctx = nullptr;
        st = h.scenes == 1 ? sph_create(params.data(), (uint32_t)h.n, stream, &ctx)
                           : sph_create_batch(params.data(), counts.data(), h.scenes, stream, &ctx);
        if (st) return st;
        st = sph_upload_aos(ctx, recs.data(), (uint32_t)h.n);
        if (!st && !order.empty()) st = sphgb::engine::apply_order(ctx, order.data());
        if (st) {
            sph_destroy(ctx);
            return st;
        }
        ctx->steps = h.steps;  // the run continues its count
        *out = ctx;
        return SPH_OK;
    } catch (const std::bad_alloc&) {
        return SPH_ERR_OUT_OF_MEMORY;
    }
}

sph_status sph_trajectory_create(sph_ctx* ctx, const char* path, uint64_t seed, sph_trajectory** out) {
    if (!ctx || !path || !out) return SPH_ERR_INVALID_ARG;
    *out = nullptr;
    if (!ctx->have_state) return fail(ctx, SPH_ERR_NOT_READY, "no particles uploaded");
    try {
        const std::vector<unsigned char> table = scene_table(ctx);
        Header h{};
        std::memcpy(h.magic, kMagicTraj, 8);
        h.version = kVersion;
        h.header_bytes = kHeader;
        h.n = (uint64_t)ctx->b.n;
        h.scenes = (uint32_t)ctx->params.size();
        h.seed = seed;
        h.checksum = fnv_words(table.data(), table.size());
        FILE* f = std::fopen(path, "wb");
        if (!f) return fail(ctx, SPH_ERR_INVALID_ARG, std::string("cannot open ") + path + " for writing");
        if (std::fwrite(&h, sizeof(h), 1, f) != 1 || std::fwrite(table.data(), 1, table.size(), f) != table.size()) {
            std::fclose(f);
            return fail(ctx, SPH_ERR_INVALID_ARG, std::string("short write to ") + path);
        }
        sph_trajectory* t = new sph_trajectory;
        t->f = f;
        t->n = h.n;
        *out = t;
        return SPH_OK;
    } catch (const std::bad_alloc&) {
        return fail(ctx, SPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
}

sph_status sph_trajectory_append(sph_trajectory* t, sph_ctx* ctx) {
    if (!t || !ctx || !t->f) return SPH_ERR_INVALID_ARG;
    if ((uint64_t)ctx->b.n != t->n) return fail(ctx, SPH_ERR_INVALID_ARG, "particle count differs from the trajectory's");
    try {
        t->buf.resize(t->n);
        sph_status st = sph_download_aos(ctx, t->buf.data(), (uint32_t)t->n);
        if (st) return st;
        const uint64_t fh[4] = {ctx->steps, t->n, fnv_words(t->buf.data(), t->n * sizeof(sph_particle)), 0};
        if (std::fwrite(fh, sizeof(fh), 1, t->f) != 1 ||
            std::fwrite(t->buf.data(), sizeof(sph_particle), t->n, t->f) != t->n)
            return fail(ctx, SPH_ERR_INVALID_ARG, "short write to the trajectory file");
        ++t->frames;
        return SPH_OK;
    } catch (const std::bad_alloc&) {
        return fail(ctx, SPH_ERR_OUT_OF_MEMORY, "host allocation failed");
    }
}

uint64_t sph_trajectory_frames(const sph_trajectory* t) { return t ? t->frames : 0; }

sph_status sph_trajectory_close(sph_trajectory* t) {
    if (!t) return SPH_ERR_INVALID_ARG;
    const bool ok = !t->f || std::fclose(t->f) == 0;
    delete t;
    return ok ? SPH_OK : SPH_ERR_INVALID_ARG;
}

uint64_t sph_checksum64(const void* data, uint64_t bytes) { return data ? fnv_words(data, (size_t)bytes) : 0; }

}  // extern "C"
