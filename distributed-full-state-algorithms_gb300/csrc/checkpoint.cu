// checkpoint.cu -- dfs_state_save / dfs_state_load: one state to and from a file (the
// format is documented with the declarations in dfs_gb300.h).  Host code over the
// public amplitude-transfer calls; amplitudes move in chunks through pinned memory.
#include <cstdio>
#include <cstring>

#include "engine.hpp"

namespace dfs {

namespace {

constexpr char kMagic[8] = {'D', 'F', 'S', 'S', 'T', 'A', 'T', 'E'};
constexpr uint32_t kVersion = 1;
constexpr uint64_t kChunkBytes = 64ull << 20;

struct FileHeader {
    char magic[8];
    uint32_t version, kind, numQubits;
    int32_t precision;
    uint64_t numAmps;
    uint32_t ampBytes, reserved;
};
static_assert(sizeof(FileHeader) == 40, "header layout");

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

struct Pinned {
    void* p = nullptr;
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
};

}  // namespace

static int save(dfs_state s, const char* path) {
    DFS_TRACE_CALL();
    if (!path) return fail(DFS_ERR_INVALID_ARG, "null path");
    dfs_state_info info;
    int rc = dfs_state_get_info(s, &info);
    if (rc) return rc;
    FileHeader h{};
    std::memcpy(h.magic, kMagic, 8);
    h.version = kVersion;
    h.kind = info.is_density_matrix ? 1u : 0u;
    h.numQubits = info.num_qubits;
    h.precision = info.precision;
    h.numAmps = info.num_amps_per_node;
    h.ampBytes = (uint32_t)elem_bytes(info.precision);
    File file;
    file.f = fopen(path, "wb");
    if (!file.f) return fail(DFS_ERR_IO, "cannot open %s for writing", path);
    if (fwrite(&h, sizeof h, 1, file.f) != 1) return fail(DFS_ERR_IO, "cannot write the header of %s", path);
    Pinned buf;
    const uint64_t perChunk = kChunkBytes / h.ampBytes;
    const uint64_t chunk = h.numAmps < perChunk ? h.numAmps : perChunk;
    cudaError_t e = cudaMallocHost(&buf.p, chunk * h.ampBytes);
    if (e != cudaSuccess) return cuda_fail(e, "pinned staging for a state file");
    for (uint64_t start = 0; start < h.numAmps; start += chunk) {
        const uint64_t count = h.numAmps - start < chunk ? h.numAmps - start : chunk;
        if ((rc = dfs_state_get_raw(s, buf.p, start, count))) return rc;
        if (fwrite(buf.p, h.ampBytes, count, file.f) != count)
            return fail(DFS_ERR_IO, "short write to %s", path);
    }
    if (fflush(file.f) != 0) return fail(DFS_ERR_IO, "cannot flush %s", path);
    return DFS_SUCCESS;
}

static int load(const char* path, dfs_state* out) {
    DFS_TRACE_CALL();
    if (!path || !out) return fail(DFS_ERR_INVALID_ARG, "null path or output handle");
    *out = nullptr;
    File file;
    file.f = fopen(path, "rb");
    if (!file.f) return fail(DFS_ERR_IO, "cannot open %s", path);
    FileHeader h;
    if (fread(&h, sizeof h, 1, file.f) != 1) return fail(DFS_ERR_IO, "%s: truncated header", path);
    if (std::memcmp(h.magic, kMagic, 8) != 0) return fail(DFS_ERR_IO, "%s is not a state file", path);
    if (h.version != kVersion) return fail(DFS_ERR_IO, "%s: unsupported version %u", path, h.version);
    if (h.kind > 1) return fail(DFS_ERR_IO, "%s: unknown state kind %u", path, h.kind);
    if (h.precision != DFS_C128 && h.precision != DFS_C128_NATIVE && h.precision != DFS_C64)
        return fail(DFS_ERR_IO, "%s: unknown precision %d", path, h.precision);
    const unsigned vq = h.kind ? 2 * h.numQubits : h.numQubits;
    if (h.numQubits > 64 || vq >= 64 || h.numAmps != (1ull << vq) || h.ampBytes != elem_bytes(h.precision))
        return fail(DFS_ERR_IO, "%s: inconsistent header", path);
    dfs_state s = nullptr;
    int rc = h.kind ? dfs_densitymatrix_create(h.numQubits, h.precision, &s)
                    : dfs_statevector_create(h.numQubits, h.precision, &s);
    if (rc) return rc;
    Pinned buf;
    const uint64_t perChunk = kChunkBytes / h.ampBytes;
    const uint64_t chunk = h.numAmps < perChunk ? h.numAmps : perChunk;
    cudaError_t e = cudaMallocHost(&buf.p, chunk * h.ampBytes);
    if (e != cudaSuccess) rc = cuda_fail(e, "pinned staging for a state file");
    for (uint64_t start = 0; !rc && start < h.numAmps; start += chunk) {
        const uint64_t count = h.numAmps - start < chunk ? h.numAmps - start : chunk;
        if (fread(buf.p, h.ampBytes, count, file.f) != count) rc = fail(DFS_ERR_IO, "%s: truncated data", path);
        else rc = dfs_state_set_raw(s, buf.p, start, count);
    }
    if (rc) {
        dfs_state_destroy(s);
        return rc;
    }
    *out = s;
    return DFS_SUCCESS;
}

}  // namespace dfs

extern "C" int dfs_state_save(dfs_state s, const char* path) { return dfs::save(s, path); }
extern "C" int dfs_state_load(const char* path, dfs_state* out) { return dfs::load(path, out); }
