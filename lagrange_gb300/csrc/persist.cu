// fwn_save / fwn_load: a built engine (single mesh or forest) written to a file and read back,
// so that a caller who queries the same meshes in several processes builds them once. The
// reference has no counterpart (lagrange's serialization covers meshes, not the winding engine).
//
// File layout (host byte order; x86-64 and aarch64 are both little-endian):
//   FileHeader                         magic, version, counts, the engine's config, which record
//                                      sets follow, and an FNV-1a 64 checksum of the payload
//   MeshInfo[num_meshes]
//   NodeF32[num_nodes]                 if the engine kept FP32 records
//   NodeF64[num_nodes]                 if it kept FP64 records
//   TriF32[num_triangles], int32[num_triangles] (original triangle id per leaf slot)
// A load checks the magic, version, sizes and checksum before it touches the device, then every
// node's links and triangle range and every mesh's root range, so that a file the walk would
// read out of bounds with is refused instead of queried.
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "fwn_internal.cuh"

namespace fwn {
namespace {

constexpr char kMagic[8] = {'F', 'W', 'N', 'G', 'B', '3', '0', '0'};
constexpr uint32_t kVersion = 1;

struct FileHeader {
    char magic[8];
    uint32_t version;
    uint32_t header_bytes;
    fwn_config cfg;
    int64_t nv, nf, nmeshes, num_nodes, num_leaves;
    int32_t has32, has64;
    uint64_t payload_bytes;
    uint64_t checksum;  // FNV-1a 64 of the payload
};

struct Fnv {
    uint64_t h = 1469598103934665603ull;
    void add(const void* p, size_t n) {
        const unsigned char* b = static_cast<const unsigned char*>(p);
        for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    }
};

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

template <class T> std::vector<T> to_host(const T* d, int64_t n) {
    std::vector<T> h((size_t)n);
    if (n) FWN_CUDA_CHECK(cudaMemcpy(h.data(), d, (size_t)n * sizeof(T), cudaMemcpyDeviceToHost));
    return h;
}

template <class T> T* to_device(const std::vector<T>& h) {
    T* d = nullptr;
    if (h.empty()) return nullptr;
    FWN_CUDA_CHECK(cudaMalloc(&d, h.size() * sizeof(T)));
    FWN_CUDA_CHECK(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return d;
}

void read_exact(FILE* f, void* p, size_t n, Fnv* sum) {
    if (n && std::fread(p, 1, n, f) != n)
        throw Error(FWN_INVALID_ARG, "engine file is truncated");
    if (sum) sum->add(p, n);
}

// The walk follows skip links forward and reads a leaf's triangles [tri_begin, tri_begin +
// tri_count); a mesh's walk runs over [root, end).
template <class Node>
void check_nodes(const std::vector<Node>& nodes, int64_t nf) {
    const int64_t E = (int64_t)nodes.size();
    for (int64_t i = 0; i < E; ++i) {
        const Node& n = nodes[(size_t)i];
        if (n.skip <= i || n.skip > E || n.tri_count < 0 || n.tri_count > 16 || n.tri_begin < 0 ||
            (int64_t)n.tri_begin + n.tri_count > nf)
            throw Error(FWN_INVALID_ARG, "engine file holds an inconsistent node " + std::to_string(i));
    }
}

}  // namespace
}  // namespace fwn

using namespace fwn;

extern "C" FWN_API fwn_status fwn_save(fwn_handle h, const char* path) {
    try {
        if (!h) throw Error(FWN_NOT_BUILT, "null handle (default-constructed or moved-from engine)");
        if (!path) throw Error(FWN_INVALID_ARG, "path is null");
        const Engine& e = *reinterpret_cast<const Engine*>(h);
        int cur = 0;
        FWN_CUDA_CHECK(cudaGetDevice(&cur));
        if (cur != e.device) FWN_CUDA_CHECK(cudaSetDevice(e.device));
        struct Restore {
            int dev, cur;
            ~Restore() {
                if (dev != cur) cudaSetDevice(cur);
            }
        } restore{e.device, cur};
        const int64_t E = e.num_nodes, nf = e.nf, M = e.nmeshes;
        const std::vector<NodeF32> n32 = e.nodes32 ? to_host(e.nodes32, E) : std::vector<NodeF32>();
        const std::vector<NodeF64> n64 = e.nodes64 ? to_host(e.nodes64, E) : std::vector<NodeF64>();
        const std::vector<TriF32> tris = to_host(e.tris, nf);
        const std::vector<int> sorted = to_host(e.sorted_tri, nf);
        FileHeader hd;
        std::memset(&hd, 0, sizeof(hd));
        std::memcpy(hd.magic, kMagic, sizeof(kMagic));
        hd.version = kVersion;
        hd.header_bytes = sizeof(FileHeader);
        hd.cfg = e.cfg;
        hd.nv = e.nv;
        hd.nf = nf;
        hd.nmeshes = M;
        hd.num_nodes = E;
        hd.num_leaves = e.num_leaves;
        hd.has32 = e.nodes32 ? 1 : 0;
        hd.has64 = e.nodes64 ? 1 : 0;
        Fnv sum;
        size_t bytes = 0;
        auto add = [&](const void* p, size_t n) {
            sum.add(p, n);
            bytes += n;
        };
        add(e.meshes_h, (size_t)M * sizeof(MeshInfo));
        add(n32.data(), n32.size() * sizeof(NodeF32));
        add(n64.data(), n64.size() * sizeof(NodeF64));
        add(tris.data(), tris.size() * sizeof(TriF32));
        add(sorted.data(), sorted.size() * sizeof(int));
        hd.payload_bytes = bytes;
        hd.checksum = sum.h;
        File f;
        f.f = std::fopen(path, "wb");
        if (!f.f) throw Error(FWN_INVALID_ARG, std::string("cannot open for writing: ") + path);
        auto put = [&](const void* p, size_t n) {
            if (n && std::fwrite(p, 1, n, f.f) != n)
                throw Error(FWN_INVALID_ARG, std::string("write failed: ") + path);
        };
        put(&hd, sizeof(hd));
        put(e.meshes_h, (size_t)M * sizeof(MeshInfo));
        put(n32.data(), n32.size() * sizeof(NodeF32));
        put(n64.data(), n64.size() * sizeof(NodeF64));
        put(tris.data(), tris.size() * sizeof(TriF32));
        put(sorted.data(), sorted.size() * sizeof(int));
        if (std::fclose(f.f) != 0) {
            f.f = nullptr;
            throw Error(FWN_INVALID_ARG, std::string("write failed: ") + path);
        }
        f.f = nullptr;
        return FWN_OK;
    } catch (const Error& err) {
        set_last_error(err.what());
        return err.status;
    } catch (const std::exception& err) {
        set_last_error(err.what());
        return FWN_INTERNAL;
    }
}

extern "C" FWN_API fwn_status fwn_load(const char* path, fwn_handle* out) {
    try {
        if (!out) throw Error(FWN_INVALID_ARG, "out is null");
        *out = nullptr;
        if (!path) throw Error(FWN_INVALID_ARG, "path is null");
        File f;
        f.f = std::fopen(path, "rb");
        if (!f.f) throw Error(FWN_INVALID_ARG, std::string("cannot open: ") + path);
        FileHeader hd;
        read_exact(f.f, &hd, sizeof(hd), nullptr);
        if (std::memcmp(hd.magic, kMagic, sizeof(kMagic)) != 0)
            throw Error(FWN_INVALID_ARG, "not an engine file (bad magic)");
        if (hd.version != kVersion || hd.header_bytes != sizeof(FileHeader))
            throw Error(FWN_INVALID_ARG, "engine file of another version");
        const int64_t E = hd.num_nodes, nf = hd.nf, M = hd.nmeshes;
        if (hd.nv < 0 || nf < 0 || nf > (int64_t)0x3fffffff || M < 1 || M > 65535 || E < 0 ||
            E > 2 * nf || hd.num_leaves < 0 || hd.num_leaves > E || (hd.has32 | hd.has64) & ~1 ||
            !(hd.has32 || hd.has64))
            throw Error(FWN_INVALID_ARG, "engine file holds inconsistent sizes");
        const uint64_t expect = (uint64_t)M * sizeof(MeshInfo) +
                                (uint64_t)E * (hd.has32 ? sizeof(NodeF32) : 0) +
                                (uint64_t)E * (hd.has64 ? sizeof(NodeF64) : 0) +
                                (uint64_t)nf * (sizeof(TriF32) + sizeof(int));
        if (hd.payload_bytes != expect) throw Error(FWN_INVALID_ARG, "engine file holds inconsistent sizes");
        // the record sets are the ones in the file (the FP64 staging moments are not saved); the
        // rest of the configuration must pass the same checks as a build's
        fwn_config cfg = hd.cfg;
        cfg.records = (hd.has32 ? FWN_RECORDS_F32 : 0) | (hd.has64 ? FWN_RECORDS_F64 : 0);
        validate_config(cfg);
        if (cfg.tuning == 7) cfg.tuning = 6;  // no structure-of-arrays copy: the same walk on the records
        Fnv sum;
        std::vector<MeshInfo> meshes((size_t)M);
        std::vector<NodeF32> n32(hd.has32 ? (size_t)E : 0);
        std::vector<NodeF64> n64(hd.has64 ? (size_t)E : 0);
        std::vector<TriF32> tris((size_t)nf);
        std::vector<int> sorted((size_t)nf);
        read_exact(f.f, meshes.data(), meshes.size() * sizeof(MeshInfo), &sum);
        read_exact(f.f, n32.data(), n32.size() * sizeof(NodeF32), &sum);
        read_exact(f.f, n64.data(), n64.size() * sizeof(NodeF64), &sum);
        read_exact(f.f, tris.data(), tris.size() * sizeof(TriF32), &sum);
        read_exact(f.f, sorted.data(), sorted.size() * sizeof(int), &sum);
        if (sum.h != hd.checksum) throw Error(FWN_INVALID_ARG, "engine file is corrupt (checksum)");
        if (hd.has32) check_nodes(n32, nf);
        if (hd.has64) check_nodes(n64, nf);
        for (const MeshInfo& m : meshes)
            if (!(m.root == -1 && m.end == -1) && !(m.root >= 0 && m.root < m.end && m.end <= E))
                throw Error(FWN_INVALID_ARG, "engine file holds an inconsistent mesh root");
        for (int s : sorted)
            if (s < 0 || (int64_t)s >= nf) throw Error(FWN_INVALID_ARG, "engine file holds an inconsistent triangle id");
        std::unique_ptr<Engine> e(new Engine());
        e->cfg = cfg;
        FWN_CUDA_CHECK(cudaGetDevice(&e->device));
        e->nv = hd.nv;
        e->nf = nf;
        e->nmeshes = M;
        e->num_nodes = E;
        e->num_leaves = hd.num_leaves;
        e->nodes32 = to_device(n32);
        e->nodes64 = to_device(n64);
        e->tris = to_device(tris);
        e->sorted_tri = to_device(sorted);
        FWN_CUDA_CHECK(cudaMalloc(&e->meshes, (size_t)M * sizeof(MeshInfo)));
        FWN_CUDA_CHECK(cudaMemcpy(e->meshes, meshes.data(), (size_t)M * sizeof(MeshInfo),
                                  cudaMemcpyHostToDevice));
        e->meshes_h = new MeshInfo[(size_t)M];
        std::memcpy(e->meshes_h, meshes.data(), (size_t)M * sizeof(MeshInfo));
        e->build_ms = 0.0;
        e->device_bytes = E * (int64_t)((hd.has32 ? sizeof(NodeF32) : 0) + (hd.has64 ? sizeof(NodeF64) : 0)) +
                          nf * (int64_t)(sizeof(TriF32) + sizeof(int)) + M * (int64_t)sizeof(MeshInfo);
        *out = reinterpret_cast<fwn_handle>(e.release());
        return FWN_OK;
    } catch (const Error& err) {
        set_last_error(err.what());
        return err.status;
    } catch (const std::exception& err) {
        set_last_error(err.what());
        return FWN_INTERNAL;
    }
}
