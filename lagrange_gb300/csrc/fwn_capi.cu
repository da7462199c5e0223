// C ABI of the engine (declared in include/fwn_gb300.h). No exception crosses this boundary:
// every entry point catches, stores the message in a thread-local slot and returns a status.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "fwn_internal.cuh"

namespace fwn {

static thread_local std::string g_last_error;

void set_last_error(const std::string& m) { g_last_error = m; }

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_pool_mutex;
// two pools per device, created on first use and kept for the process lifetime: one for query
// scratch, one for build temporaries, so that the gigabytes a large build frees (in block sizes
// of its own) never stand in for a query's scratch and push the query pool over its threshold
cudaMemPool_t g_pools[2][kMaxDevices] = {};
constexpr uint64_t kRetain[2] = {kScratchRetainBytes, kBuildRetainBytes};

cudaMemPool_t scratch_pool(int dev, int kind) {
    if (dev < 0 || dev >= kMaxDevices) throw Error(FWN_INTERNAL, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (!g_pools[kind][dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        FWN_CUDA_CHECK(cudaMemPoolCreate(&pool, &props));
        uint64_t keep = kRetain[kind];
        const cudaError_t err = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        if (err != cudaSuccess) {
            cudaMemPoolDestroy(pool);
            FWN_CUDA_CHECK(err);
        }
        g_pools[kind][dev] = pool;
    }
    return g_pools[kind][dev];
}

void* pool_alloc(size_t bytes, cudaStream_t st, int kind) {
    void* p = nullptr;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    FWN_CUDA_CHECK(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) {
        FWN_CUDA_CHECK(cudaMallocAsync(&p, bytes, st));
        return p;
    }
    int dev = 0;
    FWN_CUDA_CHECK(cudaGetDevice(&dev));
    FWN_CUDA_CHECK(cudaMallocFromPoolAsync(&p, bytes, scratch_pool(dev, kind), st));
    return p;
}
}  // namespace

// Usage of the query scratch pool of `dev` (zeros when no call has created it yet); reset_high
// restarts the high-water mark of used bytes from the current value.
void scratch_pool_stats(int dev, bool reset_high, uint64_t* reserved, uint64_t* used,
                        uint64_t* used_high) {
    if (dev < 0 || dev >= kMaxDevices) throw Error(FWN_INVALID_ARG, "device ordinal out of range");
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_pool_mutex);
        pool = g_pools[0][dev];
    }
    uint64_t r = 0, u = 0, h = 0;
    if (pool) {
        if (reset_high) {
            uint64_t zero = 0;
            FWN_CUDA_CHECK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero));
        }
        FWN_CUDA_CHECK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &r));
        FWN_CUDA_CHECK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &u));
        FWN_CUDA_CHECK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &h));
    }
    if (reserved) *reserved = r;
    if (used) *used = u;
    if (used_high) *used_high = h;
}

void* scratch_alloc(size_t bytes, cudaStream_t st) { return pool_alloc(bytes, st, 0); }

void* build_alloc(size_t bytes, cudaStream_t st) { return pool_alloc(bytes, st, 1); }

Engine::~Engine() {
    // free on the engine's device, then give the caller back its current device
    int cur = -1;
    const bool swap = cudaGetDevice(&cur) == cudaSuccess && cur != device &&
                      cudaSetDevice(device) == cudaSuccess;
    if (nodes32) cudaFree(nodes32);
    if (nodes64) cudaFree(nodes64);
    if (soa) cudaFree(soa);
    if (tris) cudaFree(tris);
    if (sorted_tri) cudaFree(sorted_tri);
    if (meshes) cudaFree(meshes);
    if (stage) cudaFree(stage);
    if (swap) cudaSetDevice(cur);
    delete[] meshes_h;
    delete[] node_tri_begin_h;
}

namespace {

template <class Fn> fwn_status guarded(Fn&& fn) {
    try {
        fn();
        return FWN_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::bad_alloc&) {
        set_last_error("host allocation failed");
        return FWN_OOM;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return FWN_INTERNAL;
    } catch (...) {
        set_last_error("unknown error");
        return FWN_INTERNAL;
    }
}


struct OwnedStream {
    cudaStream_t s = nullptr;
    OwnedStream() { FWN_CUDA_CHECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
    ~OwnedStream() {
        if (s) cudaStreamDestroy(s);
    }
};

// The streams of the synchronous host-buffer queries: non-blocking streams per (host thread,
// device), created on first use and kept for the thread's lifetime; creating and destroying a
// stream on every call costs more than a small query. Stream 0 runs the queries; in
// fwn_query_host_batches streams 1 and 2 copy batches in and out, and odd batches run on stream 3
// (so that a batch's key sort can start while the previous batch's walk finishes).
constexpr int kHostStreams = 4;

cudaStream_t host_stream(int k = 0) {
    struct Streams {
        cudaStream_t s[kMaxDevices][kHostStreams] = {};
        ~Streams() {
            for (auto& d : s)
                for (cudaStream_t x : d)
                    if (x) cudaStreamDestroy(x);
        }
    };
    thread_local Streams t;
    int dev = 0;
    FWN_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw Error(FWN_INTERNAL, "device ordinal out of range");
    if (!t.s[dev][k]) FWN_CUDA_CHECK(cudaStreamCreateWithFlags(&t.s[dev][k], cudaStreamNonBlocking));
    return t.s[dev][k];
}

Engine* engine_of(fwn_handle h) {
    if (!h) throw Error(FWN_NOT_BUILT, "null handle (default-constructed or moved-from engine)");
    return reinterpret_cast<Engine*>(h);
}

Engine* new_engine(const fwn_config* cfg) {
    fwn_config c;
    fwn_config_default(&c);
    if (cfg) c = *cfg;
    validate_config(c);
    Engine* e = new Engine();
    e->cfg = c;
    FWN_CUDA_CHECK(cudaGetDevice(&e->device));
    return e;
}

void build_into(Engine* e, const float* d_V, const int64_t* voff, const int32_t* d_F,
                const int64_t* foff, int64_t nmeshes, cudaStream_t st) {
    build_forest(*e, d_V, voff, d_F, foff, nmeshes, st);
}

void check_points(int64_t n, const void* p) {
    if (n < 0) throw Error(FWN_INVALID_ARG, "number of points must be >= 0");
    if (n > 0 && !p) throw Error(FWN_INVALID_ARG, "points pointer is null");
    if (n > (int64_t)INT32_MAX) throw Error(FWN_INVALID_ARG, "at most 2^31-1 points per call");
}

void check_mesh_args(const void* V, int64_t nv, const void* F, int64_t nf) {
    if (nv < 0 || nf < 0) throw Error(FWN_INVALID_ARG, "sizes must be >= 0");
    if (nv > 0 && !V) throw Error(FWN_INVALID_ARG, "vertices pointer is null");
    if (nf > 0 && !F) throw Error(FWN_INVALID_ARG, "triangles pointer is null");
}

}  // namespace

void validate_config(const fwn_config& c) {
    if (!(c.beta > 0.f) || !std::isfinite(c.beta)) throw Error(FWN_INVALID_ARG, "beta must be finite and > 0");
    if (c.leaf_size < 1 || c.leaf_size > 16) throw Error(FWN_INVALID_ARG, "leaf_size must be in [1, 16]");
    if (!(c.records & (FWN_RECORDS_F32 | FWN_RECORDS_F64)))
        throw Error(FWN_INVALID_ARG, "records must include FWN_RECORDS_F32 or FWN_RECORDS_F64");
    if (c.precision != FWN_PRECISION_MIXED && c.precision != FWN_PRECISION_FP64)
        throw Error(FWN_INVALID_ARG, "unknown precision");
    if (c.traversal < FWN_TRAVERSAL_AUTO || c.traversal > FWN_TRAVERSAL_WARP)
        throw Error(FWN_INVALID_ARG, "unknown traversal");
    if (c.block_size < 0 || c.block_size > 1024 || c.block_size % 32 != 0)
        throw Error(FWN_INVALID_ARG, "block_size must be 0 or a multiple of 32 <= 1024");
    if (!(c.fp64_near_scale >= 0.f) || !std::isfinite(c.fp64_near_scale))
        throw Error(FWN_INVALID_ARG, "fp64_near_scale must be finite and >= 0");
    if (!(c.fp64_cond >= 0.f) || !std::isfinite(c.fp64_cond))
        throw Error(FWN_INVALID_ARG, "fp64_cond must be finite and >= 0");
    if (c.tuning < 0 || c.tuning > 7) throw Error(FWN_INVALID_ARG, "tuning must be in [0, 7]");
    if (c.builder != FWN_BUILDER_LBVH && c.builder != FWN_BUILDER_SPLIT &&
        c.builder != FWN_BUILDER_BINNED)
        throw Error(FWN_INVALID_ARG,
                    "builder must be FWN_BUILDER_LBVH, FWN_BUILDER_SPLIT or FWN_BUILDER_BINNED");
}

}  // namespace fwn

using namespace fwn;

extern "C" {

FWN_API void fwn_config_default(fwn_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->beta = 2.0f;
    c->leaf_size = 8;
    c->records = FWN_RECORDS_F32;
    c->precision = FWN_PRECISION_MIXED;
    c->traversal = FWN_TRAVERSAL_AUTO;
    c->block_size = 0;
    c->sort_queries = 1;
    c->fp64_near_scale = 1e-3f;
    c->fp64_cond = 4.0f;
}

FWN_API size_t fwn_last_error(char* buf, size_t n) {
    const std::string& m = g_last_error;
    if (buf && n) {
        size_t k = m.size() < n - 1 ? m.size() : n - 1;
        std::memcpy(buf, m.data(), k);
        buf[k] = '\0';
    }
    return m.size();
}

FWN_API const char* fwn_version(void) { return "0.1.0 sm_103a"; }

FWN_API fwn_status fwn_build(const float* V, int64_t nv, const int32_t* F, int64_t nf,
                             const fwn_config* cfg, fwn_handle* out) {
    return guarded([&] {
        if (!out) throw Error(FWN_INVALID_ARG, "out is null");
        *out = nullptr;
        check_mesh_args(V, nv, F, nf);
        std::unique_ptr<Engine> e(new_engine(cfg));
        OwnedStream os;
        Scratch dv(nv * 3 * sizeof(float), os.s), df(nf * 3 * sizeof(int32_t), os.s);
        if (nv) FWN_CUDA_CHECK(cudaMemcpyAsync(dv.p, V, nv * 3 * sizeof(float), cudaMemcpyHostToDevice, os.s));
        if (nf) FWN_CUDA_CHECK(cudaMemcpyAsync(df.p, F, nf * 3 * sizeof(int32_t), cudaMemcpyHostToDevice, os.s));
        const int64_t voff[2] = {0, nv}, foff[2] = {0, nf};
        build_into(e.get(), dv.as<float>(), voff, df.as<int32_t>(), foff, 1, os.s);
        FWN_CUDA_CHECK(cudaStreamSynchronize(os.s));
        *out = reinterpret_cast<fwn_handle>(e.release());
    });
}

FWN_API fwn_status fwn_build_device(const float* d_V, int64_t nv, const int32_t* d_F, int64_t nf,
                                    const fwn_config* cfg, void* stream, fwn_handle* out) {
    return guarded([&] {
        if (!out) throw Error(FWN_INVALID_ARG, "out is null");
        *out = nullptr;
        check_mesh_args(d_V, nv, d_F, nf);
        std::unique_ptr<Engine> e(new_engine(cfg));
        const int64_t voff[2] = {0, nv}, foff[2] = {0, nf};
        build_into(e.get(), d_V, voff, d_F, foff, 1, static_cast<cudaStream_t>(stream));
        *out = reinterpret_cast<fwn_handle>(e.release());
    });
}

FWN_API fwn_status fwn_destroy(fwn_handle h) {
    return guarded([&] {
        if (!h) return;
        delete reinterpret_cast<Engine*>(h);
    });
}

FWN_API fwn_status fwn_get_info(fwn_handle h, fwn_info* info) {
    return guarded([&] {
        Engine* e = engine_of(h);
        if (!info) throw Error(FWN_INVALID_ARG, "info is null");
        std::memset(info, 0, sizeof(*info));
        info->num_vertices = e->nv;
        info->num_triangles = e->nf;
        info->num_nodes = e->num_nodes;
        info->num_leaves = e->num_leaves;
        info->num_meshes = e->nmeshes;
        info->device_bytes = e->device_bytes;
        info->build_ms = e->build_ms;
        for (int a = 0; a < 3; ++a) {
            info->bbox_min[a] = e->meshes_h[0].lo[a];
            info->bbox_max[a] = e->meshes_h[0].hi[a];
        }
        info->leaf_size = e->cfg.leaf_size;
        info->records = e->cfg.records;
    });
}

FWN_API fwn_status fwn_query(fwn_handle h, const float* d_points, int64_t n, float* d_omega,
                             uint8_t* d_inside, void* stream) {
    return fwn_query_ex(h, nullptr, d_points, n, d_omega, d_inside, nullptr, nullptr, stream);
}

FWN_API fwn_status fwn_query_ex(fwn_handle h, const fwn_query_opts* opts, const float* d_points,
                                int64_t n, float* d_omega, uint8_t* d_inside, double* d_omega64,
                                fwn_query_stats* stats, void* stream) {
    return guarded([&] {
        Engine* e = engine_of(h);
        require_engine_device(*e);
        check_points(n, d_points);
        if (e->nmeshes != 1) throw Error(FWN_INVALID_ARG, "forest handle: use fwn_forest_query");
        QueryArgs a = resolve_query_args(*e, opts);
        query_mesh(*e, 0, a, d_points, n, d_omega, d_inside, d_omega64, stats,
                   static_cast<cudaStream_t>(stream));
    });
}

FWN_API fwn_status fwn_query_order(fwn_handle h, const float* d_points, int64_t n,
                                   uint32_t* d_order, void* stream) {
    return guarded([&] {
        Engine* e = engine_of(h);
        require_engine_device(*e);
        check_points(n, d_points);
        if (e->nmeshes != 1) throw Error(FWN_INVALID_ARG, "forest handle: build one engine per mesh");
        if (n > 0 && !d_order) throw Error(FWN_INVALID_ARG, "order pointer is null");
        query_order(*e, 0, d_points, n, d_order, static_cast<cudaStream_t>(stream));
    });
}

FWN_API fwn_status fwn_query_host(fwn_handle h, const float* points, int64_t n, float* omega,
                                  uint8_t* inside) {
    return guarded([&] {
        Engine* e = engine_of(h);
        require_engine_device(*e);
        check_points(n, points);
        if (e->nmeshes != 1) throw Error(FWN_INVALID_ARG, "forest handle: use fwn_forest_query");
        if (n == 0) return;
        QueryArgs a = resolve_query_args(*e, nullptr);
        const cudaStream_t st = host_stream();
        Scratch dq(n * 3 * sizeof(float), st);
        Scratch dw(omega ? n * sizeof(float) : 0, st);
        Scratch di(inside ? n * sizeof(uint8_t) : 0, st);
        FWN_CUDA_CHECK(cudaMemcpyAsync(dq.p, points, n * 3 * sizeof(float), cudaMemcpyHostToDevice, st));
        query_mesh(*e, 0, a, dq.as<float>(), n, dw.as<float>(), di.as<uint8_t>(), nullptr, nullptr,
                   st, /*check=*/true);
        if (omega) FWN_CUDA_CHECK(cudaMemcpyAsync(omega, dw.p, n * sizeof(float), cudaMemcpyDeviceToHost, st));
        if (inside) FWN_CUDA_CHECK(cudaMemcpyAsync(inside, di.p, n, cudaMemcpyDeviceToHost, st));
        FWN_CUDA_CHECK(cudaStreamSynchronize(st));
    });
}

FWN_API fwn_status fwn_query_host_batches(fwn_handle h, int64_t num_batches,
                                          const float* const* points, const int64_t* counts,
                                          float* const* omega, uint8_t* const* inside) {
    return guarded([&] {
        Engine* e = engine_of(h);
        require_engine_device(*e);
        if (e->nmeshes != 1) throw Error(FWN_INVALID_ARG, "forest handle: use fwn_forest_query");
        if (num_batches < 0) throw Error(FWN_INVALID_ARG, "num_batches must be >= 0");
        if (num_batches == 0) return;
        if (!points || !counts) throw Error(FWN_INVALID_ARG, "points or counts is null");
        int64_t nmax = 0;
        for (int64_t b = 0; b < num_batches; ++b) {
            check_points(counts[b], points[b]);
            nmax = std::max(nmax, counts[b]);
        }
        if (nmax == 0) return;
        QueryArgs a = resolve_query_args(*e, nullptr);
        const cudaStream_t st = host_stream(0), in_st = host_stream(1), out_st = host_stream(2);
        const cudaStream_t qst[2] = {st, host_stream(3)};  // slot s's batches run on qst[s]
        // two device slots: batch b copies into slot b % 2 while batch b - 1 runs in the other
        Scratch dq[2] = {Scratch(nmax * 3 * sizeof(float), st), Scratch(nmax * 3 * sizeof(float), st)};
        Scratch dw[2] = {Scratch(omega ? nmax * sizeof(float) : 0, st),
                         Scratch(omega ? nmax * sizeof(float) : 0, st)};
        Scratch di[2] = {Scratch(inside ? nmax : 0, st), Scratch(inside ? nmax : 0, st)};
        cudaEvent_t ev[7];  // slot buffers ready, batch in (x2), query done (x2), batch out (x2)
        for (cudaEvent_t& x : ev) FWN_CUDA_CHECK(cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
        std::unique_ptr<cudaEvent_t[], void (*)(cudaEvent_t*)> guard(
            new cudaEvent_t[7]{ev[0], ev[1], ev[2], ev[3], ev[4], ev[5], ev[6]}, [](cudaEvent_t* p) {
                for (int i = 0; i < 7; ++i) cudaEventDestroy(p[i]);
                delete[] p;
            });
        cudaEvent_t ready = ev[0], in_done[2] = {ev[1], ev[2]}, q_done[2] = {ev[3], ev[4]},
                    out_done[2] = {ev[5], ev[6]};
        // on every exit, an error included, the side streams finish before the slots (freed on
        // stream 0 when they go out of scope, after this guard) can be reused
        struct Drain {
            cudaStream_t s[3];
            ~Drain() {
                for (cudaStream_t x : s) cudaStreamSynchronize(x);
            }
        } drain{{in_st, out_st, qst[1]}};
        FWN_CUDA_CHECK(cudaEventRecord(ready, st));  // the slots' stream-ordered allocations
        FWN_CUDA_CHECK(cudaStreamWaitEvent(in_st, ready, 0));
        FWN_CUDA_CHECK(cudaStreamWaitEvent(out_st, ready, 0));
        FWN_CUDA_CHECK(cudaStreamWaitEvent(qst[1], ready, 0));
        for (int64_t b = 0; b < num_batches; ++b) {
            const int s = (int)(b & 1);
            const int64_t n = counts[b];
            if (b >= 2) {  // slot s was batch b - 2's: its points are read, its results out
                FWN_CUDA_CHECK(cudaStreamWaitEvent(in_st, q_done[s], 0));
                FWN_CUDA_CHECK(cudaStreamWaitEvent(qst[s], out_done[s], 0));
            }
            if (n > 0)
                FWN_CUDA_CHECK(cudaMemcpyAsync(dq[s].p, points[b], n * 3 * sizeof(float),
                                               cudaMemcpyHostToDevice, in_st));
            FWN_CUDA_CHECK(cudaEventRecord(in_done[s], in_st));
            FWN_CUDA_CHECK(cudaStreamWaitEvent(qst[s], in_done[s], 0));
            // the walk's consistency check (a corrupt tree shows in every batch) is read back
            // once, on the last batch, so that no batch waits for the host
            query_mesh(*e, 0, a, dq[s].as<float>(), n, dw[s].as<float>(), di[s].as<uint8_t>(),
                       nullptr, nullptr, qst[s], /*check=*/b == num_batches - 1);
            FWN_CUDA_CHECK(cudaEventRecord(q_done[s], qst[s]));
            FWN_CUDA_CHECK(cudaStreamWaitEvent(out_st, q_done[s], 0));
            if (n > 0 && omega && omega[b])
                FWN_CUDA_CHECK(cudaMemcpyAsync(omega[b], dw[s].p, n * sizeof(float),
                                               cudaMemcpyDeviceToHost, out_st));
            if (n > 0 && inside && inside[b])
                FWN_CUDA_CHECK(cudaMemcpyAsync(inside[b], di[s].p, n, cudaMemcpyDeviceToHost, out_st));
            FWN_CUDA_CHECK(cudaEventRecord(out_done[s], out_st));
        }
        FWN_CUDA_CHECK(cudaStreamSynchronize(out_st));
        FWN_CUDA_CHECK(cudaStreamSynchronize(in_st));
        FWN_CUDA_CHECK(cudaStreamSynchronize(qst[1]));
        // the slots are freed on stream 0 (stream-ordered) after every copy that used them
        FWN_CUDA_CHECK(cudaStreamWaitEvent(st, out_done[0], 0));
        FWN_CUDA_CHECK(cudaStreamWaitEvent(st, out_done[1], 0));
    });
}

FWN_API fwn_status fwn_export_tree(fwn_handle h, int32_t* skip, int32_t* tri_begin,
                                   int32_t* tri_count, double* center_radius, int32_t* sorted_tri,
                                   int32_t* mesh_root) {
    return guarded([&] {
        Engine* e = engine_of(h);
        const int64_t E = e->num_nodes;
        if (E > 0 && (skip || tri_begin || tri_count || center_radius)) {
            if (e->nodes32) {
                std::vector<NodeF32> nodes(E);
                FWN_CUDA_CHECK(cudaMemcpy(nodes.data(), e->nodes32, E * sizeof(NodeF32), cudaMemcpyDeviceToHost));
                for (int64_t i = 0; i < E; ++i) {
                    if (skip) skip[i] = nodes[i].skip;
                    if (tri_begin) tri_begin[i] = nodes[i].tri_begin;
                    if (tri_count) tri_count[i] = nodes[i].tri_count;
                    if (center_radius) {
                        center_radius[4 * i + 0] = nodes[i].s0.x;
                        center_radius[4 * i + 1] = nodes[i].s0.y;
                        center_radius[4 * i + 2] = nodes[i].s0.z;
                        center_radius[4 * i + 3] = nodes[i].s0.w;
                    }
                }
            } else {
                std::vector<NodeF64> nodes(E);
                FWN_CUDA_CHECK(cudaMemcpy(nodes.data(), e->nodes64, E * sizeof(NodeF64), cudaMemcpyDeviceToHost));
                for (int64_t i = 0; i < E; ++i) {
                    if (skip) skip[i] = nodes[i].skip;
                    if (tri_begin) tri_begin[i] = nodes[i].tri_begin;
                    if (tri_count) tri_count[i] = nodes[i].tri_count;
                    if (center_radius) {
                        for (int a = 0; a < 3; ++a) center_radius[4 * i + a] = nodes[i].P[a];
                        center_radius[4 * i + 3] = nodes[i].r;
                    }
                }
            }
        }
        if (sorted_tri && e->nf > 0)
            FWN_CUDA_CHECK(cudaMemcpy(sorted_tri, e->sorted_tri, e->nf * sizeof(int32_t), cudaMemcpyDeviceToHost));
        if (mesh_root)
            for (int64_t m = 0; m < e->nmeshes; ++m) {
                mesh_root[2 * m] = e->meshes_h[m].root;
                mesh_root[2 * m + 1] = e->meshes_h[m].end;
            }
    });
}

FWN_API fwn_status fwn_export_moments(fwn_handle h, double* moments) {
    return guarded([&] {
        Engine* e = engine_of(h);
        if (!moments) throw Error(FWN_INVALID_ARG, "moments is null");
        if (!e->stage && e->num_nodes > 0)
            throw Error(FWN_INVALID_ARG, "engine was built without FWN_RECORDS_MOMENTS");
        const int64_t E = e->num_nodes;
        std::vector<StageRec> recs(E);
        if (E) FWN_CUDA_CHECK(cudaMemcpy(recs.data(), e->stage, E * sizeof(StageRec), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < E; ++i) {
            double* o = moments + 33 * i;
            for (int a = 0; a < 3; ++a) o[a] = recs[i].P[a];
            for (int a = 0; a < 3; ++a) o[3 + a] = recs[i].N[a];
            for (int a = 0; a < 9; ++a) o[6 + a] = recs[i].M1[a];
            for (int a = 0; a < 18; ++a) o[15 + a] = recs[i].M2[a];
        }
    });
}

FWN_API fwn_status fwn_export_nodes(fwn_handle h, void* nodes32, void* nodes64) {
    return guarded([&] {
        Engine* e = engine_of(h);
        const int64_t E = e->num_nodes;
        if (nodes32 && !e->nodes32) throw Error(FWN_INVALID_ARG, "engine keeps no FP32 records");
        if (nodes64 && !e->nodes64) throw Error(FWN_INVALID_ARG, "engine keeps no FP64 records");
        if (E && nodes32)
            FWN_CUDA_CHECK(cudaMemcpy(nodes32, e->nodes32, E * sizeof(NodeF32), cudaMemcpyDeviceToHost));
        if (E && nodes64)
            FWN_CUDA_CHECK(cudaMemcpy(nodes64, e->nodes64, E * sizeof(NodeF64), cudaMemcpyDeviceToHost));
    });
}

FWN_API fwn_status fwn_forest_build(const float* V, const int64_t* voff, const int32_t* F,
                                    const int64_t* foff, int64_t nmeshes, const fwn_config* cfg,
                                    fwn_handle* out) {
    return guarded([&] {
        if (!out) throw Error(FWN_INVALID_ARG, "out is null");
        *out = nullptr;
        if (nmeshes < 1 || !voff || !foff) throw Error(FWN_INVALID_ARG, "bad forest offsets");
        const int64_t nv = voff[nmeshes], nf = foff[nmeshes];
        check_mesh_args(V, nv, F, nf);
        std::unique_ptr<Engine> e(new_engine(cfg));
        OwnedStream os;
        Scratch dv(nv * 3 * sizeof(float), os.s), df(nf * 3 * sizeof(int32_t), os.s);
        if (nv) FWN_CUDA_CHECK(cudaMemcpyAsync(dv.p, V, nv * 3 * sizeof(float), cudaMemcpyHostToDevice, os.s));
        if (nf) FWN_CUDA_CHECK(cudaMemcpyAsync(df.p, F, nf * 3 * sizeof(int32_t), cudaMemcpyHostToDevice, os.s));
        build_into(e.get(), dv.as<float>(), voff, df.as<int32_t>(), foff, nmeshes, os.s);
        FWN_CUDA_CHECK(cudaStreamSynchronize(os.s));
        *out = reinterpret_cast<fwn_handle>(e.release());
    });
}

FWN_API fwn_status fwn_forest_build_device(const float* d_V, const int64_t* voff,
                                           const int32_t* d_F, const int64_t* foff,
                                           int64_t nmeshes, const fwn_config* cfg, void* stream,
                                           fwn_handle* out) {
    return guarded([&] {
        if (!out) throw Error(FWN_INVALID_ARG, "out is null");
        *out = nullptr;
        if (nmeshes < 1 || !voff || !foff) throw Error(FWN_INVALID_ARG, "bad forest offsets");
        check_mesh_args(d_V, voff[nmeshes], d_F, foff[nmeshes]);
        std::unique_ptr<Engine> e(new_engine(cfg));
        build_into(e.get(), d_V, voff, d_F, foff, nmeshes, static_cast<cudaStream_t>(stream));
        *out = reinterpret_cast<fwn_handle>(e.release());
    });
}

FWN_API fwn_status fwn_forest_query(fwn_handle h, const float* d_points, const int64_t* qoff,
                                    float* d_omega, uint8_t* d_inside, const fwn_query_opts* opts,
                                    void* stream) {
    return guarded([&] {
        Engine* e = engine_of(h);
        require_engine_device(*e);
        if (!qoff) throw Error(FWN_INVALID_ARG, "query offsets are null");
        if (qoff[0] != 0) throw Error(FWN_INVALID_ARG, "query offsets must start at 0");
        for (int64_t m = 0; m < e->nmeshes; ++m)
            if (qoff[m + 1] < qoff[m]) throw Error(FWN_INVALID_ARG, "query offsets must not decrease");
        check_points(qoff[e->nmeshes], d_points);
        QueryArgs a = resolve_query_args(*e, opts);
        query_forest(*e, a, d_points, qoff, d_omega, d_inside, static_cast<cudaStream_t>(stream));
    });
}

FWN_API fwn_status fwn_scratch_pool_stats(int32_t device, int32_t reset_high,
                                          uint64_t* reserved_bytes, uint64_t* used_bytes,
                                          uint64_t* used_high_bytes) {
    return guarded([&] {
        scratch_pool_stats(device, reset_high != 0, reserved_bytes, used_bytes, used_high_bytes);
    });
}

FWN_API fwn_status fwn_forest_sort_key_bits(int64_t num_meshes, const int64_t* qoff,
                                            int32_t* key_bits) {
    return guarded([&] {
        if (num_meshes < 1 || !qoff || !key_bits) throw Error(FWN_INVALID_ARG, "bad arguments");
        if (qoff[0] != 0) throw Error(FWN_INVALID_ARG, "query offsets must start at 0");
        for (int64_t m = 0; m < num_meshes; ++m)
            if (qoff[m + 1] < qoff[m]) throw Error(FWN_INVALID_ARG, "query offsets must not decrease");
        *key_bits = forest_keys(num_meshes, qoff).key_bits;
    });
}

}  // extern "C"
