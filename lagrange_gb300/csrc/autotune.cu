// Autotuner: picks the tree builder and leaf size (build), the traversal schedule, block size
// and warp-schedule variant (queries per lane, register cap) for one mesh and a representative
// query sample, by timing every candidate with CUDA events on the device. beta does not enter the choice (the schedule and block shape are
// tuned at the caller's beta, which only changes how deep the walk goes).
//
// Optional cache: a text file with one line per (GPU name, log2 triangles, log2 queries) key:
//   t2|<gpu name>|<log2 nf>|<log2 n> <leaf> <traversal> <block> <tuning> <builder> <ms>
// A hit skips the timing; a miss appends the new line.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "fwn_internal.cuh"

namespace fwn {
namespace {

struct Candidate {
    int traversal, block, tuning;
};

const Candidate kCandidates[] = {
    {FWN_TRAVERSAL_WARP, 128, 3},    // warp cursor, 1 query per lane, 64-register cap
    {FWN_TRAVERSAL_WARP, 128, 1},    // 1 query per lane, 72-register cap
    {FWN_TRAVERSAL_WARP, 128, 2},    // 1 query per lane, no register cap
    {FWN_TRAVERSAL_WARP, 128, 4},    // 2 queries per lane, 64-register cap
    {FWN_TRAVERSAL_WARP, 128, 5},    // 2 queries per lane, 80-register cap
    {FWN_TRAVERSAL_WARP, 128, 6},    // 2 queries per lane, 64-register cap, paired Taylor terms
    {FWN_TRAVERSAL_THREAD, 64, 0},   // thread per query
    {FWN_TRAVERSAL_THREAD, 128, 0},
    {FWN_TRAVERSAL_THREAD, 256, 0},
};
const int kLeafSizes[] = {4, 8, 12, 16};
// One mesh (queried many times) tries all three builders; a forest, built for each batch, the two
// whose build suits that (the binned splits add a binning pass per level for ~2% on the query).
const int kBuilders[] = {FWN_BUILDER_LBVH, FWN_BUILDER_SPLIT, FWN_BUILDER_BINNED};
const int kForestBuilders[] = {FWN_BUILDER_LBVH, FWN_BUILDER_SPLIT};

std::mutex g_cache_mutex;

int log2_bucket(int64_t x) {
    int b = 0;
    while (x > 1) {
        x >>= 1;
        ++b;
    }
    return b;
}

std::string cache_key(int64_t nf, int64_t n) {
    int dev = 0;
    cudaDeviceProp prop;
    FWN_CUDA_CHECK(cudaGetDevice(&dev));
    FWN_CUDA_CHECK(cudaGetDeviceProperties(&prop, dev));
    std::string name(prop.name);
    for (char& ch : name)
        if (ch == ' ' || ch == '|') ch = '_';
    return "t2|" + name + "|" + std::to_string(log2_bucket(nf)) + "|" + std::to_string(log2_bucket(n));
}

bool cache_lookup(const char* path, const std::string& key, fwn_tune_result* out) {
    std::lock_guard<std::mutex> lock(g_cache_mutex);
    std::ifstream f(path);
    if (!f) return false;
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string k;
        fwn_tune_result r;
        std::memset(&r, 0, sizeof(r));
        if (!(is >> k >> r.leaf_size >> r.traversal >> r.block_size >> r.tuning >> r.builder >> r.ms))
            continue;
        // an entry a caller could not apply (edited or damaged file) is ignored: tune again
        if (r.leaf_size < 1 || r.leaf_size > 16 || r.traversal < FWN_TRAVERSAL_AUTO ||
            r.traversal > FWN_TRAVERSAL_WARP || r.block_size < 0 || r.block_size > 1024 ||
            r.block_size % 32 != 0 || r.tuning < 0 || r.tuning > 6 ||
            (r.builder != FWN_BUILDER_LBVH && r.builder != FWN_BUILDER_SPLIT &&
             r.builder != FWN_BUILDER_BINNED))
            continue;
        if (k == key) {
            r.from_cache = 1;
            *out = r;
            return true;
        }
    }
    return false;
}

void cache_store(const char* path, const std::string& key, const fwn_tune_result& r) {
    std::lock_guard<std::mutex> lock(g_cache_mutex);
    std::ofstream f(path, std::ios::app);
    if (!f) return;  // a read-only cache location only loses the caching
    f << key << " " << r.leaf_size << " " << r.traversal << " " << r.block_size << " " << r.tuning
      << " " << r.builder << " " << r.ms << "\n";
}

}  // namespace
}  // namespace fwn

using namespace fwn;

extern "C" FWN_API fwn_status fwn_autotune(const float* d_V, int64_t nv, const int32_t* d_F,
                                           int64_t nf, const float* d_Q, int64_t n,
                                           const fwn_config* base, const char* cache_path,
                                           fwn_tune_result* out, void* stream) {
    try {
        if (!out) throw Error(FWN_INVALID_ARG, "out is null");
        std::memset(out, 0, sizeof(*out));
        if (nv < 0 || nf < 0 || n <= 0) throw Error(FWN_INVALID_ARG, "sizes must be >= 0 (n > 0)");
        if ((nv && !d_V) || (nf && !d_F) || !d_Q) throw Error(FWN_INVALID_ARG, "null pointer");
        if (n > (int64_t)INT32_MAX) throw Error(FWN_INVALID_ARG, "at most 2^31-1 sample points");
        fwn_config cfg;
        fwn_config_default(&cfg);
        if (base) cfg = *base;
        cfg.records = FWN_RECORDS_F32;
        const std::string key = cache_key(nf, n);
        if (cache_path && cache_lookup(cache_path, key, out)) return FWN_OK;
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        Scratch wbuf((size_t)n * sizeof(float), st), ibuf((size_t)n, st);
        cudaEvent_t e0, e1;
        FWN_CUDA_CHECK(cudaEventCreate(&e0));
        FWN_CUDA_CHECK(cudaEventCreate(&e1));
        std::unique_ptr<cudaEvent_t[], void (*)(cudaEvent_t*)> guard(
            new cudaEvent_t[2]{e0, e1}, [](cudaEvent_t* p) {
                cudaEventDestroy(p[0]);
                cudaEventDestroy(p[1]);
                delete[] p;
            });
        fwn_tune_result best;
        std::memset(&best, 0, sizeof(best));
        best.ms = 1e300;
        int evaluated = 0;
        for (int builder : kBuilders)
        for (int leaf : kLeafSizes) {
            Engine e;
            e.cfg = cfg;
            e.cfg.leaf_size = leaf;
            e.cfg.builder = builder;
            FWN_CUDA_CHECK(cudaGetDevice(&e.device));
            const int64_t voff[2] = {0, nv}, foff[2] = {0, nf};
            build_forest(e, d_V, voff, d_F, foff, 1, st);
            for (const Candidate& cand : kCandidates) {
                QueryArgs a = resolve_query_args(e, nullptr);
                a.precision = FWN_PRECISION_MIXED;
                a.traversal = cand.traversal;
                a.block_size = cand.traversal == FWN_TRAVERSAL_WARP ? 128 : cand.block;
                a.tuning = cand.tuning;
                // one warm-up, then the median of three timed passes
                query_mesh(e, 0, a, d_Q, n, wbuf.as<float>(), ibuf.as<uint8_t>(), nullptr,
                           nullptr, st);
                float t[3];
                for (int r = 0; r < 3; ++r) {
                    FWN_CUDA_CHECK(cudaEventRecord(e0, st));
                    query_mesh(e, 0, a, d_Q, n, wbuf.as<float>(), ibuf.as<uint8_t>(), nullptr,
                               nullptr, st);
                    FWN_CUDA_CHECK(cudaEventRecord(e1, st));
                    FWN_CUDA_CHECK(cudaEventSynchronize(e1));
                    FWN_CUDA_CHECK(cudaEventElapsedTime(&t[r], e0, e1));
                }
                std::sort(t, t + 3);
                ++evaluated;
                if (t[1] < best.ms) {
                    best.ms = t[1];
                    best.leaf_size = leaf;
                    best.traversal = a.traversal;
                    best.block_size = a.block_size;
                    best.tuning = a.tuning;
                    best.builder = builder;
                }
            }
        }
        best.candidates = evaluated;
        *out = best;
        if (cache_path) cache_store(cache_path, key, best);
        return FWN_OK;
    } catch (const Error& err) {
        set_last_error(err.what());
        return err.status;
    } catch (const std::exception& err) {
        set_last_error(err.what());
        return FWN_INTERNAL;
    } catch (...) {
        set_last_error("unknown error");
        return FWN_INTERNAL;
    }
}

// Forest form: the mixed forest query is one persistent kernel, so its knobs are the leaf size
// and the warp-schedule variant (queries per lane, register cap). Each leaf size builds the whole
// forest; each (leaf, variant) pair times the forest query on the caller's queries (median of
// three after a warm-up).
extern "C" FWN_API fwn_status fwn_forest_autotune(const float* d_V, const int64_t* vertex_offsets,
                                                  const int32_t* d_F,
                                                  const int64_t* triangle_offsets,
                                                  int64_t num_meshes, const float* d_Q,
                                                  const int64_t* query_offsets,
                                                  const fwn_config* base, const char* cache_path,
                                                  fwn_tune_result* out, void* stream) {
    try {
        if (!out) throw Error(FWN_INVALID_ARG, "out is null");
        std::memset(out, 0, sizeof(*out));
        if (num_meshes < 1) throw Error(FWN_INVALID_ARG, "num_meshes must be >= 1");
        if (!vertex_offsets || !triangle_offsets || !query_offsets)
            throw Error(FWN_INVALID_ARG, "offset arrays are null");
        const int64_t nv = vertex_offsets[num_meshes], nf = triangle_offsets[num_meshes];
        const int64_t n = query_offsets[num_meshes];
        if (nv < 0 || nf < 0 || n <= 0) throw Error(FWN_INVALID_ARG, "sizes must be >= 0 (queries > 0)");
        if ((nv && !d_V) || (nf && !d_F) || !d_Q) throw Error(FWN_INVALID_ARG, "null pointer");
        for (int64_t m = 0; m < num_meshes; ++m)
            if (vertex_offsets[m + 1] < vertex_offsets[m] || triangle_offsets[m + 1] < triangle_offsets[m] ||
                query_offsets[m + 1] < query_offsets[m])
                throw Error(FWN_INVALID_ARG, "offsets must be non-decreasing");
        fwn_config cfg;
        fwn_config_default(&cfg);
        if (base) cfg = *base;
        cfg.records = FWN_RECORDS_F32;
        const std::string key = "forest|" + cache_key(nf, n) + "|" + std::to_string(log2_bucket(num_meshes));
        if (cache_path && cache_lookup(cache_path, key, out)) return FWN_OK;
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        Scratch wbuf((size_t)n * sizeof(float), st), ibuf((size_t)n, st);
        cudaEvent_t e0, e1;
        FWN_CUDA_CHECK(cudaEventCreate(&e0));
        FWN_CUDA_CHECK(cudaEventCreate(&e1));
        std::unique_ptr<cudaEvent_t[], void (*)(cudaEvent_t*)> guard(
            new cudaEvent_t[2]{e0, e1}, [](cudaEvent_t* p) {
                cudaEventDestroy(p[0]);
                cudaEventDestroy(p[1]);
                delete[] p;
            });
        fwn_tune_result best;
        std::memset(&best, 0, sizeof(best));
        best.ms = 1e300;
        int evaluated = 0;
        for (int builder : kForestBuilders)
        for (int leaf : kLeafSizes) {
            Engine e;
            e.cfg = cfg;
            e.cfg.leaf_size = leaf;
            e.cfg.builder = builder;
            FWN_CUDA_CHECK(cudaGetDevice(&e.device));
            build_forest(e, d_V, vertex_offsets, d_F, triangle_offsets, num_meshes, st);
            for (int tuning : {3, 1, 4, 5, 6}) {  // warp-schedule variants (queries per lane, cap)
                QueryArgs a = resolve_query_args(e, nullptr);
                a.precision = FWN_PRECISION_MIXED;
                a.tuning = tuning;
                query_forest(e, a, d_Q, query_offsets, wbuf.as<float>(), ibuf.as<uint8_t>(), st);
                float t[3];
                for (int r = 0; r < 3; ++r) {
                    FWN_CUDA_CHECK(cudaEventRecord(e0, st));
                    query_forest(e, a, d_Q, query_offsets, wbuf.as<float>(), ibuf.as<uint8_t>(), st);
                    FWN_CUDA_CHECK(cudaEventRecord(e1, st));
                    FWN_CUDA_CHECK(cudaEventSynchronize(e1));
                    FWN_CUDA_CHECK(cudaEventElapsedTime(&t[r], e0, e1));
                }
                std::sort(t, t + 3);
                ++evaluated;
                if (t[1] < best.ms) {
                    best.ms = t[1];
                    best.leaf_size = leaf;
                    best.traversal = FWN_TRAVERSAL_WARP;
                    best.block_size = 128;
                    best.tuning = tuning;
                    best.builder = builder;
                }
            }
        }
        best.candidates = evaluated;
        *out = best;
        if (cache_path) cache_store(cache_path, key, best);
        return FWN_OK;
    } catch (const Error& err) {
        set_last_error(err.what());
        return err.status;
    } catch (const std::exception& err) {
        set_last_error(err.what());
        return FWN_INTERNAL;
    } catch (...) {
        set_last_error("unknown error");
        return FWN_INTERNAL;
    }
}
