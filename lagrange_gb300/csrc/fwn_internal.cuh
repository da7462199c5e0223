// Internal declarations of the GB300 fast-winding-number engine (not part of the C ABI).
//
// Data layout in HBM (all arrays are device allocations owned by the engine):
//   NodeF32[num_nodes]  128 B records in DFS pre-order (traversal order). Sector 0 (32 B) holds
//                       what the far test and the skip walk need; sectors 1-3 (96 B) hold the
//                       order-0/1/2 far-field coefficients, read only when the node is far.
//   NodeF64[num_nodes]  256 B FP64 records of the same tree (plain FP64 form).
//   TriF32[num_tris]    48 B records, leaf triangles in Morton (= DFS leaf) order, so a leaf's
//                       triangles are one contiguous run.
//   MeshInfo[num_meshes] per-mesh root/end node, bbox and FP64 near-field radius.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stddef.h>
#include <stdint.h>

#include <stdexcept>
#include <string>

#include "../../include/fwn_gb300.h"

namespace fwn {

// ---------------------------------------------------------------------------------------------
// Records
// ---------------------------------------------------------------------------------------------

// Far-field coefficients are pre-scaled so that, with d = P - q (centre minus query) and
// R = |d|, the order-2 expansion of the solid angle is
//   T = R^-3 (d.N + trM1) + R^-5 (d^T C d + W.d) + R^-7 (sum_m D_m * monomial_m(d)).
// Derivation (Barill et al. 2018, "Fast Winding Numbers for Soups and Clouds", eq. for the
// dipole expansion): Omega = sum_t int (x-q).n/|x-q|^3 dA; expand K(r)=r/|r|^3 about d:
//   order 0: K(d).N
//   order 1: sum_ij M1_ij dK_i/dd_j = trM1/R^3 - 3 d^T M1 d/R^5
//   order 2: 1/2 sum_ijk M2_ijk d2K_i/dd_j dd_k = -3/2 (2u+v).d/R^5 + 15/2 S(d)/R^7
// with N = sum a_t n_t, M1_ij = sum n_i int (x-P)_j, M2_ijk = sum n_i int (x-P)_j (x-P)_k,
// u_k = sum_i M2_iik, v_i = sum_j M2_ijj, S(d) = sum_ijk M2_ijk d_i d_j d_k.
// So C = -3 sym(M1) (off-diagonals doubled), W = -3/2 (2u+v), D = 15/2 * monomial sums of M2.
struct __align__(128) NodeF32 {
    float4 s0;   // P.x P.y P.z r
    int skip;    // index of the next node when this subtree is skipped (DFS escape link)
    int tri_begin;
    int tri_count;  // 0 for internal nodes
    float trM1;
    float4 m0;   // N.x N.y N.z W.x
    float4 m1;   // W.y W.z Cxx Cyy
    float4 m2;   // Czz Cxy Cxz Cyz
    float4 m3;   // Dxxx Dyyy Dzzz Dxxy
    float4 m4;   // Dxxz Dxyy Dyyz Dxzz
    float4 m5;   // Dyzz Dxyz 0 0
};
static_assert(sizeof(NodeF32) == 128, "NodeF32 must be one 128 B line");

struct __align__(16) NodeF64 {
    double P[3];
    double r;
    int skip;
    int tri_begin;
    int tri_count;
    int pad0;
    double trM1;
    double N[3];
    double W[3];
    double C[6];   // xx yy zz xy xz yz
    double D[10];  // xxx yyy zzz xxy xxz xyy yyz xzz yzz xyz
    double pad1[3];
};
static_assert(sizeof(NodeF64) == 256, "NodeF64 must be 256 B");

// Triangle record: vertices (float, exact copies of the input), the radius of the bounding
// sphere about the centroid (rounded up) and 1/|(v1-v0)x(v2-v0)| (0 when degenerate).
struct __align__(16) TriF32 {
    float4 t0;  // v0.x v0.y v0.z v1.x
    float4 t1;  // v1.y v1.z v2.x v2.y
    float4 t2;  // v2.z Rt inv_nlen 0
};
static_assert(sizeof(TriF32) == 48, "TriF32 must be 48 B");

struct MeshInfo {
    int root;          // first node of the mesh's subtree (-1: empty mesh)
    int end;           // escape index of the root (one past the subtree)
    float tau;         // FP64 near-field distance: fp64_near_scale * bbox diagonal
    float cond;        // FP64 near-field condition threshold (fwn_config::fp64_cond)
    float lo[3];       // vertex bbox
    float hi[3];
    float inv_ext[3];  // 1/(hi-lo) per axis (0 for flat axes), Morton normalisation
    float pad2;
};

// FP64 staging record written by the refit (one per emitted node, indexed by DFS position).
struct __align__(32) StageRec {
    double P[3];     // expansion centre (a float value, see refit)
    double area;
    double N[3];
    double M1[9];    // [i*3+j], i: normal component, j: offset component
    double M2[18];   // [i*6+s], s: xx yy zz xy xz yz
    double r;        // radius about P: farthest vertex of the node's triangles (a float value,
                     // rounded up); internal nodes get it after the refit (k_node_radius)
    double pad;      // 288 B: records start on 32 B sectors, so reads of one record share them
};
static_assert(sizeof(StageRec) == 288, "StageRec must be 9 sectors");
static_assert(offsetof(StageRec, area) == 24 && offsetof(StageRec, N) == 32 &&
                  offsetof(StageRec, M1) == 56 && offsetof(StageRec, M2) == 128,
              "the refit reads a record as P, area, N, M1 (128 B) then M2, in 16 B pairs");

// ---------------------------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------------------------

struct Error : std::runtime_error {
    fwn_status status;
    Error(fwn_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void set_last_error(const std::string& msg);

#define FWN_CUDA_CHECK(expr)                                                                   \
    do {                                                                                       \
        cudaError_t _e = (expr);                                                               \
        if (_e != cudaSuccess) {                                                               \
            throw ::fwn::Error(_e == cudaErrorMemoryAllocation ? FWN_OOM : FWN_CUDA_ERROR,     \
                               std::string(#expr) + ": " + cudaGetErrorString(_e) + " (" +     \
                                   __FILE__ + ":" + std::to_string(__LINE__) + ")");           \
        }                                                                                      \
    } while (0)

// Device status word bits (set by kernels, read by the host after a launch).
enum : unsigned {
    ST_BAD_INDEX = 1u,       // triangle index out of [0, nv)
    ST_NONFINITE = 2u,       // referenced vertex coordinate is NaN/inf
    ST_BAD_LINK = 4u,        // traversal met a skip link that does not advance
    ST_REFIT_ORPHAN = 8u,    // refit inconsistency (missing child or parent)
    ST_BUILD_BOUND = 16u     // a split build passed its node or depth bound
};

// ---------------------------------------------------------------------------------------------
// Tracing: an NVTX range over a host-side phase (build stages, query sort / walk). The ranges
// mark when each phase is enqueued; a profiler such as Nsight Systems lines them up with the
// kernels they launch. Without a profiler attached an NVTX call returns at once.
// ---------------------------------------------------------------------------------------------
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// ---------------------------------------------------------------------------------------------
// Stream-ordered scratch buffer
// ---------------------------------------------------------------------------------------------
// Scratch comes from a memory pool per device owned by the library, which keeps up to
// kScratchRetainBytes of freed memory across synchronisations. (The device's default pool
// returns freed memory to the driver at every synchronisation, so a host-synchronous call would
// map all of its scratch again on every call.) During stream capture the allocation goes to the
// default pool instead, so that it becomes a graph memory node. Freed with cudaFreeAsync.
constexpr uint64_t kScratchRetainBytes = uint64_t(8) << 30;
void* scratch_alloc(size_t bytes, cudaStream_t stream);
// Build temporaries come from a second pool of the same kind, which keeps up to
// kBuildRetainBytes mapped for the next build (a 42M-triangle forest's are ~10 GB).
constexpr uint64_t kBuildRetainBytes = uint64_t(12) << 30;
void* build_alloc(size_t bytes, cudaStream_t stream);

struct Scratch {
    void* p = nullptr;
    cudaStream_t s = 0;
    Scratch() = default;
    Scratch(size_t bytes, cudaStream_t st) : s(st) {
        if (bytes) p = scratch_alloc(bytes, st);
    }
    Scratch(const Scratch&) = delete;
    Scratch& operator=(const Scratch&) = delete;
    ~Scratch() {
        if (p) cudaFreeAsync(p, s);
    }
    template <class T> T* as() const { return static_cast<T*>(p); }
};

// ---------------------------------------------------------------------------------------------
// Radix sort (radix_sort.cu): stable LSD sort of (key, value) pairs, 8-bit digits.
// Sorts keys_a/vals_a using keys_b/vals_b as ping-pong buffers; returns true when the result
// ended in the *_b buffers. temp holds 256 digit counts per tile of kSortTileKeys keys, plus the
// 256 digit totals (radix_sort_temp_bytes).
// ---------------------------------------------------------------------------------------------
constexpr int kSortTileKeys = 2048;  // keys per sort tile: 256 threads x 8 keys
size_t radix_sort_temp_bytes(int64_t n, int key_bytes);
bool radix_sort_u32(uint32_t* keys_a, uint32_t* vals_a, uint32_t* keys_b, uint32_t* vals_b,
                    int64_t n, int key_bits, void* temp, cudaStream_t stream);
bool radix_sort_u64(uint64_t* keys_a, uint32_t* vals_a, uint64_t* keys_b, uint32_t* vals_b,
                    int64_t n, int key_bits, void* temp, cudaStream_t stream);

// Exclusive scan of n int32 values in place (radix_sort.cu).
size_t exclusive_scan_temp_bytes(int64_t n);
void exclusive_scan_i32(int* data, int64_t n, void* temp, cudaStream_t stream);

// ---------------------------------------------------------------------------------------------
// Engine
// ---------------------------------------------------------------------------------------------
struct Engine {
    fwn_config cfg;
    int64_t nv = 0, nf = 0, nmeshes = 0;
    int64_t num_nodes = 0, num_leaves = 0;
    NodeF32* nodes32 = nullptr;
    NodeF64* nodes64 = nullptr;
    float4* soa = nullptr;         // the FP32 records as 8 float4 arrays (tuning 7 builds only)
    TriF32* tris = nullptr;
    int* sorted_tri = nullptr;     // original triangle id per leaf slot
    MeshInfo* meshes = nullptr;    // device
    MeshInfo* meshes_h = nullptr;  // host copy
    StageRec* stage = nullptr;     // kept only when FWN_RECORDS_MOMENTS is requested
    int* node_tri_begin_h = nullptr;
    double build_ms = 0.0;
    int64_t device_bytes = 0;
    int device = 0;
    ~Engine();
};

// Throws FWN_INVALID_ARG naming the first field of c out of range (fwn_capi.cu).
void validate_config(const fwn_config& c);

// Queries launch on the current device with the engine's device pointers, so the current device
// must be the one the engine was built on (a stream passed by the caller belongs to it as well).
inline void require_engine_device(const Engine& e) {
    int dev = 0;
    FWN_CUDA_CHECK(cudaGetDevice(&dev));
    if (dev != e.device)
        throw Error(FWN_INVALID_ARG, "the engine was built on device " + std::to_string(e.device) +
                                         " but the current device is " + std::to_string(dev));
}

// lbvh_build.cu: builds the forest. d_vertices / d_triangles are device arrays with LOCAL
// indices per mesh; offsets are host arrays of num_meshes+1 entries.
void build_forest(Engine& e, const float* d_vertices, const int64_t* vertex_offsets,
                  const int32_t* d_triangles, const int64_t* triangle_offsets,
                  int64_t num_meshes, cudaStream_t stream);

// traverse.cu: single-mesh style query over queries of mesh `mesh` (forest queries use
// query_forest). Outputs may be null.
struct QueryArgs {
    int precision = FWN_PRECISION_MIXED;
    int traversal = FWN_TRAVERSAL_THREAD;
    int block_size = 128;
    int sort_queries = 1;
    float beta = 2.0f;
    int tuning = 0;
};
// `check` (or a non-null `stats`) synchronises the stream and turns device status bits into
// errors.
void query_mesh(const Engine& e, int mesh, const QueryArgs& a, const float* d_points, int64_t n,
                float* d_omega, uint8_t* d_inside, double* d_omega64, fwn_query_stats* stats,
                cudaStream_t stream, bool check = false);
// Regular voxel-centre grid of mesh `mesh` (no point array); outputs indexed i + nx (j + ny k).
void query_grid(const Engine& e, int mesh, const QueryArgs& a, const float origin[3],
                const float spacing[3], const int64_t dims[3], float* d_omega, uint8_t* d_inside,
                cudaStream_t stream);
void query_forest(const Engine& e, const QueryArgs& a, const float* d_points,
                  const int64_t* query_offsets, float* d_omega, uint8_t* d_inside,
                  cudaStream_t stream);

QueryArgs resolve_query_args(const Engine& e, const fwn_query_opts* opts);

// Sort keys of the forest query for host query offsets [nmeshes + 1]: 32-bit keys (narrow) hold
// the mesh id above the top hilbert_bits of the 30-bit Hilbert index, 64-bit keys all 30 bits.
struct ForestKeys {
    int mesh_bits = 0, hilbert_bits = 30, key_bits = 30;
    bool narrow = true;
};
ForestKeys forest_keys(int64_t nmeshes, const int64_t* query_offsets);

// The permutation query_mesh applies when sort_queries is set (Hilbert-curve order of the points in
// mesh `mesh`'s frame): d_order[k] = index of the k-th point. Async.
void query_order(const Engine& e, int mesh, const float* d_points, int64_t n, uint32_t* d_order,
                 cudaStream_t stream);

// Query with caller-provided device scratch (no allocation): `scratch` holds the status word and
// the query-sort buffers, at least query_prealloc_bytes(n) bytes, 256-byte aligned. Async.
size_t query_prealloc_bytes(int64_t n);
void query_mesh_prealloc(const Engine& e, int mesh, const QueryArgs& a, const float* d_points,
                         int64_t n, float* d_omega, uint8_t* d_inside, void* scratch,
                         size_t scratch_bytes, cudaStream_t stream);

}  // namespace fwn
