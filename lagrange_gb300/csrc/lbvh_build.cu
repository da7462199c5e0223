// LBVH build of the winding-number forest (replaces the tree + moment precompute done by
// UT_SolidAngle<float,float>::init, called at modules/winding/src/FastWindingNumber.cpp:57).
//
// Stages (each ONE launch over all meshes of the forest):
//   K0  per-mesh vertex bbox (ordered-int atomics), mesh info (Morton frame, FP64 radius)
//   K1  triangle keys: (mesh id << 30) | 30-bit Morton code of the float centroid
//   K2  device radix sort of (key, triangle id)                       (radix_sort.cu)
//   K3  Karras 2012 binary radix tree over the sorted keys (equal keys tie-broken by index)
//   K3b collapse subtrees of <= leaf_size triangles into leaves and assign DFS pre-order
//       positions + escape ("skip") links with one scan:  pos(v) = base[first(v)] + rank(v),
//       skip(v) = base[last(v)+1], where base = exclusive scan of #emitted nodes per first leaf
//       and rank(v) = #ancestors sharing first(v)
//   K4  bottom-up FP64 refit of order-0/1/2 moments: leaves grouped by triangle count, one
//       thread each; parents by recentring children, level by level over dense lists (split
//       tree: its levels; LBVH: node heights from an integer atomic-counter ascent)
//   K4a exact node radii (farthest vertex, float screen + FP64 terms for the candidates), then
//       conversion to 128 B FP32 / 256 B FP64 records in DFS order
// The alternative top-down builders (FWN_BUILDER_SPLIT, FWN_BUILDER_BINNED) replace K1-K3b with
// level-synchronous splits of each segment's centroid box (its midpoint; or, for the binned
// builder and segments of the level loop, the binned plane of least cost) and share K4-K4a.
//
// This translation unit is compiled with -fmad=false: every floating-point operation is
// individually rounded, in the order written, so the CPU restatement of the same build
// (oracle/fwn_oracle.c, compiled with -ffp-contract=off) reproduces keys, topology, centres and
// radii bit for bit.
#include <cmath>
#include <utility>
#include <vector>

#include "fwn_internal.cuh"

namespace fwn {
namespace {

constexpr int MORTON_BITS = 30;

__device__ __forceinline__ unsigned enc_float(float f) {
    unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__host__ __device__ __forceinline__ float dec_float(unsigned u) {
    unsigned b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, 4);
    return f;
#endif
}

// Spreads the low 10 bits of x so that bit k moves to bit 3k.
__device__ __forceinline__ unsigned spread3(unsigned x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

__device__ __forceinline__ unsigned quantize10(float c, float lo, float inv) {
    float u = (c - lo) * inv;
    float s = u * 1024.0f;
    int q = (s >= 0.0f) ? (int)floorf(s) : 0;  // also maps NaN to 0
    return (unsigned)min(q, 1023);
}

__device__ __forceinline__ int find_mesh(const int64_t* off, int nmeshes, int64_t x) {
    // last m with off[m] <= x (offsets non-decreasing; empty meshes skipped naturally)
    int lo = 0, hi = nmeshes - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (off[mid] <= x) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ---- K0: per-mesh vertex bbox -----------------------------------------------------------------
__global__ void k_mesh_bbox(const float* __restrict__ V, const int64_t* __restrict__ voff,
                            int chunk, unsigned* __restrict__ enc) {
    const int m = blockIdx.y;
    const int64_t v0 = voff[m] + (int64_t)blockIdx.x * chunk;
    const int64_t v1 = min(voff[m + 1], v0 + chunk);
    if (v0 >= v1) return;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float x = V[3 * v + a];
            lo[a] = fminf(lo[a], x);  // fminf/fmaxf ignore NaN
            hi[a] = fmaxf(hi[a], x);
        }
    }
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            atomicMin(&enc[6 * m + a], enc_float(lo[a]));
            atomicMax(&enc[6 * m + 3 + a], enc_float(hi[a]));
        }
    }
}

__global__ void k_init_bbox(unsigned* enc, int nmeshes) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 6 * nmeshes) enc[i] = (i % 6) < 3 ? 0xffffffffu : 0u;
}

__global__ void k_mesh_info(const unsigned* __restrict__ enc, const int64_t* __restrict__ voff,
                            int nmeshes, float near_scale, float cond,
                            MeshInfo* __restrict__ mi) {
    int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmeshes) return;
    MeshInfo r;
    r.root = -1;
    r.end = -1;
    r.cond = cond;
    r.pad2 = 0.f;
    const bool has = voff[m + 1] > voff[m];
    float diag2 = 0.f;
    for (int a = 0; a < 3; ++a) {
        float lo = has ? dec_float(enc[6 * m + a]) : 0.f;
        float hi = has ? dec_float(enc[6 * m + 3 + a]) : 0.f;
        if (!(lo <= hi)) { lo = 0.f; hi = 0.f; }  // all-NaN axis
        r.lo[a] = lo;
        r.hi[a] = hi;
        float ext = hi - lo;
        r.inv_ext[a] = ext > 0.f ? 1.0f / ext : 0.f;
        diag2 = diag2 + ext * ext;
    }
    r.tau = near_scale * sqrtf(diag2);
    mi[m] = r;
}

// ---- K1: triangle keys ------------------------------------------------------------------------
__global__ void k_tri_keys(const float* __restrict__ V, const int32_t* __restrict__ F,
                           const int64_t* __restrict__ voff, const int64_t* __restrict__ foff,
                           int nmeshes, int64_t nf, const MeshInfo* __restrict__ mi,
                           uint64_t* __restrict__ keys, uint32_t* __restrict__ vals,
                           unsigned* __restrict__ status) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nf) return;
    const int m = find_mesh(foff, nmeshes, t);
    const int64_t nvm = voff[m + 1] - voff[m];
    float c[3] = {0.f, 0.f, 0.f};
    bool ok = true;
    int32_t idx[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        idx[j] = F[3 * t + j];
        if (idx[j] < 0 || (int64_t)idx[j] >= nvm) ok = false;
    }
    if (!ok) {
        atomicOr(status, ST_BAD_INDEX);
    } else {
        float v[3][3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float* p = V + 3 * (voff[m] + idx[j]);
            v[j][0] = p[0];
            v[j][1] = p[1];
            v[j][2] = p[2];
            if (!isfinite(v[j][0]) || !isfinite(v[j][1]) || !isfinite(v[j][2])) ok = false;
        }
        if (!ok) atomicOr(status, ST_NONFINITE);
#pragma unroll
        for (int a = 0; a < 3; ++a) c[a] = ((v[0][a] + v[1][a]) + v[2][a]) / 3.0f;
    }
    const MeshInfo& M = mi[m];
    unsigned code = (spread3(quantize10(c[0], M.lo[0], M.inv_ext[0])) << 2) |
                    (spread3(quantize10(c[1], M.lo[1], M.inv_ext[1])) << 1) |
                    spread3(quantize10(c[2], M.lo[2], M.inv_ext[2]));
    keys[t] = ((uint64_t)m << MORTON_BITS) | code;
    vals[t] = (uint32_t)t;
}

// ---- K3: Karras hierarchy ---------------------------------------------------------------------
// Node ids: internal nodes 0..n-2, leaf k -> n-1+k. Root is 0 (internal 0, or leaf 0 if n==1).
__device__ __forceinline__ int kdelta(const uint64_t* __restrict__ keys, int n, int i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = keys[i], b = keys[j];
    if (a == b) return 64 + __clz((unsigned)(i ^ (int)j));
    return __clzll(a ^ b);
}

__global__ void k_leaf_init(int n, int* __restrict__ first, int* __restrict__ last) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    first[n - 1 + k] = k;
    last[n - 1 + k] = k;
}

__global__ void k_karras(const uint64_t* __restrict__ keys, int n, int* __restrict__ left,
                         int* __restrict__ right, int* __restrict__ parent,
                         int* __restrict__ first, int* __restrict__ last) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    const int d = (kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    const int dmin = kdelta(keys, n, i, i - d);
    int64_t lmax = 2;
    while (kdelta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(keys, n, i, i + (l + t) * d) > dmin) l += (int)t;
    const int j = i + l * d;
    const int dnode = kdelta(keys, n, i, j);
    int s = 0, step = l;
    do {
        step = (step + 1) >> 1;
        if (kdelta(keys, n, i, (int64_t)i + (int64_t)(s + step) * d) > dnode) s += step;
    } while (step > 1);
    const int g = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int lc = (lo == g) ? (n - 1 + g) : g;
    const int rc = (hi == g + 1) ? (n - 1 + g + 1) : g + 1;
    left[i] = lc;
    right[i] = rc;
    parent[lc] = i;
    parent[rc] = i;
    first[i] = lo;
    last[i] = hi;
    if (i == 0) parent[0] = -1;
}

__device__ __forceinline__ bool is_cross(const uint64_t* keys, const int* first, const int* last,
                                         int u) {
    return (keys[first[u]] >> MORTON_BITS) != (keys[last[u]] >> MORTON_BITS);
}
// A node is "big" (never collapsed into a leaf) if it spans meshes or holds > K triangles.
__device__ __forceinline__ bool is_big(const uint64_t* keys, const int* first, const int* last,
                                       int u, int K) {
    return is_cross(keys, first, last, u) || (last[u] - first[u] + 1) > K;
}

// ---- K3b: collapse + DFS layout ---------------------------------------------------------------
// Position in a list for the lanes where `pred` holds: one atomicAdd per warp on the list's
// counter (a single counter bumped by every thread serialises at L2). Every active lane of the
// warp calls it at the same point; the order within the list is immaterial to its users.
__device__ __forceinline__ int warp_append(int* __restrict__ counter, bool pred) {
    const unsigned mask = __activemask();
    const unsigned bal = __ballot_sync(mask, pred);
    if (!bal) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(bal) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(bal));
    base = __shfl_sync(mask, base, leader);
    return pred ? base + __popc(bal & ((1u << lane) - 1u)) : -1;
}

// The same with one atomicAdd per block, for kernels over millions of threads (one counter
// bumped once per warp still serialises ~n / 32 atomics at one L2 address). Every thread of the
// block calls it at the same point (blockDim a multiple of 32, no thread returned before).
__device__ __forceinline__ int block_append(int* __restrict__ counter, bool pred) {
    __shared__ int s_warp[32];
    __shared__ int s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned bal = __ballot_sync(0xffffffffu, pred);
    if (lane == 0) s_warp[warp] = __popc(bal);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            const int c = s_warp[w];
            s_warp[w] = acc;
            acc += c;
        }
        s_base = acc ? atomicAdd(counter, acc) : 0;
    }
    __syncthreads();
    const int at = pred ? s_base + s_warp[warp] + __popc(bal & ((1u << lane) - 1u)) : -1;
    __syncthreads();  // the shared words are reused by the next call
    return at;
}

// flags: bit0 emitted, bit1 leaf
__global__ void k_emit_count(int n, int K, const uint64_t* __restrict__ keys,
                             const int* __restrict__ parent, const int* __restrict__ first,
                             const int* __restrict__ last, int* __restrict__ cnt_first,
                             uint8_t* __restrict__ flags, int* __restrict__ leaf_list,
                             int* __restrict__ leaf_list_len) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    bool pred = false;
    if (u < 2 * n - 1) {
        const int pu = parent[u];
        const bool emitted = (u == 0) || (pu >= 0 && is_big(keys, first, last, pu, K));
        const bool leaf = (u >= n - 1) || !is_big(keys, first, last, u, K);
        flags[u] = (uint8_t)((emitted ? 1 : 0) | (leaf ? 2 : 0));
        if (emitted) atomicAdd(&cnt_first[first[u]], 1);
        pred = emitted && leaf && !is_cross(keys, first, last, u);
    }
    // emitted leaves (never a node spanning meshes: such a node is "big") feed the refit, one
    // thread each; the list order does not matter (each node's arithmetic is fixed)
    const int at = block_append(leaf_list_len, pred);
    if (at >= 0) leaf_list[at] = u;
}

__global__ void k_positions(int num_nodes, const int* __restrict__ parent,
                            const int* __restrict__ first, const int* __restrict__ last,
                            const uint8_t* __restrict__ flags, const int* __restrict__ base,
                            int* __restrict__ pos, int* __restrict__ skip) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= num_nodes) return;
    if (!(flags[u] & 1)) {
        pos[u] = -1;
        skip[u] = -1;
        return;
    }
    const int f = first[u];
    int rank = 0, v = u;
    while (v != 0) {
        const int p = parent[v];
        if (p < 0 || first[p] != f) break;  // p < 0 only for an unlinked node (never)
        ++rank;
        v = p;
    }
    pos[u] = base[f] + rank;
    skip[u] = base[last[u] + 1];
}

__global__ void k_mesh_roots(int nmeshes, const int64_t* __restrict__ foff, int n,
                             const int* __restrict__ parent, const int* __restrict__ first,
                             const int* __restrict__ last, const int* __restrict__ pos,
                             const int* __restrict__ skip, MeshInfo* __restrict__ mi) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmeshes) return;
    const int64_t lo = foff[m], hi = foff[m + 1] - 1;
    if (hi < lo) {
        mi[m].root = -1;
        mi[m].end = -1;
        return;
    }
    int u = (n - 1) + (int)lo;
    while (u != 0) {
        const int p = parent[u];
        if (p < 0 || first[p] < lo || last[p] > hi) break;
        u = p;
    }
    mi[m].root = pos[u];
    mi[m].end = skip[u];
}

// ---- K1-K3 (builder 1): top-down splitting build ----------------------------------------------
// Level-synchronous, all meshes at once. Every active segment (a node of > leaf_size triangles)
// splits the bounding box of its triangles' centroids at the midpoint of its longest axis (ties:
// the lowest axis), split = (lo + hi) * 0.5f; the left child takes the centroids below the split,
// both children keeping the segment's order (a stable partition by one scan of the left flags).
// When every centroid coincides, or the midpoint rounds down to the low end, the segment splits
// by position instead (the first m / 2 left). A child of <= leaf_size triangles is a leaf and its
// triangles take their final slots. Roots (one per non-empty mesh) are nodes 0.., the children of
// active segment s at a level are nodes base + 2s and base + 2s + 1; DFS positions and skip links
// come from the node ranges afterwards with the same formula as for the LBVH (k_positions).
// Below level kSpatialLevels every split is by position, which bounds the depth by
// kSpatialLevels + log2(n) whatever the geometry (midpoint splits of float boxes could otherwise
// go on for hundreds of levels on adversarial inputs).
constexpr int kSpatialLevels = 96;
// Segments of at most kFinishSlots triangles leave the level loop: one block each finishes their
// subtrees in shared memory (k_split_finish), with the same splits.
constexpr int kFinishSlots = 1024;
constexpr int kFinishThreads = 512;
// Segments of the level loop (more than kFinishSlots triangles) split at a binned plane: kSplitBins
// bins per axis over the centroid box, bin(x) = min((int)((x - lo) / ext * 16), 15) in float, and
// the plane with the least nL * dL + nR * dR (d = squared diagonal of a side's centroid bounds, in
// double); ties go to the lower axis, then the lower plane; left = bin <= plane. A bin holds its
// count and its centroid bounds (ordered-int encodings): kBinWords words.
constexpr int kSplitBins = 16;
constexpr int kBinWords = 7;
constexpr int kSegBinWords = 3 * kSplitBins * kBinWords;  // 336 per segment
constexpr int kBinChunk = 2048;  // slots per block of k_split_bins: at most 3 level-loop segments

__device__ __forceinline__ int split_bin(float x, float lo, float ext) {
    const int b = (int)((x - lo) / ext * (float)kSplitBins);
    return b < 0 ? 0 : (b > kSplitBins - 1 ? kSplitBins - 1 : b);
}

struct SplitSlots {
    int* perm;  // triangle id per slot
    float* cx;  // its centroid
    float* cy;
    float* cz;
    int* seg;   // active segment of the slot at this level (-1: in a leaf)
};

// A level of at most kBoxCopyKeys segments accumulates its boxes in kBoxCopies copies (block b
// adds to copy b % kBoxCopies, copies kBoxCopyKeys boxes apart), merged by k_split_decide: at the
// top levels every block of the grid adds to the same one or two boxes, and one copy's six words
// share an L2 slice that would serialise all of the grid's atomics.
constexpr int kBoxCopies = 16;
constexpr int kBoxCopyKeys = 256;
constexpr int kBoxCopyStride = 6 * kBoxCopyKeys;  // words between copies

__device__ __forceinline__ int box_copy_offset(bool copies) {
    return copies ? (int)(blockIdx.x % kBoxCopies) * kBoxCopyStride : 0;
}

// Centroid boxes: lanes that add to the same box reduce together first (ordered-int encodings,
// so min / max are integer reductions), then one atomic per group and axis. When the whole
// block adds to one box (the top levels, where a segment spans many blocks) the block reduces
// in shared memory and issues six atomics; otherwise each warp groups its lanes by box. Every
// thread of the block must call it; threads with key < 0 add nothing. `box` already points at
// the block's copy (box_copy_offset).
__device__ __forceinline__ void box_add(int key, float cx, float cy, float cz,
                                        unsigned* __restrict__ box) {
    __shared__ int s_key;
    __shared__ unsigned s_box[6];
    if (threadIdx.x == 0) {
        s_key = key;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            s_box[a] = 0xffffffffu;
            s_box[3 + a] = 0u;
        }
    }
    __syncthreads();
    if (__syncthreads_and(key >= 0 && key == s_key)) {  // uniform over the block
        const float c[3] = {cx, cy, cz};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const unsigned e = enc_float(c[a]);
            const unsigned lo = __reduce_min_sync(0xffffffffu, e);
            const unsigned hi = __reduce_max_sync(0xffffffffu, e);
            if ((threadIdx.x & 31) == 0) {
                atomicMin(&s_box[a], lo);
                atomicMax(&s_box[3 + a], hi);
            }
        }
        __syncthreads();
        if (threadIdx.x < 3) atomicMin(&box[6 * key + threadIdx.x], s_box[threadIdx.x]);
        else if (threadIdx.x < 6) atomicMax(&box[6 * key + threadIdx.x], s_box[threadIdx.x]);
        return;
    }
    const unsigned act = __ballot_sync(0xffffffffu, key >= 0);
    if (key < 0) return;
    const unsigned peers = __match_any_sync(act, key);
    const bool leader = (threadIdx.x & 31) == (unsigned)(__ffs(peers) - 1);
    const float c[3] = {cx, cy, cz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const unsigned e = enc_float(c[a]);
        const unsigned lo = __reduce_min_sync(peers, e), hi = __reduce_max_sync(peers, e);
        if (leader) {
            atomicMin(&box[6 * key + a], lo);
            atomicMax(&box[6 * key + 3 + a], hi);
        }
    }
}

__device__ __forceinline__ void box_clear(unsigned* __restrict__ b) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        b[a] = 0xffffffffu;  // min of nothing
        b[3 + a] = 0u;       // max of nothing
    }
}

// Clears box k in every copy that a level may use (all copies for k < kBoxCopyKeys).
__device__ __forceinline__ void box_clear_level(unsigned* __restrict__ box, int k) {
    if (k < kBoxCopyKeys) {
#pragma unroll 1
        for (int c = 0; c < kBoxCopies; ++c) box_clear(box + c * kBoxCopyStride + 6 * k);
    } else {
        box_clear(box + 6 * k);
    }
}

__global__ void k_split_box_init(int nact, unsigned* __restrict__ box) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nact) box_clear_level(box, i);
}

// Validation, centroids and the first level's slots; the boxes of the first level's segments
// (the meshes of > leaf_size triangles) accumulate here too.
__global__ void k_split_init(const float* __restrict__ V, const int32_t* __restrict__ F,
                             const int64_t* __restrict__ voff, const int64_t* __restrict__ foff,
                             int nmeshes, int64_t nf, const int* __restrict__ mesh_seg,
                             SplitSlots out, int* __restrict__ final_perm,
                             uint64_t* __restrict__ keys, unsigned* __restrict__ box,
                             bool box_copies, unsigned* __restrict__ status) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1;
    float c[3] = {0.f, 0.f, 0.f};
    if (t < nf) {
        const int m = find_mesh(foff, nmeshes, t);
        const int64_t nvm = voff[m + 1] - voff[m];
        bool ok = true;
        int32_t idx[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            idx[j] = F[3 * t + j];
            if (idx[j] < 0 || (int64_t)idx[j] >= nvm) ok = false;
        }
        if (!ok) {
            atomicOr(status, ST_BAD_INDEX);
        } else {
            float v[3][3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const float* p = V + 3 * (voff[m] + idx[j]);
                v[j][0] = p[0];
                v[j][1] = p[1];
                v[j][2] = p[2];
                if (!isfinite(v[j][0]) || !isfinite(v[j][1]) || !isfinite(v[j][2])) ok = false;
            }
            if (!ok) atomicOr(status, ST_NONFINITE);
#pragma unroll
            for (int a = 0; a < 3; ++a) c[a] = ((v[0][a] + v[1][a]) + v[2][a]) / 3.0f;
        }
        key = mesh_seg[m];
        out.perm[t] = (int)t;
        out.cx[t] = c[0];
        out.cy[t] = c[1];
        out.cz[t] = c[2];
        out.seg[t] = key;
        if (key == -1) final_perm[t] = (int)t;  // the whole mesh is one leaf (-2: a small root)
        keys[t] = (uint64_t)m << MORTON_BITS;
    }
    box_add(key, c[0], c[1], c[2], box + box_copy_offset(box_copies));
}

// The split of one segment from its centroid box (lo[a] = dec(box[a]), hi[a] = dec(box[3 + a])
// at stride `stride`): the longest axis (the first on ties), its midpoint, and whether the split is
// spatial (else by position).
__device__ __forceinline__ void split_decide(const unsigned* __restrict__ box, int stride,
                                             bool by_position, int& axis_out, float& split_out,
                                             int& spatial_out) {
    float lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = dec_float(box[a * stride]);
        hi[a] = dec_float(box[(3 + a) * stride]);
    }
    int axis = 0;
    float ext = hi[0] - lo[0];
#pragma unroll
    for (int a = 1; a < 3; ++a) {
        const float x = hi[a] - lo[a];
        if (x > ext) {
            ext = x;
            axis = a;
        }
    }
    const float split = (lo[axis] + hi[axis]) * 0.5f;
    axis_out = axis;
    split_out = split;
    spatial_out = (!by_position && ext > 0.f && split > lo[axis]) ? 1 : 0;
}

__global__ void k_split_decide(int nact, bool by_position, const unsigned* __restrict__ box,
                               int* __restrict__ axis_of, float* __restrict__ split_of,
                               int* __restrict__ spatial_of, float* __restrict__ seg_box) {
    const int sg = blockIdx.x * blockDim.x + threadIdx.x;
    if (sg >= nact) return;
    unsigned b[6];
#pragma unroll
    for (int a = 0; a < 6; ++a) b[a] = box[6 * sg + a];
    if (nact <= kBoxCopyKeys) {  // merge the copies (all loads in flight together)
#pragma unroll
        for (int c = 1; c < kBoxCopies; ++c) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                b[a] = min(b[a], box[c * kBoxCopyStride + 6 * sg + a]);
                b[3 + a] = max(b[3 + a], box[c * kBoxCopyStride + 6 * sg + 3 + a]);
            }
        }
    }
    split_decide(b, 1, by_position, axis_of[sg], split_of[sg], spatial_of[sg]);
#pragma unroll
    for (int a = 0; a < 6; ++a) seg_box[6 * sg + a] = dec_float(b[a]);  // lo[3], hi[3]
}

__global__ void k_split_bins_init(int nwords, unsigned* __restrict__ bins) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nwords) return;
    const int w = i % kBinWords;
    bins[i] = w == 0 ? 0u : (w < 4 ? 0xffffffffu : 0u);  // count, lo (min of nothing), hi
}

// Per-segment bins of one level: a block takes kBinChunk consecutive slots, which meet at most
// three of the level's segments (each holds more than kFinishSlots), accumulates their bins in
// shared memory, then adds the non-empty ones to the segments' global bins.
__global__ void __launch_bounds__(256) k_split_bins(int64_t n, SplitSlots cur,
                                                    const float* __restrict__ seg_box,
                                                    unsigned* __restrict__ bins,
                                                    unsigned* __restrict__ status) {
    constexpr int kLocal = 4;
    __shared__ int tab[kLocal];
    __shared__ int ntab;
    __shared__ unsigned sb[kLocal * kSegBinWords];
    for (int i = threadIdx.x; i < kLocal * kSegBinWords; i += blockDim.x) {
        const int w = i % kBinWords;
        sb[i] = w == 0 ? 0u : (w < 4 ? 0xffffffffu : 0u);
    }
    if (threadIdx.x < kLocal) tab[threadIdx.x] = -1;
    if (threadIdx.x == 0) ntab = 0;
    __syncthreads();
    const int64_t c0 = (int64_t)blockIdx.x * kBinChunk;
    // a segment's slots are one run of positions: the run's first slot in the chunk claims the
    // segment's local bins
    for (int r = 0; r < kBinChunk / 256; ++r) {
        const int64_t i = c0 + r * 256 + threadIdx.x;
        if (i >= n) break;
        const int sg = cur.seg[i];
        if (sg >= 0 && (i == c0 || cur.seg[i - 1] != sg)) {
            const int k = atomicAdd(&ntab, 1);
            if (k < kLocal) tab[k] = sg;
            else atomicOr(status, ST_BUILD_BOUND);  // cannot happen: segments hold > 1024 slots
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    for (int r = 0; r < kBinChunk / 256; ++r) {  // uniform trip count: every lane takes part
        const int64_t i = c0 + r * 256 + threadIdx.x;
        const int sg = i < n ? cur.seg[i] : -1;
        int slot = -1;
        if (sg >= 0)
#pragma unroll
            for (int k = 0; k < kLocal; ++k)
                if (tab[k] == sg) slot = k;  // at most three segments meet a chunk
        float c[3] = {0.f, 0.f, 0.f};
        if (slot >= 0) {
            c[0] = cur.cx[i];
            c[1] = cur.cy[i];
            c[2] = cur.cz[i];
        }
        const unsigned ec[3] = {enc_float(c[0]), enc_float(c[1]), enc_float(c[2])};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            // lanes adding to the same bin reduce together; one atomic per bin and word
            int key = -1;
            if (slot >= 0) {
                const float lo = seg_box[6 * sg + a], ext = seg_box[6 * sg + 3 + a] - lo;
                if (ext > 0.f) key = (slot * 3 + a) * kSplitBins + split_bin(c[a], lo, ext);
            }
            const unsigned act = __ballot_sync(0xffffffffu, key >= 0);
            if (key >= 0) {
                const unsigned peers = __match_any_sync(act, key);
                const bool leader = lane == __ffs(peers) - 1;
                unsigned lo3[3], hi3[3];
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    lo3[d] = __reduce_min_sync(peers, ec[d]);
                    hi3[d] = __reduce_max_sync(peers, ec[d]);
                }
                if (leader) {
                    unsigned* bw = sb + key * kBinWords;
                    atomicAdd(&bw[0], (unsigned)__popc(peers));
#pragma unroll
                    for (int d = 0; d < 3; ++d) {
                        atomicMin(&bw[1 + d], lo3[d]);
                        atomicMax(&bw[4 + d], hi3[d]);
                    }
                }
            }
        }
    }
    __syncthreads();
    for (int slot = 0; slot < kLocal; ++slot) {
        const int sg = tab[slot];
        if (sg < 0) continue;
        const unsigned* src = sb + slot * kSegBinWords;
        unsigned* dst = bins + (int64_t)sg * kSegBinWords;
        for (int k = threadIdx.x; k < 3 * kSplitBins; k += blockDim.x) {
            const unsigned* bw = src + k * kBinWords;
            if (!bw[0]) continue;
            atomicAdd(&dst[k * kBinWords], bw[0]);
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                atomicMin(&dst[k * kBinWords + 1 + d], bw[1 + d]);
                atomicMax(&dst[k * kBinWords + 4 + d], bw[4 + d]);
            }
        }
    }
}

__device__ __forceinline__ double split_diag2(const float* lo, const float* hi) {
    double t = 0.0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double d = (double)hi[a] - (double)lo[a];
        t = t + d * d;
    }
    return t;
}

// The binned plane of each segment (when some axis has extent): spatial_of = 2, axis_of, bin_of.
// One warp per segment: lane k holds bin k of an axis, the left sides are inclusive prefix scans
// over the lanes and the right sides suffix scans (min, max and integer counts are exact in any
// order), lane j prices plane j, and the warp keeps the least (cost, axis, plane), the first
// minimum in axis-then-plane order.
__device__ __forceinline__ void bin_scan_up(unsigned& n, float (&lo)[3], float (&hi)[3], int lane) {
#pragma unroll
    for (int o = 1; o < kSplitBins; o <<= 1) {
        const unsigned m = __shfl_up_sync(0xffffffffu, n, o);
        float l[3], h[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            l[d] = __shfl_up_sync(0xffffffffu, lo[d], o);
            h[d] = __shfl_up_sync(0xffffffffu, hi[d], o);
        }
        if (lane >= o) {
            n += m;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                lo[d] = fminf(lo[d], l[d]);
                hi[d] = fmaxf(hi[d], h[d]);
            }
        }
    }
}

__device__ __forceinline__ void bin_scan_down(unsigned& n, float (&lo)[3], float (&hi)[3], int lane) {
#pragma unroll
    for (int o = 1; o < kSplitBins; o <<= 1) {
        const unsigned m = __shfl_down_sync(0xffffffffu, n, o);
        float l[3], h[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            l[d] = __shfl_down_sync(0xffffffffu, lo[d], o);
            h[d] = __shfl_down_sync(0xffffffffu, hi[d], o);
        }
        if (lane + o < kSplitBins) {
            n += m;
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                lo[d] = fminf(lo[d], l[d]);
                hi[d] = fmaxf(hi[d], h[d]);
            }
        }
    }
}

__global__ void k_split_choose(int nact, const float* __restrict__ seg_box,
                               const unsigned* __restrict__ bins, int* __restrict__ axis_of,
                               int* __restrict__ bin_of, int* __restrict__ spatial_of) {
    const int sg = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (sg >= nact) return;  // warp-uniform
    const unsigned* sgb = bins + (int64_t)sg * kSegBinWords;
    double best = INFINITY;
    int best_a = 3, best_j = kSplitBins;
    for (int a = 0; a < 3; ++a) {
        if (!(seg_box[6 * sg + 3 + a] - seg_box[6 * sg + a] > 0.f)) continue;  // warp-uniform
        unsigned n = 0;
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        if (lane < kSplitBins) {
            const unsigned* bw = sgb + (a * kSplitBins + lane) * kBinWords;
            n = bw[0];
            if (n) {  // an empty bin's bounds are the identity
#pragma unroll
                for (int d = 0; d < 3; ++d) {
                    lo[d] = dec_float(bw[1 + d]);
                    hi[d] = dec_float(bw[4 + d]);
                }
            }
        }
        unsigned nL = n, nR = n;
        float Llo[3], Lhi[3], Rlo[3], Rhi[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            Llo[d] = Rlo[d] = lo[d];
            Lhi[d] = Rhi[d] = hi[d];
        }
        bin_scan_up(nL, Llo, Lhi, lane);    // bins 0..lane
        bin_scan_down(nR, Rlo, Rhi, lane);  // bins lane..15
        // plane j = lane: left = bins 0..j, right = bins j+1..15 (the next lane's suffix)
        const unsigned nRn = __shfl_down_sync(0xffffffffu, nR, 1);
        float rlo[3], rhi[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            rlo[d] = __shfl_down_sync(0xffffffffu, Rlo[d], 1);
            rhi[d] = __shfl_down_sync(0xffffffffu, Rhi[d], 1);
        }
        if (lane < kSplitBins - 1 && nL > 0 && nRn > 0) {
            const double cost = (double)nL * split_diag2(Llo, Lhi) + (double)nRn * split_diag2(rlo, rhi);
            if (cost < best) {  // axes in order: a lane keeps its first minimum
                best = cost;
                best_a = a;
                best_j = lane;
            }
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {  // least (cost, axis, plane) over the lanes
        const double c2 = __shfl_xor_sync(0xffffffffu, best, o);
        const int a2 = __shfl_xor_sync(0xffffffffu, best_a, o);
        const int j2 = __shfl_xor_sync(0xffffffffu, best_j, o);
        if (c2 < best || (c2 == best && (a2 < best_a || (a2 == best_a && j2 < best_j)))) {
            best = c2;
            best_a = a2;
            best_j = j2;
        }
    }
    if (lane == 0 && best_a < 3) {
        axis_of[sg] = best_a;
        bin_of[sg] = best_j;
        spatial_of[sg] = 2;
    }
}

__global__ void k_split_flags(int64_t n, SplitSlots cur, const int* __restrict__ s_start,
                              const int* __restrict__ s_end, const int* __restrict__ axis_of,
                              const float* __restrict__ split_of,
                              const int* __restrict__ spatial_of, const int* __restrict__ bin_of,
                              const float* __restrict__ seg_box, int* __restrict__ flags) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    int f = 0;
    if (i < n) {
        const int sg = cur.seg[i];
        if (sg >= 0) {
            if (spatial_of[sg] == 2) {
                const int a = axis_of[sg];
                const float c = a == 0 ? cur.cx[i] : a == 1 ? cur.cy[i] : cur.cz[i];
                const float lo = seg_box[6 * sg + a], ext = seg_box[6 * sg + 3 + a] - lo;
                f = split_bin(c, lo, ext) <= bin_of[sg] ? 1 : 0;
            } else if (spatial_of[sg]) {
                const int a = axis_of[sg];
                const float c = a == 0 ? cur.cx[i] : a == 1 ? cur.cy[i] : cur.cz[i];
                f = c < split_of[sg] ? 1 : 0;
            } else {
                f = (i - s_start[sg]) < (s_end[sg] - s_start[sg]) / 2 ? 1 : 0;
            }
        }
    }
    flags[i] = f;  // flags[n] = 0: the scan's total entry
}

// Children of every active segment (lf = exclusive scan of the left flags): the two nodes (at
// depth level + 1), and for each child of more than kFinishSlots triangles a slot of the next
// level (allocated with an atomic counter, its box cleared); a child of K < size <= kFinishSlots
// triangles goes to the small list {start, end, node, depth} that k_split_finish completes.
// child_next[2s + c] = the next level's slot, -2 for a small child or -1 for a leaf. The order
// of segments in either list is immaterial: positions come from the node ranges alone.
// counts[0] / counts[1]: the next level's segments / the small list's length.
__global__ void k_split_children(int nact, int node_base, int level, int K,
                                 const int* __restrict__ s_start, const int* __restrict__ s_end,
                                 const int* __restrict__ s_node, const int* __restrict__ lf,
                                 int* __restrict__ nfirst, int* __restrict__ nlast,
                                 int* __restrict__ nparent, int* __restrict__ nleft,
                                 int* __restrict__ nright, int* __restrict__ depth_of,
                                 int* __restrict__ counts, int* __restrict__ n_start,
                                 int* __restrict__ n_end, int* __restrict__ n_node,
                                 unsigned* __restrict__ n_box, int4* __restrict__ small,
                                 int* __restrict__ child_next) {
    const int sg = blockIdx.x * blockDim.x + threadIdx.x;
    if (sg >= nact) return;
    const int b = s_start[sg], e = s_end[sg], mid = b + (lf[e] - lf[b]);
    const int l = node_base + 2 * sg, r = l + 1, p = s_node[sg];
    nfirst[l] = b;
    nlast[l] = mid - 1;
    nfirst[r] = mid;
    nlast[r] = e - 1;
    nparent[l] = p;
    nparent[r] = p;
    nleft[l] = nright[l] = nleft[r] = nright[r] = -1;
    nleft[p] = l;
    nright[p] = r;
    depth_of[l] = depth_of[r] = level + 1;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const int cb = c == 0 ? b : mid, ce = c == 0 ? mid : e;
        const int k = warp_append(&counts[0], ce - cb > kFinishSlots);
        if (k >= 0) {
            n_start[k] = cb;
            n_end[k] = ce;
            n_node[k] = l + c;
            box_clear_level(n_box, k);
        }
        const int j = warp_append(&counts[1], ce - cb > K && ce - cb <= kFinishSlots);
        if (j >= 0) small[j] = make_int4(cb, ce, l + c, level + 1);
        child_next[2 * sg + c] = k >= 0 ? k : j >= 0 ? -2 : -1;
    }
}

// Stable partition of every active segment: left-flagged slots first, each side in its order.
// Slots of children that stay active go to the next level's buffers (and into their child's
// box); those of leaves are final.
__global__ void k_split_scatter(int64_t n, SplitSlots cur, SplitSlots nxt,
                                const int* __restrict__ lf, const int* __restrict__ s_start,
                                const int* __restrict__ s_end, const int* __restrict__ child_next,
                                int* __restrict__ final_perm, unsigned* __restrict__ n_box,
                                const int* __restrict__ next_count) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int key = -1;
    float cx = 0.f, cy = 0.f, cz = 0.f;
    if (i < n) {
        const int sg = cur.seg[i];
        if (sg < 0) {
            nxt.seg[i] = -1;
        } else {
            const int b = s_start[sg], e = s_end[sg];
            const int fb = lf[b], nl = lf[e] - fb, left_before = lf[i] - fb;
            const bool left = lf[i + 1] != lf[i];  // the exclusive scan steps where the flag is set
            const int64_t dest = left ? b + left_before : b + nl + ((int)(i - b) - left_before);
            const int k = child_next[2 * sg + (left ? 0 : 1)];
            if (k >= 0 || k == -2) {  // active next level, or a small segment's slots
                cx = cur.cx[i];
                cy = cur.cy[i];
                cz = cur.cz[i];
                nxt.perm[dest] = cur.perm[i];
                nxt.cx[dest] = cx;
                nxt.cy[dest] = cy;
                nxt.cz[dest] = cz;
                nxt.seg[dest] = k >= 0 ? k : -1;
                key = k >= 0 ? k : -1;
            } else {
                final_perm[dest] = cur.perm[i];
                nxt.seg[dest] = -1;
            }
        }
    }
    box_add(key, cx, cy, cz, n_box + box_copy_offset(*next_count <= kBoxCopyKeys));
}

// A small segment in shared memory. Sub-segments are named by their first position, so a
// split names its children itself (b and mid); the slots carry their original local index, and
// centroids stay where they were loaded.
struct FinishShared {
    float c[3][kFinishSlots];              // centroid of each original local slot
    int perm[kFinishSlots];                // triangle of each original local slot
    unsigned short orig[2][kFinishSlots];  // original local slot at each position
    short sid[2][kFinishSlots];            // first position of the position's segment (-1: leaf)
    short send[2][kFinishSlots];           // end of the segment that starts at a position
    int snode[2][kFinishSlots];            // node of the segment that starts at a position
    unsigned box[6][kFinishSlots];         // centroid box of the segment that starts there
    int scan[kFinishSlots + 1];
    int wsum[kFinishThreads / 32];
    int ns[2], rank, node_base;
};

// Exclusive scan of a[0 .. count) in shared memory by the whole block (count <= 8 * blockDim).
__device__ void block_exclusive_scan(int* a, int count, int* wsum) {
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarps = blockDim.x >> 5;
    const int per = (count + blockDim.x - 1) / blockDim.x;
    const int b = min(tid * per, count), e = min(b + per, count);
    int sum = 0;
    for (int i = b; i < e; ++i) sum += a[i];
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nwarps ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nwarps) wsum[lane] = w;
    }
    __syncthreads();
    int run = x - sum + (warp > 0 ? wsum[warp - 1] : 0);
    for (int i = b; i < e; ++i) {
        const int v = a[i];
        a[i] = run;
        run += v;
    }
    __syncthreads();
}

// One block per small segment small[blockIdx.x] = {start, end, node, depth}: its subtree, split
// by split by the level loop's rules (split_decide and the flags, children and stable partition
// of k_split_flags / k_split_children / k_split_scatter) in shared memory. The slots are in A for
// an even depth and in B for an odd one (the level that made the segment wrote them there, and
// later levels write only other segments' ranges). Each step's node ids are one allocation from
// node_count.
__global__ void __launch_bounds__(kFinishThreads) k_split_finish(
    const int4* __restrict__ small, SplitSlots A, SplitSlots B, int K, int* __restrict__ node_count,
    int cap, int* __restrict__ nfirst, int* __restrict__ nlast, int* __restrict__ nparent,
    int* __restrict__ nleft, int* __restrict__ nright, int* __restrict__ depth_of,
    int* __restrict__ final_perm, unsigned* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char finish_smem[];
    FinishShared& S = *reinterpret_cast<FinishShared*>(finish_smem);
    const int4 seg = small[blockIdx.x];
    const int gb = seg.x, size = seg.y - seg.x, d0 = seg.w, tid = threadIdx.x;
    if (size > kFinishSlots || size <= K) {  // never made so by k_split_children
        if (tid == 0) atomicOr(status, ST_BUILD_BOUND);
        return;
    }
    const SplitSlots& X = (d0 & 1) ? B : A;
    for (int i = tid; i < size; i += kFinishThreads) {
        S.c[0][i] = X.cx[gb + i];
        S.c[1][i] = X.cy[gb + i];
        S.c[2][i] = X.cz[gb + i];
        S.perm[i] = X.perm[gb + i];
        S.orig[0][i] = (unsigned short)i;
        S.sid[0][i] = 0;
    }
    if (tid == 0) {
        S.ns[0] = 1;
        S.send[0][0] = (short)size;
        S.snode[0][0] = seg.z;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            S.box[a][0] = 0xffffffffu;
            S.box[3 + a][0] = 0u;
        }
    }
    __syncthreads();
    int cur = 0;
    for (int depth = d0;; ++depth) {
        const int ns = S.ns[cur];
        if (ns == 0) break;
        if (depth > kSpatialLevels + 64) {  // position splits halve every segment
            if (tid == 0) atomicOr(status, ST_BUILD_BOUND);
            return;
        }
        // centroid boxes: lanes of one segment reduce together, then one atomic per axis
        for (int i0 = 0; i0 < size; i0 += kFinishThreads) {
            const int i = i0 + tid;
            const int key = i < size ? S.sid[cur][i] : -1;
            const unsigned act = __ballot_sync(0xffffffffu, key >= 0);
            if (key >= 0) {
                const unsigned peers = __match_any_sync(act, key);
                const bool leader = (tid & 31) == __ffs(peers) - 1;
                const int o = S.orig[cur][i];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const unsigned ev = enc_float(S.c[a][o]);
                    const unsigned lo = __reduce_min_sync(peers, ev), hi = __reduce_max_sync(peers, ev);
                    if (leader) {
                        atomicMin(&S.box[a][key], lo);
                        atomicMax(&S.box[3 + a][key], hi);
                    }
                }
            }
        }
        // the step's node ids (every active segment splits): the atomic's result is stored only
        // after the flags, so the block does not wait for it at the next barrier
        int nb = 0;
        if (tid == 0) {
            nb = atomicAdd(node_count, 2 * ns);
            S.rank = 0;
            S.ns[cur ^ 1] = 0;
        }
        __syncthreads();
        // left flags, each slot deciding its segment's split from the box
        const bool by_position = depth >= kSpatialLevels;
        for (int i = tid; i <= size; i += kFinishThreads) {
            int f = 0;
            if (i < size) {
                const int b = S.sid[cur][i];
                if (b >= 0) {
                    int axis, spatial;
                    float split;
                    split_decide(&S.box[0][b], kFinishSlots, by_position, axis, split, spatial);
                    const int e = S.send[cur][b];
                    f = spatial ? (S.c[axis][S.orig[cur][i]] < split ? 1 : 0)
                                : ((i - b) < (e - b) / 2 ? 1 : 0);
                }
            }
            S.scan[i] = f;
        }
        if (tid == 0) S.node_base = nb;
        __syncthreads();
        if (S.node_base + 2 * ns > cap) {  // uniform: no node of this step could be written
            if (tid == 0) atomicOr(status, ST_BUILD_BOUND);
            return;
        }
        block_exclusive_scan(S.scan, size + 1, S.wsum);
        // stable partition; a segment's first position makes its two nodes and next segments
        const int node_base = S.node_base;
        for (int i = tid; i < size; i += kFinishThreads) {
            const int b = S.sid[cur][i];
            if (b < 0) {
                S.sid[cur ^ 1][i] = -1;  // no moving slot lands outside its own segment
                continue;
            }
            const int e = S.send[cur][b];
            const int fb = S.scan[b], mid = b + (S.scan[e] - fb), left_before = S.scan[i] - fb;
            const bool left = S.scan[i + 1] != S.scan[i];
            const int dest = left ? b + left_before : mid + ((i - b) - left_before);
            const int cb = left ? b : mid, ce = left ? mid : e;
            if (i == b) {
                const int p = S.snode[cur][b];
                const int l = node_base + 2 * atomicAdd(&S.rank, 1), r = l + 1;  // r < cap
                nfirst[l] = gb + b;
                nlast[l] = gb + mid - 1;
                nfirst[r] = gb + mid;
                nlast[r] = gb + e - 1;
                nparent[l] = p;
                nparent[r] = p;
                nleft[l] = nright[l] = nleft[r] = nright[r] = -1;
                nleft[p] = l;
                nright[p] = r;
                depth_of[l] = depth_of[r] = depth + 1;
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const int xb = c == 0 ? b : mid, xe = c == 0 ? mid : e;
                    if (xe - xb > K) {
                        S.send[cur ^ 1][xb] = (short)xe;
                        S.snode[cur ^ 1][xb] = l + c;
#pragma unroll
                        for (int a = 0; a < 3; ++a) {
                            S.box[a][xb] = 0xffffffffu;
                            S.box[3 + a][xb] = 0u;
                        }
                        atomicAdd(&S.ns[cur ^ 1], 1);
                    }
                }
            }
            const int o = S.orig[cur][i];
            if (ce - cb > K) {
                S.sid[cur ^ 1][dest] = (short)cb;
                S.orig[cur ^ 1][dest] = (unsigned short)o;
            } else {
                S.sid[cur ^ 1][dest] = -1;
                final_perm[gb + dest] = S.perm[o];
            }
        }
        __syncthreads();
        cur ^= 1;
    }
}

// Node flags of the split tree (every node emitted; leaves = no children), the per-first-slot
// node counts of the position scan, and the refit's leaf list.
__global__ void k_split_emit(int num_nodes, const int* __restrict__ nfirst,
                             const int* __restrict__ nleft, uint8_t* __restrict__ flags,
                             int* __restrict__ cnt_first, int* __restrict__ leaf_list,
                             int* __restrict__ leaf_list_len) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    bool leaf = false;
    if (u < num_nodes) {
        leaf = nleft[u] < 0;
        flags[u] = (uint8_t)(1 | (leaf ? 2 : 0));
        atomicAdd(&cnt_first[nfirst[u]], 1);
    }
    const int at = block_append(leaf_list_len, leaf);
    if (at >= 0) leaf_list[at] = u;
}

__global__ void k_split_mesh_roots(int nmeshes, const int* __restrict__ root_node,
                                   const int* __restrict__ pos, const int* __restrict__ skip,
                                   MeshInfo* __restrict__ mi) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmeshes) return;
    const int r = root_node[m];
    mi[m].root = r < 0 ? -1 : pos[r];
    mi[m].end = r < 0 ? -1 : skip[r];
}

// ---- K4: FP64 refit ---------------------------------------------------------------------------
// Exact float <-> double conversions on the integer pipes. GB300 runs conversions on its FP64 pipe
// (2 operations per SM per cycle), which the refit's FP64 arithmetic already saturates; these give
// the hardware's results bit for bit (IEEE: float -> double is exact, double -> float rounds to
// nearest even) and fall back to the hardware conversion for the rare operands outside the
// normal range (subnormal results, infinities, NaN).
__device__ __forceinline__ double f2d(float x) {
    const unsigned b = __float_as_uint(x);
    const unsigned e = (b >> 23) & 0xffu;
    if ((b & 0x7fffffffu) == 0u) return __hiloint2double((int)b, 0);  // +-0
    if (e == 0u || e == 0xffu) return (double)x;
    const unsigned hi = (b & 0x80000000u) | ((e + 896u) << 20) | ((b & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(b << 29));
}

__device__ __forceinline__ float d2f(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned e = (hi >> 20) & 0x7ffu;
    if ((hi & 0x7fffffffu) == 0u && lo == 0u) return __uint_as_float(hi);  // +-0
    if (e < 897u || e > 1150u) return (float)x;  // float subnormal / overflow, inf, NaN
    // 52-bit fraction = (hi & 0xfffff) : lo; keep its top 23 bits, round the 29 below to even
    const unsigned f = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    const unsigned up = (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) ? 1u : 0u;
    // a carry out of the fraction steps the exponent (to infinity past the largest float)
    return __uint_as_float((hi & 0x80000000u) + (((e - 896u) << 23) | f) + up);
}

__device__ __forceinline__ double round_up_float(double x) {
    float f = d2f(x);
    if (f2d(f) < x) f = nextafterf(f, INFINITY);
    return f2d(f);
}

__device__ __forceinline__ void load_tri_d(const float* __restrict__ V, const int32_t* __restrict__ F,
                                           int64_t vbase, int64_t t, double v[3][3]) {
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const int64_t vi = vbase + F[3 * t + j];
        v[j][0] = f2d(V[3 * vi + 0]);
        v[j][1] = f2d(V[3 * vi + 1]);
        v[j][2] = f2d(V[3 * vi + 2]);
    }
}

// Moments of the triangles in sorted slots [f, l] about their area-weighted centroid P.
// Per triangle t (vertices v0,v1,v2, area-weighted normal n = (v1-v0)x(v2-v0)/2, centroid c,
// d = c - X about a point X):  N += n,  M1[i][j] += n_i d_j,
// M2[i][jk] += n_i (d_j d_k + (1/12) sum_v (v-c)_j (v-c)_k)   (exact area integral of
// (x-X)_j (x-X)_k over the triangle divided by its area).
// One pass accumulates the moments about X = the first triangle's centroid c0 together with the
// area-weighted centroid; they are then moved to P with the same recentring formulas a parent
// uses for its children (e = c0 - P). A second, vertex-only pass gives r = max |v - P|
// (vertex_r2, the same bound k_node_radius computes for internal nodes).
constexpr double kThird = 1.0 / 3.0;
constexpr double kTwelfth = 1.0 / 12.0;

// Fused multiply-add, correctly rounded. This file is compiled with -fmad=false so that no
// product is contracted implicitly; every fused operation of the refit is written out, at the
// same places as in the oracle's restatement (C fma()), which keeps the two bit-identical.
__device__ __forceinline__ double fmad(double a, double b, double c) { return __fma_rn(a, b, c); }

// Squared distance of a vertex from P in FP64, fused at fixed places: the term whose maximum over
// a node's vertices gives the node radius (leaves in leaf_moments, internal nodes in
// k_node_radius; a maximum does not depend on the order of its terms).
__device__ __forceinline__ double vertex_r2(float x, float y, float z, const double* P) {
    const double dx = f2d(x) - P[0], dy = f2d(y) - P[1], dz = f2d(z) - P[2];
    return fmad(dx, dx, fmad(dy, dy, dz * dz));
}

// Float estimate of |v - P|^2 (P a float value; every step rounded once, so within 6e-7 of the
// exact value while no step underflows).
__device__ __forceinline__ float vertex_est(float x, float y, float z, const float* Pf) {
    const float dx = x - Pf[0], dy = y - Pf[1], dz = z - Pf[2];
    return (dx * dx + dy * dy) + dz * dz;
}

// One lane's share of a one-pass radius screen: the running maximum m of the estimates, and the
// two largest estimates (with their vertices) among the vertices that came within 1e-5 of the
// running maximum when they were seen, plus the largest such estimate pushed out of the two. A
// vertex whose estimate reaches the final threshold M (1 - 1e-5) (M the warp's maximum, at least
// every running maximum) was within 1e-5 of the running maximum when seen, so it is one of the
// two or it raised `dropped` to the threshold; in that case (ties, e.g. a node centred on a
// sphere) the caller makes a second pass over its slots.
struct LaneTop2 {
    float m = 0.f;
    float e0 = -INFINITY, e1 = -INFINITY, dropped = -INFINITY;
    float x0 = 0.f, y0 = 0.f, z0 = 0.f, x1 = 0.f, y1 = 0.f, z1 = 0.f;
    __device__ __forceinline__ void add(float x, float y, float z, float e) {
        if (!(e < m * 0.99999f - 1e-37f)) {
            if (e > e0) {
                dropped = fmaxf(dropped, e1);
                e1 = e0; x1 = x0; y1 = y0; z1 = z0;
                e0 = e; x0 = x; y0 = y; z0 = z;
            } else if (e > e1) {
                dropped = fmaxf(dropped, e1);
                e1 = e; x1 = x; y1 = y; z1 = z;
            } else {
                dropped = fmaxf(dropped, e);
            }
        }
        m = fmaxf(m, e);
    }
    __device__ __forceinline__ void add_slot(const TriF32& t, const float* Pf) {
        const float4 t0 = t.t0, t1 = t.t1, t2 = t.t2;
        add(t0.x, t0.y, t0.z, vertex_est(t0.x, t0.y, t0.z, Pf));
        add(t0.w, t1.x, t1.y, vertex_est(t0.w, t1.x, t1.y, Pf));
        add(t1.z, t1.w, t2.x, vertex_est(t1.z, t1.w, t2.x, Pf));
    }
};

__device__ void leaf_moments(const float* __restrict__ V, const int32_t* __restrict__ F,
                             const int64_t* __restrict__ voff, const uint64_t* __restrict__ keys,
                             const uint32_t* __restrict__ tri_of_slot, int f, int l,
                             StageRec& R) {
    double A = 0.0, S[3] = {0.0, 0.0, 0.0}, c0[3] = {0.0, 0.0, 0.0};
    double N[3] = {0.0, 0.0, 0.0}, M1[9], M2[18];
    for (int i = 0; i < 9; ++i) M1[i] = 0.0;
    for (int i = 0; i < 18; ++i) M2[i] = 0.0;
    const int SJ[6] = {0, 1, 2, 0, 0, 1};
    const int SK[6] = {0, 1, 2, 1, 2, 2};
    for (int s = f; s <= l; ++s) {
        const int64_t t = tri_of_slot[s];
        const int m = (int)(keys[s] >> MORTON_BITS);
        double v[3][3];
        load_tri_d(V, F, voff[m], t, v);
        double e1[3], e2[3], nn[3], c[3], d[3], w[3][3], Q[6];
        for (int a = 0; a < 3; ++a) {
            e1[a] = v[1][a] - v[0][a];
            e2[a] = v[2][a] - v[0][a];
        }
        nn[0] = 0.5 * fmad(e1[1], e2[2], -(e1[2] * e2[1]));
        nn[1] = 0.5 * fmad(e1[2], e2[0], -(e1[0] * e2[2]));
        nn[2] = 0.5 * fmad(e1[0], e2[1], -(e1[1] * e2[0]));
        const double a_t = sqrt(fmad(nn[0], nn[0], fmad(nn[1], nn[1], nn[2] * nn[2])));
        for (int a = 0; a < 3; ++a) c[a] = ((v[0][a] + v[1][a]) + v[2][a]) * kThird;
        if (s == f)
            for (int a = 0; a < 3; ++a) c0[a] = c[a];
        for (int a = 0; a < 3; ++a) {
            S[a] = fmad(a_t, c[a], S[a]);
            d[a] = c[a] - c0[a];
        }
        A = A + a_t;
        for (int j = 0; j < 3; ++j)
            for (int a = 0; a < 3; ++a) w[j][a] = v[j][a] - c[a];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int j = SJ[q], k = SK[q];
            const double cov = fmad(w[0][j], w[0][k], fmad(w[1][j], w[1][k], w[2][j] * w[2][k])) * kTwelfth;
            Q[q] = fmad(d[j], d[k], cov);
        }
        for (int i = 0; i < 3; ++i) {
            N[i] = N[i] + nn[i];
            for (int j = 0; j < 3; ++j) M1[3 * i + j] = fmad(nn[i], d[j], M1[3 * i + j]);
#pragma unroll
            for (int q = 0; q < 6; ++q) M2[6 * i + q] = fmad(nn[i], Q[q], M2[6 * i + q]);
        }
    }
    // a leaf of zero area is centred at the plain mean of its centroids (Cs / count); that sum is
    // only needed then, so it is formed in a second pass, with the same additions in the same order
    double Cs[3] = {0.0, 0.0, 0.0};
    if (!(A > 0.0))
        for (int s = f; s <= l; ++s) {
            double v[3][3];
            load_tri_d(V, F, voff[(int)(keys[s] >> MORTON_BITS)], tri_of_slot[s], v);
            for (int a = 0; a < 3; ++a) Cs[a] = Cs[a] + ((v[0][a] + v[1][a]) + v[2][a]) * kThird;
        }
    const double cnt = (double)(l - f + 1);
    double P[3], e[3];
    for (int a = 0; a < 3; ++a) {
        const double pe = A > 0.0 ? S[a] / A : Cs[a] / cnt;
        P[a] = f2d(d2f(pe));
        e[a] = c0[a] - P[a];
    }
    for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            const int j = SJ[q], k = SK[q];
            R.M2[6 * i + q] =
                fmad(N[i], e[j] * e[k], fmad(M1[3 * i + k], e[j], fmad(M1[3 * i + j], e[k], M2[6 * i + q])));
        }
        for (int j = 0; j < 3; ++j) R.M1[3 * i + j] = fmad(N[i], e[j], M1[3 * i + j]);
    }
    // radius: the leaf's farthest vertex from P, screened in float in one pass (LaneTop2 on this
    // thread's own vertices), with exact FP64 terms for the one or two candidates kept, or for
    // every vertex reaching the threshold in a second pass when ties may have pushed one out
    const float Pf[3] = {d2f(P[0]), d2f(P[1]), d2f(P[2])};
    auto vertex_of = [&](int s, int j) {
        const int64_t t = tri_of_slot[s];
        const int m = (int)(keys[s] >> MORTON_BITS);
        return V + 3 * (voff[m] + F[3 * t + j]);
    };
    LaneTop2 top;
    for (int s = f; s <= l; ++s)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const float* vp = vertex_of(s, j);
            top.add(vp[0], vp[1], vp[2], vertex_est(vp[0], vp[1], vp[2], Pf));
        }
    const float thr = top.m * 0.99999f - 1e-37f;
    double r2 = 0.0;
    if (!(top.m < INFINITY) || !(top.dropped < thr)) {
        const bool all = !(top.m < INFINITY);
        for (int s = f; s <= l; ++s)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const float* vp = vertex_of(s, j);
                if (all || vertex_est(vp[0], vp[1], vp[2], Pf) >= thr)
                    r2 = fmax(r2, vertex_r2(vp[0], vp[1], vp[2], P));
            }
    } else {
        if (top.e0 >= thr) r2 = vertex_r2(top.x0, top.y0, top.z0, P);
        if (top.e1 >= thr) r2 = fmax(r2, vertex_r2(top.x1, top.y1, top.z1, P));
    }
    for (int a = 0; a < 3; ++a) {
        R.P[a] = P[a];
        R.N[a] = N[a];
    }
    R.area = A;
    R.r = round_up_float(sqrt(r2));
    R.pad = 0.0;
}

// Children's records: plain cached loads (an earlier launch wrote them), so the fields of one
// record share its L1 sectors.
__device__ __forceinline__ double2 ld_rec2(const double* p) {  // p 16 B aligned
    return *reinterpret_cast<const double2*>(p);
}

__device__ void combine_moments(const StageRec* __restrict__ a_, const StageRec* __restrict__ b_,
                                StageRec& R) {
    // a record as doubles: P[0..2], area, N[0..2], M1[0..8] (the first 128 B), then M2[0..17];
    // records are 32 B aligned, so every even index starts a 16 B pair
    const double* ra = reinterpret_cast<const double*>(a_);
    const double* rb = reinterpret_cast<const double*>(b_);
    double ha[16], hb[16];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const double2 x = ld_rec2(ra + 2 * k), y = ld_rec2(rb + 2 * k);
        ha[2 * k] = x.x;
        ha[2 * k + 1] = x.y;
        hb[2 * k] = y.x;
        hb[2 * k + 1] = y.y;
    }
    const double* Pa = ha;
    const double* Pb = hb;
    const double Aa = ha[3], Ab = hb[3];
    const double* Na = ha + 4;
    const double* Nb = hb + 4;
    const double* M1a = ha + 7;
    const double* M1b = hb + 7;
    const double A = Aa + Ab;
    double P[3], ea[3], eb[3];
    for (int i = 0; i < 3; ++i) {
        const double pe = A > 0.0 ? fmad(Aa, Pa[i], Ab * Pb[i]) / A : (Pa[i] + Pb[i]) * 0.5;
        P[i] = f2d(d2f(pe));
        ea[i] = Pa[i] - P[i];
        eb[i] = Pb[i] - P[i];
    }
    for (int i = 0; i < 3; ++i) {
        R.P[i] = P[i];
        R.N[i] = Na[i] + Nb[i];
        for (int j = 0; j < 3; ++j)
            R.M1[3 * i + j] = fmad(Na[i], ea[j], M1a[3 * i + j]) + fmad(Nb[i], eb[j], M1b[3 * i + j]);
    }
    const int SJ[6] = {0, 1, 2, 0, 0, 1};
    const int SK[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int q = 0; q < 6; q += 2) {
            const double2 ma = ld_rec2(ra + 16 + 6 * i + q), mb = ld_rec2(rb + 16 + 6 * i + q);
            const double m2a[2] = {ma.x, ma.y}, m2b[2] = {mb.x, mb.y};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int j = SJ[q + h], k = SK[q + h];
                const double ta = fmad(Na[i], ea[j] * ea[k],
                                       fmad(M1a[3 * i + k], ea[j], fmad(M1a[3 * i + j], ea[k], m2a[h])));
                const double tb = fmad(Nb[i], eb[j] * eb[k],
                                       fmad(M1b[3 * i + k], eb[j], fmad(M1b[3 * i + j], eb[k], m2b[h])));
                R.M2[6 * i + q + h] = ta + tb;
            }
        }
    R.area = A;
    R.r = 0.0;  // exact radius about P from the node's vertices: k_node_radius, after the refit
    R.pad = 0.0;
}

__device__ __forceinline__ void store_rec(StageRec* dst, const StageRec& R) {
    *dst = R;  // read by a later launch (k_refit_level)
}

// The leaf pass: one emitted leaf per thread (k_refit_level then combines the internal nodes).
__global__ void k_refit(int num_leaves, const int* __restrict__ leaf_list,
                        const uint64_t* __restrict__ keys, const int* __restrict__ first,
                        const int* __restrict__ last, const int* __restrict__ pos,
                        const uint32_t* __restrict__ tri_of_slot, const float* __restrict__ V,
                        const int32_t* __restrict__ F, const int64_t* __restrict__ voff,
                        StageRec* __restrict__ stage) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= num_leaves) return;
    const int e = leaf_list[k];
    StageRec R;
    leaf_moments(V, F, voff, keys, tri_of_slot, first[e], last[e], R);
    store_rec(&stage[pos[e]], R);
}

// The refit's leaf list grouped by triangle count (a counting sort over 1..16), so that the 32
// leaves of a warp run the same number of triangle iterations: the FP64 pipe costs the same for
// a warp instruction whatever the number of active lanes.
constexpr int kLeafSizes = 17;  // counts 0..16 (WARP_LEAF_MAX); 0 does not occur

__device__ __forceinline__ int leaf_size_of(const int* __restrict__ first,
                                            const int* __restrict__ last, int u) {
    return min(max(last[u] - first[u] + 1, 0), kLeafSizes - 1);
}

__global__ void k_leaf_hist(int nl, const int* __restrict__ leaves, const int* __restrict__ first,
                            const int* __restrict__ last, int* __restrict__ hist) {
    __shared__ int h[kLeafSizes];
    if (threadIdx.x < kLeafSizes) h[threadIdx.x] = 0;
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nl) atomicAdd(&h[leaf_size_of(first, last, leaves[k])], 1);
    __syncthreads();
    if (threadIdx.x < kLeafSizes && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

__global__ void k_leaf_offsets(int* __restrict__ hist) {  // one thread: exclusive scan in place
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int acc = 0;
    for (int i = 0; i < kLeafSizes; ++i) {
        const int c = hist[i];
        hist[i] = acc;
        acc += c;
    }
}

__global__ void k_leaf_sort(int nl, const int* __restrict__ leaves, const int* __restrict__ first,
                            const int* __restrict__ last, int* __restrict__ offset,
                            int* __restrict__ sorted) {
    __shared__ int cnt[kLeafSizes];   // the block's leaves per size (ranks from shared atomics)
    __shared__ int base[kLeafSizes];  // where they go: one global atomic per non-zero size
    if (threadIdx.x < kLeafSizes) cnt[threadIdx.x] = 0;
    __syncthreads();
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    int u = -1, sz = 0, rank = 0;
    if (k < nl) {
        u = leaves[k];
        sz = leaf_size_of(first, last, u);
        rank = atomicAdd(&cnt[sz], 1);
    }
    __syncthreads();
    if (threadIdx.x < kLeafSizes && cnt[threadIdx.x])
        base[threadIdx.x] = atomicAdd(&offset[threadIdx.x], cnt[threadIdx.x]);
    __syncthreads();
    if (u >= 0) sorted[base[sz] + rank] = u;
}

// The internal nodes of one level of a split tree, or of one height of the LBVH
// (nodes[0 .. count)): each combines its two children, whose records the leaf pass or an
// earlier (deeper, or lower) list wrote.
__global__ void __launch_bounds__(128, 4) k_refit_level(int count, const int* __restrict__ nodes,
                              const int* __restrict__ left, const int* __restrict__ right,
                              const int* __restrict__ pos, StageRec* __restrict__ stage,
                              unsigned* __restrict__ status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const int p = nodes[k];
    const int l = left[p], r = right[p];
    if (l < 0 || r < 0 || pos[l] < 0 || pos[r] < 0) {
        atomicOr(status, ST_REFIT_ORPHAN);
        return;
    }
    StageRec R;
    combine_moments(&stage[pos[l]], &stage[pos[r]], R);
    store_rec(&stage[pos[p]], R);
}

// LBVH: the height of every emitted internal node (a leaf is 0, a node one more than its taller
// child), by an integer ascent from the emitted leaves (the second child to arrive continues);
// the FP64 combine then runs height by height over dense lists (k_refit_level), like the split
// tree's levels, instead of on the ascent's ever sparser warps.
constexpr int kMaxHeight = 4 * 64 + 64;  // key bits + index bits bound the depth

__global__ void k_heights(int num_leaves, const int* __restrict__ leaf_list,
                          const uint64_t* __restrict__ keys, const int* __restrict__ parent,
                          const int* __restrict__ first, const int* __restrict__ last,
                          int* __restrict__ visit, int* __restrict__ height,
                          unsigned* __restrict__ status) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= num_leaves) return;
    int v = leaf_list[k], h = 0;
    for (int guard = 0; v != 0; ++guard) {
        const int p = parent[v];
        if (p < 0) {  // in the LBVH only node 0 has no parent
            atomicOr(status, ST_REFIT_ORPHAN);
            return;
        }
        if (is_cross(keys, first, last, p)) return;  // v is a mesh root
        if (guard >= kMaxHeight - 1) {
            atomicOr(status, ST_REFIT_ORPHAN);
            return;
        }
        atomicMax(&height[p], h + 1);
        __threadfence();
        if (atomicAdd(&visit[p], 1) == 0) return;  // first arrival: the sibling continues
        __threadfence();
        h = atomicAdd(&height[p], 0);  // both children's contributions are in
        v = p;
    }
}

// Counting sort of the emitted internal nodes (not spanning meshes) by height: hist[h] counts,
// then (after an exclusive scan) list[offset[h] + rank] = node.
__device__ __forceinline__ bool refit_internal(const uint64_t* __restrict__ keys,
                                               const int* __restrict__ first,
                                               const int* __restrict__ last,
                                               const uint8_t* __restrict__ flags, int u) {
    const uint8_t fl = flags[u];
    return (fl & 1) && !(fl & 2) && !is_cross(keys, first, last, u);
}

__global__ void k_height_hist(int nint, const uint64_t* __restrict__ keys,
                              const int* __restrict__ first, const int* __restrict__ last,
                              const uint8_t* __restrict__ flags, const int* __restrict__ height,
                              int* __restrict__ hist, unsigned* __restrict__ status) {
    __shared__ int h_s[kMaxHeight];  // the block's counts, then one atomic per non-zero entry
    for (int i = threadIdx.x; i < kMaxHeight; i += blockDim.x) h_s[i] = 0;
    __syncthreads();
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u < nint && refit_internal(keys, first, last, flags, u)) {
        if (height[u] < 0 || height[u] >= kMaxHeight) atomicOr(status, ST_REFIT_ORPHAN);
        atomicAdd(&h_s[min(max(height[u], 0), kMaxHeight - 1)], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kMaxHeight; i += blockDim.x)
        if (h_s[i]) atomicAdd(&hist[i], h_s[i]);
}

__global__ void k_height_offsets(int* __restrict__ hist) {  // one thread: exclusive scan in place
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int acc = 0;
    for (int i = 0; i < kMaxHeight; ++i) {
        const int c = hist[i];
        hist[i] = acc;
        acc += c;
    }
}

__global__ void k_height_sort(int nint, const uint64_t* __restrict__ keys,
                              const int* __restrict__ first, const int* __restrict__ last,
                              const uint8_t* __restrict__ flags, const int* __restrict__ height,
                              int* __restrict__ offset, int* __restrict__ list) {
    __shared__ int cnt[kMaxHeight];   // the block's nodes per key (ranks from shared atomics)
    __shared__ int base[kMaxHeight];  // where they go: one global atomic per non-zero key
    for (int i = threadIdx.x; i < kMaxHeight; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    int h = -1, rank = 0;
    if (u < nint && refit_internal(keys, first, last, flags, u)) {
        h = min(max(height[u], 0), kMaxHeight - 1);
        rank = atomicAdd(&cnt[h], 1);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kMaxHeight; i += blockDim.x)
        if (cnt[i]) base[i] = atomicAdd(&offset[i], cnt[i]);
    __syncthreads();
    if (h >= 0) list[base[h] + rank] = u;
}

// ---- K4a: exact node radii ------------------------------------------------------------------------
// The far test of a node compares |q - P| with beta * r, so r must bound the distance from P to
// every point of the node's triangles; the tightest such bound is the distance to the farthest
// vertex (triangles are convex hulls of their vertices). Leaves compute it in leaf_moments. An
// internal node's triangles are the contiguous run of sorted slots [first, last]. Every internal
// node of at most kRadiusChunk triangles (all but the top few levels) takes one warp of its own
// (a compacted list, so large and small nodes spread evenly over the warps); larger ones are
// split into chunks of kRadiusChunk slots, one warp per chunk, whose maxima meet in an atomicMax
// on the bit pattern (non-negative doubles order like their bits). A maximum does not depend on
// the order, so it equals the serial one bit for bit.
constexpr int kRadiusChunk = 2048;

// The warp's threshold after a one-pass screen, and whether a second pass is needed (some lane
// dropped a vertex that reaches it, or the estimates left float's range).
__device__ __forceinline__ bool top2_threshold(const LaneTop2& t, float& thr) {
    float m = t.m;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    thr = m * 0.99999f - 1e-37f;
    return __any_sync(0xffffffffu, !(m < INFINITY) || !(t.dropped < thr));
}

// Largest vertex_r2 over slots [s0, s1), one warp: a one-pass float screen (LaneTop2), then the
// exact FP64 term of the vertices whose estimate reaches M (1 - 1e-5) only, M being the largest
// estimate (a second pass over the slots finds them when the two kept per lane may not hold them
// all, or near float's underflow or overflow, where every vertex is taken). The vertex with the
// largest exact term always qualifies, so the result is the plain FP64 maximum bit for bit, at a
// few FP64 terms per run instead of three per triangle.
__device__ __forceinline__ double slots_r2(const TriF32* __restrict__ tris, int s0, int s1,
                                           const double* P, int lane) {
    const float Pf[3] = {d2f(P[0]), d2f(P[1]), d2f(P[2])};
    LaneTop2 t;
    for (int s = s0 + lane; s < s1; s += 32) t.add_slot(tris[s], Pf);
    float thr;
    double r2 = 0.0;
    if (top2_threshold(t, thr)) {
        const bool all = !(thr < INFINITY);
        for (int s = s0 + lane; s < s1; s += 32) {
            const float4 t0 = tris[s].t0, t1 = tris[s].t1, t2 = tris[s].t2;
            if (all || vertex_est(t0.x, t0.y, t0.z, Pf) >= thr) r2 = fmax(r2, vertex_r2(t0.x, t0.y, t0.z, P));
            if (all || vertex_est(t0.w, t1.x, t1.y, Pf) >= thr) r2 = fmax(r2, vertex_r2(t0.w, t1.x, t1.y, P));
            if (all || vertex_est(t1.z, t1.w, t2.x, Pf) >= thr) r2 = fmax(r2, vertex_r2(t1.z, t1.w, t2.x, P));
        }
    } else {
        if (t.e0 >= thr) r2 = vertex_r2(t.x0, t.y0, t.z0, P);
        if (t.e1 >= thr) r2 = fmax(r2, vertex_r2(t.x1, t.y1, t.z1, P));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r2 = fmax(r2, __shfl_xor_sync(0xffffffffu, r2, o));
    return r2;
}

__device__ __forceinline__ bool internal_emitted(const uint64_t* __restrict__ keys,
                                                 const int* __restrict__ first,
                                                 const int* __restrict__ last,
                                                 const uint8_t* __restrict__ flags, int u) {
    const uint8_t fl = flags[u];
    return (fl & 1) && !(fl & 2) && !is_cross(keys, first, last, u);
}

// chunks[u] for the nodes u < num_nodes (0 unless an emitted single-mesh internal node of more than
// kRadiusChunk triangles); chunks[num_nodes] = 0 becomes the total after the exclusive scan.
__global__ void k_radius_chunks(int num_nodes, const uint64_t* __restrict__ keys,
                                const int* __restrict__ first, const int* __restrict__ last,
                                const uint8_t* __restrict__ flags, int* __restrict__ chunks) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u > num_nodes) return;
    chunks[u] = (u < num_nodes && internal_emitted(keys, first, last, flags, u) &&
                 last[u] - first[u] + 1 > kRadiusChunk)
                    ? (last[u] - first[u] + kRadiusChunk) / kRadiusChunk
                    : 0;
}

// The internal nodes of at most kRadiusChunk triangles, in any order (list[0 .. *count)).
__global__ void k_radius_list(int num_nodes, const uint64_t* __restrict__ keys,
                              const int* __restrict__ first, const int* __restrict__ last,
                              const uint8_t* __restrict__ flags, int* __restrict__ list,
                              int* __restrict__ count) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    const bool pred = u < num_nodes && internal_emitted(keys, first, last, flags, u) &&
                      last[u] - first[u] + 1 <= kRadiusChunk;
    const int at = block_append(count, pred);
    if (at >= 0) list[at] = u;
}

// One warp per listed node (grid-stride), all lanes on its slot run. The float screen runs per
// node in one pass (LaneTop2; a second pass only on ties); the vertices that pass it (a few per
// node) queue in the warp's shared buffer across the
// warp's nodes and get their exact FP64 terms 32 at a time, one per lane, so the FP64 pipe (2
// operations per SM per cycle on GB300, whatever the number of active lanes) sees full warps;
// each term goes to its node's maximum by atomicMax on the bit pattern (r2bits starts at 0).
constexpr int kRadiusWarps = 8;      // warps per block of k_node_radius_small
constexpr int kRadiusQueue = 64;     // queued vertices per warp (< 32 left + 32 added)

struct RadiusQueue {
    float x[kRadiusQueue], y[kRadiusQueue], z[kRadiusQueue];
    int node[kRadiusQueue];
};

__device__ __forceinline__ void radius_flush(RadiusQueue& q, int count,
                                             const StageRec* __restrict__ stage,
                                             unsigned long long* __restrict__ r2bits, int lane) {
    __syncwarp();
    if (lane < count) {
        const int i = q.node[lane];
        const double P[3] = {stage[i].P[0], stage[i].P[1], stage[i].P[2]};
        const double r2 = vertex_r2(q.x[lane], q.y[lane], q.z[lane], P);
        atomicMax(&r2bits[i], (unsigned long long)__double_as_longlong(r2));
    }
    __syncwarp();
}

__global__ void __launch_bounds__(32 * kRadiusWarps)
k_node_radius_small(const int* __restrict__ list, const int* __restrict__ count,
                    const int* __restrict__ first, const int* __restrict__ last,
                    const int* __restrict__ pos, const StageRec* __restrict__ stage,
                    const TriF32* __restrict__ tris, unsigned long long* __restrict__ r2bits) {
    __shared__ RadiusQueue queues[kRadiusWarps];
    RadiusQueue& q = queues[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    const int total = *count;
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    int queued = 0;  // warp-uniform
    // queue one vertex per lane where c holds (a warp-wide step), evaluating full groups of 32
    auto enqueue = [&](bool c, float x, float y, float z, int node) {
        const unsigned bal = __ballot_sync(0xffffffffu, c);
        if (c) {
            const int k = queued + __popc(bal & lt);
            q.x[k] = x;
            q.y[k] = y;
            q.z[k] = z;
            q.node[k] = node;
        }
        queued += __popc(bal);
        while (queued >= 32) {  // evaluate 32, move the rest down (each lane its own column)
            radius_flush(q, 32, stage, r2bits, lane);
            for (int k = 32 + lane; k < queued; k += 32) {
                q.x[k - 32] = q.x[k];
                q.y[k - 32] = q.y[k];
                q.z[k - 32] = q.z[k];
                q.node[k - 32] = q.node[k];
            }
            __syncwarp();
            queued -= 32;
        }  // queued < 32 here: the next step adds at most 32 (< kRadiusQueue)
    };
    for (int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < total; w += nwarps) {
        const int v = list[w];
        const int i = pos[v];
        const int s0 = first[v], s1 = last[v] + 1;
        const float Pf[3] = {d2f(stage[i].P[0]), d2f(stage[i].P[1]), d2f(stage[i].P[2])};
        LaneTop2 t;
        for (int s = s0 + lane; s < s1; s += 32) t.add_slot(tris[s], Pf);
        float thr;
        if (!top2_threshold(t, thr)) {  // the two kept per lane hold every candidate
            enqueue(t.e0 >= thr, t.x0, t.y0, t.z0, i);
            enqueue(t.e1 >= thr, t.x1, t.y1, t.z1, i);
            continue;
        }
        const bool all = !(thr < INFINITY);
        for (int base = s0; base < s1; base += 32) {  // second pass, warp-uniform trip count
            const int s = base + lane;
            float vx[3] = {0.f, 0.f, 0.f}, vy[3] = {0.f, 0.f, 0.f}, vz[3] = {0.f, 0.f, 0.f};
            if (s < s1) {
                const float4 t0 = tris[s].t0, t1 = tris[s].t1, t2 = tris[s].t2;
                vx[0] = t0.x; vy[0] = t0.y; vz[0] = t0.z;
                vx[1] = t0.w; vy[1] = t1.x; vz[1] = t1.y;
                vx[2] = t1.z; vy[2] = t1.w; vz[2] = t2.x;
            }
#pragma unroll
            for (int j = 0; j < 3; ++j)
                enqueue(s < s1 && (all || vertex_est(vx[j], vy[j], vz[j], Pf) >= thr), vx[j], vy[j],
                        vz[j], i);
        }
    }
    if (queued > 0) radius_flush(q, queued, stage, r2bits, lane);
}

// Grid-stride over the chunks: chunk c belongs to the last node u with off[u] <= c.
__global__ void k_node_radius(int num_nodes, const int* __restrict__ off,
                              const int* __restrict__ first, const int* __restrict__ last,
                              const int* __restrict__ pos, const StageRec* __restrict__ stage,
                              const TriF32* __restrict__ tris,
                              unsigned long long* __restrict__ r2bits) {
    const int lane = threadIdx.x & 31;
    const int total = off[num_nodes];
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); c < total; c += nwarps) {
        int lo = 0, hi = num_nodes - 1;  // off[num_nodes] = total > c
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (off[mid] <= c) lo = mid; else hi = mid - 1;
        }
        const int u = lo;
        const int s0 = first[u] + (c - off[u]) * kRadiusChunk;
        const int s1 = min(last[u] + 1, s0 + kRadiusChunk);
        const int i = pos[u];
        const double P[3] = {stage[i].P[0], stage[i].P[1], stage[i].P[2]};
        const double r2 = slots_r2(tris, s0, s1, P, lane);
        if (lane == 0) atomicMax(&r2bits[i], (unsigned long long)__double_as_longlong(r2));
    }
}

// ---- K4b: records -------------------------------------------------------------------------------
struct Coeffs {
    double trM1, N[3], W[3], C[6], D[10];
};

__device__ void derive_coeffs(const StageRec& R, Coeffs& c) {
    const double* M1 = R.M1;
    const double* M2 = R.M2;  // [i*6 + s], s: xx yy zz xy xz yz
    c.trM1 = (M1[0] + M1[4]) + M1[8];
    for (int i = 0; i < 3; ++i) c.N[i] = R.N[i];
    // C = -3 sym(M1): d^T C d with off-diagonals doubled
    c.C[0] = -3.0 * M1[0];
    c.C[1] = -3.0 * M1[4];
    c.C[2] = -3.0 * M1[8];
    c.C[3] = -3.0 * (M1[1] + M1[3]);
    c.C[4] = -3.0 * (M1[2] + M1[6]);
    c.C[5] = -3.0 * (M1[5] + M1[7]);
    // u_k = sum_i M2[i][ik], v_i = sum_j M2[i][jj]; W = -1.5 (2u + v)
    auto m2 = [&](int i, int j, int k) -> double {
        // symmetric pair (j,k) -> slot
        int a = j < k ? j : k, b = j < k ? k : j;
        int s = (a == b) ? a : (a == 0 ? (b == 1 ? 3 : 4) : 5);
        return M2[6 * i + s];
    };
    for (int k = 0; k < 3; ++k) {
        const double u = (m2(0, 0, k) + m2(1, 1, k)) + m2(2, 2, k);
        const double v = (m2(k, 0, 0) + m2(k, 1, 1)) + m2(k, 2, 2);
        c.W[k] = -1.5 * (2.0 * u + v);
    }
    // D = 7.5 * coefficients of the cubic sum_ijk M2_ijk d_i d_j d_k per monomial
    const double xxx = m2(0, 0, 0), yyy = m2(1, 1, 1), zzz = m2(2, 2, 2);
    const double xxy = 2.0 * m2(0, 0, 1) + m2(1, 0, 0);
    const double xxz = 2.0 * m2(0, 0, 2) + m2(2, 0, 0);
    const double xyy = 2.0 * m2(1, 0, 1) + m2(0, 1, 1);
    const double yyz = 2.0 * m2(1, 1, 2) + m2(2, 1, 1);
    const double xzz = 2.0 * m2(2, 0, 2) + m2(0, 2, 2);
    const double yzz = 2.0 * m2(2, 1, 2) + m2(1, 2, 2);
    const double xyz = 2.0 * ((m2(0, 1, 2) + m2(1, 0, 2)) + m2(2, 0, 1));
    const double mono[10] = {xxx, yyy, zzz, xxy, xxz, xyy, yyz, xzz, yzz, xyz};
    for (int i = 0; i < 10; ++i) c.D[i] = 7.5 * mono[i];
}

// The emitted node at each DFS position (node_of_pos[pos[u]] = u), so that the conversion runs
// one thread per record: the LBVH's emitted nodes are scattered among its 2n - 1 Karras nodes,
// and a thread per Karras node leaves the FP64 work of the conversion on sparse warps.
__global__ void k_node_of_pos(int num_nodes, const uint8_t* __restrict__ flags,
                              const int* __restrict__ pos, int* __restrict__ node_of_pos) {
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u < num_nodes && (flags[u] & 1)) node_of_pos[pos[u]] = u;
}

__global__ void k_convert(int num_records, const int* __restrict__ node_of_pos,
                          const uint64_t* __restrict__ keys, const int* __restrict__ first,
                          const int* __restrict__ last, const uint8_t* __restrict__ flags,
                          const int* __restrict__ skip,
                          StageRec* __restrict__ stage, const unsigned long long* __restrict__ r2bits,
                          NodeF32* __restrict__ n32, NodeF64* __restrict__ n64,
                          int* __restrict__ leaf_count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int u = i < num_records ? node_of_pos[i] : 0;
    const bool cross = i < num_records && is_cross(keys, first, last, u);
    const bool leaf = i < num_records && (flags[u] & 2) && !cross;
    const int nleaf = __syncthreads_count(leaf);  // counts the leaves, one atomic per block
    if (threadIdx.x == 0 && nleaf) atomicAdd(leaf_count, nleaf);
    if (i >= num_records) return;
    const int tb = first[u];
    const int tc = leaf ? (last[u] - first[u] + 1) : 0;
    Coeffs c;
    StageRec R;
    if (!cross) {
        R = stage[i];
        if (!leaf) {  // internal: the exact radius of k_node_radius
            R.r = round_up_float(sqrt(__longlong_as_double((long long)r2bits[i])));
            stage[i].r = R.r;
        }
        derive_coeffs(R, c);
    } else {
        memset(&R, 0, sizeof(R));
        memset(&c, 0, sizeof(c));
    }
    if (n32) {
        NodeF32 o;
        o.s0 = make_float4(d2f(R.P[0]), d2f(R.P[1]), d2f(R.P[2]), d2f(R.r));
        o.skip = skip[u];
        o.tri_begin = tb;
        o.tri_count = tc;
        o.trM1 = d2f(c.trM1);
        o.m0 = make_float4(d2f(c.N[0]), d2f(c.N[1]), d2f(c.N[2]), d2f(c.W[0]));
        o.m1 = make_float4(d2f(c.W[1]), d2f(c.W[2]), d2f(c.C[0]), d2f(c.C[1]));
        o.m2 = make_float4(d2f(c.C[2]), d2f(c.C[3]), d2f(c.C[4]), d2f(c.C[5]));
        o.m3 = make_float4(d2f(c.D[0]), d2f(c.D[1]), d2f(c.D[2]), d2f(c.D[3]));
        o.m4 = make_float4(d2f(c.D[4]), d2f(c.D[5]), d2f(c.D[6]), d2f(c.D[7]));
        o.m5 = make_float4(d2f(c.D[8]), d2f(c.D[9]), 0.f, 0.f);
        n32[i] = o;
    }
    if (n64) {
        NodeF64 o;
        for (int a = 0; a < 3; ++a) {
            o.P[a] = R.P[a];
            o.N[a] = c.N[a];
            o.W[a] = c.W[a];
        }
        o.r = R.r;
        o.skip = skip[u];
        o.tri_begin = tb;
        o.tri_count = tc;
        o.pad0 = 0;
        o.trM1 = c.trM1;
        for (int a = 0; a < 6; ++a) o.C[a] = c.C[a];
        for (int a = 0; a < 10; ++a) o.D[a] = c.D[a];
        o.pad1[0] = o.pad1[1] = o.pad1[2] = 0.0;
        n64[i] = o;
    }
}

// Structure-of-arrays copy of the FP32 records (tuning variant 7): float4 k of node i goes to
// soa[k * num_nodes + i].
__global__ void k_aos_to_soa(int64_t num_nodes, const NodeF32* __restrict__ n32,
                             float4* __restrict__ soa) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num_nodes) return;
    const float4* r = reinterpret_cast<const float4*>(n32 + i);
#pragma unroll
    for (int k = 0; k < 8; ++k) soa[k * num_nodes + i] = r[k];
}

__global__ void k_tri_records(int n, const uint32_t* __restrict__ tri_of_slot,
                              const uint64_t* __restrict__ keys, const float* __restrict__ V,
                              const int32_t* __restrict__ F, const int64_t* __restrict__ voff,
                              TriF32* __restrict__ tris, int* __restrict__ sorted_tri) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int64_t t = tri_of_slot[s];
    const int m = (int)(keys[s] >> MORTON_BITS);
    float v[3][3];
    for (int j = 0; j < 3; ++j) {
        const int64_t vi = voff[m] + F[3 * t + j];
        v[j][0] = V[3 * vi];
        v[j][1] = V[3 * vi + 1];
        v[j][2] = V[3 * vi + 2];
    }
    float c[3];
    for (int a = 0; a < 3; ++a) c[a] = ((v[0][a] + v[1][a]) + v[2][a]) / 3.0f;
    float rt = 0.f;
    for (int j = 0; j < 3; ++j) {
        const float dx = v[j][0] - c[0], dy = v[j][1] - c[1], dz = v[j][2] - c[2];
        rt = fmaxf(rt, sqrtf(dx * dx + dy * dy + dz * dz));
    }
    rt = rt * 1.0000010f + 1e-30f;  // conservative: the bound only selects the FP64 near field
    const float e1x = v[1][0] - v[0][0], e1y = v[1][1] - v[0][1], e1z = v[1][2] - v[0][2];
    const float e2x = v[2][0] - v[0][0], e2y = v[2][1] - v[0][1], e2z = v[2][2] - v[0][2];
    const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
    const float nl = sqrtf(nx * nx + ny * ny + nz * nz);
    TriF32 o;
    o.t0 = make_float4(v[0][0], v[0][1], v[0][2], v[1][0]);
    o.t1 = make_float4(v[1][1], v[1][2], v[2][0], v[2][1]);
    o.t2 = make_float4(v[2][2], rt, nl > 0.f ? 1.0f / nl : 0.f, 0.f);
    tris[s] = o;
    sorted_tri[s] = (int)t;
}

// Build temporaries come from the library's build pool, which keeps freed memory mapped across
// synchronisations (up to kBuildRetainBytes): a rebuild, or the next mesh of a batch, reuses it
// instead of mapping gigabytes of new pages (the device's default pool returns freed memory at
// every synchronisation).
template <class T> T* dalloc(size_t count, cudaStream_t s) {
    return count ? static_cast<T*>(build_alloc(count * sizeof(T), s)) : nullptr;
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace

void build_forest(Engine& e, const float* d_V, const int64_t* voff_h, const int32_t* d_F,
                  const int64_t* foff_h, int64_t nmeshes, cudaStream_t st) {
    if (nmeshes <= 0 || nmeshes > 65535)
        throw Error(FWN_INVALID_ARG, "number of meshes must be in [1, 65535]");
    for (int64_t m = 0; m < nmeshes; ++m) {
        if (voff_h[m + 1] < voff_h[m] || foff_h[m + 1] < foff_h[m] || voff_h[0] != 0 ||
            foff_h[0] != 0)
            throw Error(FWN_INVALID_ARG, "vertex/triangle offsets must start at 0 and not decrease");
    }
    const int64_t nv = voff_h[nmeshes], nf = foff_h[nmeshes];
    if (nf > (int64_t)0x3fffffff)
        throw Error(FWN_INVALID_ARG, "at most 2^30-1 triangles per forest");
    e.nv = nv;
    e.nf = nf;
    e.nmeshes = nmeshes;
    const int K = e.cfg.leaf_size;
    NvtxRange trace_build("fwn build");

    cudaEvent_t ev0, ev1;
    FWN_CUDA_CHECK(cudaEventCreate(&ev0));
    FWN_CUDA_CHECK(cudaEventCreate(&ev1));
    FWN_CUDA_CHECK(cudaEventRecord(ev0, st));

    int64_t* voff = dalloc<int64_t>(nmeshes + 1, st);
    int64_t* foff = dalloc<int64_t>(nmeshes + 1, st);
    FWN_CUDA_CHECK(cudaMemcpyAsync(voff, voff_h, (nmeshes + 1) * sizeof(int64_t),
                                   cudaMemcpyHostToDevice, st));
    FWN_CUDA_CHECK(cudaMemcpyAsync(foff, foff_h, (nmeshes + 1) * sizeof(int64_t),
                                   cudaMemcpyHostToDevice, st));
    FWN_CUDA_CHECK(cudaMalloc(&e.meshes, nmeshes * sizeof(MeshInfo)));
    e.meshes_h = new MeshInfo[nmeshes];
    unsigned* enc = dalloc<unsigned>(6 * nmeshes, st);
    unsigned* status = dalloc<unsigned>(1, st);
    FWN_CUDA_CHECK(cudaMemsetAsync(status, 0, sizeof(unsigned), st));
    k_init_bbox<<<grid_for(6 * nmeshes, 256), 256, 0, st>>>(enc, (int)nmeshes);
    int64_t maxv = 0;
    for (int64_t m = 0; m < nmeshes; ++m) maxv = std::max(maxv, voff_h[m + 1] - voff_h[m]);
    if (maxv > 0) {
        const int chunk = 16384;
        dim3 g((unsigned)((maxv + chunk - 1) / chunk), (unsigned)nmeshes);
        k_mesh_bbox<<<g, 256, 0, st>>>(d_V, voff, chunk, enc);
    }
    k_mesh_info<<<grid_for(nmeshes, 128), 128, 0, st>>>(enc, voff, (int)nmeshes,
                                                        e.cfg.fp64_near_scale, e.cfg.fp64_cond,
                                                        e.meshes);
    FWN_CUDA_CHECK(cudaGetLastError());

    struct TmpList {  // stream-ordered frees on every exit path
        std::vector<void*> v;
        cudaStream_t s;
        ~TmpList() {
            for (void* p : v) cudaFreeAsync(p, s);
        }
    } tmp{{}, st};
    auto track = [&](void* p) { tmp.v.push_back(p); return p; };
    track(voff);
    track(foff);
    track(enc);
    track(status);

    if (nf > 0) {
        const int n = (int)nf;
        const bool split = e.cfg.builder != FWN_BUILDER_LBVH;  // top-down (midpoint or binned)
        const bool binned = e.cfg.builder == FWN_BUILDER_BINNED;
        // node arrays: the LBVH's Karras tree has 2n - 1 nodes (internal 0..n-2, leaves after);
        // a split tree at most 2n - 1 as well, ids in creation order
        const int cap = split ? 2 * n : 2 * n - 1;
        const int nint = split ? cap : std::max(n - 1, 1);  // left / right / visit entries
        int* parent = (int*)track(dalloc<int>(cap, st));
        int* first = (int*)track(dalloc<int>(cap, st));
        int* last = (int*)track(dalloc<int>(cap, st));
        int* left = (int*)track(dalloc<int>(nint, st));
        int* right = (int*)track(dalloc<int>(nint, st));
        int* cnt = (int*)track(dalloc<int>(n + 1, st));
        uint8_t* flags = (uint8_t*)track(dalloc<uint8_t>(cap, st));
        int* pos = (int*)track(dalloc<int>(cap, st));
        int* skip = (int*)track(dalloc<int>(cap, st));
        void* scan_tmp = track(dalloc<char>(exclusive_scan_temp_bytes(cap + 1), st));
        int* visit = (int*)track(dalloc<int>(nint, st));
        int* leaf_list = (int*)track(dalloc<int>(n, st));
        int* leaf_list_len = (int*)track(dalloc<int>(1, st));
        int* leaf_count = (int*)track(dalloc<int>(1, st));
        const uint64_t* keys = nullptr;
        const uint32_t* tri_of_slot = nullptr;
        int num_nodes = 0;
        unsigned st_h = 0;
        // split tree: every node's depth (roots 0), the order of the level-by-level refit
        int* depth_of = split ? (int*)track(dalloc<int>(cap, st)) : nullptr;
        auto check_input = [&]() {
            FWN_CUDA_CHECK(cudaMemcpyAsync(&st_h, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
            FWN_CUDA_CHECK(cudaStreamSynchronize(st));
            if (st_h & ST_BAD_INDEX) throw Error(FWN_INVALID_ARG, "triangle vertex index out of range");
            if (st_h & ST_NONFINITE)
                throw Error(FWN_INVALID_ARG, "non-finite vertex coordinate referenced by a triangle");
        };

        if (!split) {
            int mesh_bits = 0;
            while ((1ll << mesh_bits) < nmeshes) ++mesh_bits;
            uint64_t* keys_a = (uint64_t*)track(dalloc<uint64_t>(n, st));
            uint64_t* keys_b = (uint64_t*)track(dalloc<uint64_t>(n, st));
            uint32_t* vals_a = (uint32_t*)track(dalloc<uint32_t>(n, st));
            uint32_t* vals_b = (uint32_t*)track(dalloc<uint32_t>(n, st));
            void* sort_tmp = track(dalloc<char>(radix_sort_temp_bytes(n, 8), st));
            NvtxRange trace_keys("fwn build: Morton keys + sort");
            k_tri_keys<<<grid_for(n, 256), 256, 0, st>>>(d_V, d_F, voff, foff, (int)nmeshes, nf,
                                                         e.meshes, keys_a, vals_a, status);
            FWN_CUDA_CHECK(cudaGetLastError());
            check_input();
            const bool in_b = radix_sort_u64(keys_a, vals_a, keys_b, vals_b, n,
                                             MORTON_BITS + mesh_bits, sort_tmp, st);
            keys = in_b ? keys_b : keys_a;
            tri_of_slot = in_b ? vals_b : vals_a;

            const int nn = 2 * n - 1;
            num_nodes = nn;
            NvtxRange trace_tree("fwn build: Karras tree + DFS layout");
            FWN_CUDA_CHECK(cudaMemsetAsync(parent, 0xff, (size_t)nn * sizeof(int), st));  // -1
            k_leaf_init<<<grid_for(n, 256), 256, 0, st>>>(n, first, last);
            if (n == 1) {
                int m1 = -1;
                FWN_CUDA_CHECK(cudaMemcpyAsync(parent, &m1, sizeof(int), cudaMemcpyHostToDevice, st));
            } else {
                k_karras<<<grid_for(n - 1, 256), 256, 0, st>>>(keys, n, left, right, parent, first, last);
            }
            FWN_CUDA_CHECK(cudaMemsetAsync(cnt, 0, (n + 1) * sizeof(int), st));
            FWN_CUDA_CHECK(cudaMemsetAsync(leaf_list_len, 0, sizeof(int), st));
            k_emit_count<<<grid_for(nn, 256), 256, 0, st>>>(n, K, keys, parent, first, last, cnt, flags,
                                                            leaf_list, leaf_list_len);
            exclusive_scan_i32(cnt, n + 1, scan_tmp, st);
            k_positions<<<grid_for(nn, 256), 256, 0, st>>>(nn, parent, first, last, flags, cnt, pos, skip);
            k_mesh_roots<<<grid_for(nmeshes, 128), 128, 0, st>>>((int)nmeshes, foff, n, parent, first,
                                                                 last, pos, skip, e.meshes);
        } else {
            NvtxRange trace_tree("fwn build: top-down splits + DFS layout");
            // roots: one node per non-empty mesh; a mesh of > kFinishSlots triangles is an active
            // segment of the first level, one of K < size <= kFinishSlots a small segment
            std::vector<int> root_node(nmeshes, -1), mesh_seg(nmeshes, -1);
            std::vector<int> h_first, h_last, s_start, s_end, s_node;
            std::vector<int4> h_small;
            for (int64_t m = 0; m < nmeshes; ++m) {
                const int64_t b = foff_h[m], en = foff_h[m + 1];
                if (en <= b) continue;
                const int id = (int)h_first.size();
                root_node[m] = id;
                h_first.push_back((int)b);
                h_last.push_back((int)(en - 1));
                if (en - b > kFinishSlots) {
                    mesh_seg[m] = (int)s_start.size();
                    s_start.push_back((int)b);
                    s_end.push_back((int)en);
                    s_node.push_back(id);
                } else if (en - b > K) {
                    mesh_seg[m] = -2;
                    h_small.push_back(make_int4((int)b, (int)en, id, 0));
                }
            }
            const int nroots = (int)h_first.size();
            const int smax = n / 2 + (int)nmeshes + 1;  // active segments hold >= 2 triangles
            uint64_t* skeys = (uint64_t*)track(dalloc<uint64_t>(n, st));
            int* final_perm = (int*)track(dalloc<int>(n, st));
            SplitSlots A, B;
            for (SplitSlots* X : {&A, &B}) {
                X->perm = (int*)track(dalloc<int>(n, st));
                X->cx = (float*)track(dalloc<float>(n, st));
                X->cy = (float*)track(dalloc<float>(n, st));
                X->cz = (float*)track(dalloc<float>(n, st));
                X->seg = (int*)track(dalloc<int>(n, st));
            }
            int* lflags = (int*)track(dalloc<int>(n + 1, st));
            int* child_next = (int*)track(dalloc<int>(2 * (size_t)smax, st));
            int* counts = (int*)track(dalloc<int>(3, st));  // next level, small list, node ids
            int4* small = (int4*)track(dalloc<int4>(smax, st));
            if (!h_small.empty())
                FWN_CUDA_CHECK(cudaMemcpyAsync(small, h_small.data(), h_small.size() * sizeof(int4),
                                               cudaMemcpyHostToDevice, st));
            FWN_CUDA_CHECK(cudaMemsetAsync(depth_of, 0, (size_t)cap * sizeof(int), st));
            int* seg_a[3], *seg_b[3];  // start, end, node of this level / the next
            for (int k = 0; k < 3; ++k) {
                seg_a[k] = (int*)track(dalloc<int>(smax, st));
                seg_b[k] = (int*)track(dalloc<int>(smax, st));
            }
            const size_t box_words = std::max(6 * (size_t)smax, (size_t)kBoxCopies * kBoxCopyStride);
            unsigned* box_a = (unsigned*)track(dalloc<unsigned>(box_words, st));
            unsigned* box_b = (unsigned*)track(dalloc<unsigned>(box_words, st));
            int* axis_of = (int*)track(dalloc<int>(smax, st));
            float* split_of = (float*)track(dalloc<float>(smax, st));
            int* spatial_of = (int*)track(dalloc<int>(smax, st));
            int* bin_of = (int*)track(dalloc<int>(smax, st));
            float* seg_box = (float*)track(dalloc<float>(6 * (size_t)smax, st));
            // level-loop segments other than the roots hold more than kFinishSlots triangles each
            const int seg_bound = std::max((int)s_start.size(), n / (kFinishSlots + 1) + 1);
            unsigned* bins = (unsigned*)track(dalloc<unsigned>((size_t)seg_bound * kSegBinWords, st));
            int* d_mesh_seg = (int*)track(dalloc<int>(nmeshes, st));
            int* d_root_node = (int*)track(dalloc<int>(nmeshes, st));
            FWN_CUDA_CHECK(cudaMemcpyAsync(d_mesh_seg, mesh_seg.data(), nmeshes * sizeof(int),
                                           cudaMemcpyHostToDevice, st));
            FWN_CUDA_CHECK(cudaMemcpyAsync(d_root_node, root_node.data(), nmeshes * sizeof(int),
                                           cudaMemcpyHostToDevice, st));
            FWN_CUDA_CHECK(cudaMemcpyAsync(first, h_first.data(), nroots * sizeof(int),
                                           cudaMemcpyHostToDevice, st));
            FWN_CUDA_CHECK(cudaMemcpyAsync(last, h_last.data(), nroots * sizeof(int),
                                           cudaMemcpyHostToDevice, st));
            FWN_CUDA_CHECK(cudaMemsetAsync(parent, 0xff, (size_t)nroots * sizeof(int), st));
            FWN_CUDA_CHECK(cudaMemsetAsync(left, 0xff, (size_t)nroots * sizeof(int), st));
            FWN_CUDA_CHECK(cudaMemsetAsync(right, 0xff, (size_t)nroots * sizeof(int), st));
            int nact = (int)s_start.size();
            if (nact) {
                FWN_CUDA_CHECK(cudaMemcpyAsync(seg_a[0], s_start.data(), nact * sizeof(int),
                                               cudaMemcpyHostToDevice, st));
                FWN_CUDA_CHECK(cudaMemcpyAsync(seg_a[1], s_end.data(), nact * sizeof(int),
                                               cudaMemcpyHostToDevice, st));
                FWN_CUDA_CHECK(cudaMemcpyAsync(seg_a[2], s_node.data(), nact * sizeof(int),
                                               cudaMemcpyHostToDevice, st));
                k_split_box_init<<<grid_for(nact, 256), 256, 0, st>>>(nact, box_a);
            }
            k_split_init<<<grid_for(n, 256), 256, 0, st>>>(d_V, d_F, voff, foff, (int)nmeshes, nf,
                                                           d_mesh_seg, A, final_perm, skeys, box_a,
                                                           nact <= kBoxCopyKeys, status);
            FWN_CUDA_CHECK(cudaGetLastError());
            check_input();
            int node_base = nroots;
            int nsmall = (int)h_small.size();
            SplitSlots* cur = &A;
            SplitSlots* nxt = &B;
            int level = 0;
            while (nact > 0) {
                if (level > kSpatialLevels + 64)  // position splits halve every segment
                    throw Error(FWN_INTERNAL, "split build did not converge");
                if (node_base + 2 * nact > cap) throw Error(FWN_INTERNAL, "split build node overflow");
                if (nact > seg_bound) throw Error(FWN_INTERNAL, "split build segment overflow");
                k_split_decide<<<grid_for(nact, 128), 128, 0, st>>>(
                    nact, level >= kSpatialLevels, box_a, axis_of, split_of, spatial_of, seg_box);
                if (binned && level < kSpatialLevels) {  // the binned plane of each segment
                    const int words = nact * kSegBinWords;
                    k_split_bins_init<<<grid_for(words, 256), 256, 0, st>>>(words, bins);
                    k_split_bins<<<(int)((n + kBinChunk - 1) / kBinChunk), 256, 0, st>>>(
                        n, *cur, seg_box, bins, status);
                    k_split_choose<<<grid_for(32 * nact, 128), 128, 0, st>>>(nact, seg_box, bins,
                                                                             axis_of, bin_of,
                                                                             spatial_of);
                }
                k_split_flags<<<grid_for(n + 1, 256), 256, 0, st>>>(n, *cur, seg_a[0], seg_a[1],
                                                                   axis_of, split_of, spatial_of,
                                                                   bin_of, seg_box, lflags);
                exclusive_scan_i32(lflags, n + 1, scan_tmp, st);
                const int h_counts[2] = {0, nsmall};
                FWN_CUDA_CHECK(cudaMemcpyAsync(counts, h_counts, sizeof(h_counts),
                                               cudaMemcpyHostToDevice, st));
                k_split_children<<<grid_for(nact, 128), 128, 0, st>>>(
                    nact, node_base, level, K, seg_a[0], seg_a[1], seg_a[2], lflags, first, last,
                    parent, left, right, depth_of, counts, seg_b[0], seg_b[1], seg_b[2], box_b,
                    small, child_next);
                // lflags now holds the exclusive scan of the left flags (a slot's flag is the
                // step from its entry to the next)
                k_split_scatter<<<grid_for(n, 256), 256, 0, st>>>(n, *cur, *nxt, lflags, seg_a[0],
                                                                 seg_a[1], child_next, final_perm,
                                                                 box_b, counts);
                FWN_CUDA_CHECK(cudaGetLastError());
                node_base += 2 * nact;
                int next[2] = {0, 0};
                FWN_CUDA_CHECK(cudaMemcpyAsync(next, counts, sizeof(next), cudaMemcpyDeviceToHost,
                                               st));
                FWN_CUDA_CHECK(cudaStreamSynchronize(st));
                nact = next[0];
                nsmall = next[1];
                ++level;
                std::swap(cur, nxt);
                std::swap(box_a, box_b);
                for (int k = 0; k < 3; ++k) std::swap(seg_a[k], seg_b[k]);
            }
            if (nsmall > 0) {  // the small segments' subtrees, one block each
                FWN_CUDA_CHECK(cudaMemcpyAsync(counts + 2, &node_base, sizeof(int),
                                               cudaMemcpyHostToDevice, st));
                FWN_CUDA_CHECK(cudaFuncSetAttribute(k_split_finish,
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                    (int)sizeof(FinishShared)));
                k_split_finish<<<nsmall, kFinishThreads, sizeof(FinishShared), st>>>(
                    small, A, B, K, counts + 2, cap, first, last, parent, left, right, depth_of,
                    final_perm, status);
                FWN_CUDA_CHECK(cudaGetLastError());
                FWN_CUDA_CHECK(cudaMemcpyAsync(&node_base, counts + 2, sizeof(int),
                                               cudaMemcpyDeviceToHost, st));
                FWN_CUDA_CHECK(cudaMemcpyAsync(&st_h, status, sizeof(unsigned),
                                               cudaMemcpyDeviceToHost, st));
                FWN_CUDA_CHECK(cudaStreamSynchronize(st));
                if ((st_h & ST_BUILD_BOUND) || node_base > cap)
                    throw Error(FWN_INTERNAL, "split build passed its node or depth bound");
            }
            num_nodes = node_base;
            keys = skeys;
            tri_of_slot = reinterpret_cast<const uint32_t*>(final_perm);
            FWN_CUDA_CHECK(cudaMemsetAsync(cnt, 0, (n + 1) * sizeof(int), st));
            FWN_CUDA_CHECK(cudaMemsetAsync(leaf_list_len, 0, sizeof(int), st));
            k_split_emit<<<grid_for(num_nodes, 256), 256, 0, st>>>(num_nodes, first, left, flags, cnt,
                                                                   leaf_list, leaf_list_len);
            exclusive_scan_i32(cnt, n + 1, scan_tmp, st);
            k_positions<<<grid_for(num_nodes, 256), 256, 0, st>>>(num_nodes, parent, first, last,
                                                                  flags, cnt, pos, skip);
            k_split_mesh_roots<<<grid_for(nmeshes, 128), 128, 0, st>>>((int)nmeshes, d_root_node,
                                                                       pos, skip, e.meshes);
            FWN_CUDA_CHECK(cudaGetLastError());
        }
        int E = 0, NL = 0;
        FWN_CUDA_CHECK(cudaMemcpyAsync(&E, cnt + n, sizeof(int), cudaMemcpyDeviceToHost, st));
        FWN_CUDA_CHECK(cudaMemcpyAsync(&NL, leaf_list_len, sizeof(int), cudaMemcpyDeviceToHost, st));
        FWN_CUDA_CHECK(cudaStreamSynchronize(st));
        e.num_nodes = E;

        NvtxRange trace_refit("fwn build: FP64 refit, radii, records");
        StageRec* stage = dalloc<StageRec>(E, st);
        if (!(e.cfg.records & FWN_RECORDS_MOMENTS)) track(stage);
        else e.stage = stage;
        // the refit reads the records in 16 B pairs: the pool's allocations are 256 B aligned,
        // and a build that got less stops here rather than launch misaligned vector loads
        if (reinterpret_cast<uintptr_t>(stage) % alignof(StageRec) != 0)
            throw Error(FWN_INTERNAL, "staging records are not 32 B aligned");
        FWN_CUDA_CHECK(cudaMemsetAsync(visit, 0, (size_t)nint * sizeof(int), st));
        FWN_CUDA_CHECK(cudaMemsetAsync(leaf_count, 0, sizeof(int), st));
        if (NL > 0) {
            int* hist = (int*)track(dalloc<int>(kLeafSizes, st));
            int* leaf_sorted = (int*)track(dalloc<int>(NL, st));
            FWN_CUDA_CHECK(cudaMemsetAsync(hist, 0, kLeafSizes * sizeof(int), st));
            k_leaf_hist<<<grid_for(NL, 256), 256, 0, st>>>(NL, leaf_list, first, last, hist);
            k_leaf_offsets<<<1, 32, 0, st>>>(hist);
            k_leaf_sort<<<grid_for(NL, 256), 256, 0, st>>>(NL, leaf_list, first, last, hist,
                                                          leaf_sorted);
            leaf_list = leaf_sorted;
        }
        if (NL > 0)
            k_refit<<<grid_for(NL, 128), 128, 0, st>>>(NL, leaf_list, keys, first, last, pos,
                                                       tri_of_slot, d_V, d_F, voff, stage);
        if (NL > 0 && n > 1) {
            // internal nodes level by level, one thread per node of a dense list (an atomic
            // ascent would leave most lanes of its warps idle on GB300's narrow FP64 pipe): the
            // split tree deepest first by node depth, the LBVH lowest first by node height
            // (k_heights); the lists come from one counting sort by that key
            const int count = split ? num_nodes : nint;
            int* key = depth_of;
            if (!split) {
                key = (int*)track(dalloc<int>(nint, st));
                FWN_CUDA_CHECK(cudaMemsetAsync(key, 0, (size_t)nint * sizeof(int), st));
                k_heights<<<grid_for(NL, 128), 128, 0, st>>>(NL, leaf_list, keys, parent, first,
                                                             last, visit, key, status);
            }
            int* hist = (int*)track(dalloc<int>(kMaxHeight, st));
            int* order = (int*)track(dalloc<int>(count, st));
            FWN_CUDA_CHECK(cudaMemsetAsync(hist, 0, kMaxHeight * sizeof(int), st));
            k_height_hist<<<grid_for(count, 1024), 1024, 0, st>>>(count, keys, first, last, flags, key,
                                                                hist, status);
            std::vector<int> h_hist(kMaxHeight);
            FWN_CUDA_CHECK(cudaMemcpyAsync(h_hist.data(), hist, kMaxHeight * sizeof(int),
                                           cudaMemcpyDeviceToHost, st));
            k_height_offsets<<<1, 32, 0, st>>>(hist);
            k_height_sort<<<grid_for(count, 1024), 1024, 0, st>>>(count, keys, first, last, flags, key,
                                                                hist, order);
            FWN_CUDA_CHECK(cudaStreamSynchronize(st));
            std::vector<int> off(kMaxHeight + 1, 0);
            for (int h = 0; h < kMaxHeight; ++h) off[h + 1] = off[h] + h_hist[h];
            for (int t = 0; t < kMaxHeight; ++t) {
                const int h = split ? kMaxHeight - 1 - t : t;
                if (h_hist[h] > 0)
                    k_refit_level<<<grid_for(h_hist[h], 128), 128, 0, st>>>(
                        h_hist[h], order + off[h], left, right, pos, stage, status);
            }
        }
        FWN_CUDA_CHECK(cudaGetLastError());
        FWN_CUDA_CHECK(cudaMalloc(&e.tris, (size_t)n * sizeof(TriF32)));
        FWN_CUDA_CHECK(cudaMalloc(&e.sorted_tri, (size_t)n * sizeof(int)));
        k_tri_records<<<grid_for(n, 256), 256, 0, st>>>(n, tri_of_slot, keys, d_V, d_F, voff,
                                                        e.tris, e.sorted_tri);
        // exact radii of the internal nodes from the triangle records: one warp per node of at
        // most kRadiusChunk triangles, chunks of the larger nodes' slot runs (the scan's last
        // entry is the chunk total)
        int* rchunk = (int*)track(dalloc<int>(num_nodes + 1, st));
        unsigned long long* r2bits = (unsigned long long*)track(dalloc<unsigned long long>(E, st));
        FWN_CUDA_CHECK(cudaMemsetAsync(r2bits, 0, (size_t)E * sizeof(unsigned long long), st));
        k_radius_chunks<<<grid_for(num_nodes + 1, 256), 256, 0, st>>>(num_nodes, keys, first, last,
                                                                      flags, rchunk);
        exclusive_scan_i32(rchunk, num_nodes + 1, scan_tmp, st);
        if (n > 1) {
            int dev = 0, sms = 0;
            FWN_CUDA_CHECK(cudaGetDevice(&dev));
            FWN_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            int* rlist = (int*)track(dalloc<int>(num_nodes + 1, st));  // [count | list]
            FWN_CUDA_CHECK(cudaMemsetAsync(rlist, 0, sizeof(int), st));
            k_radius_list<<<grid_for(num_nodes, 256), 256, 0, st>>>(num_nodes, keys, first, last,
                                                                    flags, rlist + 1, rlist);
            k_node_radius_small<<<sms * 8, 32 * kRadiusWarps, 0, st>>>(rlist + 1, rlist, first,
                                                                       last, pos, stage, e.tris,
                                                                       r2bits);
            k_node_radius<<<sms * 4, 256, 0, st>>>(num_nodes, rchunk, first, last, pos, stage,
                                                   e.tris, r2bits);
        }
        FWN_CUDA_CHECK(cudaGetLastError());
        if (e.cfg.records & FWN_RECORDS_F32) FWN_CUDA_CHECK(cudaMalloc(&e.nodes32, E * sizeof(NodeF32)));
        if (e.cfg.records & FWN_RECORDS_F64) FWN_CUDA_CHECK(cudaMalloc(&e.nodes64, E * sizeof(NodeF64)));
        int* node_of_pos = (int*)track(dalloc<int>(E, st));
        k_node_of_pos<<<grid_for(num_nodes, 256), 256, 0, st>>>(num_nodes, flags, pos, node_of_pos);
        k_convert<<<grid_for(E, 128), 128, 0, st>>>(E, node_of_pos, keys, first, last, flags, skip,
                                                    stage, r2bits, e.nodes32, e.nodes64,
                                                    leaf_count);
        FWN_CUDA_CHECK(cudaGetLastError());
        if (e.cfg.tuning == 7 && e.nodes32 && E > 0) {  // the structure-of-arrays layout variant
            FWN_CUDA_CHECK(cudaMalloc(&e.soa, (size_t)E * sizeof(NodeF32)));
            k_aos_to_soa<<<grid_for(E, 256), 256, 0, st>>>(E, e.nodes32, e.soa);
            FWN_CUDA_CHECK(cudaGetLastError());
        }
        int lc = 0;
        FWN_CUDA_CHECK(cudaMemcpyAsync(&lc, leaf_count, sizeof(int), cudaMemcpyDeviceToHost, st));
        FWN_CUDA_CHECK(cudaMemcpyAsync(&st_h, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        FWN_CUDA_CHECK(cudaStreamSynchronize(st));
        e.num_leaves = lc;
        if (st_h & ST_REFIT_ORPHAN) throw Error(FWN_INTERNAL, "refit found an inconsistent tree");
        if (st_h & ST_BUILD_BOUND) throw Error(FWN_INTERNAL, "split build passed its node or depth bound");
    }
    FWN_CUDA_CHECK(cudaEventRecord(ev1, st));
    FWN_CUDA_CHECK(cudaMemcpyAsync(e.meshes_h, e.meshes, nmeshes * sizeof(MeshInfo),
                                   cudaMemcpyDeviceToHost, st));
    FWN_CUDA_CHECK(cudaStreamSynchronize(st));
    float ms = 0.f;
    FWN_CUDA_CHECK(cudaEventElapsedTime(&ms, ev0, ev1));
    e.build_ms = ms;
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    e.device_bytes = (int64_t)e.num_nodes * ((e.nodes32 ? sizeof(NodeF32) : 0) +
                                             (e.soa ? sizeof(NodeF32) : 0) +
                                             (e.nodes64 ? sizeof(NodeF64) : 0) +
                                             (e.stage ? sizeof(StageRec) : 0)) +
                     (int64_t)nf * (sizeof(TriF32) + sizeof(int)) + nmeshes * sizeof(MeshInfo);
}

}  // namespace fwn
