// Device LSD radix sort of (key, value) pairs and an int32 exclusive scan.
//
// Sort: 8-bit digits, three launches per pass (reduce-then-scan):
//   upsweep   : per-tile digit histogram (per-warp shared counters), digit-major output
//   scan      : one block per digit scans that digit's per-tile counts, writes digit totals
//   downsweep : tile keys ranked stably within each warp (lanes holding the same digit found
//               with one ballot per digit bit), scattered into shared memory in digit order,
//               then written out with runs of consecutive addresses
// Stability comes from the warp-striped load order (warp, round, lane) = input order.
// Used for the triangle Morton keys (u64: mesh id above 30 Morton bits) and the query keys.
#include "fwn_internal.cuh"

namespace fwn {
namespace {

constexpr int RADIX_BITS = 8;
constexpr int RADIX = 1 << RADIX_BITS;
constexpr int SORT_THREADS = 256;  // == RADIX: one thread per digit in the digit loops
constexpr int SORT_WARPS = SORT_THREADS / 32;
static_assert(SORT_THREADS == RADIX, "digit loops assume one thread per digit");

// 8 keys per thread for both key widths: the downsweep's per-thread key, value, rank and digit
// arrays then fit in under 64 registers (4 blocks of 256 threads per SM). At 16 keys per thread
// the 32-bit sort needed 114 registers, ran at 2 blocks per SM and was latency-bound.
template <class K> struct TileCfg {
    static constexpr int KPT = 8;
    static constexpr int TILE = SORT_THREADS * KPT;
    static_assert(TILE == kSortTileKeys, "tile size shared with the fixed no-alloc region");
};

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Exclusive scan of one int per thread over a block of SORT_THREADS threads.
__device__ __forceinline__ int block_exclusive_scan_256(int v, int* warp_tot) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < SORT_WARPS ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < SORT_WARPS) warp_tot[lane] = t;  // inclusive warp totals
    }
    __syncthreads();
    int off = w > 0 ? warp_tot[w - 1] : 0;
    int res = off + x - v;
    __syncthreads();
    return res;
}

template <class K>
__global__ void __launch_bounds__(SORT_THREADS)
k_upsweep(const K* __restrict__ keys, int64_t n, int shift, int* __restrict__ hist, int nblocks) {
    constexpr int KPT = TileCfg<K>::KPT, TILE = TileCfg<K>::TILE;
    __shared__ int wh[SORT_WARPS][RADIX];
    const int tid = threadIdx.x, w = tid >> 5;
    for (int i = tid; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&wh[0][0])[i] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * TILE;
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        int64_t idx = base + (int64_t)j * SORT_THREADS + tid;
        if (idx < n) {
            unsigned d = (unsigned)(keys[idx] >> shift) & (RADIX - 1);
            atomicAdd(&wh[w][d], 1);
        }
    }
    __syncthreads();
    int s = 0;
#pragma unroll
    for (int ww = 0; ww < SORT_WARPS; ++ww) s += wh[ww][tid];
    hist[(int64_t)tid * nblocks + blockIdx.x] = s;
}

// One block per digit: exclusive scan of that digit's per-tile counts (in place).
__global__ void __launch_bounds__(1024)
k_scan_digits(int* __restrict__ hist, int nblocks, int* __restrict__ digit_totals) {
    __shared__ int wt[32];
    __shared__ int carry_s;
    int* row = hist + (int64_t)blockIdx.x * nblocks;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid == 0) carry_s = 0;
    __syncthreads();
    for (int b = 0; b < nblocks; b += 1024) {
        int i = b + tid;
        int v = i < nblocks ? row[i] : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wt[w] = x;
        __syncthreads();
        if (w == 0) {
            int t = wt[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += y;
            }
            wt[lane] = t;
        }
        __syncthreads();
        int carry = carry_s;
        int ex = carry + (w > 0 ? wt[w - 1] : 0) + x - v;
        if (i < nblocks) row[i] = ex;
        __syncthreads();
        if (tid == 0) carry_s = carry + wt[31];
        __syncthreads();
    }
    if (tid == 0) digit_totals[blockIdx.x] = carry_s;
}

template <class K>
__global__ void __launch_bounds__(SORT_THREADS)
k_downsweep(const K* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
            K* __restrict__ keys_out, uint32_t* __restrict__ vals_out, int64_t n, int shift,
            const int* __restrict__ hist, const int* __restrict__ digit_totals, int nblocks) {
    constexpr int KPT = TileCfg<K>::KPT, TILE = TileCfg<K>::TILE;
    __shared__ K skeys[TILE];
    __shared__ uint32_t svals[TILE];
    __shared__ int wc[SORT_WARPS][RADIX];
    __shared__ int tile_start[RADIX];
    __shared__ int gbase[RADIX];
    __shared__ int warp_tot[SORT_WARPS];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int i = tid; i < SORT_WARPS * RADIX; i += SORT_THREADS) (&wc[0][0])[i] = 0;

    // The tile's keys and values are requested first, so that their loads are in flight while
    // the block computes the digits' global bases.
    const int64_t base = (int64_t)blockIdx.x * TILE;
    K k[KPT];
    uint32_t v[KPT];
    int r[KPT];
    unsigned dg[KPT];
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        int64_t idx = base + (int64_t)w * (KPT * 32) + j * 32 + lane;
        bool valid = idx < n;
        k[j] = valid ? keys_in[idx] : (K)0;
        v[j] = valid ? vals_in[idx] : 0u;
    }
    // Global base of each digit for this tile: exclusive scan of the digit totals plus this
    // tile's exclusive offset within the digit.
    {
        const int tile_off = hist[(int64_t)tid * nblocks + blockIdx.x];
        int dt = digit_totals[tid];
        int ex = block_exclusive_scan_256(dt, warp_tot);
        gbase[tid] = ex + tile_off;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        int64_t idx = base + (int64_t)w * (KPT * 32) + j * 32 + lane;
        dg[j] = idx < n ? ((unsigned)(k[j] >> shift) & (RADIX - 1)) : (unsigned)RADIX;
    }
    const unsigned lt = lanemask_lt();
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        unsigned d = dg[j];
        // lanes holding the same digit: one ballot per bit of d (8 digit bits and the invalid
        // flag d == RADIX), which is cheaper here than __match_any_sync
        unsigned peers = 0xffffffffu;
#pragma unroll
        for (int bt = 0; bt <= RADIX_BITS; ++bt) {
            const bool bit = (d >> bt) & 1u;
            const unsigned m = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? m : ~m;
        }
        int leader = __ffs(peers) - 1;
        int before = __popc(peers & lt);
        int cnt = d < RADIX ? wc[w][d] : 0;
        __syncwarp();
        if (lane == leader && d < RADIX) wc[w][d] = cnt + __popc(peers);
        __syncwarp();
        r[j] = cnt + before;
    }
    __syncthreads();
    int tile_cnt = 0;
    {
        const int d = tid;
#pragma unroll
        for (int ww = 0; ww < SORT_WARPS; ++ww) {
            int t = wc[ww][d];
            wc[ww][d] = tile_cnt;
            tile_cnt += t;
        }
    }
    int ts = block_exclusive_scan_256(tile_cnt, warp_tot);
    tile_start[tid] = ts;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < KPT; ++j) {
        unsigned d = dg[j];
        if (d < RADIX) {
            int pos = tile_start[d] + wc[w][d] + r[j];
            skeys[pos] = k[j];
            svals[pos] = v[j];
        }
    }
    __syncthreads();
    const int tile_n = (int)min((int64_t)TILE, n - base);
    for (int i = tid; i < tile_n; i += SORT_THREADS) {
        K kk = skeys[i];
        unsigned d = (unsigned)(kk >> shift) & (RADIX - 1);
        int64_t out = (int64_t)gbase[d] + (i - tile_start[d]);
        keys_out[out] = kk;
        vals_out[out] = svals[i];
    }
}

template <class K>
bool radix_sort_impl(K* ka, uint32_t* va, K* kb, uint32_t* vb, int64_t n, int key_bits,
                     void* temp, cudaStream_t stream) {
    if (n <= 1 || key_bits <= 0) return false;
    constexpr int TILE = TileCfg<K>::TILE;
    const int nblocks = (int)((n + TILE - 1) / TILE);
    int* hist = static_cast<int*>(temp);
    int* totals = hist + (int64_t)RADIX * nblocks;
    K* ks = ka;
    K* kd = kb;
    uint32_t* vs = va;
    uint32_t* vd = vb;
    bool in_b = false;
    for (int shift = 0; shift < key_bits; shift += RADIX_BITS) {
        k_upsweep<K><<<nblocks, SORT_THREADS, 0, stream>>>(ks, n, shift, hist, nblocks);
        k_scan_digits<<<RADIX, 1024, 0, stream>>>(hist, nblocks, totals);
        k_downsweep<K><<<nblocks, SORT_THREADS, 0, stream>>>(ks, vs, kd, vd, n, shift, hist,
                                                              totals, nblocks);
        std::swap(ks, kd);
        std::swap(vs, vd);
        in_b = !in_b;
    }
    FWN_CUDA_CHECK(cudaGetLastError());
    return in_b;
}

// ---- exclusive scan of int32 (three phases: tile sums, scan of sums, tile scan) ----
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_IPT = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_IPT;

__device__ __forceinline__ int block_scan_1024(int v, int* wt, int* total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wt[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = wt[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        wt[lane] = t;
    }
    __syncthreads();
    int res = (w > 0 ? wt[w - 1] : 0) + x - v;
    *total = wt[31];
    __syncthreads();
    return res;
}

static_assert(SCAN_IPT == 4, "a thread's items are one int4");

// A thread's SCAN_IPT consecutive items: one 16 B load where the run is whole and aligned.
__device__ __forceinline__ void load_items(const int* __restrict__ data, int64_t i0, int64_t n,
                                           int (&v)[SCAN_IPT]) {
    if (i0 + SCAN_IPT <= n && (reinterpret_cast<uintptr_t>(data + i0) & 15) == 0) {
        const int4 x = *reinterpret_cast<const int4*>(data + i0);
        v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
    } else {
#pragma unroll
        for (int j = 0; j < SCAN_IPT; ++j) v[j] = i0 + j < n ? data[i0 + j] : 0;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_tile_sums(const int* __restrict__ data, int64_t n, int* __restrict__ sums) {
    __shared__ int wt[32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int v[SCAN_IPT];
    load_items(data, base + (int64_t)threadIdx.x * SCAN_IPT, n, v);
    int s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) s += v[j];
    int total;
    block_scan_1024(s, wt, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_sums(int* __restrict__ sums, int m) {
    __shared__ int wt[32];
    int carry = 0;
    for (int b = 0; b < m; b += SCAN_THREADS) {
        int i = b + threadIdx.x;
        int v = i < m ? sums[i] : 0;
        int total;
        int ex = block_scan_1024(v, wt, &total);
        if (i < m) sums[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(SCAN_THREADS)
k_scan_tiles(int* __restrict__ data, int64_t n, const int* __restrict__ sums) {
    __shared__ int wt[32];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    const int64_t i0 = base + (int64_t)threadIdx.x * SCAN_IPT;
    int v[SCAN_IPT];
    load_items(data, i0, n, v);
    int s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) s += v[j];
    int total;
    int ex = block_scan_1024(s, wt, &total) + sums[blockIdx.x];
    int o[SCAN_IPT];
#pragma unroll
    for (int j = 0; j < SCAN_IPT; ++j) {
        o[j] = ex;
        ex += v[j];
    }
    if (i0 + SCAN_IPT <= n && (reinterpret_cast<uintptr_t>(data + i0) & 15) == 0) {
        *reinterpret_cast<int4*>(data + i0) = make_int4(o[0], o[1], o[2], o[3]);
    } else {
#pragma unroll
        for (int j = 0; j < SCAN_IPT; ++j)
            if (i0 + j < n) data[i0 + j] = o[j];
    }
}

}  // namespace

size_t radix_sort_temp_bytes(int64_t n, int key_bytes) {
    const int tile = key_bytes == 8 ? TileCfg<uint64_t>::TILE : TileCfg<uint32_t>::TILE;
    const int64_t nblocks = (n + tile - 1) / tile;
    return (size_t)(RADIX * nblocks + RADIX) * sizeof(int) + 256;
}

bool radix_sort_u32(uint32_t* ka, uint32_t* va, uint32_t* kb, uint32_t* vb, int64_t n,
                    int key_bits, void* temp, cudaStream_t stream) {
    return radix_sort_impl<uint32_t>(ka, va, kb, vb, n, key_bits, temp, stream);
}

bool radix_sort_u64(uint64_t* ka, uint32_t* va, uint64_t* kb, uint32_t* vb, int64_t n,
                    int key_bits, void* temp, cudaStream_t stream) {
    return radix_sort_impl<uint64_t>(ka, va, kb, vb, n, key_bits, temp, stream);
}

size_t exclusive_scan_temp_bytes(int64_t n) {
    return (size_t)((n + SCAN_TILE - 1) / SCAN_TILE + 1) * sizeof(int) + 256;
}

void exclusive_scan_i32(int* data, int64_t n, void* temp, cudaStream_t stream) {
    if (n <= 0) return;
    const int m = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
    int* sums = static_cast<int*>(temp);
    k_scan_tile_sums<<<m, SCAN_THREADS, 0, stream>>>(data, n, sums);
    k_scan_sums<<<1, SCAN_THREADS, 0, stream>>>(sums, m);
    k_scan_tiles<<<m, SCAN_THREADS, 0, stream>>>(data, n, sums);
    FWN_CUDA_CHECK(cudaGetLastError());
}

}  // namespace fwn
