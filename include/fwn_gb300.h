/*
 * fwn_gb300.h — C ABI of the GB300 (sm_103a) fast-winding-number engine.
 *
 * This is the drop-in boundary for the `lagrange::winding::FastWindingNumber` path of
 * adobe/lagrange. Every entry point is plain C: POD arguments, raw pointers and sizes, a status
 * code instead of exceptions, no CUDA or torch types (streams are passed as `void*` holding a
 * `cudaStream_t`, 0 meaning the legacy default stream).
 *
 * Reference interfaces replaced (paths relative to the adobe/lagrange tree):
 *   - fwn_build          <- FastWindingNumber::FastWindingNumber(const SurfaceMesh<S,I>&)
 *                           modules/winding/src/FastWindingNumber.cpp:87-98, whose Impl::initialize
 *                           (:31-58) casts vertices to float and indices to int and calls
 *                           UT_SolidAngle<float,float>::init (:57).
 *   - fwn_query[_host]   <- FastWindingNumber::solid_angle / is_inside
 *                           modules/winding/src/FastWindingNumber.cpp:105-113 -> Impl::is_inside
 *                           (:60-67, `Omega / (4*pi) > 0.5f`) and Impl::solid_angle (:69-76), both
 *                           per point; here they are batched.
 *   - fwn_destroy        <- FastWindingNumber::~FastWindingNumber (:101, value_ptr<Impl> release).
 *   - fwn_forest_*       <- no single reference call: the reference builds one engine per mesh
 *                           and queries per point; the forest batches many meshes.
 *
 * Threading: a built handle is immutable. Concurrent fwn_query calls on one handle from several
 * host threads are safe (each call allocates its own stream-ordered scratch), matching the
 * reference's const query methods called from OpenVDB worker threads
 * (modules/volume/src/mesh_to_volume.cpp:175-183).
 *
 * Devices: an engine lives on the device that was current when it was built. Every query call
 * (fwn_query*, fwn_forest_query, fwn_query_grid, fwn_orientation_criterion) must be made with
 * that device current and returns FWN_INVALID_ARG otherwise; fwn_destroy may be called from any.
 */
#ifndef FWN_GB300_H
#define FWN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define FWN_API __declspec(dllexport)
#else
#define FWN_API __attribute__((visibility("default")))
#endif

/* Status codes. Every entry point returns one; fwn_last_error() gives the message. */
typedef enum fwn_status {
    FWN_OK = 0,
    FWN_INVALID_ARG = 1,   /* bad sizes, null pointers, out-of-range indices, non-finite vertices */
    FWN_OOM = 2,           /* device allocation failed */
    FWN_CUDA_ERROR = 3,    /* a CUDA runtime call or kernel failed */
    FWN_TIMEOUT = 4,       /* reserved: no kernel of this library waits on a flag or a peer */
    FWN_INTERNAL = 5,      /* a device-side consistency check failed (corrupt tree links) */
    FWN_NOT_BUILT = 6      /* handle is null / default-constructed */
} fwn_status;

/* Precision forms of the query. */
enum {
    FWN_PRECISION_MIXED = 0, /* FP32 traversal + far field, Kahan sum, FP64 for close triangles */
    FWN_PRECISION_FP64 = 1   /* plain form: FP64 everywhere */
};

/* Traversal schedules. AUTO is the warp schedule for the mixed form and the thread schedule
 * (the plain form) for the FP64 form; the FP64 form runs on the warp schedule when WARP is asked
 * for explicitly (same cursor and leaf pairs, FP64 arithmetic, same sums as the thread form). */
enum {
    FWN_TRAVERSAL_AUTO = 0,   /* mixed: autotuned warp schedule; FP64: thread schedule */
    FWN_TRAVERSAL_THREAD = 1, /* one thread per query, stackless skip-link walk */
    FWN_TRAVERSAL_WARP = 2    /* warp-shared cursor over 32 queries, leaf triangles in smem */
};

/* Tree builders. All give a binary tree in DFS order with leaves of <= leaf_size triangles and
 * the same refit; they differ in how the triangles are grouped. */
enum {
    FWN_BUILDER_LBVH = 0,   /* 30-bit Morton codes, device radix sort, Karras 2012 hierarchy */
    FWN_BUILDER_SPLIT = 1,  /* top-down: split each node's centroid box at the midpoint of its
                               longest axis (level by level on the device); fewer, more compact
                               nodes: ~15% fewer far tests per query, a slower build */
    FWN_BUILDER_BINNED = 2  /* as FWN_BUILDER_SPLIT, but nodes of more than 1024 triangles split
                               at the binned plane (16 bins per axis of the centroid box) with the
                               least n_L d_L + n_R d_R, d the squared diagonal of a side's centroid
                               bounds: ~2% faster queries, a slower build (a binning pass per level);
                               for one mesh queried many times */
};

/* Which node-record sets a build keeps (bit mask). */
enum {
    FWN_RECORDS_F32 = 1, /* 128 B FP32 records for the mixed form */
    FWN_RECORDS_F64 = 2, /* 256 B FP64 records for the plain FP64 form */
    FWN_RECORDS_MOMENTS = 4 /* keep the FP64 refit moments (fwn_export_moments, tests) */
};

typedef struct fwn_config {
    float beta;            /* far-field accuracy scale: node is far if |q-P| > beta*r. Default 2 */
    int32_t leaf_size;     /* max triangles per tree leaf, 1..16. Default 8 */
    int32_t records;       /* FWN_RECORDS_* mask. Default FWN_RECORDS_F32 */
    int32_t precision;     /* default query form, FWN_PRECISION_*. Default MIXED */
    int32_t traversal;     /* default schedule, FWN_TRAVERSAL_*. Default AUTO */
    int32_t block_size;    /* query kernel block size (multiple of 32, <= 1024); 0 = tuned */
    int32_t sort_queries;  /* 1: sort queries along a Hilbert curve first (default), 0: input order */
    float fp64_near_scale; /* FP64 near field if triangle is within scale*bbox_diagonal. 1e-3 */
    float fp64_cond;       /* ... and its FP32 evaluation is ill-conditioned: |a||b||c| >
                              fp64_cond * |(det, D)|, or det is within rounding of 0 with D <= 0.
                              0 = every triangle within the distance. Default 4 */
    int32_t tuning;        /* warp-schedule variant (set by fwn_autotune): queries per lane and
                              register cap. 1: 1 query per lane, 72 registers; 2: 1, no cap;
                              3: 1, 64 registers; 4: 2 queries per lane, 64 registers; 5: 2, 80;
                              6: as 4 with both query slots' Taylor terms in paired f32x2
                              arithmetic (same results bit for bit); 7: as 6 reading the node
                              records from a structure-of-arrays copy (eight float4 arrays,
                              128 B more per node) that a build with tuning 7 keeps: the layout
                              comparison, one mesh's point queries only (grids and forests run 6).
                              0 (default): 4 for batches that fill the GPU, else 3 */
    int32_t builder;       /* FWN_BUILDER_*. Default FWN_BUILDER_LBVH */
    int32_t reserved[5];
} fwn_config;

/* Per-query options (override the handle's defaults; pass NULL for defaults). */
typedef struct fwn_query_opts {
    int32_t precision;     /* FWN_PRECISION_* or -1 for the handle default */
    int32_t traversal;     /* FWN_TRAVERSAL_* or -1 */
    int32_t block_size;    /* 0 = handle default */
    int32_t sort_queries;  /* -1 = handle default */
    float beta;            /* <= 0: handle default */
    int32_t tuning;        /* schedule-specific variant for the autotuner (0 = default) */
    int32_t reserved[6];
} fwn_query_opts;

/* Work counters of one query call (filled when a non-NULL pointer is passed to fwn_query_ex). */
typedef struct fwn_query_stats {
    uint64_t nodes_tested;     /* node visits (far test evaluated) */
    uint64_t far_evals;        /* order-2 Taylor evaluations */
    uint64_t tri_evals;        /* exact triangle solid angles (all precisions) */
    uint64_t tri_evals_fp64;   /* of which evaluated in FP64 (mixed form only) */
    uint64_t warp_steps;       /* node steps summed over warps (max over the warp's lanes);
                                  the warp schedule counts with the variant's queries per lane
                                  (qpl = 2 for tunings >= 4): nodes_tested / (32 * qpl *
                                  warp_steps) = slot utilisation */
} fwn_query_stats;

/* Result of fwn_autotune: the fastest (builder, leaf_size, traversal, block_size, tuning) on the
 * sample. */
typedef struct fwn_tune_result {
    int32_t leaf_size;
    int32_t traversal;
    int32_t block_size;
    int32_t tuning;
    double ms;                 /* median device time of the winning configuration on the sample */
    int32_t candidates;        /* configurations timed (0 when the result came from the cache) */
    int32_t from_cache;
    int32_t builder;           /* FWN_BUILDER_* of the winning configuration */
    int32_t reserved[3];
} fwn_tune_result;

typedef struct fwn_info {
    int64_t num_vertices;
    int64_t num_triangles;
    int64_t num_nodes;         /* nodes in traversal order (all meshes) */
    int64_t num_leaves;
    int64_t num_meshes;
    int64_t device_bytes;      /* resident bytes of the built structure */
    double build_ms;           /* device time of the last build (CUDA events) */
    float bbox_min[3];         /* bbox of mesh 0 */
    float bbox_max[3];
    int32_t leaf_size;
    int32_t records;
} fwn_info;

typedef struct fwn_engine* fwn_handle;

FWN_API void fwn_config_default(fwn_config* cfg);

/* Copies the last error message of the calling thread into buf (always NUL-terminated) and
 * returns the full message length. */
FWN_API size_t fwn_last_error(char* buf, size_t buflen);

/* Library version string, e.g. "0.1.0 sm_103a". */
FWN_API const char* fwn_version(void);

/* Build from HOST arrays: vertices [nv x 3] float row-major, triangles [nf x 3] int32.
 * Mirrors FastWindingNumber.cpp:40-57 (float vertices, int indices). nf == 0 gives an engine
 * whose solid angle is 0 everywhere. Out-of-range indices or non-finite referenced vertex
 * coordinates return FWN_INVALID_ARG. Synchronous. */
FWN_API fwn_status fwn_build(const float* vertices, int64_t num_vertices,
                             const int32_t* triangles, int64_t num_triangles,
                             const fwn_config* cfg, fwn_handle* out);

/* Same, from DEVICE arrays (already resident in HBM). Synchronous on `stream`. */
FWN_API fwn_status fwn_build_device(const float* d_vertices, int64_t num_vertices,
                                    const int32_t* d_triangles, int64_t num_triangles,
                                    const fwn_config* cfg, void* stream, fwn_handle* out);

FWN_API fwn_status fwn_destroy(fwn_handle h);

FWN_API fwn_status fwn_get_info(fwn_handle h, fwn_info* info);

/* Queries on DEVICE buffers: points [n x 3] float; omega [n] float (solid angle, steradians) and
 * inside [n] uint8 (Omega/(4*pi) > 0.5, FastWindingNumber.cpp:66), either output may be NULL.
 * Asynchronous on `stream`; scratch is stream-ordered. The device-side consistency check of the
 * walk (a skip link that does not advance, i.e. a corrupt tree) is read back only by the
 * synchronous calls (fwn_query_host, and fwn_query_ex with work counters). */
FWN_API fwn_status fwn_query(fwn_handle h, const float* d_points, int64_t n,
                             float* d_omega, uint8_t* d_inside, void* stream);

/* Extended query: per-call options, optional FP64 solid-angle output (plain FP64 form only,
 * may be NULL), optional work counters (synchronises the stream when non-NULL). */
FWN_API fwn_status fwn_query_ex(fwn_handle h, const fwn_query_opts* opts,
                                const float* d_points, int64_t n, float* d_omega,
                                uint8_t* d_inside, double* d_omega_f64,
                                fwn_query_stats* stats, void* stream);

/* No counterpart in the reference (it answers one point per call). Writes the permutation the
 * query applies to group nearby points into warps: d_order[k] (uint32, device) is the index of
 * the k-th point in Hilbert-curve order of the mesh's frame. A caller that queries the same points
 * repeatedly can gather them once in this order and pass sort_queries = 0 in fwn_query_opts;
 * the results are the same. Asynchronous on `stream`. */
FWN_API fwn_status fwn_query_order(fwn_handle h, const float* d_points, int64_t n,
                                   uint32_t* d_order, void* stream);

/* Queries on HOST buffers (pinned or pageable): copies in, runs, copies out. Synchronous. */
FWN_API fwn_status fwn_query_host(fwn_handle h, const float* points, int64_t n,
                                  float* omega, uint8_t* inside);

/* No counterpart in the reference (a serving loop over many point sets). Queries num_batches
 * HOST batches: batch b is points[b] ([counts[b] x 3] float), its results go to omega[b] and
 * inside[b] (either array, or any entry of one, may be NULL). Each batch's results equal
 * fwn_query_host on it. Batch b is copied in while batch b - 1 is queried and batch b - 1's
 * results are copied out while batch b is queried (two device slots, the library's per-thread
 * copy streams), so that for batches of millions of points the host link hides behind the walk;
 * the copies overlap only from pinned host memory (pageable buffers are staged by the driver and
 * serialise). The walk's device-side consistency check is read back after the last batch.
 * Synchronous: returns when every batch's results are in host memory. */
FWN_API fwn_status fwn_query_host_batches(fwn_handle h, int64_t num_batches,
                                          const float* const* points, const int64_t* counts,
                                          float* const* omega, uint8_t* const* inside);

/* No counterpart in the reference. Same result as fwn_query with the handle's defaults, but it
 * allocates nothing: for callers that must not allocate device memory while they query (a
 * voxelizer or renderer working under a fixed per-frame device budget, or code where a
 * cudaMalloc/cudaFree could fail or would synchronize the device). Its sort buffers live in one
 * fixed region built into the library (about 17.3 MB per GPU that loads it, held until exit),
 * which limits a call to FWN_NOALLOC_MAX_POINTS points (larger n: FWN_INVALID_ARG; split the
 * batch). All calls share that region: calls whose GPU work overlaps (other streams or host
 * threads) race and must be serialized. The first call on each device looks up the region's
 * device address; make it before any stream capture. Asynchronous on `stream`; like fwn_query,
 * it does not read back the walk's device-side consistency check (that would need a
 * synchronisation): use fwn_query_host or fwn_query_ex with work counters for that check. */
#define FWN_NOALLOC_MAX_POINTS (1 << 20)
FWN_API fwn_status fwn_query_noalloc(fwn_handle h, const float* d_points, int64_t n,
                                     float* d_omega, uint8_t* d_inside, void* stream);

/* Exports the tree for inspection/tests into HOST arrays (any may be NULL):
 *   skip [num_nodes] int32, tri_begin [num_nodes] int32, tri_count [num_nodes] int32
 *   (0 for internal nodes), center_radius [num_nodes x 4] double (P.xyz, r) from the FP64
 *   refit, sorted_tri [num_triangles] int32 (original triangle id of each leaf slot),
 *   mesh_root [num_meshes x 2] int32 (first node, end node) */
FWN_API fwn_status fwn_export_tree(fwn_handle h, int32_t* skip, int32_t* tri_begin,
                                   int32_t* tri_count, double* center_radius,
                                   int32_t* sorted_tri, int32_t* mesh_root);

/* Exports the FP64 moments of every node [num_nodes x 33] double: P(3) N(3) M1(9, row i=normal
 * component, column j=offset component) M2(18, [i][xx,yy,zz,xy,xz,yz]). Needs FWN_RECORDS_F64 or
 * a build that kept the staging records (tests). */
FWN_API fwn_status fwn_export_moments(fwn_handle h, double* moments);

/* Copies the node records as they are on the device into HOST buffers (either may be NULL):
 * nodes32 [num_nodes x 128 B] (float4 P.xyz r; int32 skip, tri_begin, tri_count; float trM1;
 * float N.xyz, W.xyz, C[6], D[10], 2 zero floats), nodes64 [num_nodes x 256 B] (double P.xyz r;
 * int32 skip, tri_begin, tri_count, 0; double trM1, N.xyz, W.xyz, C[6], D[10], 3 zero doubles).
 * FWN_INVALID_ARG when a requested record set is not kept. Inspection and tests: every FP32
 * coefficient is the FP64 one rounded to nearest. */
FWN_API fwn_status fwn_export_nodes(fwn_handle h, void* nodes32, void* nodes64);

/* Autotuner (no reference counterpart: the reference has no tunable parameters). For one mesh
 * (DEVICE arrays) and a representative DEVICE sample of query points, builds the tree with both
 * builders for leaf sizes 4, 8, 12 and 16 and times every query schedule (the warp cursor's variants 1-6; thread per
 * query with blocks of 64/128/256) with CUDA events; returns the fastest. Apply it
 * with cfg.builder, cfg.leaf_size, cfg.traversal, cfg.block_size, cfg.tuning. `base` gives beta and the
 * precision knobs (NULL = defaults). cache_path (may be NULL) names a text file keyed by GPU name
 * and log2 of the triangle and query counts: a hit returns without timing, a miss appends.
 * Synchronous on `stream`. */
FWN_API fwn_status fwn_autotune(const float* d_vertices, int64_t num_vertices,
                                const int32_t* d_triangles, int64_t num_triangles,
                                const float* d_points, int64_t num_points, const fwn_config* base,
                                const char* cache_path, fwn_tune_result* out, void* stream);

/* Forest autotuner (no reference counterpart). The mixed forest query is one persistent kernel,
 * so its knobs are the builder, the leaf size and the register cap: builds the forest (DEVICE
 * vertex/triangle arrays, HOST offset arrays as in fwn_forest_build_device) with both builders
 * for leaf sizes 4, 8, 12 and 16 and
 * times the forest query with tuning 3, 1, 4, 5 and 6 on the DEVICE points with HOST query_offsets
 * [num_meshes + 1]. Returns the fastest (builder, leaf size, tuning; traversal WARP, block 128). Cache as
 * in fwn_autotune, keyed also by log2 of the mesh count. Synchronous on `stream`. */
FWN_API fwn_status fwn_forest_autotune(const float* d_vertices, const int64_t* vertex_offsets,
                                       const int32_t* d_triangles,
                                       const int64_t* triangle_offsets, int64_t num_meshes,
                                       const float* d_points, const int64_t* query_offsets,
                                       const fwn_config* base, const char* cache_path,
                                       fwn_tune_result* out, void* stream);

/* Voxel-grid sign pass (batched form of the winding-number signing in volume::mesh_to_volume,
 * modules/volume/src/mesh_to_volume.cpp:156-183, which calls is_inside once per voxel). Classifies
 * the centres of an nx x ny x nz grid of mesh `mesh` (0 for a single-mesh handle): voxel
 * (i, j, k) has centre fmaf(i + 0.5, spacing[0], origin[0]) (and likewise for y, z); outputs are
 * DEVICE arrays indexed i + nx * (j + ny * k). The centres are generated on the device (no point
 * array, no sort). Either output may be NULL. Asynchronous on `stream`. */
FWN_API fwn_status fwn_query_grid(fwn_handle h, int64_t mesh, const float* origin,
                                  const float* spacing, const int64_t* dims, float* d_omega,
                                  uint8_t* d_inside, void* stream);

/* Orientation test of modules/winding/examples/fix_orientation.cpp:75-115 for every triangle f of
 * a second mesh (DEVICE arrays, local indices): with unit normal n_f (zero for a degenerate
 * triangle) and barycentre b_f, criterion_f = (Omega(b_f + eps n_f) - Omega(b_f - eps n_f)) /
 * (4 pi) against this handle's (reference) mesh, and flip_f = criterion_f > threshold. The
 * example's defaults are eps = 1e-2, threshold = 0.8. Either output may be NULL. Synchronous. */
FWN_API fwn_status fwn_orientation_criterion(fwn_handle h, const float* d_vertices,
                                             int64_t num_vertices, const int32_t* d_triangles,
                                             int64_t num_triangles, float eps, float threshold,
                                             float* d_criterion, uint8_t* d_flip, void* stream);

/* ---- Forest: many meshes built and queried together (one launch per stage over all meshes).
 * vertices/triangles are concatenated; triangle indices are LOCAL to their mesh.
 * vertex_offsets [num_meshes+1], triangle_offsets [num_meshes+1] (host int64 prefix offsets).
 * Host arrays; synchronous. */
FWN_API fwn_status fwn_forest_build(const float* vertices, const int64_t* vertex_offsets,
                                    const int32_t* triangles, const int64_t* triangle_offsets,
                                    int64_t num_meshes, const fwn_config* cfg, fwn_handle* out);

/* Forest build from DEVICE vertex/triangle arrays (offsets stay on the host). */
FWN_API fwn_status fwn_forest_build_device(const float* d_vertices,
                                           const int64_t* vertex_offsets,
                                           const int32_t* d_triangles,
                                           const int64_t* triangle_offsets, int64_t num_meshes,
                                           const fwn_config* cfg, void* stream,
                                           fwn_handle* out);

/* Forest query on DEVICE buffers: points of mesh m are d_points[query_offsets[m] ..
 * query_offsets[m+1]) (host int64 offsets, num_meshes+1 entries). One persistent launch over
 * a work queue of (mesh, chunk) items.
 * Graph capture: the call reads query_offsets on the host when it is made (to choose the sort-key
 * width and the persistent grid) and copies them to the device with an async copy. A captured
 * call therefore replays with the offsets' values at capture time baked into those choices:
 * keep the offsets unchanged between replays (the copy re-reads the pinned array, but the key
 * width and grid would not follow a change), or capture again. */
FWN_API fwn_status fwn_forest_query(fwn_handle h, const float* d_points,
                                    const int64_t* query_offsets, float* d_omega,
                                    uint8_t* d_inside, const fwn_query_opts* opts,
                                    void* stream);

/* No counterpart in the reference (lagrange serializes meshes, not the winding engine). Writes a
 * built engine, single mesh or forest, to a file: a header with its sizes and configuration, its
 * per-mesh data, node records (FP32 and/or FP64, as built) and triangle records, and a checksum.
 * Reading it back with fwn_load skips the build. Synchronous. */
FWN_API fwn_status fwn_save(fwn_handle h, const char* path);

/* Reads an engine written by fwn_save onto the current device (the FP64 staging moments kept for
 * fwn_export_moments, and the structure-of-arrays copy of tuning 7, are not saved). The header,
 * the sizes, the configuration (the checks of a build), the checksum and every node's skip link
 * and triangle range are checked before any device work: a foreign, truncated or corrupt file
 * returns FWN_INVALID_ARG. Queries on the loaded engine equal those on the saved one.
 * Synchronous. */
FWN_API fwn_status fwn_load(const char* path, fwn_handle* out);

/* No counterpart in the reference (a diagnostic). Usage of the library's per-device pool of
 * stream-ordered query scratch, which keeps up to 8 GB of freed memory mapped (build temporaries
 * use a second pool, not reported here; zeros if no call has used the pool on `device` yet):
 * bytes the
 * pool holds from the driver, bytes handed out, and the high-water mark of handed-out bytes since
 * the last reset (reset_high != 0 restarts it from the current value before reading). Any output
 * may be NULL. Host-side; no device work. */
FWN_API fwn_status fwn_scratch_pool_stats(int32_t device, int32_t reset_high,
                                          uint64_t* reserved_bytes, uint64_t* used_bytes,
                                          uint64_t* used_high_bytes);

/* No counterpart in the reference (its per-point queries sort nothing). The key width, in bits,
 * of the radix sort that fwn_forest_query runs for these HOST query offsets [num_meshes + 1]: the
 * mesh id above the top bits of the 30-bit Hilbert index, 32-bit keys while every mesh keeps at
 * least 8 curve cells per query at that level, else 64-bit keys with all 30 bits. The sort makes
 * ceil(bits / 8) passes. Host-only (no device work). */
FWN_API fwn_status fwn_forest_sort_key_bits(int64_t num_meshes, const int64_t* query_offsets,
                                            int32_t* key_bits);

/* No counterpart in the reference (a measurement aid). The device's FP32 fused-multiply-add
 * throughput, which bounds the traversal kernels: a full-occupancy grid of independent FMA chains
 * on the current device, timed with CUDA events (median of 5 launches after 2 warm-ups).
 * form 0: scalar fma.rn.f32; form 1: paired fma.rn.f32x2. Writes the flops of one launch
 * (FMA = 2) and its device milliseconds. Allocates 4 bytes. Synchronous on `stream`. */
FWN_API fwn_status fwn_probe_fp32_peak(int32_t form, double* flops, double* ms, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FWN_GB300_H */
