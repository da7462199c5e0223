/*
 * fwn_oracle.c — CPU oracle for the fast-winding-number path. TEST INFRASTRUCTURE ONLY: imported
 * by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker; never part
 * of the product path.
 *
 * Parity status: the reference arithmetic lives in the third-party library jdumas/WindingNumber
 * pinned at a48b8f555b490afe7aab9159c7daaf83fa2cdf8e (fetched by
 * cmake/recipes/external/winding_number.cmake:21-26), which is absent here, and the reference's
 * own tests pin no values (modules/winding/tests/test_fast_winding_number.cpp:80-83 is a no-op,
 * :85-125 an assertion-free benchmark). PARITY IS UNPINNED against the reference; the oracle is
 * pinned instead by analytic known answers (tests/test_oracle.py, tests/golden/).
 *
 * Three oracles:
 *   O1  oracle_brute_f64 : FP64 sum of exact triangle solid angles over ALL triangles (ground
 *                          truth, Van Oosterom & Strackee 1983).
 *   O2  oracle_ref_*     : restatement of the reference path: float vertices / int indices
 *                          (FastWindingNumber.cpp:40-52), a float BVH with order-2 dipole moments
 *                          (Barill et al. 2018, "Fast Winding Numbers for Soups and Clouds"),
 *                          far field when |q-P| > beta*r (beta = 2), exact near field, float
 *                          accumulation, is_inside = Omega/(4 pi) > 0.5 (FastWindingNumber.cpp:66).
 *                          Per-point queries threaded over host cores, as the OpenVDB caller does
 *                          (modules/volume/src/mesh_to_volume.cpp:175-183).
 *   O3  oracle_lbvh_*    : CPU restatement of the GPU build (30-bit Morton keys, stable sort,
 *                          Karras 2012 radix tree, leaf collapse, DFS layout, FP64 refit) and of
 *                          the plain FP64 traversal. Compiled with -ffp-contract=off so keys,
 *                          topology, centres and radii match the device build bit for bit.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#if FLT_EVAL_METHOD != 0
#error "float arithmetic must round to float (the shared far predicate)"
#endif

#define MORTON_BITS 30

/* ------------------------------------------------------------------------------------------- */
/* Exact triangle solid angle (Van Oosterom & Strackee 1983):                                   */
/*   tan(Omega/2) = a.(b x c) / (|a||b||c| + (a.b)|c| + (b.c)|a| + (c.a)|b|),  a,b,c = v - q.   */
/* A query on a vertex or in the triangle's plane contributes 0.                               */
/* ------------------------------------------------------------------------------------------- */
double oracle_tri_solid_angle_f64(const double* v0, const double* v1, const double* v2,
                                  const double* q) {
    const double ax = v0[0] - q[0], ay = v0[1] - q[1], az = v0[2] - q[2];
    const double bx = v1[0] - q[0], by = v1[1] - q[1], bz = v1[2] - q[2];
    const double cx = v2[0] - q[0], cy = v2[1] - q[1], cz = v2[2] - q[2];
    const double la = sqrt(ax * ax + ay * ay + az * az);
    const double lb = sqrt(bx * bx + by * by + bz * bz);
    const double lc = sqrt(cx * cx + cy * cy + cz * cz);
    if (la == 0.0 || lb == 0.0 || lc == 0.0) return 0.0;
    const double det = ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
    if (det == 0.0) return 0.0;
    const double D = la * lb * lc + (ax * bx + ay * by + az * bz) * lc +
                     (bx * cx + by * cy + bz * cz) * la + (cx * ax + cy * ay + cz * az) * lb;
    return 2.0 * atan2(det, D);
}

static float tri_solid_angle_f32(const float* v0, const float* v1, const float* v2, const float* q) {
    const float ax = v0[0] - q[0], ay = v0[1] - q[1], az = v0[2] - q[2];
    const float bx = v1[0] - q[0], by = v1[1] - q[1], bz = v1[2] - q[2];
    const float cx = v2[0] - q[0], cy = v2[1] - q[1], cz = v2[2] - q[2];
    const float la = sqrtf(ax * ax + ay * ay + az * az);
    const float lb = sqrtf(bx * bx + by * by + bz * bz);
    const float lc = sqrtf(cx * cx + cy * cy + cz * cz);
    if (la == 0.f || lb == 0.f || lc == 0.f) return 0.f;
    const float det = ax * (by * cz - bz * cy) + ay * (bz * cx - bx * cz) + az * (bx * cy - by * cx);
    if (det == 0.f) return 0.f;
    const float D = la * lb * lc + (ax * bx + ay * by + az * bz) * lc +
                    (bx * cx + by * cy + bz * cz) * la + (cx * ax + cy * ay + cz * az) * lb;
    return 2.0f * atan2f(det, D);
}

/* ---------------------------------- thread pool helper ------------------------------------ */
typedef void (*range_fn)(void* ctx, int64_t b, int64_t e);
typedef struct {
    range_fn fn;
    void* ctx;
    int64_t b, e;
} job_t;

static void* job_run(void* p) {
    job_t* j = (job_t*)p;
    j->fn(j->ctx, j->b, j->e);
    return NULL;
}

static void parallel_for(int64_t n, int nthreads, range_fn fn, void* ctx) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 512) nthreads = 512;
    if ((int64_t)nthreads > n) nthreads = (int)(n > 0 ? n : 1);
    if (nthreads == 1) {
        fn(ctx, 0, n);
        return;
    }
    pthread_t th[512];
    job_t jobs[512];
    /* interleaved small chunks would balance better; contiguous ranges keep per-thread locality
       (queries are typically spatially ordered). */
    for (int t = 0; t < nthreads; ++t) {
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].b = n * t / nthreads;
        jobs[t].e = n * (t + 1) / nthreads;
        pthread_create(&th[t], NULL, job_run, &jobs[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
}

/* ========================================================================================== */
/* O1: FP64 brute force                                                                        */
/* ========================================================================================== */
typedef struct {
    const float* V;
    const int32_t* F;
    int64_t nf;
    const float* Q;
    double* out;
} brute_ctx;

static void brute_range(void* p, int64_t b, int64_t e) {
    brute_ctx* c = (brute_ctx*)p;
    for (int64_t i = b; i < e; ++i) {
        const double q[3] = {c->Q[3 * i], c->Q[3 * i + 1], c->Q[3 * i + 2]};
        double s = 0.0;
        for (int64_t t = 0; t < c->nf; ++t) {
            double v[3][3];
            for (int j = 0; j < 3; ++j)
                for (int a = 0; a < 3; ++a) v[j][a] = c->V[3 * (int64_t)c->F[3 * t + j] + a];
            s += oracle_tri_solid_angle_f64(v[0], v[1], v[2], q);
        }
        c->out[i] = s;
    }
}

/* Omega(q) = sum over all triangles, FP64. Indices must be valid (checked by the caller). */
void oracle_brute_f64(const float* V, int64_t nv, const int32_t* F, int64_t nf, const float* Q,
                      int64_t nq, double* out, int nthreads) {
    (void)nv;
    brute_ctx c = {V, F, nf, Q, out};
    parallel_for(nq, nthreads, brute_range, &c);
}

/* ========================================================================================== */
/* O2: float Barill tree (restatement of the reference UT_SolidAngle<float,float> path)        */
/* ========================================================================================== */
typedef struct {
    float P[3], r;
    float N[3];
    float M1[9];  /* [i*3+j] */
    float M2[18]; /* [i*6+s], s: xx yy zz xy xz yz */
    int32_t left, right; /* children (-1 for leaves) */
    int32_t begin, count;
} ref_node;

typedef struct {
    int64_t nf;
    float* tv;        /* [nf][9] triangle vertices in tree order */
    ref_node* nodes;
    int64_t nnodes, cap;
    int leaf_size;
} ref_tree;

typedef struct {
    float* cen;      /* centroids [nf*3] */
    int32_t* perm;
    int axis;
} ref_sort_ctx;

static ref_sort_ctx* g_sort_ctx; /* qsort has no context argument: set before each call (single thread build) */

static int cmp_axis(const void* a, const void* b) {
    const int32_t ia = *(const int32_t*)a, ib = *(const int32_t*)b;
    const float ca = g_sort_ctx->cen[3 * ia + g_sort_ctx->axis];
    const float cb = g_sort_ctx->cen[3 * ib + g_sort_ctx->axis];
    if (ca < cb) return -1;
    if (ca > cb) return 1;
    return (ia > ib) - (ia < ib);
}

static int32_t ref_new_node(ref_tree* T) {
    if (T->nnodes == T->cap) {
        T->cap = T->cap ? 2 * T->cap : 1024;
        T->nodes = (ref_node*)realloc(T->nodes, T->cap * sizeof(ref_node));
    }
    memset(&T->nodes[T->nnodes], 0, sizeof(ref_node));
    return (int32_t)T->nnodes++;
}

/* float moments of triangles [b, e) of perm, about their area-weighted centroid */
static void ref_moments(const float* V, const int32_t* F, const int32_t* perm, int64_t b, int64_t e,
                        ref_node* nd) {
    float A = 0.f, S[3] = {0, 0, 0}, C[3] = {0, 0, 0};
    for (int64_t k = b; k < e; ++k) {
        const int32_t t = perm[k];
        const float* v0 = V + 3 * (int64_t)F[3 * t];
        const float* v1 = V + 3 * (int64_t)F[3 * t + 1];
        const float* v2 = V + 3 * (int64_t)F[3 * t + 2];
        float e1[3], e2[3], n[3];
        for (int a = 0; a < 3; ++a) {
            e1[a] = v1[a] - v0[a];
            e2[a] = v2[a] - v0[a];
        }
        n[0] = 0.5f * (e1[1] * e2[2] - e1[2] * e2[1]);
        n[1] = 0.5f * (e1[2] * e2[0] - e1[0] * e2[2]);
        n[2] = 0.5f * (e1[0] * e2[1] - e1[1] * e2[0]);
        const float at = sqrtf(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int a = 0; a < 3; ++a) {
            const float c = (v0[a] + v1[a] + v2[a]) / 3.f;
            S[a] += at * c;
            C[a] += c;
        }
        A += at;
    }
    for (int a = 0; a < 3; ++a) nd->P[a] = A > 0.f ? S[a] / A : C[a] / (float)(e - b);
    float r2 = 0.f;
    for (int64_t k = b; k < e; ++k) {
        const int32_t t = perm[k];
        const float* v[3] = {V + 3 * (int64_t)F[3 * t], V + 3 * (int64_t)F[3 * t + 1],
                             V + 3 * (int64_t)F[3 * t + 2]};
        float e1[3], e2[3], n[3], c[3], d[3];
        for (int a = 0; a < 3; ++a) {
            e1[a] = v[1][a] - v[0][a];
            e2[a] = v[2][a] - v[0][a];
        }
        n[0] = 0.5f * (e1[1] * e2[2] - e1[2] * e2[1]);
        n[1] = 0.5f * (e1[2] * e2[0] - e1[0] * e2[2]);
        n[2] = 0.5f * (e1[0] * e2[1] - e1[1] * e2[0]);
        for (int a = 0; a < 3; ++a) {
            c[a] = (v[0][a] + v[1][a] + v[2][a]) / 3.f;
            d[a] = c[a] - nd->P[a];
        }
        static const int SJ[6] = {0, 1, 2, 0, 0, 1}, SK[6] = {0, 1, 2, 1, 2, 2};
        float Qm[6];
        for (int s = 0; s < 6; ++s) {
            const int j = SJ[s], kk = SK[s];
            float cov = 0.f;
            for (int w = 0; w < 3; ++w) cov += (v[w][j] - c[j]) * (v[w][kk] - c[kk]);
            Qm[s] = d[j] * d[kk] + cov / 12.f;
        }
        for (int i = 0; i < 3; ++i) {
            nd->N[i] += n[i];
            for (int j = 0; j < 3; ++j) nd->M1[3 * i + j] += n[i] * d[j];
            for (int s = 0; s < 6; ++s) nd->M2[6 * i + s] += n[i] * Qm[s];
        }
        for (int w = 0; w < 3; ++w) {
            const float dx = v[w][0] - nd->P[0], dy = v[w][1] - nd->P[1], dz = v[w][2] - nd->P[2];
            const float q2 = dx * dx + dy * dy + dz * dz;
            if (q2 > r2) r2 = q2;
        }
    }
    nd->r = sqrtf(r2);
}

static int32_t ref_build_rec(ref_tree* T, const float* V, const int32_t* F, ref_sort_ctx* sc,
                             int64_t b, int64_t e) {
    const int32_t id = ref_new_node(T);
    ref_moments(V, F, sc->perm, b, e, &T->nodes[id]);
    T->nodes[id].begin = (int32_t)b;
    T->nodes[id].count = (int32_t)(e - b);
    T->nodes[id].left = T->nodes[id].right = -1;
    if (e - b <= T->leaf_size) return id;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t k = b; k < e; ++k)
        for (int a = 0; a < 3; ++a) {
            const float c = sc->cen[3 * sc->perm[k] + a];
            if (c < lo[a]) lo[a] = c;
            if (c > hi[a]) hi[a] = c;
        }
    int axis = 0;
    for (int a = 1; a < 3; ++a)
        if (hi[a] - lo[a] > hi[axis] - lo[axis]) axis = a;
    sc->axis = axis;
    g_sort_ctx = sc;
    qsort(sc->perm + b, (size_t)(e - b), sizeof(int32_t), cmp_axis);
    const int64_t mid = b + (e - b) / 2;
    const int32_t l = ref_build_rec(T, V, F, sc, b, mid);
    const int32_t r = ref_build_rec(T, V, F, sc, mid, e);
    T->nodes[id].left = l;
    T->nodes[id].right = r;
    T->nodes[id].count = 0;
    return id;
}

void* oracle_ref_build(const float* V, int64_t nv, const int32_t* F, int64_t nf, int leaf_size) {
    (void)nv;
    ref_tree* T = (ref_tree*)calloc(1, sizeof(ref_tree));
    T->nf = nf;
    T->leaf_size = leaf_size < 1 ? 1 : leaf_size;
    if (nf == 0) return T;
    ref_sort_ctx sc;
    sc.cen = (float*)malloc(nf * 3 * sizeof(float));
    sc.perm = (int32_t*)malloc(nf * sizeof(int32_t));
    for (int64_t t = 0; t < nf; ++t) {
        sc.perm[t] = (int32_t)t;
        for (int a = 0; a < 3; ++a)
            sc.cen[3 * t + a] = (V[3 * (int64_t)F[3 * t] + a] + V[3 * (int64_t)F[3 * t + 1] + a] +
                                 V[3 * (int64_t)F[3 * t + 2] + a]) / 3.f;
    }
    ref_build_rec(T, V, F, &sc, 0, nf);
    T->tv = (float*)malloc(nf * 9 * sizeof(float));
    for (int64_t k = 0; k < nf; ++k)
        for (int j = 0; j < 3; ++j)
            for (int a = 0; a < 3; ++a) T->tv[9 * k + 3 * j + a] = V[3 * (int64_t)F[3 * sc.perm[k] + j] + a];
    free(sc.cen);
    free(sc.perm);
    return T;
}

void oracle_ref_free(void* h) {
    ref_tree* T = (ref_tree*)h;
    if (!T) return;
    free(T->tv);
    free(T->nodes);
    free(T);
}

int64_t oracle_ref_num_nodes(void* h) { return ((ref_tree*)h)->nnodes; }

/* Order-2 dipole expansion of one node at d = P - q (float). See the derivation in the engine:
 * T = K(d).N + sum M1_ij dK_i/dd_j + 1/2 sum M2_ijk d2K_i/dd_j dd_k, K(r) = r/|r|^3. */
static float ref_taylor(const ref_node* nd, const float* d) {
    const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float rinv = 1.f / sqrtf(r2);
    const float r3 = rinv * rinv * rinv, r5 = r3 * rinv * rinv, r7 = r5 * rinv * rinv;
    float t0 = 0.f, tr = 0.f, q = 0.f;
    for (int i = 0; i < 3; ++i) {
        t0 += d[i] * nd->N[i];
        tr += nd->M1[3 * i + i];
        for (int j = 0; j < 3; ++j) q += nd->M1[3 * i + j] * d[i] * d[j];
    }
    static const int SJ[6] = {0, 1, 2, 0, 0, 1}, SK[6] = {0, 1, 2, 1, 2, 2};
    float u[3] = {0, 0, 0}, v[3] = {0, 0, 0}, S = 0.f;
    for (int i = 0; i < 3; ++i)
        for (int s = 0; s < 6; ++s) {
            const int j = SJ[s], k = SK[s];
            const float m = nd->M2[6 * i + s];
            const float mult = (j == k) ? 1.f : 2.f; /* symmetric pair counted twice */
            S += mult * m * d[i] * d[j] * d[k];
            if (j == k) v[i] += m;
            if (i == j) u[k] += m;
            if (i == k && j != k) u[j] += m;
        }
    const float wr = (2.f * u[0] + v[0]) * d[0] + (2.f * u[1] + v[1]) * d[1] + (2.f * u[2] + v[2]) * d[2];
    return t0 * r3 + tr * r3 - 3.f * q * r5 - 1.5f * wr * r5 + 7.5f * S * r7;
}

static float ref_query_one(const ref_tree* T, const float* q, float beta) {
    if (T->nnodes == 0) return 0.f;
    int32_t stack[256];
    int sp = 0;
    stack[sp++] = 0;
    float sum = 0.f;
    const float b2 = beta * beta;
    while (sp) {
        const ref_node* nd = &T->nodes[stack[--sp]];
        const float d[3] = {nd->P[0] - q[0], nd->P[1] - q[1], nd->P[2] - q[2]};
        const float dd = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (dd > b2 * nd->r * nd->r) {
            sum += ref_taylor(nd, d);
        } else if (nd->left < 0) {
            for (int32_t k = nd->begin; k < nd->begin + nd->count; ++k) {
                const float* tv = T->tv + 9 * (int64_t)k;
                sum += tri_solid_angle_f32(tv, tv + 3, tv + 6, q);
            }
        } else {
            if (sp + 2 > 256) return NAN; /* depth bound exceeded: cannot happen for median splits */
            stack[sp++] = nd->right;
            stack[sp++] = nd->left;
        }
    }
    return sum;
}

typedef struct {
    const ref_tree* T;
    const float* Q;
    float beta;
    float* omega;
    uint8_t* inside;
} ref_q_ctx;

static void ref_q_range(void* p, int64_t b, int64_t e) {
    ref_q_ctx* c = (ref_q_ctx*)p;
    const double four_pi = 4.0 * 3.14159265358979323846264338327950288;
    for (int64_t i = b; i < e; ++i) {
        const float w = ref_query_one(c->T, c->Q + 3 * i, c->beta);
        if (c->omega) c->omega[i] = w;
        /* FastWindingNumber.cpp:66: float / (4.f * double pi) > 0.5f, evaluated in double */
        if (c->inside) c->inside[i] = ((double)w / four_pi > 0.5) ? 1 : 0;
    }
}

void oracle_ref_query(void* h, const float* Q, int64_t nq, float beta, float* omega,
                      uint8_t* inside, int nthreads) {
    ref_q_ctx c = {(const ref_tree*)h, Q, beta, omega, inside};
    parallel_for(nq, nthreads, ref_q_range, &c);
}

/* ========================================================================================== */
/* O3: restatement of the GPU LBVH build and the plain FP64 traversal                         */
/* ========================================================================================== */
typedef struct {
    double P[3], area, N[3], M1[9], M2[18], r;
} lb_stage;

typedef struct {
    int64_t nmeshes, nf, E;
    int32_t* root;     /* [nmeshes] DFS position of each mesh root (-1 empty) */
    int32_t* end;      /* [nmeshes] */
    float* tau;        /* [nmeshes] */
    float* mlo;        /* [nmeshes*3] */
    float* mhi;
    int32_t* skip;     /* [E] */
    int32_t* tbeg;     /* [E] */
    int32_t* tcnt;     /* [E] */
    lb_stage* st;      /* [E] */
    int32_t* sorted_tri; /* [nf] global triangle id per slot */
    float* tv;         /* [nf*9] vertices per slot */
    uint64_t* keys;    /* [nf] sorted keys */
} lb_tree;

static unsigned spread3(unsigned x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

static unsigned quantize10(float c, float lo, float inv) {
    const float u = (c - lo) * inv;
    const float s = u * 1024.0f;
    int q = (s >= 0.0f) ? (int)floorf(s) : 0;
    return (unsigned)(q < 1023 ? q : 1023);
}

typedef struct {
    uint64_t key;
    uint32_t idx;
} kv_t;

static int cmp_kv(const void* a, const void* b) {
    const kv_t* x = (const kv_t*)a;
    const kv_t* y = (const kv_t*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

static int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }
static int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }

static int kdelta(const uint64_t* keys, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    if (keys[i] == keys[j]) return 64 + clz32((uint32_t)(i ^ j));
    return clz64(keys[i] ^ keys[j]);
}

static double round_up_float(double x) {
    float f = (float)x;
    if ((double)f < x) f = nextafterf(f, INFINITY);
    return (double)f;
}

static void lb_tri_d(const lb_tree* T, int64_t s, double v[3][3]) {
    for (int j = 0; j < 3; ++j)
        for (int a = 0; a < 3; ++a) v[j][a] = (double)T->tv[9 * s + 3 * j + a];
}

/* Leaf moments (same steps as the device refit): one pass accumulates the area-weighted
 * centroid and the moments about the first triangle's centroid c0; the moments are then moved to
 * P = float(area-weighted centroid) with the parent recentring formulas (e = c0 - P); a second,
 * vertex-only pass gives r = max |v - P| (rounded up to a float, lb_node_r2). */
/* The refit's fused multiply-adds are written out (C fma(), correctly rounded) at the same places
 * as in the device refit, which is compiled without implicit contraction. */
/* Squared radius of the sphere about P through the farthest vertex of the triangles in sorted
 * slots [f, l]: max fma(dx, dx, fma(dy, dy, dz * dz)) with d = v - P in FP64. A maximum does not
 * depend on the order of its terms, so the device's chunked warp reduction gives the same value.
 * Every node's radius, leaf or internal, is this exact bound, rounded up to a float. */
static double lb_node_r2(const lb_tree* T, int64_t f, int64_t l, const double* P) {
    double r2 = 0.0;
    for (int64_t s = f; s <= l; ++s) {
        double v[3][3];
        lb_tri_d(T, s, v);
        for (int j = 0; j < 3; ++j) {
            const double dx = v[j][0] - P[0], dy = v[j][1] - P[1], dz = v[j][2] - P[2];
            r2 = fmax(r2, fma(dx, dx, fma(dy, dy, dz * dz)));
        }
    }
    return r2;
}

static void lb_leaf(const lb_tree* T, int64_t f, int64_t l, lb_stage* R) {
    static const double kThird = 1.0 / 3.0, kTwelfth = 1.0 / 12.0;
    static const int SJ[6] = {0, 1, 2, 0, 0, 1}, SK[6] = {0, 1, 2, 1, 2, 2};
    double A = 0.0, S[3] = {0, 0, 0}, Cs[3] = {0, 0, 0}, c0[3] = {0, 0, 0};
    double N[3] = {0, 0, 0}, M1[9] = {0}, M2[18] = {0};
    for (int64_t s = f; s <= l; ++s) {
        double v[3][3], e1[3], e2[3], nn[3], c[3], d[3], w[3][3], Q[6];
        lb_tri_d(T, s, v);
        for (int a = 0; a < 3; ++a) {
            e1[a] = v[1][a] - v[0][a];
            e2[a] = v[2][a] - v[0][a];
        }
        nn[0] = 0.5 * fma(e1[1], e2[2], -(e1[2] * e2[1]));
        nn[1] = 0.5 * fma(e1[2], e2[0], -(e1[0] * e2[2]));
        nn[2] = 0.5 * fma(e1[0], e2[1], -(e1[1] * e2[0]));
        const double at = sqrt(fma(nn[0], nn[0], fma(nn[1], nn[1], nn[2] * nn[2])));
        for (int a = 0; a < 3; ++a) c[a] = ((v[0][a] + v[1][a]) + v[2][a]) * kThird;
        if (s == f)
            for (int a = 0; a < 3; ++a) c0[a] = c[a];
        for (int a = 0; a < 3; ++a) {
            S[a] = fma(at, c[a], S[a]);
            Cs[a] = Cs[a] + c[a];
            d[a] = c[a] - c0[a];
        }
        A = A + at;
        for (int j = 0; j < 3; ++j)
            for (int a = 0; a < 3; ++a) w[j][a] = v[j][a] - c[a];
        for (int q = 0; q < 6; ++q) {
            const int j = SJ[q], k = SK[q];
            const double cov = fma(w[0][j], w[0][k], fma(w[1][j], w[1][k], w[2][j] * w[2][k])) * kTwelfth;
            Q[q] = fma(d[j], d[k], cov);
        }
        for (int i = 0; i < 3; ++i) {
            N[i] = N[i] + nn[i];
            for (int j = 0; j < 3; ++j) M1[3 * i + j] = fma(nn[i], d[j], M1[3 * i + j]);
            for (int q = 0; q < 6; ++q) M2[6 * i + q] = fma(nn[i], Q[q], M2[6 * i + q]);
        }
    }
    const double cnt = (double)(l - f + 1);
    double P[3], e[3];
    for (int a = 0; a < 3; ++a) {
        const double pe = A > 0.0 ? S[a] / A : Cs[a] / cnt;
        P[a] = (double)(float)pe;
        e[a] = c0[a] - P[a];
    }
    for (int i = 0; i < 3; ++i) {
        for (int q = 0; q < 6; ++q) {
            const int j = SJ[q], k = SK[q];
            R->M2[6 * i + q] =
                fma(N[i], e[j] * e[k], fma(M1[3 * i + k], e[j], fma(M1[3 * i + j], e[k], M2[6 * i + q])));
        }
        for (int j = 0; j < 3; ++j) R->M1[3 * i + j] = fma(N[i], e[j], M1[3 * i + j]);
    }
    for (int a = 0; a < 3; ++a) {
        R->P[a] = P[a];
        R->N[a] = N[a];
    }
    R->area = A;
    R->r = round_up_float(sqrt(lb_node_r2(T, f, l, P)));
}

static void lb_combine(const lb_stage* a, const lb_stage* b, lb_stage* R) {
    const double A = a->area + b->area;
    double P[3], ea[3], eb[3];
    for (int i = 0; i < 3; ++i) {
        const double pe = A > 0.0 ? fma(a->area, a->P[i], b->area * b->P[i]) / A : (a->P[i] + b->P[i]) * 0.5;
        P[i] = (double)(float)pe;
        ea[i] = a->P[i] - P[i];
        eb[i] = b->P[i] - P[i];
    }
    lb_stage o;
    for (int i = 0; i < 3; ++i) {
        o.P[i] = P[i];
        o.N[i] = a->N[i] + b->N[i];
        for (int j = 0; j < 3; ++j)
            o.M1[3 * i + j] = fma(a->N[i], ea[j], a->M1[3 * i + j]) + fma(b->N[i], eb[j], b->M1[3 * i + j]);
    }
    static const int SJ[6] = {0, 1, 2, 0, 0, 1}, SK[6] = {0, 1, 2, 1, 2, 2};
    for (int i = 0; i < 3; ++i)
        for (int q = 0; q < 6; ++q) {
            const int j = SJ[q], k = SK[q];
            const double ta = fma(a->N[i], ea[j] * ea[k],
                                  fma(a->M1[3 * i + k], ea[j], fma(a->M1[3 * i + j], ea[k], a->M2[6 * i + q])));
            const double tb = fma(b->N[i], eb[j] * eb[k],
                                  fma(b->M1[3 * i + k], eb[j], fma(b->M1[3 * i + j], eb[k], b->M2[6 * i + q])));
            o.M2[6 * i + q] = ta + tb;
        }
    o.area = A;
    o.r = 0.0; /* set from the node's vertices once P is known (lb_node_r2) */
    *R = o;
}

/* Builds the forest; voff/foff are [nmeshes+1] prefix offsets, triangle indices local per mesh.
 * Returns NULL on invalid input (bad index / non-finite referenced vertex). */
/* Top-down splitting builds (builders 1 and 2), restating the device's level-synchronous build: a node
 * of m > K triangles splits its centroids' bounding box at the midpoint of its longest axis
 * (ties: the lowest axis), split = (lo + hi) * 0.5f, left = centroids below the split, both sides
 * keeping their order (a stable partition); when every centroid coincides, or the midpoint rounds
 * down to lo, it splits by position instead (the first m / 2 left), as every node at depth
 * >= SP_SPATIAL_LEVELS does. Nodes are created here in DFS pre-order, which is the order the
 * device reaches with its position formula. */
#define SP_SPATIAL_LEVELS 96
/* Builder 2 (binned): nodes of more than SP_FINISH_SLOTS triangles (the device's level loop;
 * smaller ones are finished per block in shared memory) split at a binned plane instead: SP_BINS bins per axis over
 * the centroid box, bin(x) = min((int)((x - lo) / ext * 16), 15) in float, and the plane with the
 * least nL * dL + nR * dR, d = the squared diagonal of a side's centroid bounds (in double from
 * the float bounds); ties go to the lower axis, then the lower plane; left = bin <= plane. */
#define SP_FINISH_SLOTS 1024
#define SP_BINS 16

static int sp_bin(float x, float lo, float ext) {
    const int b = (int)((x - lo) / ext * (float)SP_BINS);
    return b < 0 ? 0 : (b > SP_BINS - 1 ? SP_BINS - 1 : b);
}

static double sp_diag2(const float* lo, const float* hi) {
    double t = 0.0;
    for (int a = 0; a < 3; ++a) {
        const double d = (double)hi[a] - (double)lo[a];
        t = t + d * d;
    }
    return t;
}

typedef struct {
    lb_tree* T;
    const float* cen;   /* [nf*3] centroids, input triangle order */
    int32_t* perm;      /* triangle ids, partitioned in place */
    int32_t* tmp;
    int K;
    int binned;         /* builder 2: binned planes above SP_FINISH_SLOTS triangles */
    int64_t E;          /* nodes created so far */
    int32_t* nfirst;    /* per node (DFS position): slot range and children */
    int32_t* nlast;
    int32_t* nleft;
    int32_t* nright;
} sp_ctx;

static int32_t sp_build_rec(sp_ctx* c, int64_t b, int64_t e, int depth) {
    const int32_t id = (int32_t)c->E++;
    c->nfirst[id] = (int32_t)b;
    c->nlast[id] = (int32_t)(e - 1);
    c->nleft[id] = c->nright[id] = -1;
    const int64_t m = e - b;
    if (m <= c->K) return id;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = b; i < e; ++i)
        for (int a = 0; a < 3; ++a) {
            const float x = c->cen[3 * (int64_t)c->perm[i] + a];
            lo[a] = fminf(lo[a], x);
            hi[a] = fmaxf(hi[a], x);
        }
    int axis = 0;
    float ext = hi[0] - lo[0];
    for (int a = 1; a < 3; ++a)
        if (hi[a] - lo[a] > ext) {
            ext = hi[a] - lo[a];
            axis = a;
        }
    const float split = (lo[axis] + hi[axis]) * 0.5f;
    const int spatial = depth < SP_SPATIAL_LEVELS && ext > 0.f && split > lo[axis];
    int64_t nl = 0;
    int bin_axis = -1, bin_plane = -1;
    if (c->binned && m > SP_FINISH_SLOTS && depth < SP_SPATIAL_LEVELS) {
        int64_t cnt[3][SP_BINS];
        float blo[3][SP_BINS][3], bhi[3][SP_BINS][3];
        for (int a = 0; a < 3; ++a)
            for (int k = 0; k < SP_BINS; ++k) {
                cnt[a][k] = 0;
                for (int d = 0; d < 3; ++d) {
                    blo[a][k][d] = INFINITY;
                    bhi[a][k][d] = -INFINITY;
                }
            }
        for (int64_t i = b; i < e; ++i) {
            const float* x = c->cen + 3 * (int64_t)c->perm[i];
            for (int a = 0; a < 3; ++a) {
                const float ea = hi[a] - lo[a];
                if (!(ea > 0.f)) continue;
                const int k = sp_bin(x[a], lo[a], ea);
                ++cnt[a][k];
                for (int d = 0; d < 3; ++d) {
                    blo[a][k][d] = fminf(blo[a][k][d], x[d]);
                    bhi[a][k][d] = fmaxf(bhi[a][k][d], x[d]);
                }
            }
        }
        double best = INFINITY;
        for (int a = 0; a < 3; ++a) {
            if (!(hi[a] - lo[a] > 0.f)) continue;
            for (int j = 0; j < SP_BINS - 1; ++j) {
                int64_t nL = 0, nR = 0;
                float Llo[3] = {INFINITY, INFINITY, INFINITY}, Lhi[3] = {-INFINITY, -INFINITY, -INFINITY};
                float Rlo[3] = {INFINITY, INFINITY, INFINITY}, Rhi[3] = {-INFINITY, -INFINITY, -INFINITY};
                for (int k = 0; k < SP_BINS; ++k) {
                    if (k <= j) {
                        nL += cnt[a][k];
                        for (int d = 0; d < 3; ++d) {
                            Llo[d] = fminf(Llo[d], blo[a][k][d]);
                            Lhi[d] = fmaxf(Lhi[d], bhi[a][k][d]);
                        }
                    } else {
                        nR += cnt[a][k];
                        for (int d = 0; d < 3; ++d) {
                            Rlo[d] = fminf(Rlo[d], blo[a][k][d]);
                            Rhi[d] = fmaxf(Rhi[d], bhi[a][k][d]);
                        }
                    }
                }
                if (nL == 0 || nR == 0) continue;
                const double cost = (double)nL * sp_diag2(Llo, Lhi) + (double)nR * sp_diag2(Rlo, Rhi);
                if (cost < best) {
                    best = cost;
                    bin_axis = a;
                    bin_plane = j;
                }
            }
        }
    }
    if (bin_axis >= 0) {
        const float la = lo[bin_axis], ea = hi[bin_axis] - lo[bin_axis];
        int64_t k = b;
        for (int64_t i = b; i < e; ++i)
            if (sp_bin(c->cen[3 * (int64_t)c->perm[i] + bin_axis], la, ea) <= bin_plane) c->tmp[k++] = c->perm[i];
        nl = k - b;
        for (int64_t i = b; i < e; ++i)
            if (!(sp_bin(c->cen[3 * (int64_t)c->perm[i] + bin_axis], la, ea) <= bin_plane)) c->tmp[k++] = c->perm[i];
        memcpy(c->perm + b, c->tmp + b, (size_t)m * sizeof(int32_t));
    } else if (spatial) {
        int64_t k = b;
        for (int64_t i = b; i < e; ++i)  /* stable partition: left run, then right run */
            if (c->cen[3 * (int64_t)c->perm[i] + axis] < split) c->tmp[k++] = c->perm[i];
        nl = k - b;
        for (int64_t i = b; i < e; ++i)
            if (!(c->cen[3 * (int64_t)c->perm[i] + axis] < split)) c->tmp[k++] = c->perm[i];
        memcpy(c->perm + b, c->tmp + b, (size_t)m * sizeof(int32_t));
    } else {
        nl = m / 2;
    }
    c->nleft[id] = sp_build_rec(c, b, b + nl, depth + 1);
    c->nright[id] = sp_build_rec(c, b + nl, e, depth + 1);
    return id;
}

/* Builder 1 after validation: per-mesh trees side by side (no node spans two meshes), then the
 * same refit and exact radii as the LBVH. */
static void lb_split_finish(lb_tree* T, const float* V, const int64_t* voff, const int32_t* F,
                            const int64_t* foff, int64_t nmeshes, int K, const float* cen,
                            int binned) {
    const int64_t n = T->nf;
    sp_ctx c;
    memset(&c, 0, sizeof(c));
    c.T = T;
    c.cen = cen;
    c.K = K;
    c.binned = binned;
    c.perm = (int32_t*)malloc(n * sizeof(int32_t));
    c.tmp = (int32_t*)malloc(n * sizeof(int32_t));
    const int64_t cap = 2 * n;
    c.nfirst = (int32_t*)malloc(cap * sizeof(int32_t));
    c.nlast = (int32_t*)malloc(cap * sizeof(int32_t));
    c.nleft = (int32_t*)malloc(cap * sizeof(int32_t));
    c.nright = (int32_t*)malloc(cap * sizeof(int32_t));
    for (int64_t t = 0; t < n; ++t) c.perm[t] = (int32_t)t;
    for (int64_t mm = 0; mm < nmeshes; ++mm) {
        if (foff[mm + 1] <= foff[mm]) continue;
        const int32_t r = sp_build_rec(&c, foff[mm], foff[mm + 1], 0);
        T->root[mm] = r;
        T->end[mm] = (int32_t)c.E;
    }
    const int64_t E = c.E;
    T->E = E;
    T->skip = (int32_t*)malloc(E * sizeof(int32_t));
    T->tbeg = (int32_t*)malloc(E * sizeof(int32_t));
    T->tcnt = (int32_t*)malloc(E * sizeof(int32_t));
    T->st = (lb_stage*)calloc(E, sizeof(lb_stage));
    T->keys = (uint64_t*)malloc(n * sizeof(uint64_t));
    T->sorted_tri = (int32_t*)malloc(n * sizeof(int32_t));
    T->tv = (float*)malloc(n * 9 * sizeof(float));
    int64_t mesh = 0;
    for (int64_t s = 0; s < n; ++s) {
        while (foff[mesh + 1] <= s) ++mesh;
        const int64_t t = c.perm[s];
        T->keys[s] = (uint64_t)mesh << MORTON_BITS;
        T->sorted_tri[s] = (int32_t)t;
        for (int j = 0; j < 3; ++j)
            for (int a = 0; a < 3; ++a) T->tv[9 * s + 3 * j + a] = V[3 * (voff[mesh] + F[3 * t + j]) + a];
    }
    /* skip links: a node's subtree is the run of positions [id, id + size); the next node after
     * it is the first one starting after its last slot (DFS order) */
    for (int64_t i = E - 1; i >= 0; --i) {
        const int leaf = c.nleft[i] < 0;
        T->tbeg[i] = c.nfirst[i];
        T->tcnt[i] = leaf ? c.nlast[i] - c.nfirst[i] + 1 : 0;
        T->skip[i] = leaf ? (int32_t)(i + 1) : T->skip[c.nright[i]];
    }
    /* refit in decreasing position (children after parents), then exact radii */
    for (int64_t i = E - 1; i >= 0; --i) {
        if (c.nleft[i] < 0) {
            lb_leaf(T, c.nfirst[i], c.nlast[i], &T->st[i]);
        } else {
            lb_combine(&T->st[c.nleft[i]], &T->st[c.nright[i]], &T->st[i]);
            T->st[i].r = round_up_float(sqrt(lb_node_r2(T, c.nfirst[i], c.nlast[i], T->st[i].P)));
        }
    }
    free(c.perm);
    free(c.tmp);
    free(c.nfirst);
    free(c.nlast);
    free(c.nleft);
    free(c.nright);
}

void* oracle_lbvh_build(const float* V, const int64_t* voff, const int32_t* F, const int64_t* foff,
                        int64_t nmeshes, int leaf_size, float near_scale, int builder) {
    lb_tree* T = (lb_tree*)calloc(1, sizeof(lb_tree));
    const int K = leaf_size;
    T->nmeshes = nmeshes;
    T->root = (int32_t*)malloc(nmeshes * sizeof(int32_t));
    T->end = (int32_t*)malloc(nmeshes * sizeof(int32_t));
    T->tau = (float*)malloc(nmeshes * sizeof(float));
    T->mlo = (float*)malloc(nmeshes * 3 * sizeof(float));
    T->mhi = (float*)malloc(nmeshes * 3 * sizeof(float));
    float* inv = (float*)malloc(nmeshes * 3 * sizeof(float));
    for (int64_t m = 0; m < nmeshes; ++m) {
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int64_t v = voff[m]; v < voff[m + 1]; ++v)
            for (int a = 0; a < 3; ++a) {
                lo[a] = fminf(lo[a], V[3 * v + a]);
                hi[a] = fmaxf(hi[a], V[3 * v + a]);
            }
        const int has = voff[m + 1] > voff[m];
        float diag2 = 0.f;
        for (int a = 0; a < 3; ++a) {
            float l = has ? lo[a] : 0.f, h = has ? hi[a] : 0.f;
            if (!(l <= h)) { l = 0.f; h = 0.f; }
            T->mlo[3 * m + a] = l;
            T->mhi[3 * m + a] = h;
            const float ext = h - l;
            inv[3 * m + a] = ext > 0.f ? 1.0f / ext : 0.f;
            diag2 = diag2 + ext * ext;
        }
        T->tau[m] = near_scale * sqrtf(diag2);
        T->root[m] = -1;
        T->end[m] = -1;
    }
    const int64_t n = foff[nmeshes];
    T->nf = n;
    if (n == 0) {
        free(inv);
        return T;
    }
    int mesh_bits = 0;
    while ((1ll << mesh_bits) < nmeshes) ++mesh_bits;
    (void)mesh_bits;
    kv_t* kv = (kv_t*)malloc(n * sizeof(kv_t));
    float* cen = (float*)malloc(n * 3 * sizeof(float));
    int64_t m = 0;
    for (int64_t t = 0; t < n; ++t) {
        while (foff[m + 1] <= t) ++m;
        float c[3];
        const int64_t nvm = voff[m + 1] - voff[m];
        for (int j = 0; j < 3; ++j) {
            const int32_t ix = F[3 * t + j];
            if (ix < 0 || ix >= nvm) goto bad;
        }
        for (int a = 0; a < 3; ++a) {
            float x[3];
            for (int j = 0; j < 3; ++j) {
                x[j] = V[3 * (voff[m] + F[3 * t + j]) + a];
                if (!isfinite(x[j])) goto bad;
            }
            c[a] = ((x[0] + x[1]) + x[2]) / 3.0f;
            cen[3 * t + a] = c[a];
        }
        {
            const unsigned code = (spread3(quantize10(c[0], T->mlo[3 * m], inv[3 * m])) << 2) |
                                  (spread3(quantize10(c[1], T->mlo[3 * m + 1], inv[3 * m + 1])) << 1) |
                                  spread3(quantize10(c[2], T->mlo[3 * m + 2], inv[3 * m + 2]));
            kv[t].key = ((uint64_t)m << MORTON_BITS) | code;
            kv[t].idx = (uint32_t)t;
        }
    }
    if (builder == 1 || builder == 2) {
        free(kv);
        lb_split_finish(T, V, voff, F, foff, nmeshes, K, cen, builder == 2);
        free(cen);
        free(inv);
        return T;
    }
    free(cen);
    qsort(kv, (size_t)n, sizeof(kv_t), cmp_kv);
    T->keys = (uint64_t*)malloc(n * sizeof(uint64_t));
    T->sorted_tri = (int32_t*)malloc(n * sizeof(int32_t));
    T->tv = (float*)malloc(n * 9 * sizeof(float));
    for (int64_t s = 0; s < n; ++s) {
        T->keys[s] = kv[s].key;
        T->sorted_tri[s] = (int32_t)kv[s].idx;
        const int64_t t = kv[s].idx, mm = (int64_t)(kv[s].key >> MORTON_BITS);
        for (int j = 0; j < 3; ++j)
            for (int a = 0; a < 3; ++a) T->tv[9 * s + 3 * j + a] = V[3 * (voff[mm] + F[3 * t + j]) + a];
    }
    free(kv);
    {
        const int64_t nn = 2 * n - 1;
        int32_t* parent = (int32_t*)malloc(nn * sizeof(int32_t));
        int32_t* first = (int32_t*)malloc(nn * sizeof(int32_t));
        int32_t* last = (int32_t*)malloc(nn * sizeof(int32_t));
        int32_t* left = (int32_t*)malloc((n > 1 ? n - 1 : 1) * sizeof(int32_t));
        int32_t* right = (int32_t*)malloc((n > 1 ? n - 1 : 1) * sizeof(int32_t));
        int32_t* cnt = (int32_t*)calloc(n + 1, sizeof(int32_t));
        uint8_t* flags = (uint8_t*)malloc(nn);
        int32_t* pos = (int32_t*)malloc(nn * sizeof(int32_t));
        const uint64_t* keys = T->keys;
        for (int64_t k = 0; k < n; ++k) first[n - 1 + k] = last[n - 1 + k] = (int32_t)k;
        parent[0] = -1;
        /* Karras 2012: one pass per internal node */
        for (int64_t i = 0; i + 1 < n; ++i) {
            const int d = (kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
            const int dmin = kdelta(keys, n, i, i - d);
            int64_t lmax = 2;
            while (kdelta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
            int64_t l = 0;
            for (int64_t t = lmax >> 1; t >= 1; t >>= 1)
                if (kdelta(keys, n, i, i + (l + t) * d) > dmin) l += t;
            const int64_t j = i + l * d;
            const int dnode = kdelta(keys, n, i, j);
            int64_t s = 0, step = l;
            do {
                step = (step + 1) >> 1;
                if (kdelta(keys, n, i, i + (s + step) * d) > dnode) s += step;
            } while (step > 1);
            const int64_t g = i + s * d + (d < 0 ? d : 0);
            const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
            const int32_t lc = (int32_t)((lo == g) ? (n - 1 + g) : g);
            const int32_t rc = (int32_t)((hi == g + 1) ? (n - 1 + g + 1) : g + 1);
            left[i] = lc;
            right[i] = rc;
            parent[lc] = (int32_t)i;
            parent[rc] = (int32_t)i;
            first[i] = (int32_t)lo;
            last[i] = (int32_t)hi;
        }
#define CROSS(u) ((keys[first[u]] >> MORTON_BITS) != (keys[last[u]] >> MORTON_BITS))
#define BIG(u) (CROSS(u) || (last[u] - first[u] + 1) > K)
        for (int64_t u = 0; u < nn; ++u) {
            const int emitted = (u == 0) || BIG(parent[u]);
            const int leaf = (u >= n - 1) || !BIG(u);
            flags[u] = (uint8_t)((emitted ? 1 : 0) | (leaf ? 2 : 0));
            if (emitted) cnt[first[u]]++;
        }
        int32_t run = 0;
        for (int64_t k = 0; k <= n; ++k) {
            const int32_t c = cnt[k];
            cnt[k] = run;
            run += c;
        }
        const int64_t E = cnt[n];
        T->E = E;
        T->skip = (int32_t*)malloc(E * sizeof(int32_t));
        T->tbeg = (int32_t*)malloc(E * sizeof(int32_t));
        T->tcnt = (int32_t*)malloc(E * sizeof(int32_t));
        T->st = (lb_stage*)calloc(E, sizeof(lb_stage));
        for (int64_t u = 0; u < nn; ++u) {
            if (!(flags[u] & 1)) {
                pos[u] = -1;
                continue;
            }
            int rank = 0;
            int64_t v = u;
            while (v != 0 && first[parent[v]] == first[v]) {
                ++rank;
                v = parent[v];
            }
            pos[u] = cnt[first[u]] + rank;
            const int32_t p = pos[u];
            const int cross = CROSS(u);
            const int leaf = (flags[u] & 2) && !cross;
            T->skip[p] = cnt[last[u] + 1];
            T->tbeg[p] = first[u];
            T->tcnt[p] = leaf ? last[u] - first[u] + 1 : 0;
        }
        /* mesh roots */
        for (int64_t mm = 0; mm < nmeshes; ++mm) {
            const int64_t lo = foff[mm], hi = foff[mm + 1] - 1;
            if (hi < lo) continue;
            int64_t u = (n - 1) + lo;
            while (u != 0) {
                const int64_t p = parent[u];
                if (first[p] < lo || last[p] > hi) break;
                u = p;
            }
            T->root[mm] = pos[u];
            T->end[mm] = T->skip[pos[u]];
        }
        /* refit in post-order (children before parents): process emitted nodes in decreasing
         * DFS position — every child has a larger position than its parent */
        int32_t* node_of_pos = (int32_t*)malloc(E * sizeof(int32_t));
        for (int64_t u = 0; u < nn; ++u)
            if (flags[u] & 1) node_of_pos[pos[u]] = (int32_t)u;
        for (int64_t p = E - 1; p >= 0; --p) {
            const int32_t u = node_of_pos[p];
            if (CROSS(u)) continue;
            if (flags[u] & 2) {
                lb_leaf(T, first[u], last[u], &T->st[p]);
            } else {
                lb_combine(&T->st[pos[left[u]]], &T->st[pos[right[u]]], &T->st[p]);
                T->st[p].r = round_up_float(sqrt(lb_node_r2(T, first[u], last[u], T->st[p].P)));
            }
        }
#undef BIG
#undef CROSS
        free(node_of_pos);
        free(parent);
        free(first);
        free(last);
        free(left);
        free(right);
        free(cnt);
        free(flags);
        free(pos);
    }
    free(inv);
    return T;
bad:
    free(kv);
    free(cen);
    free(inv);
    free(T->root);
    free(T->end);
    free(T->tau);
    free(T->mlo);
    free(T->mhi);
    free(T);
    return NULL;
}

void oracle_lbvh_free(void* h) {
    lb_tree* T = (lb_tree*)h;
    if (!T) return;
    free(T->root);
    free(T->end);
    free(T->tau);
    free(T->mlo);
    free(T->mhi);
    free(T->skip);
    free(T->tbeg);
    free(T->tcnt);
    free(T->st);
    free(T->sorted_tri);
    free(T->tv);
    free(T->keys);
    free(T);
}

int64_t oracle_lbvh_num_nodes(void* h) { return ((lb_tree*)h)->E; }

/* Exports (any pointer may be NULL): skip/tbeg/tcnt [E], center_radius [E*4],
 * moments [E*33] (P N M1 M2), sorted_tri [nf], mesh_root [nmeshes*2], tau [nmeshes]. */
void oracle_lbvh_export(void* h, int32_t* skip, int32_t* tbeg, int32_t* tcnt, double* cr,
                        double* moments, int32_t* sorted_tri, int32_t* mesh_root, float* tau) {
    const lb_tree* T = (const lb_tree*)h;
    for (int64_t p = 0; p < T->E; ++p) {
        if (skip) skip[p] = T->skip[p];
        if (tbeg) tbeg[p] = T->tbeg[p];
        if (tcnt) tcnt[p] = T->tcnt[p];
        if (cr) {
            for (int a = 0; a < 3; ++a) cr[4 * p + a] = T->st[p].P[a];
            cr[4 * p + 3] = T->st[p].r;
        }
        if (moments) {
            double* o = moments + 33 * p;
            for (int a = 0; a < 3; ++a) o[a] = T->st[p].P[a];
            for (int a = 0; a < 3; ++a) o[3 + a] = T->st[p].N[a];
            for (int a = 0; a < 9; ++a) o[6 + a] = T->st[p].M1[a];
            for (int a = 0; a < 18; ++a) o[15 + a] = T->st[p].M2[a];
        }
    }
    if (sorted_tri)
        for (int64_t s = 0; s < T->nf; ++s) sorted_tri[s] = T->sorted_tri[s];
    for (int64_t m = 0; m < T->nmeshes; ++m) {
        if (mesh_root) {
            mesh_root[2 * m] = T->root[m];
            mesh_root[2 * m + 1] = T->end[m];
        }
        if (tau) tau[m] = T->tau[m];
    }
}

/* order-2 expansion in FP64 from the raw moments (independent of the device's pre-scaled
 * coefficients): T = K(d).N + sum M1_ij dK_i/dd_j + 1/2 sum M2_ijk d2K_i/dd_j dd_k */
static double lb_taylor(const lb_stage* s, const double* d) {
    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double r = sqrt(r2);
    const double r3 = 1.0 / (r2 * r), r5 = r3 / r2, r7 = r5 / r2;
    double t = 0.0;
    for (int i = 0; i < 3; ++i) t += s->N[i] * d[i] * r3;
    /* dK_i/dd_j = delta_ij/r^3 - 3 d_i d_j / r^5 */
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            t += s->M1[3 * i + j] * ((i == j ? r3 : 0.0) - 3.0 * d[i] * d[j] * r5);
    /* d2K_i/dd_j dd_k = -3 (delta_ij d_k + delta_ik d_j + delta_jk d_i)/r^5 + 15 d_i d_j d_k / r^7 */
    static const int SJ[6] = {0, 1, 2, 0, 0, 1}, SK[6] = {0, 1, 2, 1, 2, 2};
    for (int i = 0; i < 3; ++i)
        for (int q = 0; q < 6; ++q) {
            const int j = SJ[q], k = SK[q];
            const double mult = (j == k) ? 1.0 : 2.0;
            const double h = -3.0 * ((i == j ? d[k] : 0.0) + (i == k ? d[j] : 0.0) + (j == k ? d[i] : 0.0)) * r5 +
                             15.0 * d[i] * d[j] * d[k] * r7;
            t += 0.5 * mult * s->M2[6 * i + q] * h;
        }
    return t;
}

/* The far/near predicate every form of the device path shares, in float, each step rounded as
 * written: fma(dx, dx, fma(dy, dy, dz * dz)) > (beta * r)^2 with d = P - q (P and r are float
 * values). The reference tree decides in float too (UT_SolidAngle<float, float>,
 * modules/winding/src/FastWindingNumber.cpp:80). Needs FLT_EVAL_METHOD == 0 and no
 * contraction (-ffp-contract=off). */
static int lb_far_pred(const lb_stage* st, const float* q, float beta) {
    const float dx = (float)st->P[0] - q[0], dy = (float)st->P[1] - q[1], dz = (float)st->P[2] - q[2];
    const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float br = beta * (float)st->r;
    return d2 > br * br;
}

typedef struct {
    const lb_tree* T;
    const float* Q;
    const int32_t* qmesh; /* per-query mesh id or NULL (mesh 0) */
    double beta;
    double* omega;
    int exact; /* 1: ignore the far field (every leaf exact) */
} lb_q_ctx;

static void lb_q_range(void* p, int64_t b, int64_t e) {
    lb_q_ctx* c = (lb_q_ctx*)p;
    const lb_tree* T = c->T;
    for (int64_t qi = b; qi < e; ++qi) {
        const int m = c->qmesh ? c->qmesh[qi] : 0;
        const double q[3] = {c->Q[3 * qi], c->Q[3 * qi + 1], c->Q[3 * qi + 2]};
        double s = 0.0;
        int64_t i = T->root[m];
        const int64_t end = T->end[m];
        if (i < 0) {
            c->omega[qi] = 0.0;
            continue;
        }
        while (i < end) {
            const lb_stage* st = &T->st[i];
            const double dx = st->P[0] - q[0], dy = st->P[1] - q[1], dz = st->P[2] - q[2];
            const int far = !c->exact && lb_far_pred(st, c->Q + 3 * qi, (float)c->beta);
            if (far) {
                const double d[3] = {dx, dy, dz};
                s += lb_taylor(st, d);
                i = T->skip[i];
            } else if (T->tcnt[i] > 0) {
                for (int32_t k = T->tbeg[i]; k < T->tbeg[i] + T->tcnt[i]; ++k) {
                    double v[3][3];
                    lb_tri_d(T, k, v);
                    s += oracle_tri_solid_angle_f64(v[0], v[1], v[2], q);
                }
                i = T->skip[i];
            } else {
                i = i + 1;
            }
        }
        c->omega[qi] = s;
    }
}

/* FP64 traversal of the restated LBVH (the device's shared FP32 far predicate, lb_far_pred;
 * FP64 far field and near field). exact=1 evaluates every triangle. */
void oracle_lbvh_query_f64(void* h, const float* Q, const int32_t* qmesh, int64_t nq, double beta,
                           int exact, double* omega, int nthreads) {
    lb_q_ctx c = {(const lb_tree*)h, Q, qmesh, beta, omega, exact};
    parallel_for(nq, nthreads, lb_q_range, &c);
}
