// Winding-number traversal (replaces UT_SolidAngle::computeSolidAngle, called per point at
// modules/winding/src/FastWindingNumber.cpp:66 and :75).
//
// Tree walk: nodes are in DFS pre-order with escape links, so the walk is stackless:
//   far  (|P-q| > beta*r)      -> add the order-2 Taylor term, jump to skip
//   near leaf                   -> add exact triangle solid angles, jump to skip
//   near internal               -> step to i+1 (the first child)
// The cursor strictly increases, so every walk ends in at most num_nodes steps.
//
// The far/near decision is one FP32 predicate shared by every form (and by the oracle):
//   far  <=>  fma(dx, dx, fma(dy, dy, dz*dz)) > (beta*r)^2,  d = P - q, each step rounded to
//   float as written. The reference tree makes this decision in float as well (its engine is
//   UT_SolidAngle<float, float>, modules/winding/src/FastWindingNumber.cpp:80), and sharing it
//   makes the mixed and FP64 forms visit exactly the same nodes, so they differ only in
//   arithmetic.
//
// Forms:
//   mixed / thread : one thread per query, FP32 far field and near field with a Kahan sum;
//                    triangles within tau = fp64_near_scale * bbox diagonal get det and the
//                    Van Oosterom denominator in FP64.
//   mixed / warp   : 32 or 64 queries (one or two per lane) share one cursor (warp-uniform
//                    node loads, query slots inactive until the cursor reaches their own resume
//                    index); the leaf's triangles are staged in shared memory once per warp.
//   fp64           : the plain comparison form, FP64 everywhere (including atan2).
#include <climits>
#include <cmath>

#include "fwn_internal.cuh"

namespace fwn {
namespace {

constexpr double TWO_PI_D = 6.283185307179586476925286766559;  // Omega/(4 pi) > 0.5 <=> Omega > 2 pi

// is_inside of a float Omega: (double)Omega > 2 pi (the reference compares in double, since its pi
// is a double). 2 pi lies strictly between the floats 0x40C90FDA and 0x40C90FDB, so for every float
// x, (double)x > 2 pi <=> x > 0x40C90FDA (NaN: false on both sides). The float comparison keeps
// the test off the FP64 pipe, which on GB300 issues 2 operations per SM per cycle.
__device__ __forceinline__ uint8_t inside_of(float res) {
    return res > __int_as_float(0x40C90FDA) ? 1 : 0;
}

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

struct QCounters {
    unsigned nodes = 0, far = 0, tri = 0, tri64 = 0, steps = 0;
};

// The mixed form's arithmetic is written with explicit roundings (_rn intrinsics, and fmaf where
// a fused operation is wanted): the compiler may not contract a product into a neighbouring add
// on its own, because its choice could differ between the kernels that inline these functions
// (point walk, grid walk, forest walk, thread walk), and a query must get the same bits from all.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

// The shared far predicate (see the top of this file); also returns d = P - q and |d|^2 in
// float. Explicit _rn intrinsics keep the compiler from contracting it differently anywhere.
__device__ __forceinline__ bool far_pred(float px, float py, float pz, float r, float qx, float qy,
                                         float qz, float beta, float& dx, float& dy, float& dz,
                                         float& d2) {
    dx = __fsub_rn(px, qx);
    dy = __fsub_rn(py, qy);
    dz = __fsub_rn(pz, qz);
    d2 = __fmaf_rn(dx, dx, __fmaf_rn(dy, dy, __fmul_rn(dz, dz)));
    const float br = __fmul_rn(beta, r);
    return d2 > __fmul_rn(br, br);
}

// Order-2 far-field term of a node (coefficients pre-scaled, see NodeF32), d = P - q.
__device__ __forceinline__ float taylor_f32(const float4 m0, const float4 m1, const float4 m2,
                                            const float4 m3, const float4 m4, const float4 m5,
                                            float dx, float dy, float dz, float d2, float trM1) {
    const float rinv = rsqrtf(d2);
    const float rinv2 = __fmul_rn(rinv, rinv);
    const float rinv3 = __fmul_rn(rinv, rinv2);
    const float xx = __fmul_rn(dx, dx), yy = __fmul_rn(dy, dy), zz = __fmul_rn(dz, dz);
    const float xy = __fmul_rn(dx, dy), xz = __fmul_rn(dx, dz), yz = __fmul_rn(dy, dz);
    const float t0 = fmaf(dx, m0.x, fmaf(dy, m0.y, fmaf(dz, m0.z, trM1)));
    float t1 = __fmul_rn(m0.w, dx);
    t1 = fmaf(m1.x, dy, t1);
    t1 = fmaf(m1.y, dz, t1);
    t1 = fmaf(m1.z, xx, t1);
    t1 = fmaf(m1.w, yy, t1);
    t1 = fmaf(m2.x, zz, t1);
    t1 = fmaf(m2.y, xy, t1);
    t1 = fmaf(m2.z, xz, t1);
    t1 = fmaf(m2.w, yz, t1);
    const float gx = fmaf(m3.x, dx, fmaf(m3.w, dy, __fmul_rn(m4.x, dz)));  // xxx xxy xxz
    const float gy = fmaf(m4.y, dx, fmaf(m3.y, dy, __fmul_rn(m4.z, dz)));  // xyy yyy yyz
    const float gz = fmaf(m4.w, dx, fmaf(m5.x, dy, __fmul_rn(m3.z, dz)));  // xzz yzz zzz
    const float t2 = fmaf(xx, gx, fmaf(yy, gy, fmaf(zz, gz, __fmul_rn(__fmul_rn(m5.y, xy), dz))));
    return __fmul_rn(rinv3, fmaf(rinv2, fmaf(rinv2, t2, t1), t0));
}

// ---- paired f32x2 arithmetic (sm_100+): two FP32 lanes per instruction on a 64-bit register
// pair. Each half rounds exactly like the scalar instruction, so a paired evaluation gives the
// scalar results bit for bit while issuing half as many FP32 instructions.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(f32x2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 bc2(float x) { return pk2(x, x); }

// taylor_f32 for two query slots at once (halves: slot 0, slot 1), the same operations in the
// same order, so each half equals the scalar taylor_f32 of its slot.
__device__ __forceinline__ void taylor_f32x2(const float4 m0, const float4 m1, const float4 m2,
                                             const float4 m3, const float4 m4, const float4 m5,
                                             float trM1, float dx0, float dy0, float dz0,
                                             float d20, float dx1, float dy1, float dz1,
                                             float d21, float& out0, float& out1) {
    const f32x2 rinv = pk2(rsqrtf(d20), rsqrtf(d21));
    const f32x2 rinv2 = mul2(rinv, rinv);
    const f32x2 rinv3 = mul2(rinv, rinv2);
    const f32x2 DX = pk2(dx0, dx1), DY = pk2(dy0, dy1), DZ = pk2(dz0, dz1);
    const f32x2 XX = mul2(DX, DX), YY = mul2(DY, DY), ZZ = mul2(DZ, DZ);
    const f32x2 XY = mul2(DX, DY), XZ = mul2(DX, DZ), YZ = mul2(DY, DZ);
    const f32x2 t0 = fma2(DX, bc2(m0.x), fma2(DY, bc2(m0.y), fma2(DZ, bc2(m0.z), bc2(trM1))));
    f32x2 t1 = mul2(bc2(m0.w), DX);
    t1 = fma2(bc2(m1.x), DY, t1);
    t1 = fma2(bc2(m1.y), DZ, t1);
    t1 = fma2(bc2(m1.z), XX, t1);
    t1 = fma2(bc2(m1.w), YY, t1);
    t1 = fma2(bc2(m2.x), ZZ, t1);
    t1 = fma2(bc2(m2.y), XY, t1);
    t1 = fma2(bc2(m2.z), XZ, t1);
    t1 = fma2(bc2(m2.w), YZ, t1);
    const f32x2 gx = fma2(bc2(m3.x), DX, fma2(bc2(m3.w), DY, mul2(bc2(m4.x), DZ)));
    const f32x2 gy = fma2(bc2(m4.y), DX, fma2(bc2(m3.y), DY, mul2(bc2(m4.z), DZ)));
    const f32x2 gz = fma2(bc2(m4.w), DX, fma2(bc2(m5.x), DY, mul2(bc2(m3.z), DZ)));
    const f32x2 t2 = fma2(XX, gx, fma2(YY, gy, fma2(ZZ, gz, mul2(mul2(bc2(m5.y), XY), DZ))));
    upk2(mul2(rinv3, fma2(rinv2, fma2(rinv2, t2, t1), t0)), out0, out1);
}

__device__ __forceinline__ double taylor_f64(const NodeF64* __restrict__ nd, double dx, double dy,
                                             double dz, double d2) {
    const double rinv = 1.0 / sqrt(d2);
    const double rinv2 = rinv * rinv;
    const double rinv3 = rinv * rinv2;
    const double xx = dx * dx, yy = dy * dy, zz = dz * dz;
    const double xy = dx * dy, xz = dx * dz, yz = dy * dz;
    const double t0 = dx * nd->N[0] + dy * nd->N[1] + dz * nd->N[2] + nd->trM1;
    const double t1 = nd->W[0] * dx + nd->W[1] * dy + nd->W[2] * dz + nd->C[0] * xx +
                      nd->C[1] * yy + nd->C[2] * zz + nd->C[3] * xy + nd->C[4] * xz +
                      nd->C[5] * yz;
    const double* D = nd->D;  // xxx yyy zzz xxy xxz xyy yyz xzz yzz xyz
    const double t2 = xx * (D[0] * dx + D[3] * dy + D[4] * dz) +
                      yy * (D[5] * dx + D[1] * dy + D[6] * dz) +
                      zz * (D[7] * dx + D[8] * dy + D[2] * dz) + D[9] * xy * dz;
    return rinv3 * (t0 + rinv2 * (t1 + rinv2 * t2));
}

// Van Oosterom & Strackee (1983): tan(Omega/2) = a.(b x c) /
//   (|a||b||c| + (a.b)|c| + (b.c)|a| + (c.a)|b|),  a,b,c = vertices - q.
// A query on a vertex, or in the triangle's plane (det == 0), contributes 0.
__device__ __forceinline__ double tri_omega_f64(double ax, double ay, double az, double bx,
                                                double by, double bz, double cx, double cy,
                                                double cz) {
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

// Mixed-form near field in FP64: det and the denominator in FP64 (the cancellation-prone part),
// then atan2 in FP32 on the exponent-normalised pair (atan2 is well conditioned in its inputs).
__device__ __noinline__ float tri_omega_near64(float v0x, float v0y, float v0z, float v1x,
                                               float v1y, float v1z, float v2x, float v2y,
                                               float v2z, float qx, float qy, float qz) {
    const double ax = (double)v0x - (double)qx, ay = (double)v0y - (double)qy,
                 az = (double)v0z - (double)qz;
    const double bx = (double)v1x - (double)qx, by = (double)v1y - (double)qy,
                 bz = (double)v1z - (double)qz;
    const double cx = (double)v2x - (double)qx, cy = (double)v2y - (double)qy,
                 cz = (double)v2z - (double)qz;
    const double la = sqrt(fma(ax, ax, fma(ay, ay, __dmul_rn(az, az))));
    const double lb = sqrt(fma(bx, bx, fma(by, by, __dmul_rn(bz, bz))));
    const double lc = sqrt(fma(cx, cx, fma(cy, cy, __dmul_rn(cz, cz))));
    if (la == 0.0 || lb == 0.0 || lc == 0.0) return 0.f;
    const double crx = fma(by, cz, -__dmul_rn(bz, cy)), cry = fma(bz, cx, -__dmul_rn(bx, cz)),
                 crz = fma(bx, cy, -__dmul_rn(by, cx));
    const double det = fma(ax, crx, fma(ay, cry, __dmul_rn(az, crz)));
    if (det == 0.0) return 0.f;
    const double ab = fma(ax, bx, fma(ay, by, __dmul_rn(az, bz)));
    const double bc = fma(bx, cx, fma(by, cy, __dmul_rn(bz, cz)));
    const double ca = fma(cx, ax, fma(cy, ay, __dmul_rn(cz, az)));
    const double D = fma(ab, lc, fma(bc, la, fma(ca, lb, __dmul_rn(__dmul_rn(la, lb), lc))));
    const double m = fmax(fabs(det), fabs(D));
    const int ex = max(-1000, min(1000, ((__double2hiint(m) >> 20) & 0x7ff) - 1023));
    const double sc = __hiloint2double((1023 - ex) << 20, 0);  // 2^-ex, exact scaling
    return __fmul_rn(2.0f, atan2f((float)__dmul_rn(det, sc), (float)__dmul_rn(D, sc)));
}

// sqrt(x) for x >= 0 as x * rsqrt(x): two instructions instead of the correctly rounded square
// root, a few ulp of error (well inside the mixed form's budget; the ill-conditioned triangles
// where it could matter are re-evaluated in FP64). Exactly 0 for x = 0.
__device__ __forceinline__ float sqrt_fast(float x) {
    return __fmul_rn(x, rsqrtf(fmaxf(x, 1e-37f)));
}

template <bool STATS>
__device__ __forceinline__ float tri_omega_mixed(float v0x, float v0y, float v0z, float v1x,
                                                 float v1y, float v1z, float v2x, float v2y,
                                                 float v2z, float rt, float inv_nlen, float qx,
                                                 float qy, float qz, float tau, float cond,
                                                 QCounters& qc) {
    const float ax = __fsub_rn(v0x, qx), ay = __fsub_rn(v0y, qy), az = __fsub_rn(v0z, qz);
    const float bx = __fsub_rn(v1x, qx), by = __fsub_rn(v1y, qy), bz = __fsub_rn(v1z, qz);
    const float cx = __fsub_rn(v2x, qx), cy = __fsub_rn(v2y, qy), cz = __fsub_rn(v2z, qz);
    const float crx = fmaf(by, cz, -__fmul_rn(bz, cy)), cry = fmaf(bz, cx, -__fmul_rn(bx, cz)),
                crz = fmaf(bx, cy, -__fmul_rn(by, cx));
    const float det = fmaf(ax, crx, fmaf(ay, cry, __fmul_rn(az, crz)));
    const float la = sqrt_fast(fmaf(ax, ax, fmaf(ay, ay, __fmul_rn(az, az))));
    const float lb = sqrt_fast(fmaf(bx, bx, fmaf(by, by, __fmul_rn(bz, bz))));
    const float lc = sqrt_fast(fmaf(cx, cx, fmaf(cy, cy, __fmul_rn(cz, cz))));
    const float ab = fmaf(ax, bx, fmaf(ay, by, __fmul_rn(az, bz)));
    const float bc = fmaf(bx, cx, fmaf(by, cy, __fmul_rn(bz, cz)));
    const float ca = fmaf(cx, ax, fmaf(cy, ay, __fmul_rn(cz, az)));
    const float prod = __fmul_rn(__fmul_rn(la, lb), lc);
    const float D = fmaf(ab, lc, fmaf(bc, la, fmaf(ca, lb, prod)));
    // FP64 near field: the triangle is within tau of q (lower bound of the distance:
    // max(plane distance, centroid distance - Rt)) AND its FP32 evaluation is ill-conditioned.
    // The FP32 rounding errors of det and D are ~eps*|a||b||c| each, so the angle error is
    // ~eps*kappa with kappa = |a||b||c| / |(det, D)|; and when D <= 0, a det within its rounding
    // error may carry the wrong sign, i.e. the wrong side of atan2's branch cut (+-pi).
    const float h = __fmul_rn(fabsf(det), inv_nlen);
    if (h < tau) {
        const float sx = __fadd_rn(__fadd_rn(ax, bx), cx), sy = __fadd_rn(__fadd_rn(ay, by), cy),
                    sz = __fadd_rn(__fadd_rn(az, bz), cz);
        const float dc = __fmul_rn(sqrt_fast(fmaf(sx, sx, fmaf(sy, sy, __fmul_rn(sz, sz)))),
                                   1.0f / 3.0f);
        if (__fsub_rn(dc, rt) < tau) {
            const bool ill = prod > __fmul_rn(cond, sqrt_fast(fmaf(det, det, __fmul_rn(D, D)))) ||
                             (D <= 0.f && fabsf(det) <= __fmul_rn(1e-6f, prod));
            if (ill) {
                if (STATS) ++qc.tri64;
                return tri_omega_near64(v0x, v0y, v0z, v1x, v1y, v1z, v2x, v2y, v2z, qx, qy, qz);
            }
        }
    }
    if (la == 0.f || lb == 0.f || lc == 0.f || det == 0.f) return 0.f;
    return __fmul_rn(2.0f, atan2f(det, D));
}

__device__ __forceinline__ void flush_stats(const QCounters& c, unsigned long long* stats) {
    // warp-aggregated: all lanes of the warp call this (no early exits in STATS kernels)
    unsigned v[4] = {c.nodes, c.far, c.tri, c.tri64};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        unsigned s = __reduce_add_sync(0xffffffffu, v[i]);
        if ((threadIdx.x & 31) == 0 && s) atomicAdd(&stats[i], (unsigned long long)s);
    }
    // warp steps: the warp runs as many steps as its longest lane (per-lane step counts) or
    // as its shared cursor (all lanes hold the same count)
    const unsigned ws = __reduce_max_sync(0xffffffffu, c.steps);
    if ((threadIdx.x & 31) == 0 && ws) atomicAdd(&stats[4], (unsigned long long)ws);
}

// ---- 256-bit record loads ----------------------------------------------------------------------
// A NodeF32 is four 32 B sectors: sector 0 = (P, r, skip, tri_begin, tri_count, trM1), sectors
// 1-3 = far-field coefficients. One ld.global.nc.v8 per sector halves the load instructions (and
// the L1 wavefronts when lanes sit on different nodes) compared with float4 loads.
__device__ __forceinline__ void ld_v8(const void* p, float4& lo, float4& hi) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(lo.x), "=f"(lo.y), "=f"(lo.z), "=f"(lo.w), "=f"(hi.x), "=f"(hi.y), "=f"(hi.z),
          "=f"(hi.w)
        : "l"(p));
}

__device__ __forceinline__ void load_sector0(const NodeF32* nd, float4& a, int4& b) {
    float4 h;
    ld_v8(nd, a, h);
    b = make_int4(__float_as_int(h.x), __float_as_int(h.y), __float_as_int(h.z),
                  __float_as_int(h.w));
}

__device__ __forceinline__ float taylor_node(const NodeF32* nd, float dx, float dy, float dz,
                                             float d2, float trM1) {
    float4 m0, m1, m2, m3, m4, m5;
    ld_v8(&nd->m0, m0, m1);
    ld_v8(&nd->m2, m2, m3);
    ld_v8(&nd->m4, m4, m5);
    return taylor_f32(m0, m1, m2, m3, m4, m5, dx, dy, dz, d2, trM1);
}

template <bool STATS>
__device__ __forceinline__ bool far_test(const float4 a, float qx, float qy, float qz, float beta,
                                         float& dx, float& dy, float& dz, float& d2,
                                         QCounters& qc) {
    if (STATS) ++qc.nodes;
    return far_pred(a.x, a.y, a.z, a.w, qx, qy, qz, beta, dx, dy, dz, d2);
}

// ---- mixed, one thread per query --------------------------------------------------------------
// "Advance, then evaluate" rounds keep the warp converged on the two expensive blocks:
//   1. every lane walks its own path through cheap near-internal steps until it reaches its next
//      far node; near leaves met on the way are queued (two slots per lane) and skipped;
//   2. the lanes holding a far node evaluate its Taylor term together;
//   3. queued leaf triangles are evaluated in a batch once half the warp holds one (or a lane's
//      slots are full, or a lane has finished its walk), one triangle per lane per iteration.
constexpr int LEAF_BATCH = 16;

template <bool STATS>
__global__ void __launch_bounds__(256)
k_query_thread(const NodeF32* __restrict__ nodes, const TriF32* __restrict__ tris,
               const MeshInfo mi, const float* __restrict__ Q, const uint32_t* __restrict__ order,
               int64_t n, float beta, float* __restrict__ omega, uint8_t* __restrict__ inside,
               unsigned* __restrict__ status, unsigned long long* __restrict__ stats) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k - (threadIdx.x & 31) >= n) return;  // whole warp out of range (warp-uniform)
    const bool valid = k < n;
    QCounters qc;
    int64_t qi = 0;
    float qx = 0.f, qy = 0.f, qz = 0.f;
    if (valid) {
        qi = order ? (int64_t)order[k] : k;
        qx = Q[3 * qi];
        qy = Q[3 * qi + 1];
        qz = Q[3 * qi + 2];
    }
    const int end = mi.end;
    const float tau = mi.tau;
    const float cond = mi.cond;
    float s = 0.f, c = 0.f;
    int i = valid ? mi.root : end;
    int pb0 = 0, pc0 = 0, pb1 = 0, pc1 = 0;  // queued leaf triangle runs
    bool bad = false;
    while (true) {
        bool far = false;
        float dx = 0.f, dy = 0.f, dz = 0.f, d2 = 1.f, trM1 = 0.f;
        int skipf = 0;
        while (i < end) {
            float4 a;
            int4 b;
            load_sector0(nodes + i, a, b);
            far = far_test<STATS>(a, qx, qy, qz, beta, dx, dy, dz, d2, qc);
            if (far) {
                trM1 = __int_as_float(b.w);
                skipf = b.x;
                break;
            }
            if (b.z > 0) {
                if (pc0 == 0) {
                    pb0 = b.y;
                    pc0 = b.z;
                } else if (pc1 == 0) {
                    pb1 = b.y;
                    pc1 = b.z;
                } else {
                    break;  // both slots full: stay on this leaf until the batch below runs
                }
                if (b.x <= i) {
                    bad = true;
                    i = end;
                    break;
                }
                i = b.x;
            } else {
                i = i + 1;
            }
        }
        const bool blocked = (i < end) && !far;
        if (far) {
            kahan_add(s, c, taylor_node(nodes + i, dx, dy, dz, d2, trM1));
            if (STATS) ++qc.far;
            if (skipf <= i) {
                bad = true;
                i = end;
            } else {
                i = skipf;
            }
        }
        if (STATS) ++qc.steps;
        const bool pend = pc0 > 0;
        const bool done = i >= end;
        const unsigned pm = __ballot_sync(0xffffffffu, pend);
        if (__any_sync(0xffffffffu, blocked || (done && pend)) || __popc(pm) >= LEAF_BATCH) {
            while (__any_sync(0xffffffffu, pc0 > 0)) {
                if (pc0 > 0) {
                    const TriF32* T = tris + pb0;
                    const float4 t0 = __ldg(&T->t0), t1 = __ldg(&T->t1), t2 = __ldg(&T->t2);
                    const float w = tri_omega_mixed<STATS>(t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z,
                                                           t1.w, t2.x, t2.y, t2.z, qx, qy, qz, tau,
                                                           cond, qc);
                    kahan_add(s, c, w);
                    if (STATS) ++qc.tri;
                    ++pb0;
                    if (--pc0 == 0) {
                        pb0 = pb1;
                        pc0 = pc1;
                        pc1 = 0;
                    }
                }
            }
        }
        if (__all_sync(0xffffffffu, i >= end && pc0 == 0)) break;
    }
    if (bad) atomicOr(status, ST_BAD_LINK);
    if (valid) {
        const float res = s - c;
        if (omega) omega[qi] = res;
        if (inside) inside[qi] = inside_of(res);
    }
    if (STATS) flush_stats(qc, stats);
}

// Mesh of forest query k: the last mesh m with qoff[m] <= k (meshes without queries are skipped
// over, since their offset equals the next mesh's). qoff has nmeshes + 1 entries, qoff[0] = 0.
__device__ __forceinline__ int mesh_of_query(const int64_t* __restrict__ qoff, int nmeshes,
                                             int64_t k) {
    int lo = 0, hi = nmeshes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (qoff[mid] <= k) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// ---- mixed, warp-shared cursor ------------------------------------------------------------------
// 32 * QPL queries (QPL = 1 or 2 per lane) share one cursor over the DFS node order: the cursor
// is the smallest "resume" index of the warp's query slots, and a slot takes part in a step only
// when the cursor equals its own resume index. Node loads are therefore warp-uniform (one L1
// wavefront each, serving every slot), while every query still visits exactly its own path, in
// DFS order (so the result does not depend on which queries share the warp). With two slots per
// lane a node record serves 64 queries and each lane has two independent far tests to issue. A
// slot is done when its resume index reaches the end of its own mesh's subtree, so one warp may
// serve queries of consecutive meshes of a forest (their subtrees are consecutive ranges of the
// DFS order). The walk is software-pipelined: the next cursor is reduced right
// after the far test and its 32 B test sector is loaded before this step's Taylor / leaf work,
// and the coefficient sectors of the current node are requested before its far test.
// Near leaves: the (query, triangle) pairs of the leaf under the cursor are spread over all 32
// lanes (triangles staged in shared memory, each query with its mesh's FP64 near-field radius)
// and each owning slot adds its results in triangle order.
constexpr int WARP_LEAF_MAX = 16;
// ceil(2^16 / c) for c = 0..WARP_LEAF_MAX (entry 0 unused): the leaf pair loop's divisor table
__constant__ unsigned kPairMagic[WARP_LEAF_MAX + 1] = {
    0u, 65536u, 32768u, 21846u, 16384u, 13108u, 10923u, 9363u, 8192u,
    7282u, 6554u, 5958u, 5462u, 5042u, 4682u, 4370u, 4096u};
constexpr int WARP_BLOCK = 128;
constexpr int DONE = INT_MAX;

// Per-lane state of one query slot. A lane holds QPL queries; slot j of lane l is query
// j * 32 + l of the warp's group of 32 * QPL.
struct Slot {
    float qx, qy, qz;
    float tau;   // FP64 near-field radius of the query's mesh
    float s, c;  // Kahan sum
    int resume;  // next node this query visits (DONE when finished)
    int end;     // escape index of the query's mesh subtree
};

template <int QPL>
struct WarpSmem {
    float4 leaf[WARP_LEAF_MAX * 3];
    float4 q[32 * QPL];  // (x, y, z, tau) of the queries that need the current leaf
    float res[32 * QPL * WARP_LEAF_MAX];
};

// UEND: every slot of the warp walks the same subtree, ending at uend (one mesh: its subtree is
// the whole node range, and no skip link points past it), so a finished slot's resume index is
// uend itself and the per-slot end test drops out of every step.
// SOA: the node records as eight float4 arrays of num_nodes entries each (soa[k * stride + i]:
// k = 0 the test sector's (P, r), 1 its (skip, tri_begin, tri_count, trM1), 2-7 the coefficient
// float4s) instead of one 128 B record per node: the structure-of-arrays layout, kept as tuning
// variant 7 for the layout comparison.
template <bool STATS, int QPL, bool PAIRED = false, bool UEND = false, bool SOA = false>
__device__ __forceinline__ void warp_walk(const NodeF32* __restrict__ nodes,
                                          const TriF32* __restrict__ tris, Slot (&sl)[QPL],
                                          float cond, float beta, WarpSmem<QPL>& sm,
                                          QCounters& qc, unsigned* __restrict__ status,
                                          int uend = DONE, const float4* __restrict__ soa = nullptr,
                                          int64_t stride = 0) {
    auto sector0 = [&](int i, float4& a, int4& b) {
        if constexpr (SOA) {
            a = __ldg(soa + i);
            const float4 h = __ldg(soa + stride + i);
            b = make_int4(__float_as_int(h.x), __float_as_int(h.y), __float_as_int(h.z),
                          __float_as_int(h.w));
        } else {
            load_sector0(nodes + i, a, b);
        }
    };
    const int lane = threadIdx.x & 31;
    const unsigned lt = lanemask_lt();
    const int stop = UEND ? uend : DONE;
    int lo = stop;
#pragma unroll
    for (int j = 0; j < QPL; ++j) {
        if (sl[j].resume >= (UEND ? uend : sl[j].end)) sl[j].resume = stop;
        lo = min(lo, sl[j].resume);
    }
    int cursor = __reduce_min_sync(0xffffffffu, lo);
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
    int4 b = make_int4(0, 0, 0, 0);
    if (cursor != stop) sector0(cursor, a, b);
    while (cursor != stop) {
        float4 m0, m1, m2, m3, m4, m5;
        if constexpr (SOA) {
            const float4* c = soa + 2 * stride + cursor;
            m0 = __ldg(c); m1 = __ldg(c + stride); m2 = __ldg(c + 2 * stride);
            m3 = __ldg(c + 3 * stride); m4 = __ldg(c + 4 * stride); m5 = __ldg(c + 5 * stride);
        } else {
            const NodeF32* nd = nodes + cursor;
            ld_v8(&nd->m0, m0, m1);
            ld_v8(&nd->m2, m2, m3);
            ld_v8(&nd->m4, m4, m5);
        }
        // far test of every slot on every lane (only slots whose resume index is the cursor use
        // the result), with no divergent branch around it and the resume update as selects
        const bool leafnode = b.z > 0;
        bool do_far[QPL], need_leaf[QPL];
        float dx[QPL], dy[QPL], dz[QPL], d2[QPL];
        int lo2 = stop;
#pragma unroll
        for (int j = 0; j < QPL; ++j) {
            const bool active = sl[j].resume == cursor;
            const bool far = far_pred(a.x, a.y, a.z, a.w, sl[j].qx, sl[j].qy, sl[j].qz, beta, dx[j],
                                      dy[j], dz[j], d2[j]);
            if (STATS && active) ++qc.nodes;
            int nr = (far || leafnode) ? b.x : cursor + 1;
            if constexpr (UEND) nr = min(nr, uend);  // a well-formed tree never exceeds it
            else nr = nr >= sl[j].end ? DONE : nr;
            sl[j].resume = active ? nr : sl[j].resume;
            do_far[j] = active && far;
            need_leaf[j] = active && !far && leafnode;
            lo2 = min(lo2, sl[j].resume);
        }
        const int nc = __reduce_min_sync(0xffffffffu, lo2);
        float4 an = a;
        int4 bn = b;
        if (nc != stop) sector0(nc, an, bn);  // next step's test sector, in flight
        if constexpr (PAIRED && QPL == 2) {
            // both slots' Taylor terms in one paired evaluation when any lane of either is far
            if (__any_sync(0xffffffffu, do_far[0] || do_far[1])) {
                float t[2];
                taylor_f32x2(m0, m1, m2, m3, m4, m5, __int_as_float(b.w), dx[0], dy[0], dz[0],
                             d2[0], dx[QPL - 1], dy[QPL - 1], dz[QPL - 1], d2[QPL - 1], t[0], t[1]);
#pragma unroll
                for (int j = 0; j < QPL; ++j)
                    if (do_far[j]) {
                        kahan_add(sl[j].s, sl[j].c, t[j]);
                        if (STATS) ++qc.far;
                    }
            }
        } else {
#pragma unroll
            for (int j = 0; j < QPL; ++j) {
                if (__any_sync(0xffffffffu, do_far[j])) {  // warp-uniform: all lanes evaluate
                    const float t = taylor_f32(m0, m1, m2, m3, m4, m5, dx[j], dy[j], dz[j], d2[j],
                                               __int_as_float(b.w));
                    if (do_far[j]) {
                        kahan_add(sl[j].s, sl[j].c, t);
                        if (STATS) ++qc.far;
                    }
                }
            }
        }
        unsigned lm[QPL];
        int off[QPL];
        int nl = 0;
#pragma unroll
        for (int j = 0; j < QPL; ++j) {
            lm[j] = __ballot_sync(0xffffffffu, need_leaf[j]);
            off[j] = nl;
            nl += __popc(lm[j]);
        }
        if (nl) {
            const int cnt = b.z;  // warp-uniform (same node for all lanes), <= WARP_LEAF_MAX
            const float4* src = reinterpret_cast<const float4*>(tris + b.y);
            for (int i = lane; i < 3 * cnt; i += 32) sm.leaf[i] = __ldg(src + i);
#pragma unroll
            for (int j = 0; j < QPL; ++j)
                if (need_leaf[j])
                    sm.q[off[j] + __popc(lm[j] & lt)] = make_float4(sl[j].qx, sl[j].qy, sl[j].qz, sl[j].tau);
            __syncwarp();
            const int np = nl * cnt;
            // p = r * cnt + t by a multiply-shift: floor(p * ceil(2^16 / cnt) / 2^16) = p / cnt
            // for every p < 4096 and cnt <= 16 (p < 64 * 16 here); integer ALU only, where a
            // float reciprocal would put two conversions per pair on GB300's narrow FP64 pipe
            const unsigned mcnt = kPairMagic[cnt];
            for (int base = 0; base < np; base += 32) {
                const int p = base + lane;
                if (p < np) {
                    const int r = (int)(((unsigned)p * mcnt) >> 16);
                    const int t = p - r * cnt;
                    const float4 qq = sm.q[r];
                    const float4 t0 = sm.leaf[3 * t], t1 = sm.leaf[3 * t + 1], t2 = sm.leaf[3 * t + 2];
                    sm.res[p] = tri_omega_mixed<STATS>(t0.x, t0.y, t0.z, t0.w, t1.x, t1.y, t1.z,
                                                       t1.w, t2.x, t2.y, t2.z, qq.x, qq.y, qq.z,
                                                       qq.w, cond, qc);
                }
            }
            __syncwarp();
#pragma unroll
            for (int j = 0; j < QPL; ++j) {
                if (need_leaf[j]) {
                    const int r = off[j] + __popc(lm[j] & lt);
                    for (int t = 0; t < cnt; ++t) kahan_add(sl[j].s, sl[j].c, sm.res[r * cnt + t]);
                    if (STATS) qc.tri += cnt;
                }
            }
            __syncwarp();
        }
        if (nc <= cursor) {  // cannot happen for a well-formed tree
            if (lane == 0) atomicOr(status, ST_BAD_LINK);
            break;
        }
        if (STATS) ++qc.steps;
        cursor = nc;
        a = an;
        b = bn;
    }
}

__device__ __forceinline__ void write_result(const Slot& s, int64_t qi, float* __restrict__ omega,
                                             uint8_t* __restrict__ inside) {
    const float res = s.s - s.c;
    if (omega) omega[qi] = res;
    if (inside) inside[qi] = inside_of(res);
}

// One mesh: each warp takes the next 32 * QPL queries of the (sorted) order. With sorted_omega
// the results go, coalesced, to position k of the sorted order (k_scatter_results then writes
// them to the callers' indices in one pass); otherwise to the callers' indices directly.
template <bool STATS, int MINB, int QPL, bool PAIRED = false, bool SOA = false>
__global__ void __launch_bounds__(WARP_BLOCK, MINB)
k_query_warp(const NodeF32* __restrict__ nodes, const TriF32* __restrict__ tris,
             const MeshInfo mi, const float* __restrict__ Q, const uint32_t* __restrict__ order,
             int64_t n, float beta, float* __restrict__ omega, uint8_t* __restrict__ inside,
             float* __restrict__ sorted_omega, unsigned* __restrict__ status,
             unsigned long long* __restrict__ stats, const float4* __restrict__ soa,
             int64_t soa_stride) {
    __shared__ WarpSmem<QPL> smem[WARP_BLOCK / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t base = ((int64_t)blockIdx.x * (WARP_BLOCK / 32) + w) * (32 * QPL);
    if (base >= n) return;  // whole warp out of range (warp-uniform)
    QCounters qc;
    Slot sl[QPL];
    int64_t qi[QPL];
#pragma unroll
    for (int j = 0; j < QPL; ++j) {
        const int64_t k = base + 32 * j + lane;
        const bool valid = k < n;
        qi[j] = valid ? (order ? (int64_t)order[k] : k) : -1;
        sl[j].qx = valid ? Q[3 * qi[j]] : 0.f;
        sl[j].qy = valid ? Q[3 * qi[j] + 1] : 0.f;
        sl[j].qz = valid ? Q[3 * qi[j] + 2] : 0.f;
        sl[j].tau = mi.tau;
        sl[j].s = sl[j].c = 0.f;
        sl[j].resume = valid ? mi.root : DONE;
        sl[j].end = mi.end;
    }
    warp_walk<STATS, QPL, PAIRED, true, SOA>(nodes, tris, sl, mi.cond, beta, smem[w], qc, status,
                                              mi.end, soa, soa_stride);
#pragma unroll
    for (int j = 0; j < QPL; ++j) {
        if (qi[j] < 0) continue;
        if (sorted_omega) sorted_omega[base + 32 * j + lane] = sl[j].s - sl[j].c;
        else write_result(sl[j], qi[j], omega, inside);
    }
    if (STATS) flush_stats(qc, stats);
}

// Writes the traversal's sorted-order results to the callers' indices: omega[order[k]] and
// inside[order[k]] from sorted_omega[k]. Reads are coalesced; the scattered 4 B and 1 B writes of a
// whole batch meet in L2 (one pass, with no tree traffic beside them), so partial sectors merge
// before they reach DRAM instead of being evicted half-written during the walk.
__global__ void k_scatter_results(const float* __restrict__ sorted_omega,
                                  const uint32_t* __restrict__ order, int64_t n,
                                  float* __restrict__ omega, uint8_t* __restrict__ inside) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float res = sorted_omega[k];
    const int64_t qi = order[k];
    if (omega) omega[qi] = res;
    if (inside) inside[qi] = inside_of(res);
}

// Regular grid: voxel (i, j, k) has centre fmaf(i + 0.5, spacing, origin) per axis and output
// index i + nx (j + ny k). Each warp takes one 4 x 4 x (2 QPL) brick of voxels (bricks in raster
// order; slot q of a lane holds layer pair q), so a warp's queries are spatially compact without
// a sort; no point array is read.
template <int MINB, int QPL, bool PAIRED = false>
__global__ void __launch_bounds__(WARP_BLOCK, MINB)
k_query_grid(const NodeF32* __restrict__ nodes, const TriF32* __restrict__ tris,
             const MeshInfo mi, float ox, float oy, float oz, float sx, float sy, float sz,
             int64_t nx, int64_t ny, int64_t nz, int64_t bx, int64_t by, int64_t nbricks,
             float beta, float* __restrict__ omega, uint8_t* __restrict__ inside,
             unsigned* __restrict__ status) {
    __shared__ WarpSmem<QPL> smem[WARP_BLOCK / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t brick = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (brick >= nbricks) return;  // warp-uniform
    const int64_t bi = brick % bx, bj = (brick / bx) % by, bk = brick / (bx * by);
    const int64_t i = bi * 4 + (lane & 3), j = bj * 4 + ((lane >> 2) & 3);
    Slot sl[QPL];
    int64_t out[QPL];
#pragma unroll
    for (int q = 0; q < QPL; ++q) {
        const int64_t k = bk * (2 * QPL) + 2 * q + (lane >> 4);
        const bool valid = i < nx && j < ny && k < nz;
        out[q] = valid ? i + nx * (j + ny * k) : -1;
        sl[q].qx = fmaf((float)i + 0.5f, sx, ox);
        sl[q].qy = fmaf((float)j + 0.5f, sy, oy);
        sl[q].qz = fmaf((float)k + 0.5f, sz, oz);
        sl[q].tau = mi.tau;
        sl[q].s = sl[q].c = 0.f;
        sl[q].resume = valid ? mi.root : DONE;
        sl[q].end = mi.end;
    }
    QCounters qc;
    warp_walk<false, QPL, PAIRED, true>(nodes, tris, sl, mi.cond, beta, smem[w], qc, status,
                                         mi.end);
#pragma unroll
    for (int q = 0; q < QPL; ++q)
        if (out[q] >= 0) write_result(sl[q], out[q], omega, inside);
}

// Forest: one persistent launch over all meshes. Queries are sorted by (mesh, Hilbert index); each
// warp takes the next 32 * QPL sorted queries from a global work counter until none are left. A
// slot's walk ends at its own mesh's subtree end, so a warp may serve queries of two meshes.
template <int MINB, int QPL, bool PAIRED = false>
__global__ void __launch_bounds__(WARP_BLOCK, MINB)
k_forest_warp(const NodeF32* __restrict__ nodes, const TriF32* __restrict__ tris,
              const MeshInfo* __restrict__ meshes, const float* __restrict__ Q,
              const int64_t* __restrict__ qoff, int nmeshes, const uint32_t* __restrict__ order,
              int64_t n, float beta, float cond, float* __restrict__ omega,
              uint8_t* __restrict__ inside, float* __restrict__ sorted_omega,
              unsigned* __restrict__ work, unsigned* __restrict__ status) {
    __shared__ WarpSmem<QPL> smem[WARP_BLOCK / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t nchunks = (n + 32 * QPL - 1) / (32 * QPL);
    QCounters qc;
    while (true) {
        unsigned chunk = 0;
        if (lane == 0) chunk = atomicAdd(work, 1u);
        chunk = __shfl_sync(0xffffffffu, chunk, 0);
        if ((int64_t)chunk >= nchunks) break;
        Slot sl[QPL];
        int64_t qi[QPL];
#pragma unroll
        for (int j = 0; j < QPL; ++j) {
            const int64_t k = (int64_t)chunk * (32 * QPL) + 32 * j + lane;
            sl[j].s = sl[j].c = 0.f;
            if (k < n) {
                qi[j] = order[k];
                sl[j].qx = Q[3 * qi[j]];
                sl[j].qy = Q[3 * qi[j] + 1];
                sl[j].qz = Q[3 * qi[j] + 2];
                const MeshInfo& mi = meshes[mesh_of_query(qoff, nmeshes, qi[j])];
                sl[j].tau = mi.tau;
                sl[j].resume = mi.root < 0 ? DONE : mi.root;
                sl[j].end = mi.end;
            } else {
                qi[j] = -1;
                sl[j].qx = sl[j].qy = sl[j].qz = sl[j].tau = 0.f;
                sl[j].resume = sl[j].end = DONE;
            }
        }
        warp_walk<false, QPL, PAIRED>(nodes, tris, sl, cond, beta, smem[w], qc, status);
#pragma unroll
        for (int j = 0; j < QPL; ++j) {
            if (qi[j] < 0) continue;
            if (sorted_omega) sorted_omega[(int64_t)chunk * (32 * QPL) + 32 * j + lane] = sl[j].s - sl[j].c;
            else write_result(sl[j], qi[j], omega, inside);
        }
    }
}

// ---- plain FP64 form ----------------------------------------------------------------------------
template <bool STATS>
__global__ void __launch_bounds__(128)
k_query_f64(const NodeF64* __restrict__ nodes, const TriF32* __restrict__ tris, const MeshInfo mi,
            const float* __restrict__ Q, const uint32_t* __restrict__ order, int64_t n,
            float beta, float* __restrict__ omega, uint8_t* __restrict__ inside,
            double* __restrict__ omega64, unsigned* __restrict__ status,
            unsigned long long* __restrict__ stats) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = k < n;
    if (!STATS && !valid) return;
    QCounters qc;
    if (valid) {
        const int64_t qi = order ? (int64_t)order[k] : k;
        const double qx = Q[3 * qi], qy = Q[3 * qi + 1], qz = Q[3 * qi + 2];
        double s = 0.0;
        int i = mi.root;
        const int end = mi.end;
        while (i < end) {
            const NodeF64* nd = nodes + i;
            const double px = nd->P[0], py = nd->P[1], pz = nd->P[2];
            float fdx, fdy, fdz, fd2;  // P, r and q are float values: the shared predicate
            const bool far = far_pred((float)px, (float)py, (float)pz, (float)nd->r, (float)qx,
                                      (float)qy, (float)qz, beta, fdx, fdy, fdz, fd2);
            if (STATS) { ++qc.nodes; ++qc.steps; }
            int next;
            const int skip = nd->skip, tc = nd->tri_count;
            if (far) {
                const double dx = px - qx, dy = py - qy, dz = pz - qz;
                s += taylor_f64(nd, dx, dy, dz, dx * dx + dy * dy + dz * dz);
                if (STATS) ++qc.far;
                next = skip;
            } else if (tc > 0) {
                const TriF32* T = tris + nd->tri_begin;
                for (int t = 0; t < tc; ++t) {
                    const float4 t0 = T[t].t0, t1 = T[t].t1, t2 = T[t].t2;
                    s += tri_omega_f64((double)t0.x - qx, (double)t0.y - qy, (double)t0.z - qz,
                                       (double)t0.w - qx, (double)t1.x - qy, (double)t1.y - qz,
                                       (double)t1.z - qx, (double)t1.w - qy, (double)t2.x - qz);
                }
                if (STATS) qc.tri += tc;
                next = skip;
            } else {
                next = i + 1;
            }
            if (next <= i) {
                atomicOr(status, ST_BAD_LINK);
                break;
            }
            i = next;
        }
        const float res = (float)s;
        if (omega) omega[qi] = res;
        if (omega64) omega64[qi] = s;
        if (inside) inside[qi] = inside_of(res);
    }
    if (STATS) flush_stats(qc, stats);
}

// ---- plain FP64 form on the warp-shared cursor ------------------------------------------------
// The FP64 form on the schedule of the mixed warp walk (one query per lane): the same cursor,
// far predicate and leaf pair distribution, with FP64 records, FP64 Taylor terms and FP64
// triangle solid angles summed in DFS order as k_query_f64 sums them. Against k_query_f64 it
// isolates what precision costs on the warp schedule; against the mixed warp walk it is the
// like-for-like FP64 comparison.
struct WarpSmem64 {
    float4 leaf[WARP_LEAF_MAX * 3];
    float4 q[32];
    double res[32 * WARP_LEAF_MAX];
};

__global__ void __launch_bounds__(WARP_BLOCK)
k_query_warp_f64(const NodeF64* __restrict__ nodes, const TriF32* __restrict__ tris,
                 const MeshInfo mi, const float* __restrict__ Q, const uint32_t* __restrict__ order,
                 int64_t n, float beta, float* __restrict__ omega, uint8_t* __restrict__ inside,
                 double* __restrict__ omega64, unsigned* __restrict__ status) {
    __shared__ WarpSmem64 smem[WARP_BLOCK / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t k = ((int64_t)blockIdx.x * (WARP_BLOCK / 32) + w) * 32 + lane;
    if (k - lane >= n) return;  // whole warp out of range (warp-uniform)
    WarpSmem64& sm = smem[w];
    const bool valid = k < n;
    const int64_t qi = valid ? (order ? (int64_t)order[k] : k) : -1;
    const float qx = valid ? Q[3 * qi] : 0.f, qy = valid ? Q[3 * qi + 1] : 0.f,
                qz = valid ? Q[3 * qi + 2] : 0.f;
    const double dqx = qx, dqy = qy, dqz = qz;
    const unsigned lt = lanemask_lt();
    double s = 0.0;
    int resume = valid ? mi.root : DONE;
    if (resume >= mi.end) resume = DONE;
    int cursor = __reduce_min_sync(0xffffffffu, resume);
    while (cursor != DONE) {
        const NodeF64* nd = nodes + cursor;
        const double px = nd->P[0], py = nd->P[1], pz = nd->P[2];
        const int skip = nd->skip, tb = nd->tri_begin, tc = nd->tri_count;
        const bool active = resume == cursor;
        float fdx, fdy, fdz, fd2;  // P, r and q are float values: the shared predicate
        const bool far = far_pred((float)px, (float)py, (float)pz, (float)nd->r, qx, qy, qz, beta,
                                  fdx, fdy, fdz, fd2);
        int nr = (far || tc > 0) ? skip : cursor + 1;
        nr = nr >= mi.end ? DONE : nr;
        const bool do_far = active && far, need_leaf = active && !far && tc > 0;
        if (active) resume = nr;
        const int nc = __reduce_min_sync(0xffffffffu, resume);
        if (__any_sync(0xffffffffu, do_far)) {
            const double dx = px - dqx, dy = py - dqy, dz = pz - dqz;
            const double t = taylor_f64(nd, dx, dy, dz, dx * dx + dy * dy + dz * dz);
            if (do_far) s += t;
        }
        const unsigned lm = __ballot_sync(0xffffffffu, need_leaf);
        if (lm) {
            const int nl = __popc(lm);
            const float4* src = reinterpret_cast<const float4*>(tris + tb);
            for (int i = lane; i < 3 * tc; i += 32) sm.leaf[i] = __ldg(src + i);
            if (need_leaf) sm.q[__popc(lm & lt)] = make_float4(qx, qy, qz, 0.f);
            __syncwarp();
            const int np = nl * tc;
            for (int p = lane; p < np; p += 32) {
                const int r = p / tc, t = p - r * tc;
                const float4 q = sm.q[r];
                const float4 t0 = sm.leaf[3 * t], t1 = sm.leaf[3 * t + 1], t2 = sm.leaf[3 * t + 2];
                const double x = q.x, y = q.y, z = q.z;
                sm.res[p] = tri_omega_f64((double)t0.x - x, (double)t0.y - y, (double)t0.z - z,
                                          (double)t0.w - x, (double)t1.x - y, (double)t1.y - z,
                                          (double)t1.z - x, (double)t1.w - y, (double)t2.x - z);
            }
            __syncwarp();
            if (need_leaf) {
                const int r = __popc(lm & lt);
                for (int t = 0; t < tc; ++t) s += sm.res[r * tc + t];
            }
            __syncwarp();
        }
        if (nc <= cursor) {  // cannot happen for a well-formed tree
            if (lane == 0) atomicOr(status, ST_BAD_LINK);
            break;
        }
        cursor = nc;
    }
    if (valid) {
        const float res = (float)s;
        if (omega) omega[qi] = res;
        if (omega64) omega64[qi] = s;
        if (inside) inside[qi] = inside_of(res);
    }
}

// ---- query sort keys -------------------------------------------------------------------------
__device__ __forceinline__ unsigned spread3q(unsigned x) {
    x &= 0x3ffu;
    x = (x | (x << 16)) & 0x030000ffu;
    x = (x | (x << 8)) & 0x0300f00fu;
    x = (x | (x << 4)) & 0x030c30c3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// 30-bit index of a cell of a 1024^3 grid along the 3-D Hilbert curve: Skilling's transpose
// algorithm ("Programming the Hilbert curve", AIP Conf. Proc. 707, 2004) undoes the excess work
// per bit plane, Gray-encodes the transposed coordinates, and interleaves their bits. Sorting
// the query points by it gives warps more compact groups than Morton order (no long jumps).
__device__ __forceinline__ unsigned hilbert3(unsigned x, unsigned y, unsigned z) {
    unsigned X[3] = {x, y, z};
    constexpr unsigned kTop = 1u << 9;
    for (unsigned q = kTop; q > 1; q >>= 1) {
        const unsigned p = q - 1;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            if (X[i] & q) {
                X[0] ^= p;  // invert the low bits of the first axis
            } else {
                const unsigned t = (X[0] ^ X[i]) & p;  // exchange the low bits with axis i
                X[0] ^= t;
                X[i] ^= t;
            }
        }
    }
    X[1] ^= X[0];
    X[2] ^= X[1];
    unsigned t = 0;
    for (unsigned q = kTop; q > 1; q >>= 1)
        if (X[2] & q) t ^= q - 1;
    X[0] ^= t;
    X[1] ^= t;
    X[2] ^= t;
    return (spread3q(X[0]) << 2) | (spread3q(X[1]) << 1) | spread3q(X[2]);
}

// Sort key of a query point in its mesh's frame (the mesh bbox grown by 25% per side, 1024
// cells per axis; NaN coordinates fall in cell 0).
__device__ __forceinline__ unsigned query_key(const MeshInfo& mi, const float* q) {
    unsigned c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float ext = mi.hi[a] - mi.lo[a];
        const float lo = mi.lo[a] - 0.25f * ext;
        const float inv = ext > 0.f ? 1.0f / (1.5f * ext) : 0.f;
        const float u = (q[a] - lo) * inv * 1024.0f;
        // floor of u clamped to [0, 1023] (NaN -> 0): adding 2^23 rounded down leaves floor(v)
        // in the low mantissa bits for 0 <= v < 2^23, the same value as the truncating (int)
        // conversion, without a conversion instruction (GB300 runs those on its narrow FP64 pipe)
        c[a] = u >= 0.f ? __float_as_uint(__fadd_rd(fminf(u, 1023.0f), 8388608.0f)) - 0x4B000000u : 0u;
    }
    return hilbert3(c[0], c[1], c[2]);
}

__global__ void k_query_keys(const float* __restrict__ Q, int64_t n, const MeshInfo mi,
                             uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    keys[k] = query_key(mi, Q + 3 * k);
    vals[k] = (uint32_t)k;
}

// Forest sort key of query k: its mesh id above the top `hb` bits of its 30-bit Hilbert index
// (the same curve, hb < 30 being a coarser level of it).
template <class K>
__global__ void k_forest_keys(const float* __restrict__ Q, int64_t n,
                              const int64_t* __restrict__ qoff, int nmeshes,
                              const MeshInfo* __restrict__ meshes, int hb, K* __restrict__ keys,
                              uint32_t* __restrict__ vals) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int m = mesh_of_query(qoff, nmeshes, k);
    keys[k] = ((K)m << hb) | (K)(query_key(meshes[m], Q + 3 * k) >> (30 - hb));
    vals[k] = (uint32_t)k;
}

__global__ void k_fill_zero(float* omega, uint8_t* inside, double* omega64, int64_t n) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (omega) omega[k] = 0.f;
    if (inside) inside[k] = 0;
    if (omega64) omega64[k] = 0.0;
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

// Warp-schedule variants (fwn_config::tuning): queries per lane and register cap.
//   1: 1 query per lane, 72 registers      2: 1 per lane, no cap     3: 1 per lane, 64 registers
//   4: 2 queries per lane, 64 registers    5: 2 per lane, 80 registers
//   6: 2 queries per lane, 64 registers, both slots' Taylor terms in paired f32x2 arithmetic
//   0 (default): 4 when the batch fills every SM's warp slots four times over at two queries per
//   lane, else 3 (with fewer queries, two per lane would leave SMs idle)
int warp_variant(int tuning, int64_t n) {
    if (tuning != 0) return tuning;
    int dev = 0, sms = 0;
    FWN_CUDA_CHECK(cudaGetDevice(&dev));
    FWN_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int64_t wave = (int64_t)sms * 32 * 64;  // 32 resident warps per SM, 64 queries each
    return n >= 4 * wave ? 4 : 3;
}

template <int MINB, int QPL, bool PAIRED = false, bool SOA = false>
void launch_query_warp(const Engine& e, const MeshInfo& mi, const float* d_points,
                       const uint32_t* order, int64_t n, float beta, float* d_omega,
                       uint8_t* d_inside, float* sorted_omega, unsigned* d_status,
                       cudaStream_t st) {
    if (SOA && !e.soa && e.num_nodes > 0)
        throw Error(FWN_INVALID_ARG, "tuning 7 (structure-of-arrays records) needs an engine built "
                                     "with tuning 7");
    k_query_warp<false, MINB, QPL, PAIRED, SOA><<<grid_for(n, WARP_BLOCK * QPL), WARP_BLOCK, 0, st>>>(
        e.nodes32, e.tris, mi, d_points, order, n, beta, d_omega, d_inside, sorted_omega,
        d_status, nullptr, e.soa, e.num_nodes);
}

// The warp walk of one mesh's queries. With a sort order and a free n-float buffer
// (sorted_omega), the results are written in sorted order and scattered to the callers'
// indices by one k_scatter_results pass.
void launch_query_warp_variant(int variant, const Engine& e, const MeshInfo& mi,
                               const float* d_points, const uint32_t* order, int64_t n,
                               float beta, float* d_omega, uint8_t* d_inside, unsigned* d_status,
                               cudaStream_t st, float* sorted_omega = nullptr) {
    float* so = (order && (d_omega || d_inside)) ? sorted_omega : nullptr;
    switch (variant) {
        case 1: launch_query_warp<7, 1>(e, mi, d_points, order, n, beta, d_omega, d_inside, so, d_status, st); break;
        case 2: launch_query_warp<1, 1>(e, mi, d_points, order, n, beta, d_omega, d_inside, so, d_status, st); break;
        case 4: launch_query_warp<8, 2>(e, mi, d_points, order, n, beta, d_omega, d_inside, so, d_status, st); break;
        case 5: launch_query_warp<6, 2>(e, mi, d_points, order, n, beta, d_omega, d_inside, so, d_status, st); break;
        case 6: launch_query_warp<8, 2, true>(e, mi, d_points, order, n, beta, d_omega, d_inside, so, d_status, st); break;
        case 7: launch_query_warp<8, 2, true, true>(e, mi, d_points, order, n, beta, d_omega, d_inside, so, d_status, st); break;
        default: launch_query_warp<8, 1>(e, mi, d_points, order, n, beta, d_omega, d_inside, so, d_status, st); break;
    }
    if (so) k_scatter_results<<<grid_for(n, 256), 256, 0, st>>>(so, order, n, d_omega, d_inside);
}

}  // namespace

QueryArgs resolve_query_args(const Engine& e, const fwn_query_opts* o) {
    QueryArgs a;
    a.precision = e.cfg.precision;
    a.traversal = e.cfg.traversal;
    a.block_size = e.cfg.block_size;
    a.sort_queries = e.cfg.sort_queries;
    a.beta = e.cfg.beta;
    a.tuning = e.cfg.tuning;
    if (o) {
        if (o->precision >= 0) a.precision = o->precision;
        if (o->traversal >= 0) a.traversal = o->traversal;
        if (o->block_size > 0) a.block_size = o->block_size;
        if (o->sort_queries >= 0) a.sort_queries = o->sort_queries;
        if (o->beta > 0.f) a.beta = o->beta;
        if (o->tuning > 0) a.tuning = o->tuning;
    }
    if (a.tuning < 0 || a.tuning > 7) throw Error(FWN_INVALID_ARG, "tuning must be in [0, 7]");
    if (a.precision != FWN_PRECISION_MIXED && a.precision != FWN_PRECISION_FP64)
        throw Error(FWN_INVALID_ARG, "unknown precision");
    // AUTO: the warp walk for the mixed form; for the FP64 form the plain thread-per-query walk
    // (the warp-schedule FP64 form runs when FWN_TRAVERSAL_WARP is asked for explicitly)
    if (a.traversal == FWN_TRAVERSAL_AUTO)
        a.traversal = a.precision == FWN_PRECISION_FP64 ? FWN_TRAVERSAL_THREAD : FWN_TRAVERSAL_WARP;
    if (a.traversal != FWN_TRAVERSAL_THREAD && a.traversal != FWN_TRAVERSAL_WARP)
        throw Error(FWN_INVALID_ARG, "unknown traversal");
    if (a.block_size <= 0) a.block_size = 128;
    if (a.block_size % 32 != 0 || a.block_size > 1024)
        throw Error(FWN_INVALID_ARG, "block_size must be a multiple of 32 and <= 1024");
    if (a.traversal == FWN_TRAVERSAL_WARP) a.block_size = 128;
    if (!(a.beta > 0.f) || !std::isfinite(a.beta)) throw Error(FWN_INVALID_ARG, "beta must be > 0");
    return a;
}

void query_order(const Engine& e, int mesh, const float* d_points, int64_t n, uint32_t* d_order,
                 cudaStream_t st) {
    if (n <= 0) return;
    const MeshInfo& mi = e.meshes_h[mesh];
    Scratch buf(3 * (size_t)n * sizeof(uint32_t) + radix_sort_temp_bytes(n, 4) + 256, st);
    uint32_t* ka = buf.as<uint32_t>();
    uint32_t* kb = ka + n;
    uint32_t* vb = kb + n;
    void* tmp = vb + n;
    k_query_keys<<<grid_for(n, 256), 256, 0, st>>>(d_points, n, mi, ka, d_order);
    FWN_CUDA_CHECK(cudaGetLastError());
    if (n > 1 && radix_sort_u32(ka, d_order, kb, vb, n, 30, tmp, st))
        FWN_CUDA_CHECK(cudaMemcpyAsync(d_order, vb, (size_t)n * sizeof(uint32_t),
                                       cudaMemcpyDeviceToDevice, st));
}

void query_mesh(const Engine& e, int mesh, const QueryArgs& a, const float* d_points, int64_t n,
                float* d_omega, uint8_t* d_inside, double* d_omega64, fwn_query_stats* stats,
                cudaStream_t st, bool check) {
    if (n <= 0) return;
    if (a.precision == FWN_PRECISION_FP64 && !e.nodes64 && e.num_nodes > 0)
        throw Error(FWN_INVALID_ARG, "engine was built without FP64 records (FWN_RECORDS_F64)");
    if (a.precision == FWN_PRECISION_MIXED && !e.nodes32 && e.num_nodes > 0)
        throw Error(FWN_INVALID_ARG, "engine was built without FP32 records (FWN_RECORDS_F32)");
    NvtxRange trace("fwn query");
    if (d_omega64 && a.precision != FWN_PRECISION_FP64)
        throw Error(FWN_INVALID_ARG, "FP64 solid-angle output needs the FP64 form");
    const MeshInfo& mi = e.meshes_h[mesh];
    // layout: [status u32 | pad to 8 B | 8 x u64 counters]
    constexpr size_t kStatusBytes = 8 + 8 * sizeof(unsigned long long);
    Scratch status(kStatusBytes, st);
    unsigned* d_status = status.as<unsigned>();
    unsigned long long* d_stats = reinterpret_cast<unsigned long long*>(status.as<char>() + 8);
    FWN_CUDA_CHECK(cudaMemsetAsync(status.p, 0, kStatusBytes, st));
    if (mi.root < 0) {
        k_fill_zero<<<grid_for(n, 256), 256, 0, st>>>(d_omega, d_inside, d_omega64, n);
        FWN_CUDA_CHECK(cudaGetLastError());
        if (stats) *stats = fwn_query_stats{0, 0, 0, 0, 0};
        return;
    }
    const uint32_t* order = nullptr;
    float* sorted_omega = nullptr;  // the sorted keys' buffer, free once the sort is done
    const bool do_sort = a.sort_queries && n > 1;
    Scratch sortbuf(do_sort ? 4 * (size_t)n * sizeof(uint32_t) + radix_sort_temp_bytes(n, 4) + 256 : 0, st);
    if (do_sort) {
        uint32_t* ka = sortbuf.as<uint32_t>();
        uint32_t* va = ka + n;
        uint32_t* kb = va + n;
        uint32_t* vb = kb + n;
        void* tmp = vb + n;
        k_query_keys<<<grid_for(n, 256), 256, 0, st>>>(d_points, n, mi, ka, va);
        const bool in_b = radix_sort_u32(ka, va, kb, vb, n, 30, tmp, st);
        order = in_b ? vb : va;
        sorted_omega = reinterpret_cast<float*>(in_b ? kb : ka);
    }
    const bool want_stats = stats != nullptr;
    const int bs = a.block_size;
    if (a.precision == FWN_PRECISION_FP64) {
        if (want_stats)  // counters: the thread walk (the counts do not depend on the schedule)
            k_query_f64<true><<<grid_for(n, 128), 128, 0, st>>>(e.nodes64, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, d_omega64, d_status, d_stats);
        else if (a.traversal == FWN_TRAVERSAL_WARP)
            k_query_warp_f64<<<grid_for(n, WARP_BLOCK), WARP_BLOCK, 0, st>>>(e.nodes64, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, d_omega64, d_status);
        else
            k_query_f64<false><<<grid_for(n, 128), 128, 0, st>>>(e.nodes64, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, d_omega64, d_status, d_stats);
    } else if (a.traversal == FWN_TRAVERSAL_WARP) {
        if (want_stats) {  // counters: no register cap, the variant's queries per lane
            if (warp_variant(a.tuning, n) >= 4)
                k_query_warp<true, 1, 2><<<grid_for(n, WARP_BLOCK * 2), WARP_BLOCK, 0, st>>>(e.nodes32, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, nullptr, d_status, d_stats, nullptr, 0);
            else
                k_query_warp<true, 1, 1><<<grid_for(n, WARP_BLOCK), WARP_BLOCK, 0, st>>>(e.nodes32, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, nullptr, d_status, d_stats, nullptr, 0);
        } else
            launch_query_warp_variant(warp_variant(a.tuning, n), e, mi, d_points, order, n, a.beta,
                                      d_omega, d_inside, d_status, st, sorted_omega);
    } else {
        if (want_stats)
            k_query_thread<true><<<grid_for(n, bs), bs, 0, st>>>(e.nodes32, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, d_status, d_stats);
        else
            k_query_thread<false><<<grid_for(n, bs), bs, 0, st>>>(e.nodes32, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, d_status, d_stats);
    }
    FWN_CUDA_CHECK(cudaGetLastError());
    if (want_stats || check) {
        unsigned long long h[8];
        unsigned sh = 0;
        FWN_CUDA_CHECK(cudaMemcpyAsync(h, d_stats, sizeof(h), cudaMemcpyDeviceToHost, st));
        FWN_CUDA_CHECK(cudaMemcpyAsync(&sh, d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        FWN_CUDA_CHECK(cudaStreamSynchronize(st));
        if (stats) {
            stats->nodes_tested = h[0];
            stats->far_evals = h[1];
            stats->tri_evals = h[2];
            stats->tri_evals_fp64 = h[3];
            stats->warp_steps = h[4];
        }
        if (sh & ST_BAD_LINK) throw Error(FWN_INTERNAL, "traversal met a non-advancing skip link");
    }
}

void query_grid(const Engine& e, int mesh, const QueryArgs& a, const float origin[3],
                const float spacing[3], const int64_t dims[3], float* d_omega, uint8_t* d_inside,
                cudaStream_t st) {
    const int64_t nx = dims[0], ny = dims[1], nz = dims[2];
    if (nx <= 0 || ny <= 0 || nz <= 0) return;
    const MeshInfo& mi = e.meshes_h[mesh];
    const int64_t n = nx * ny * nz;
    NvtxRange trace("fwn grid query");
    if (mi.root < 0) {
        k_fill_zero<<<grid_for(n, 256), 256, 0, st>>>(d_omega, d_inside, nullptr, n);
        FWN_CUDA_CHECK(cudaGetLastError());
        return;
    }
    if (!e.nodes32) throw Error(FWN_INVALID_ARG, "engine was built without FP32 records (FWN_RECORDS_F32)");
    // schedule variants as in the point query (warp_variant); two voxels per lane stack two
    // 4 x 4 x 2 layers in one brick
    // (variant 7, the structure-of-arrays records, exists for one mesh's point walk: grids run 6)
    const int v = std::min(warp_variant(a.tuning, nx * ny * nz), 6);
    const int qpl = v >= 4 ? 2 : 1;
    const int64_t bx = (nx + 3) / 4, by = (ny + 3) / 4, bz = (nz + 2 * qpl - 1) / (2 * qpl);
    const int64_t nbricks = bx * by * bz;
    Scratch status(sizeof(unsigned), st);
    FWN_CUDA_CHECK(cudaMemsetAsync(status.p, 0, sizeof(unsigned), st));
    const int64_t threads = nbricks * 32;
    auto kern = v == 1 ? k_query_grid<7, 1> : v == 2 ? k_query_grid<1, 1> : v == 4 ? k_query_grid<8, 2>
              : v == 5 ? k_query_grid<6, 2> : v == 6 ? k_query_grid<8, 2, true> : k_query_grid<8, 1>;
    kern<<<grid_for(threads, WARP_BLOCK), WARP_BLOCK, 0, st>>>(
        e.nodes32, e.tris, mi, origin[0], origin[1], origin[2], spacing[0], spacing[1], spacing[2],
        nx, ny, nz, bx, by, nbricks, a.beta, d_omega, d_inside, status.as<unsigned>());
    FWN_CUDA_CHECK(cudaGetLastError());
}

// 32-bit keys (mesh id above the top hb bits of the Hilbert index) whenever every mesh keeps at
// least 8 curve cells per query at that level, else 64-bit keys with all 30 bits. A 32-bit pass
// moves 20 B per key against 32 B, and 39 key bits would need a fifth pass.
ForestKeys forest_keys(int64_t nmeshes, const int64_t* query_offsets) {
    ForestKeys k;
    while ((1ll << k.mesh_bits) < nmeshes) ++k.mesh_bits;
    int64_t max_q = 0;
    for (int64_t m = 0; m < nmeshes; ++m)
        max_q = std::max(max_q, query_offsets[m + 1] - query_offsets[m]);
    const int hb = std::min(30, 32 - k.mesh_bits);
    k.narrow = hb >= 30 || (hb >= 3 && max_q <= (int64_t(1) << (hb - 3)));
    k.hilbert_bits = k.narrow ? hb : 30;
    k.key_bits = k.mesh_bits + k.hilbert_bits;
    return k;
}

void query_forest(const Engine& e, const QueryArgs& a, const float* d_points,
                  const int64_t* query_offsets, float* d_omega, uint8_t* d_inside,
                  cudaStream_t st) {
    const int64_t n = query_offsets[e.nmeshes];
    if (n <= 0) return;
    if (a.precision == FWN_PRECISION_FP64 || e.num_nodes == 0) {
        // the plain form: one launch per mesh
        for (int64_t m = 0; m < e.nmeshes; ++m) {
            const int64_t q0 = query_offsets[m], q1 = query_offsets[m + 1];
            if (q1 <= q0) continue;
            query_mesh(e, (int)m, a, d_points + 3 * q0, q1 - q0, d_omega ? d_omega + q0 : nullptr,
                       d_inside ? d_inside + q0 : nullptr, nullptr, nullptr, st);
        }
        return;
    }
    if (!e.nodes32) throw Error(FWN_INVALID_ARG, "engine was built without FP32 records (FWN_RECORDS_F32)");
    if (n > (int64_t)UINT32_MAX) throw Error(FWN_INVALID_ARG, "too many forest queries");
    NvtxRange trace("fwn forest query");
    const ForestKeys fk = forest_keys(e.nmeshes, query_offsets);
    const int mesh_bits = fk.mesh_bits, hb = fk.hilbert_bits;
    const bool narrow = fk.narrow;
    const size_t nb = (size_t)n;
    const size_t bytes = 256 + (e.nmeshes + 1) * sizeof(int64_t) + 2 * nb * sizeof(uint64_t) +
                         2 * nb * sizeof(uint32_t) + radix_sort_temp_bytes(n, 8) + 1024;
    Scratch buf(bytes, st);
    char* p = buf.as<char>();
    unsigned* d_status = reinterpret_cast<unsigned*>(p);          // [0]: status, [1]: work counter
    int64_t* d_qoff = reinterpret_cast<int64_t*>(p + 256);
    uint64_t* ka = reinterpret_cast<uint64_t*>(p + 256 + ((e.nmeshes + 1) * sizeof(int64_t) + 255) / 256 * 256);
    uint64_t* kb = ka + nb;
    uint32_t* va = reinterpret_cast<uint32_t*>(kb + nb);
    uint32_t* vb = va + nb;
    void* tmp = vb + nb;
    FWN_CUDA_CHECK(cudaMemsetAsync(d_status, 0, 2 * sizeof(unsigned), st));
    FWN_CUDA_CHECK(cudaMemcpyAsync(d_qoff, query_offsets, (e.nmeshes + 1) * sizeof(int64_t),
                                   cudaMemcpyHostToDevice, st));
    const uint32_t* order = nullptr;
    // after the sort, the first key area (n u32 at least) holds the sorted-order results
    float* sorted_omega = (d_omega || d_inside) ? reinterpret_cast<float*>(ka) : nullptr;
    if (narrow) {
        uint32_t* ka32 = reinterpret_cast<uint32_t*>(ka);  // the 64-bit key areas hold n u32 each
        uint32_t* kb32 = reinterpret_cast<uint32_t*>(kb);
        k_forest_keys<uint32_t><<<grid_for(n, 256), 256, 0, st>>>(
            d_points, n, d_qoff, (int)e.nmeshes, e.meshes, hb, ka32, va);
        order = radix_sort_u32(ka32, va, kb32, vb, n, mesh_bits + hb, tmp, st) ? vb : va;
    } else {
        k_forest_keys<uint64_t><<<grid_for(n, 256), 256, 0, st>>>(
            d_points, n, d_qoff, (int)e.nmeshes, e.meshes, 30, ka, va);
        order = radix_sort_u64(ka, va, kb, vb, n, 30 + mesh_bits, tmp, st) ? vb : va;
    }
    int dev = 0, sms = 0, per_sm = 0;
    FWN_CUDA_CHECK(cudaGetDevice(&dev));
    FWN_CUDA_CHECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // schedule variants as in the point query (warp_variant)
    // (variant 7, the structure-of-arrays records, exists for one mesh's point walk: forests run 6)
    const int v = std::min(warp_variant(a.tuning, n), 6);
    const int qpl = v >= 4 ? 2 : 1;
    auto kern = v == 1 ? k_forest_warp<7, 1> : v == 2 ? k_forest_warp<1, 1> : v == 4 ? k_forest_warp<8, 2>
              : v == 5 ? k_forest_warp<6, 2> : v == 6 ? k_forest_warp<8, 2, true> : k_forest_warp<8, 1>;
    FWN_CUDA_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WARP_BLOCK, 0));
    const int64_t chunks = (n + 32 * qpl - 1) / (32 * qpl);
    const int64_t want = (chunks + WARP_BLOCK / 32 - 1) / (WARP_BLOCK / 32);
    const unsigned grid = (unsigned)std::min<int64_t>(want, (int64_t)sms * std::max(per_sm, 1));
    kern<<<grid, WARP_BLOCK, 0, st>>>(e.nodes32, e.tris, e.meshes, d_points, d_qoff,
                                      (int)e.nmeshes, order, n, a.beta, e.meshes_h[0].cond,
                                      d_omega, d_inside, sorted_omega, d_status + 1, d_status);
    if (sorted_omega)
        k_scatter_results<<<grid_for(n, 256), 256, 0, st>>>(sorted_omega, order, n, d_omega, d_inside);
    FWN_CUDA_CHECK(cudaGetLastError());
}

// Scratch layout of query_mesh_prealloc: [status word, 256 B][4 x n u32 sort keys/values]
// [radix-sort histogram].
size_t query_prealloc_bytes(int64_t n) {
    return 256 + 4 * (size_t)n * sizeof(uint32_t) + radix_sort_temp_bytes(n, 4);
}

void query_mesh_prealloc(const Engine& e, int mesh, const QueryArgs& a, const float* d_points,
                         int64_t n, float* d_omega, uint8_t* d_inside, void* scratch,
                         size_t scratch_bytes, cudaStream_t st) {
    if (n <= 0) return;
    if (query_prealloc_bytes(n) > scratch_bytes)
        throw Error(FWN_INTERNAL, "scratch region smaller than the query needs");
    if (a.precision == FWN_PRECISION_FP64 && !e.nodes64 && e.num_nodes > 0)
        throw Error(FWN_INVALID_ARG, "engine was built without FP64 records (FWN_RECORDS_F64)");
    if (a.precision == FWN_PRECISION_MIXED && !e.nodes32 && e.num_nodes > 0)
        throw Error(FWN_INVALID_ARG, "engine was built without FP32 records (FWN_RECORDS_F32)");
    const MeshInfo& mi = e.meshes_h[mesh];
    char* base = static_cast<char*>(scratch);
    unsigned* d_status = reinterpret_cast<unsigned*>(base);
    // the previous call's status bits are still in the shared region: clear them
    FWN_CUDA_CHECK(cudaMemsetAsync(d_status, 0, sizeof(unsigned), st));
    if (mi.root < 0) {
        k_fill_zero<<<grid_for(n, 256), 256, 0, st>>>(d_omega, d_inside, nullptr, n);
        FWN_CUDA_CHECK(cudaGetLastError());
        return;
    }
    const uint32_t* order = nullptr;
    float* sorted_omega = nullptr;  // the sorted keys' slot of the region, free after the sort
    if (a.sort_queries && n > 1) {
        uint32_t* ka = reinterpret_cast<uint32_t*>(base + 256);
        uint32_t* va = ka + n;
        uint32_t* kb = va + n;
        uint32_t* vb = kb + n;
        void* tmp = vb + n;  // histogram: every entry is written by each pass before it is read
        k_query_keys<<<grid_for(n, 256), 256, 0, st>>>(d_points, n, mi, ka, va);
        const bool in_b = radix_sort_u32(ka, va, kb, vb, n, 30, tmp, st);
        order = in_b ? vb : va;
        sorted_omega = reinterpret_cast<float*>(in_b ? kb : ka);
    }
    const int bs = a.block_size;
    if (a.precision == FWN_PRECISION_FP64) {
        if (a.traversal == FWN_TRAVERSAL_WARP)
            k_query_warp_f64<<<grid_for(n, WARP_BLOCK), WARP_BLOCK, 0, st>>>(e.nodes64, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, nullptr, d_status);
        else
            k_query_f64<false><<<grid_for(n, 128), 128, 0, st>>>(e.nodes64, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, nullptr, d_status, nullptr);
    } else if (a.traversal == FWN_TRAVERSAL_WARP) {
        launch_query_warp_variant(warp_variant(a.tuning, n), e, mi, d_points, order, n, a.beta,
                                  d_omega, d_inside, d_status, st, sorted_omega);
    } else {
        k_query_thread<false><<<grid_for(n, bs), bs, 0, st>>>(e.nodes32, e.tris, mi, d_points, order, n, a.beta, d_omega, d_inside, d_status, nullptr);
    }
    FWN_CUDA_CHECK(cudaGetLastError());
}

}  // namespace fwn
