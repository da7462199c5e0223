// Batched forms of the reference's winding-number callers (the "next" rows around the path):
//   fwn_query_grid            the winding-number sign pass of volume::mesh_to_volume
//                             (modules/volume/src/mesh_to_volume.cpp:156-183 calls is_inside once
//                             per voxel from OpenVDB's threads): one launch over a voxel grid
//                             whose centres are generated on the device.
//   fwn_orientation_criterion the per-facet orientation test of
//                             modules/winding/examples/fix_orientation.cpp:75-115: two queries per
//                             facet at barycentre +- eps * unit normal, one batched query.
#include <cmath>
#include <string>

#include "fwn_internal.cuh"

namespace fwn {
namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;

// Query points of the orientation test, as the example computes them in float:
// normal = ((b - a) x (c - a)).normalized() (a zero normal stays zero), barycentre =
// (a + b + c) / 3, points barycentre +- eps * normal.
__global__ void k_orient_points(const float* __restrict__ V, int64_t nv,
                                const int32_t* __restrict__ F, int64_t nf, float eps,
                                float* __restrict__ Q, unsigned* __restrict__ status) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    int32_t id[3];
    bool ok = true;
    for (int j = 0; j < 3; ++j) {
        id[j] = F[3 * f + j];
        if (id[j] < 0 || (int64_t)id[j] >= nv) ok = false;
    }
    float p[3] = {0.f, 0.f, 0.f}, m[3] = {0.f, 0.f, 0.f};
    if (!ok) {
        atomicOr(status, ST_BAD_INDEX);
    } else {
        const float* a = V + 3 * (int64_t)id[0];
        const float* b = V + 3 * (int64_t)id[1];
        const float* c = V + 3 * (int64_t)id[2];
        // every float operation is rounded on its own, in the order written (no contraction into
        // fused multiply-adds), as the example's host code evaluates it, so that a host
        // restatement gives the same points bit for bit
        const float ux = __fsub_rn(b[0], a[0]), uy = __fsub_rn(b[1], a[1]), uz = __fsub_rn(b[2], a[2]);
        const float vx = __fsub_rn(c[0], a[0]), vy = __fsub_rn(c[1], a[1]), vz = __fsub_rn(c[2], a[2]);
        float nx = __fsub_rn(__fmul_rn(uy, vz), __fmul_rn(uz, vy));
        float ny = __fsub_rn(__fmul_rn(uz, vx), __fmul_rn(ux, vz));
        float nz = __fsub_rn(__fmul_rn(ux, vy), __fmul_rn(uy, vx));
        const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)),
                                               __fmul_rn(nz, nz)));
        if (len > 0.f) {
            nx = __fdiv_rn(nx, len);
            ny = __fdiv_rn(ny, len);
            nz = __fdiv_rn(nz, len);
        }
        const float n3[3] = {nx, ny, nz};
        for (int k = 0; k < 3; ++k) {
            const float bary = __fdiv_rn(__fadd_rn(__fadd_rn(a[k], b[k]), c[k]), 3.0f);
            p[k] = __fadd_rn(bary, __fmul_rn(eps, n3[k]));
            m[k] = __fsub_rn(bary, __fmul_rn(eps, n3[k]));
        }
    }
    for (int k = 0; k < 3; ++k) {
        Q[6 * f + k] = p[k];
        Q[6 * f + 3 + k] = m[k];
    }
}

// criterion = (Omega(p) - Omega(q)) / (4 pi): float difference, double division (as in the
// example's `(float - float) / (4.f * pi)` with pi a double constant); flip = criterion > threshold
__global__ void k_orient_criterion(const float* __restrict__ omega, int64_t nf, float threshold,
                                   float* __restrict__ crit, uint8_t* __restrict__ flip) {
    const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const double c = (double)(omega[2 * f] - omega[2 * f + 1]) / (4.0 * kPi);
    if (crit) crit[f] = (float)c;
    if (flip) flip[f] = c > (double)threshold ? 1 : 0;
}

inline unsigned grid_for(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

template <class Fn> fwn_status guarded(Fn&& fn) {
    try {
        fn();
        return FWN_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return FWN_INTERNAL;
    } catch (...) {
        set_last_error("unknown error");
        return FWN_INTERNAL;
    }
}

const Engine& engine_ref(fwn_handle h) {
    if (!h) throw Error(FWN_NOT_BUILT, "null handle (default-constructed or moved-from engine)");
    const Engine& e = *reinterpret_cast<const Engine*>(h);
    require_engine_device(e);
    return e;
}

}  // namespace
}  // namespace fwn

using namespace fwn;

extern "C" {

FWN_API fwn_status fwn_query_grid(fwn_handle h, int64_t mesh, const float* origin,
                                  const float* spacing, const int64_t* dims, float* d_omega,
                                  uint8_t* d_inside, void* stream) {
    return guarded([&] {
        const Engine& e = engine_ref(h);
        if (!origin || !spacing || !dims) throw Error(FWN_INVALID_ARG, "origin/spacing/dims are null");
        if (mesh < 0 || mesh >= e.nmeshes) throw Error(FWN_INVALID_ARG, "mesh index out of range");
        for (int a = 0; a < 3; ++a) {
            if (dims[a] < 0) throw Error(FWN_INVALID_ARG, "grid dimensions must be >= 0");
            if (!std::isfinite(origin[a]) || !std::isfinite(spacing[a]))
                throw Error(FWN_INVALID_ARG, "grid origin and spacing must be finite");
        }
        if (dims[0] > 0 && dims[1] > 0 && dims[2] > 0 &&
            (double)dims[0] * (double)dims[1] * (double)dims[2] > 9.0e15)
            throw Error(FWN_INVALID_ARG, "grid too large");
        const QueryArgs a = resolve_query_args(e, nullptr);
        query_grid(e, (int)mesh, a, origin, spacing, dims, d_omega, d_inside,
                   static_cast<cudaStream_t>(stream));
    });
}

FWN_API fwn_status fwn_orientation_criterion(fwn_handle h, const float* d_vertices, int64_t nv,
                                             const int32_t* d_triangles, int64_t nf, float eps,
                                             float threshold, float* d_criterion,
                                             uint8_t* d_flip, void* stream) {
    return guarded([&] {
        const Engine& e = engine_ref(h);
        if (e.nmeshes != 1) throw Error(FWN_INVALID_ARG, "forest handle: build one engine per reference mesh");
        if (nv < 0 || nf < 0) throw Error(FWN_INVALID_ARG, "sizes must be >= 0");
        if ((nv && !d_vertices) || (nf && !d_triangles)) throw Error(FWN_INVALID_ARG, "null pointer");
        if (!std::isfinite(eps) || !std::isfinite(threshold))
            throw Error(FWN_INVALID_ARG, "eps and threshold must be finite");
        if (nf == 0) return;
        if (2 * nf > (int64_t)INT32_MAX) throw Error(FWN_INVALID_ARG, "too many triangles");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        Scratch buf(256 + (size_t)nf * (6 * sizeof(float) + 2 * sizeof(float)), st);
        unsigned* d_status = buf.as<unsigned>();
        float* Q = reinterpret_cast<float*>(buf.as<char>() + 256);
        float* omega = Q + 6 * nf;
        FWN_CUDA_CHECK(cudaMemsetAsync(d_status, 0, sizeof(unsigned), st));
        k_orient_points<<<grid_for(nf, 256), 256, 0, st>>>(d_vertices, nv, d_triangles, nf, eps, Q,
                                                           d_status);
        FWN_CUDA_CHECK(cudaGetLastError());
        const QueryArgs a = resolve_query_args(e, nullptr);
        query_mesh(e, 0, a, Q, 2 * nf, omega, nullptr, nullptr, nullptr, st);
        k_orient_criterion<<<grid_for(nf, 256), 256, 0, st>>>(omega, nf, threshold, d_criterion,
                                                              d_flip);
        FWN_CUDA_CHECK(cudaGetLastError());
        unsigned sh = 0;
        FWN_CUDA_CHECK(cudaMemcpyAsync(&sh, d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        FWN_CUDA_CHECK(cudaStreamSynchronize(st));
        if (sh & ST_BAD_INDEX) throw Error(FWN_INVALID_ARG, "triangle vertex index out of range");
    });
}

}  // extern "C"
