// C interface to the reference itself — adobe/lagrange's lagrange::winding::FastWindingNumber
// (modules/winding/src/FastWindingNumber.cpp:57 init, :66 is_inside, :75 solid_angle) — for the
// CPU legs of the benchmark and the oracle tests. TEST / MEASUREMENT INFRASTRUCTURE ONLY.
//
// oracle/__init__.py compiles it only when a built reference is present (its headers and
// liblagrange_winding under baseline/_ref); otherwise the CPU legs use the restatement O2. It
// calls the reference's stock path: a SurfaceMesh<float, uint32_t> built from the arrays, the
// FastWindingNumber constructor, and one solid_angle call per point, spread over host threads the
// way volume::mesh_to_volume's OpenVDB workers call it (modules/volume/src/mesh_to_volume.cpp:
// 175-183). is_inside is Omega / (4 pi) > 0.5f as in FastWindingNumber.cpp:66.
#include <lagrange/SurfaceMesh.h>
#include <lagrange/winding/FastWindingNumber.h>

#include <cstdint>
#include <thread>
#include <vector>

extern "C" {

void* refshim_build(const float* V, int64_t nv, const int32_t* F, int64_t nf) {
    lagrange::SurfaceMesh<float, uint32_t> mesh;
    mesh.add_vertices(static_cast<uint32_t>(nv), {V, static_cast<size_t>(3 * nv)});
    std::vector<uint32_t> idx(F, F + 3 * nf);
    mesh.add_triangles(static_cast<uint32_t>(nf), {idx.data(), idx.size()});
    return new lagrange::winding::FastWindingNumber(mesh);
}

void refshim_free(void* h) { delete static_cast<lagrange::winding::FastWindingNumber*>(h); }

void refshim_query(void* h, const float* Q, int64_t n, float* omega, uint8_t* inside,
                   int nthreads) {
    const auto* eng = static_cast<const lagrange::winding::FastWindingNumber*>(h);
    const double four_pi = 4.0 * 3.14159265358979323846264338327950288;
    auto run = [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; ++i) {
            const float w = eng->solid_angle({Q[3 * i], Q[3 * i + 1], Q[3 * i + 2]});
            if (omega) omega[i] = w;
            if (inside) inside[i] = (double)w / four_pi > 0.5 ? 1 : 0;
        }
    };
    if (nthreads <= 1 || n < 2 * nthreads) {
        run(0, n);
        return;
    }
    std::vector<std::thread> pool;
    const int64_t chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        const int64_t b = t * chunk, e = b + chunk < n ? b + chunk : n;
        if (b < e) pool.emplace_back(run, b, e);
    }
    for (auto& th : pool) th.join();
}

}  // extern "C"
