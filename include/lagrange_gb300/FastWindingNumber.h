/*
 * lagrange_gb300::winding::FastWindingNumber — header-only C++ surface over the C ABI in
 * fwn_gb300.h, mirroring lagrange::winding::FastWindingNumber
 * (modules/winding/include/lagrange/winding/FastWindingNumber.h:24-108).
 *
 * Same members and semantics as the reference:
 *   - templated constructor from a triangle SurfaceMesh; vertices are cast to float and indices
 *     to int (FastWindingNumber.cpp:40-52); a mesh whose dimension is not 3 or that is not a
 *     triangle mesh throws with the reference's messages (FastWindingNumber.cpp:91-96);
 *   - default constructor, move construction/assignment, copy deleted (FastWindingNumber.h:45-82);
 *   - is_inside(pos): Omega/(4*pi) > 0.5 (FastWindingNumber.cpp:60-67);
 *   - solid_angle(pos): Omega in steradians (FastWindingNumber.cpp:69-76).
 * Added: batched host/device queries (the single-point members forward to a batch of one).
 * Querying a default-constructed or moved-from object throws (the reference dereferences a null
 * PIMPL there).
 *
 * The mesh constructor is duck-typed on Lagrange's SurfaceMesh API (get_dimension,
 * is_triangle_mesh, get_num_vertices, get_num_facets, get_position, get_facet_vertex), so
 * `lagrange::SurfaceMesh<S, I>` for all four (S, I) instantiations of the reference
 * (FastWindingNumber.cpp:115-118) is accepted without including Lagrange headers here.
 */
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "../fwn_gb300.h"

namespace lagrange_gb300 {

/// Error raised by the C++ surface (the reference raises lagrange::Error, a std::runtime_error).
class Error : public std::runtime_error
{
public:
    Error(const std::string& msg, fwn_status status = FWN_INTERNAL)
        : std::runtime_error(msg)
        , m_status(status)
    {}
    fwn_status status() const noexcept { return m_status; }

private:
    fwn_status m_status;
};

namespace detail {
inline void check(fwn_status s)
{
    if (s == FWN_OK) return;
    char buf[512];
    fwn_last_error(buf, sizeof(buf));
    throw Error(buf, s);
}
} // namespace detail

namespace winding {

class FastWindingNumber
{
public:
    /// Builds the acceleration structure on a triangle mesh (any SurfaceMesh-like type).
    template <
        typename MeshType,
        typename = decltype(std::declval<const MeshType&>().get_facet_vertex(0, 0))>
    explicit FastWindingNumber(const MeshType& mesh, const fwn_config* cfg = nullptr)
    {
        if (mesh.get_dimension() != 3) {
            throw Error("Fast winding number engine only supports 3D meshes", FWN_INVALID_ARG);
        }
        if (!mesh.is_triangle_mesh()) {
            throw Error(
                "Fast winding number engine only supports triangle meshes",
                FWN_INVALID_ARG);
        }
        const size_t nv = static_cast<size_t>(mesh.get_num_vertices());
        const size_t nf = static_cast<size_t>(mesh.get_num_facets());
        std::vector<float> V(3 * nv);
        std::vector<int32_t> F(3 * nf);
        for (size_t v = 0; v < nv; ++v) {
            auto p = mesh.get_position(static_cast<decltype(mesh.get_num_vertices())>(v));
            for (int k = 0; k < 3; ++k) V[3 * v + k] = static_cast<float>(p[k]);
        }
        for (size_t f = 0; f < nf; ++f) {
            for (int k = 0; k < 3; ++k) {
                using I = decltype(mesh.get_num_facets());
                F[3 * f + k] =
                    static_cast<int32_t>(mesh.get_facet_vertex(static_cast<I>(f), static_cast<I>(k)));
            }
        }
        init(V.data(), nv, F.data(), nf, cfg);
    }

    /// Builds from raw row-major arrays (vertices [nv x 3], triangles [nf x 3]).
    template <typename Scalar, typename Index>
    FastWindingNumber(
        const Scalar* vertices,
        size_t num_vertices,
        const Index* triangles,
        size_t num_triangles,
        const fwn_config* cfg = nullptr)
    {
        if (std::is_same<Scalar, float>::value && std::is_same<Index, int32_t>::value) {
            init(
                reinterpret_cast<const float*>(vertices),
                num_vertices,
                reinterpret_cast<const int32_t*>(triangles),
                num_triangles,
                cfg);
            return;
        }
        std::vector<float> V(3 * num_vertices);
        std::vector<int32_t> F(3 * num_triangles);
        for (size_t i = 0; i < V.size(); ++i) V[i] = static_cast<float>(vertices[i]);
        for (size_t i = 0; i < F.size(); ++i) F[i] = static_cast<int32_t>(triangles[i]);
        init(V.data(), num_vertices, F.data(), num_triangles, cfg);
    }

    FastWindingNumber() noexcept = default;

    ~FastWindingNumber()
    {
        if (m_handle) fwn_destroy(m_handle);
    }

    FastWindingNumber(FastWindingNumber&& other) noexcept
        : m_handle(other.m_handle)
    {
        other.m_handle = nullptr;
    }

    FastWindingNumber& operator=(FastWindingNumber&& other) noexcept
    {
        if (this != &other) {
            if (m_handle) fwn_destroy(m_handle);
            m_handle = other.m_handle;
            other.m_handle = nullptr;
        }
        return *this;
    }

    FastWindingNumber(const FastWindingNumber&) = delete;
    FastWindingNumber& operator=(const FastWindingNumber&) = delete;

    /// Omega(pos) / (4 pi) > 0.5 (strict: w == 0.5 is outside).
    bool is_inside(const std::array<float, 3>& pos) const
    {
        uint8_t r = 0;
        detail::check(fwn_query_host(m_handle, pos.data(), 1, nullptr, &r));
        return r != 0;
    }

    /// Solid angle at pos, in steradians (4 pi inside a closed outward-oriented surface).
    float solid_angle(const std::array<float, 3>& pos) const
    {
        float r = 0.f;
        detail::check(fwn_query_host(m_handle, pos.data(), 1, &r, nullptr));
        return r;
    }

    /// Batched solid angles of n points (host buffers, xyz row-major).
    void solid_angle(const float* xyz, size_t n, float* omega) const
    {
        detail::check(fwn_query_host(m_handle, xyz, static_cast<int64_t>(n), omega, nullptr));
    }

    /// Batched inside flags of n points (host buffers).
    void is_inside(const float* xyz, size_t n, uint8_t* inside) const
    {
        detail::check(fwn_query_host(m_handle, xyz, static_cast<int64_t>(n), nullptr, inside));
    }

    /// A serving loop's host point sets in one call (fwn_query_host_batches): batch b is
    /// xyz[b] (counts[b] points); omega / inside (either may be null, as may any entry) receive
    /// its results. Copies of one batch overlap the walk of its neighbour when the buffers are
    /// pinned.
    void query_batches(
        size_t num_batches,
        const float* const* xyz,
        const size_t* counts,
        float* const* omega,
        uint8_t* const* inside) const
    {
        std::vector<int64_t> n(counts, counts + num_batches);
        detail::check(fwn_query_host_batches(
            m_handle,
            static_cast<int64_t>(num_batches),
            xyz,
            n.data(),
            omega,
            inside));
    }

    /// Batched query on device buffers (asynchronous on `stream`, a cudaStream_t).
    void query_device(
        const float* d_xyz,
        size_t n,
        float* d_omega,
        uint8_t* d_inside,
        void* stream = nullptr) const
    {
        detail::check(fwn_query(m_handle, d_xyz, static_cast<int64_t>(n), d_omega, d_inside, stream));
    }

    fwn_info info() const
    {
        fwn_info i;
        detail::check(fwn_get_info(m_handle, &i));
        return i;
    }

    fwn_handle handle() const noexcept { return m_handle; }

private:
    void init(const float* V, size_t nv, const int32_t* F, size_t nf, const fwn_config* cfg)
    {
        detail::check(fwn_build(
            V,
            static_cast<int64_t>(nv),
            F,
            static_cast<int64_t>(nf),
            cfg,
            &m_handle));
    }

    fwn_handle m_handle = nullptr;
};

} // namespace winding
} // namespace lagrange_gb300
