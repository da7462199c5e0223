// Exercises the C++ surface lagrange_gb300::winding::FastWindingNumber the way the reference's
// callers use lagrange::winding::FastWindingNumber (construct from a SurfaceMesh, then
// is_inside / solid_angle per point; modules/winding/examples/sample_points_in_mesh.cpp:66-76,
// modules/volume/src/mesh_to_volume.cpp:160-183), for all four (Scalar, Index) instantiations
// of the reference (FastWindingNumber.cpp:115-118). Needs a GPU; run by tests/test_cpp_class.py.
#include <lagrange_gb300/FastWindingNumber.h>

#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// Stand-in for lagrange::SurfaceMesh<Scalar, Index> with the accessors the engine reads.
template <typename Scalar, typename Index>
struct MiniMesh
{
    Index dim = 3;
    bool tri = true;
    std::vector<Scalar> V;
    std::vector<Index> F;
    Index get_dimension() const { return dim; }
    bool is_triangle_mesh() const { return tri; }
    Index get_num_vertices() const { return static_cast<Index>(V.size() / 3); }
    Index get_num_facets() const { return static_cast<Index>(F.size() / 3); }
    const Scalar* get_position(Index v) const { return &V[3 * v]; }
    Index get_facet_vertex(Index f, Index lv) const { return F[3 * f + lv]; }
};

template <typename Scalar, typename Index>
MiniMesh<Scalar, Index> octahedron(Scalar s)
{
    MiniMesh<Scalar, Index> m;
    m.V = {s, 0, 0, -s, 0, 0, 0, s, 0, 0, -s, 0, 0, 0, s, 0, 0, -s};
    m.F = {0, 2, 4, 2, 1, 4, 1, 3, 4, 3, 0, 4, 2, 0, 5, 1, 2, 5, 3, 1, 5, 0, 3, 5};
    return m;
}

int g_fail = 0;
#define CHECK(cond)                                                                  \
    do {                                                                             \
        if (!(cond)) {                                                               \
            std::fprintf(stderr, "CHECK failed %s:%d: %s\n", __FILE__, __LINE__, #cond); \
            ++g_fail;                                                                \
        }                                                                            \
    } while (0)

template <typename Fn>
bool throws_with(Fn&& fn, const char* msg, fwn_status st)
{
    try {
        fn();
    } catch (const lagrange_gb300::Error& e) {
        const bool ok_msg = msg == nullptr || std::string(e.what()).find(msg) != std::string::npos;
        return ok_msg && e.status() == st;
    }
    return false;
}

template <typename Scalar, typename Index>
void run_instantiation()
{
    using lagrange_gb300::winding::FastWindingNumber;
    const double four_pi = 4.0 * 3.14159265358979323846;
    auto mesh = octahedron<Scalar, Index>(Scalar(1));
    FastWindingNumber engine(mesh);
    CHECK(engine.is_inside({0.f, 0.f, 0.f}));
    CHECK(engine.is_inside({0.1f, 0.2f, -0.1f}));
    CHECK(!engine.is_inside({2.f, 0.f, 0.f}));
    CHECK(!engine.is_inside({0.5f, 0.5f, 0.5f}));  // outside the face x+y+z=1
    CHECK(std::fabs(engine.solid_angle({0.f, 0.f, 0.f}) - four_pi) < 1e-5);
    CHECK(std::fabs(engine.solid_angle({3.f, -2.f, 1.f})) < 1e-5);

    // batched == single-point
    const std::vector<float> pts = {0.f, 0.f, 0.f, 0.3f, 0.3f, 0.3f, 0.4f, 0.4f, 0.4f, 1.f, 1.f, 1.f};
    std::vector<float> om(4);
    std::vector<uint8_t> in(4);
    engine.solid_angle(pts.data(), 4, om.data());
    engine.is_inside(pts.data(), 4, in.data());
    for (int i = 0; i < 4; ++i) {
        std::array<float, 3> p = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        CHECK(om[i] == engine.solid_angle(p));
        CHECK((in[i] != 0) == engine.is_inside(p));
    }
    CHECK(in[0] == 1 && in[1] == 1 && in[2] == 0 && in[3] == 0);

    // several host batches in one call == one call each
    const float* bx[3] = {pts.data(), pts.data() + 3, pts.data()};
    const size_t bn[3] = {4, 2, 0};
    std::vector<float> o0(4), o1(2);
    std::vector<uint8_t> i0(4), i1(2);
    float* bo[3] = {o0.data(), o1.data(), nullptr};
    uint8_t* bi[3] = {i0.data(), i1.data(), nullptr};
    engine.query_batches(3, bx, bn, bo, bi);
    for (int i = 0; i < 4; ++i) CHECK(o0[i] == om[i] && i0[i] == in[i]);
    for (int i = 0; i < 2; ++i) CHECK(o1[i] == om[i + 1] && i1[i] == in[i + 1]);

    // move semantics: moved-from objects are empty and throw NOT_BUILT when queried
    FastWindingNumber moved(std::move(engine));
    CHECK(moved.is_inside({0.f, 0.f, 0.f}));
    CHECK(throws_with([&] { (void)engine.is_inside({0.f, 0.f, 0.f}); }, nullptr, FWN_NOT_BUILT));
    FastWindingNumber assigned;
    assigned = std::move(moved);
    CHECK(assigned.is_inside({0.f, 0.f, 0.f}));
    CHECK(throws_with([&] { (void)moved.solid_angle({0.f, 0.f, 0.f}); }, nullptr, FWN_NOT_BUILT));
}

} // namespace

int main()
{
    run_instantiation<float, uint32_t>();
    run_instantiation<double, uint32_t>();
    run_instantiation<float, uint64_t>();
    run_instantiation<double, uint64_t>();

    using lagrange_gb300::winding::FastWindingNumber;
    // reference ctor checks (FastWindingNumber.cpp:91-96), same messages
    auto m2 = octahedron<float, uint32_t>(1.f);
    m2.dim = 2;
    CHECK(throws_with([&] { FastWindingNumber e(m2); }, "only supports 3D meshes", FWN_INVALID_ARG));
    auto mq = octahedron<float, uint32_t>(1.f);
    mq.tri = false;
    CHECK(throws_with(
        [&] { FastWindingNumber e(mq); },
        "only supports triangle meshes",
        FWN_INVALID_ARG));
    // out-of-range index -> INVALID_ARG
    auto mb = octahedron<float, uint32_t>(1.f);
    mb.F[5] = 99;
    CHECK(throws_with([&] { FastWindingNumber e(mb); }, "out of range", FWN_INVALID_ARG));
    // default-constructed engine
    FastWindingNumber empty;
    CHECK(throws_with([&] { (void)empty.is_inside({0.f, 0.f, 0.f}); }, nullptr, FWN_NOT_BUILT));
    // empty mesh: solid angle 0 everywhere
    MiniMesh<float, uint32_t> none;
    FastWindingNumber e0(none);
    CHECK(e0.solid_angle({0.f, 0.f, 0.f}) == 0.f);
    CHECK(!e0.is_inside({0.f, 0.f, 0.f}));
    // raw-array constructor with double / int64 input
    const double Vd[] = {0, 0, 0, 1, 0, 0, 0, 1, 0};
    const int64_t Fd[] = {0, 1, 2};
    FastWindingNumber tri(Vd, 3, Fd, 1);
    // octant triangle seen from (0,0,0)... query below the triangle plane: solid angle of the
    // right triangle from (0,0,-1): 2*atan2(det, D) computed on the host for comparison
    const float om = tri.solid_angle({0.25f, 0.25f, -1.f});
    CHECK(om > 0.f && om < 2.f * 3.1415927f);

    if (g_fail) {
        std::fprintf(stderr, "%d checks failed\n", g_fail);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
