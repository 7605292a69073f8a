// A C++ caller of libprgpu.so through include/prgpu.h only: one reconstruction,
// a batch of two clouds, the octree's OctNode fields, and the error path.
// Prints "ok" and returns 0 when every check holds.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include "prgpu.h"

#define CHECK(c)                                                              \
    do {                                                                      \
        if (!(c)) {                                                           \
            std::fprintf(stderr, "check failed: %s (%s)\n", #c, prgpu_last_error()); \
            return 1;                                                         \
        }                                                                     \
    } while (0)

// points on a sphere of radius r around (0.5, 0.5, 0.5), outward normals (a Fibonacci lattice)
static void sphere(int n, float r, std::vector<float>& xyz, std::vector<float>& nrm) {
    const double ga = 3.14159265358979323846 * (3.0 - std::sqrt(5.0));
    for (int i = 0; i < n; ++i) {
        const double z = 1.0 - 2.0 * (i + 0.5) / n, rho = std::sqrt(1.0 - z * z), t = ga * i;
        const double d[3] = {rho * std::cos(t), rho * std::sin(t), z};
        for (int a = 0; a < 3; ++a) {
            xyz.push_back((float)(0.5 + r * d[a]));
            nrm.push_back((float)d[a]);
        }
    }
}

int main() {
    prgpu_params p;
    CHECK(prgpu_params_default(&p) == PRGPU_OK);
    p.depth = 6;
    void* ctx = nullptr;
    CHECK(prgpu_create(&p, &ctx) == PRGPU_OK);

    std::vector<float> xyz, nrm;
    sphere(4000, 0.35f, xyz, nrm);
    prgpu_mesh m;
    CHECK(prgpu_reconstruct(ctx, xyz.data(), nrm.data(), 4000, &m) == PRGPU_OK);
    CHECK(m.n_vertices > 0 && m.n_triangles > 0);
    for (int64_t v = 0; v < m.n_vertices; ++v) {
        const float dx = m.vertices[3 * v] - 0.5f, dy = m.vertices[3 * v + 1] - 0.5f, dz = m.vertices[3 * v + 2] - 0.5f;
        CHECK(std::fabs(std::sqrt(dx * dx + dy * dy + dz * dz) - 0.35f) < 0.03f);
    }
    for (int64_t t = 0; t < 3 * m.n_triangles; ++t) CHECK(m.triangles[t] >= 0 && m.triangles[t] < m.n_vertices);
    const int64_t ntri = m.n_triangles;

    // the octree's node fields, sized by a first call
    prgpu_node_arrays na;
    std::memset(&na, 0, sizeof na);
    CHECK(prgpu_get_node_arrays(ctx, &na) == PRGPU_OK);
    CHECK(na.n_nodes > 0 && na.max_depth == 6);
    std::vector<int64_t> base(na.max_depth + 2);
    std::vector<int32_t> parent(na.n_nodes), children(8 * na.n_nodes);
    na.base = base.data();
    na.parent = parent.data();
    na.children = children.data();
    CHECK(prgpu_get_node_arrays(ctx, &na) == PRGPU_OK);
    CHECK(base[0] == 0 && base[na.max_depth + 1] == na.n_nodes && parent[0] == -1);
    for (int64_t i = 1; i < na.n_nodes; ++i) CHECK(children[8 * parent[i] + (i - 1) % 8] == i);

    // two clouds in one call: the first is the cloud above
    std::vector<float> xyz2 = xyz, nrm2 = nrm;
    sphere(2500, 0.25f, xyz2, nrm2);
    const int64_t offsets[3] = {0, 4000, 6500};
    const int32_t depths[2] = {6, 5};
    prgpu_mesh out[2];
    CHECK(prgpu_reconstruct_batch(ctx, xyz2.data(), nrm2.data(), offsets, depths, 2, out) == PRGPU_OK);
    CHECK(out[0].n_triangles == ntri && out[1].n_triangles > 0);
    CHECK(prgpu_mesh_free(&out[0]) == PRGPU_OK && out[0].vertices == nullptr);
    CHECK(prgpu_mesh_free(&out[1]) == PRGPU_OK);

    // errors are statuses with a message, and the context stays usable
    const int32_t bad[2] = {6, 1};
    CHECK(prgpu_reconstruct_batch(ctx, xyz2.data(), nrm2.data(), offsets, bad, 2, out) == PRGPU_ERR_ARG);
    CHECK(std::strstr(prgpu_last_error(), "cloud 1") != nullptr);
    CHECK(prgpu_reconstruct(ctx, xyz.data(), nrm.data(), 4000, &m) == PRGPU_OK && m.n_triangles == ntri);

    CHECK(prgpu_destroy(ctx) == PRGPU_OK);
    std::printf("ok\n");
    return 0;
}
