// prgpu: command-line front end of the library.
//   prgpu --in points.ply --out mesh.ply [--depth 8] [--binary] [--relative TOL]
//         [--maxIter N] [--device K] [--weld] [--density] [--cascadic] [--refine]
//         [--stable-basis] [--learned CHECKPOINT] [--samples-per-node K] [--stats]
// The reference takes its input/output paths and maxDepth at compile time
// (main.cu:69,3251-3252); the flag names follow the Kazhdan-style "--name value"
// convention of its CmdLineParser (CmdLineParser.cu:205-240).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/prgpu.h"

static void usage() {
    fprintf(stderr,
            "usage: prgpu --in <points.ply|.bnpts|ascii> --out <mesh.ply> [--depth D] [--binary]\n"
            "             [--relative TOL] [--maxIter N] [--device K] [--weld] [--density] [--cascadic]\n"
            "             [--refine] [--stable-basis] [--learned CHECKPOINT] [--samples-per-node K] [--stats]\n"
            "  --samples-per-node K: the depth is the finest (at most --depth) whose occupied nodes\n"
            "                        hold K points each on average\n");
}

int main(int argc, char** argv) {
    const char* in = nullptr;
    const char* out = nullptr;
    prgpu_params p;
    prgpu_params_default(&p);
    int binary = 0, stats = 0;
    const char* learned = nullptr;
    double samples_per_node = 0.0;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto next = [&]() -> const char* {
            if (i + 1 >= argc) { usage(); exit(2); }
            return argv[++i];
        };
        if (a == "--in") in = next();
        else if (a == "--out") out = next();
        else if (a == "--depth") p.depth = atoi(next());
        else if (a == "--binary") binary = 1;
        else if (a == "--weld") p.weld = 1;
        else if (a == "--density") p.density_weights = 1;
        else if (a == "--cascadic") p.cascadic = 1;
        else if (a == "--relative") { p.solve_mode = PRGPU_SOLVE_RELATIVE; p.cg_tol = atof(next()); }
        else if (a == "--maxIter") p.cg_max_iter = atoi(next());
        else if (a == "--device") p.device = atoi(next());
        else if (a == "--refine") p.refine = 1;
        else if (a == "--stable-basis") p.stable_basis = 1;
        else if (a == "--learned") { learned = next(); p.learned = 1; }
        else if (a == "--samples-per-node") samples_per_node = atof(next());
        else if (a == "--stats") stats = 1;
        else { usage(); return 2; }
    }
    if (!in || !out) { usage(); return 2; }
    auto t0 = std::chrono::steady_clock::now();
    int64_t n = 0;
    const float *xyz = nullptr, *nrm = nullptr;
    int rc = prgpu_read_points(in, &n, &xyz, &nrm);
    if (rc) { fprintf(stderr, "read failed (%d): %s\n", rc, prgpu_last_error()); return 1; }
    if (samples_per_node > 0.0) {
        int32_t d = 0;
        if ((rc = prgpu_choose_depth(xyz, nrm, n, p.depth, samples_per_node, p.device, &d, nullptr))) {
            fprintf(stderr, "depth choice failed (%d): %s\n", rc, prgpu_last_error());
            return 1;
        }
        fprintf(stderr, "depth %d (at most %d, %.1f points per node)\n", d, p.depth, samples_per_node);
        p.depth = d;
    }
    void* ctx = nullptr;
    if ((rc = prgpu_create(&p, &ctx))) { fprintf(stderr, "create failed (%d): %s\n", rc, prgpu_last_error()); return 1; }
    if (learned && (rc = prgpu_load_preconditioner(ctx, learned))) {
        fprintf(stderr, "preconditioner failed (%d): %s\n", rc, prgpu_last_error());
        prgpu_destroy(ctx);
        return 1;
    }
    prgpu_mesh m;
    rc = prgpu_reconstruct(ctx, xyz, nrm, n, &m);
    if (rc) { fprintf(stderr, "reconstruction failed (%d): %s\n", rc, prgpu_last_error()); prgpu_destroy(ctx); return 1; }
    rc = prgpu_write_mesh_ply(out, &m, binary);
    if (rc) { fprintf(stderr, "write failed (%d): %s\n", rc, prgpu_last_error()); prgpu_destroy(ctx); return 1; }
    auto t1 = std::chrono::steady_clock::now();
    if (stats) {
        char buf[4096];
        prgpu_stats_json(ctx, buf, sizeof buf);
        printf("%s\n", buf);
    }
    fprintf(stderr, "%lld points -> %lld vertices, %lld triangles in %.3f s\n", (long long)n, (long long)m.n_vertices,
            (long long)m.n_triangles, std::chrono::duration<double>(t1 - t0).count());
    prgpu_destroy(ctx);
    return 0;
}
