// Driver of the reference's own CUDA build (test infrastructure and GPU
// baseline; never part of the library).  Linked with the reference's main.cu,
// CmdLineParser.cu, Geometry.cu, plyfile.cu and Factor.cu, compiled unchanged
// by oracle/ref_cuda.sh (main() renamed to prgpu_reference_main at compile time).
//
//   ref_cuda octree <in.ply> <out.bin>
//       pipelineBuildNodeArray (main.cu:511-841) on the file, then its outputs
//       to out.bin (little endian):
//         char[8] "PRREFOCT", int32 version (1), int32 maxDepth, int32 points,
//         int32 nodes, int32 NodeArrayCount[maxDepth+1],
//         int32 BaseAddressArray[maxDepth+1], float center[3], float scale,
//         float points[3*points] (sorted, normalised), float normals[3*points],
//         int32 PointToNodeArrayD[points],
//         int32 per node: key, pidx, pnum, parent, children[8], neighs[27], didx,
//         dnum (OctNode.cuh:8-19, the first 41 fields)
//   ref_cuda pipeline
//       the stock main() (main.cu:3247-4573): reads bunny.points.ply and writes
//       bunny.ply in $PRGPU_REF_IO_DIR (oracle/ref_shim/ref_io.cpp maps its fixed
//       /home/davidxu/ paths there); the CUDA context is created first, then the
//       wall time of main() is printed as "prgpu_ref_wall_s <seconds>".
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "Geometry.cuh"
#include "OctNode.cuh"

// defined in the reference's main.cu (maxDepth 8, main.cu:69)
void pipelineBuildNodeArray(char* fileName, Point3D<float>& center, float& scale, int& count, int& NodeArray_sz,
                            int NodeArrayCount_h[], int BaseAddressArray_h[], Point3D<float>*& samplePoints_d,
                            Point3D<float>*& sampleNormals_d, int*& PointToNodeArrayD, OctNode*& NodeArray);
int prgpu_reference_main();

static const int REF_MAX_DEPTH = 8;

static int check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
        exit(3);
    }
    return 0;
}

static int dump_octree(const char* in, const char* out) {
    std::vector<char> path(in, in + strlen(in) + 1);
    Point3D<float> center;
    float scale = 0.f;
    int count = 0, nodes = 0;
    int counts[REF_MAX_DEPTH + 1], base[REF_MAX_DEPTH + 1];
    Point3D<float>*pts = nullptr, *nrm = nullptr;
    int* p2n = nullptr;
    OctNode* na = nullptr;
    pipelineBuildNodeArray(path.data(), center, scale, count, nodes, counts, base, pts, nrm, p2n, na);
    check(cudaDeviceSynchronize(), "pipelineBuildNodeArray");
    std::vector<float> hp(3 * (size_t)count), hn(3 * (size_t)count);
    std::vector<int> hp2n(count);
    std::vector<OctNode> hna(nodes);
    check(cudaMemcpy(hp.data(), pts, hp.size() * 4, cudaMemcpyDeviceToHost), "points");
    check(cudaMemcpy(hn.data(), nrm, hn.size() * 4, cudaMemcpyDeviceToHost), "normals");
    check(cudaMemcpy(hp2n.data(), p2n, hp2n.size() * 4, cudaMemcpyDeviceToHost), "point to node");
    check(cudaMemcpy(hna.data(), na, (size_t)nodes * sizeof(OctNode), cudaMemcpyDeviceToHost), "node array");
    FILE* f = fopen(out, "wb");
    if (!f) return 1;
    const int version = 1, D = REF_MAX_DEPTH;
    fwrite("PRREFOCT", 1, 8, f);
    fwrite(&version, 4, 1, f);
    fwrite(&D, 4, 1, f);
    fwrite(&count, 4, 1, f);
    fwrite(&nodes, 4, 1, f);
    fwrite(counts, 4, D + 1, f);
    fwrite(base, 4, D + 1, f);
    fwrite(center.coords, 4, 3, f);
    fwrite(&scale, 4, 1, f);
    fwrite(hp.data(), 4, hp.size(), f);
    fwrite(hn.data(), 4, hn.size(), f);
    fwrite(hp2n.data(), 4, hp2n.size(), f);
    std::vector<int> rec(41);
    for (int i = 0; i < nodes; ++i) {
        const OctNode& n = hna[i];
        rec[0] = n.key;
        rec[1] = n.pidx;
        rec[2] = n.pnum;
        rec[3] = n.parent;
        for (int k = 0; k < 8; ++k) rec[4 + k] = n.children[k];
        for (int k = 0; k < 27; ++k) rec[12 + k] = n.neighs[k];
        rec[39] = n.didx;
        rec[40] = n.dnum;
        fwrite(rec.data(), 4, 41, f);
    }
    fclose(f);
    printf("octree: %d points, %d nodes\n", count, nodes);
    return 0;
}

int main(int argc, char** argv) {
    if (argc >= 4 && !strcmp(argv[1], "octree")) return dump_octree(argv[2], argv[3]);
    if (argc >= 2 && !strcmp(argv[1], "pipeline")) {
        if (!getenv("PRGPU_REF_IO_DIR")) {
            fprintf(stderr, "PRGPU_REF_IO_DIR is not set\n");
            return 2;
        }
        setvbuf(stdout, nullptr, _IONBF, 0);   // the stage lines survive an abort
        check(cudaFree(0), "context");
        const auto t0 = std::chrono::steady_clock::now();
        prgpu_reference_main();
        check(cudaDeviceSynchronize(), "reference main");
        const auto t1 = std::chrono::steady_clock::now();
        printf("prgpu_ref_wall_s %.6f\n", std::chrono::duration<double>(t1 - t0).count());
        fflush(stdout);
        return 0;
    }
    fprintf(stderr, "usage: ref_cuda octree <in.ply> <out.bin> | ref_cuda pipeline\n");
    return 2;
}
