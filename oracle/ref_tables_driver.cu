// Golden-vector driver (test infrastructure): links the reference's own
// host-side basis code (FunctionData.inl, PPolynomial.inl, Polynomial.inl, read
// from the reference tree at build time, never copied) and dumps what it
// computes for one maxDepth:
//   <out>.tables : res*res doubles each of dotTable, dDotTable, d2DotTable
//   stdout       : the normalised base function pieces, hex floats
// Built by oracle/ref_build.sh into oracle/_ref/.
#include <cstdio>
#include <cstdlib>
#include "PPolynomial.cuh"
#include "FunctionData.cuh"

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: ref_tables <maxDepth> <out.tables>\n"); return 2; }
    const int D = atoi(argv[1]);
    PPolynomial<2> F = PPolynomial<2>::GaussianApproximation();
    FunctionData<2, double> fd;
    fd.set(D, F, 0, 0);   // normalize = 0, useDotRatios = 0 as in main.cu:3308-3310
    fd.setDotTables(fd.DOT_FLAG | fd.D_DOT_FLAG | fd.D2_DOT_FLAG);
    FILE* f = fopen(argv[2], "wb");
    if (!f) return 1;
    const size_t n = (size_t)fd.res * fd.res;
    fwrite(fd.dotTable, sizeof(double), n, f);
    fwrite(fd.dDotTable, sizeof(double), n, f);
    fwrite(fd.d2DotTable, sizeof(double), n, f);
    fclose(f);
    for (size_t i = 0; i < fd.baseFunction.polyCount; ++i) {
        printf("%a", fd.baseFunction.polys[i].start);
        for (int k = 0; k < 3; ++k) printf(" %a", fd.baseFunction.polys[i].p.coefficients[k]);
        printf("\n");
    }
    return 0;
}
