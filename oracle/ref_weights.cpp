// Test-oracle driver: evaluates the reference's own computeNodalWeight2D
// (mathTools/math.cpp:229-312, with solvec and newtonSolve2D) on a batch of
// (cell, point) queries.  Test infrastructure only.
//
// usage: ref_weights IN.bin OUT.bin
//   IN:  int32 n, then n records {int32 nvert, double xv[4][2], double xp[2]}
//   OUT: n records of double frac[4] (unused entries 0)
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

void computeNodalWeight2D(double xv[8][3], double* xp, double* frac, int nvert);

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s IN OUT\n", argv[0]);
        return 2;
    }
    FILE* fi = fopen(argv[1], "rb");
    if (!fi) return 3;
    int n = 0;
    if (fread(&n, 4, 1, fi) != 1) return 3;
    std::vector<double> out(4 * (size_t)n, 0.0);
    for (int q = 0; q < n; q++) {
        int nv;
        double v[8], p[2];
        if (fread(&nv, 4, 1, fi) != 1 || fread(v, 8, 8, fi) != 8 || fread(p, 8, 2, fi) != 2) return 3;
        double xv[8][3] = {{0}};
        for (int i = 0; i < 4; i++) {
            xv[i][0] = v[2 * i];
            xv[i][1] = v[2 * i + 1];
        }
        double frac[8] = {0};
        try {
            computeNodalWeight2D(xv, p, frac, nv);
        } catch (const std::exception&) {
            frac[0] = frac[1] = frac[2] = frac[3] = -1e300;  // degenerate triangle
        }
        for (int i = 0; i < 4; i++) out[4 * (size_t)q + i] = frac[i];
    }
    fclose(fi);
    FILE* fo = fopen(argv[2], "wb");
    if (!fo) return 4;
    fwrite(out.data(), 8, out.size(), fo);
    fclose(fo);
    return 0;
}
