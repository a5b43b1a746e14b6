// Reads a matrixIO .bin file with the header-only readers of glsu_io.hpp,
// writes it back, and round-trips a complex .fp text file.
// usage: test_io <in.bin> <out.bin> <tmp.fp>; prints "rows cols sum".
#include <cstdio>
#include <fstream>
#include <vector>

#include "glsu_io.hpp"

int main(int argc, char **argv)
{
    if (argc < 4) return 2;
    int rows = 0, cols = 0;
    std::vector<float> m;
    if (WFT_FPA::Utils::ReadMatrixFromDisk<float>(argv[1], &rows, &cols, m) != 0) return 3;
    if (WFT_FPA::Utils::WriteMatrixToDisk<float>(argv[2], rows, cols, m.data()) != 0) return 4;
    double sum = 0;
    for (float v : m) sum += v;
    std::vector<cuFloatComplex> f(6);
    for (int i = 0; i < 6; i++) f[i] = make_cuFloatComplex(0.25f * i, -1.5f + i);
    {
        std::ofstream o(argv[3]);
        WFT_FPA::Utils::cufftComplexMatWrite2D(o, f.data(), 2, 3);
    }
    std::ifstream in(argv[3]);
    std::vector<cuFloatComplex> g;
    int r2 = 0, c2 = 0;
    if (!WFT_FPA::Utils::cufftComplexMatRead2D(in, g, r2, c2) || r2 != 2 || c2 != 3) return 5;
    for (int i = 0; i < 6; i++)
        if (g[i].x != f[i].x || g[i].y != f[i].y) return 6;
    std::printf("%d %d %.9g\n", rows, cols, sum);
    return 0;
}
