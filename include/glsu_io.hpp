// glsu_io.hpp -- the reference's matrix file formats, header-only.
//
//   WFT_FPA::Utils::ReadMatrixFromDisk / WriteMatrixToDisk
//       the matrixIO binary format (Utils/matrixIO.h:17-55): int32 rows,
//       int32 cols, rows*cols row-major elements.
//   WFT_FPA::Utils::cufftComplexMatRead2D / cufftComplexMatWrite2D
//       the ".fp" text format (Utils/Utils.cpp:80-123): "rows,cols", then
//       one "re,im" line per element.
// Return values follow the reference: 0 (read/write) or true (text read)
// on success.  Matrices are returned in std::vector (the reference's
// malloc'd T** variants leave ownership to the caller).
#pragma once

#include <cuComplex.h>

#include <cstdint>
#include <cstdio>
#include <istream>
#include <ostream>
#include <sstream>
#include <string>
#include <vector>

namespace WFT_FPA {
namespace Utils {

template <class T> int ReadMatrixFromDisk(const char *filename, int *rows, int *cols, std::vector<T> &matrix)
{
    FILE *f = std::fopen(filename, "rb");
    if (!f) return 1;
    int32_t hdr[2];
    int rc = 1;
    if (std::fread(hdr, sizeof(int32_t), 2, f) == 2 && hdr[0] >= 0 && hdr[1] >= 0) {
        *rows = hdr[0];
        *cols = hdr[1];
        matrix.resize((size_t)hdr[0] * hdr[1]);
        if (std::fread(matrix.data(), sizeof(T), matrix.size(), f) == matrix.size()) rc = 0;
    }
    std::fclose(f);
    return rc;
}

template <class T> int WriteMatrixToDisk(const char *filename, int rows, int cols, const T *matrix)
{
    FILE *f = std::fopen(filename, "wb");
    if (!f) return 1;
    const int32_t hdr[2] = {rows, cols};
    int rc = 1;
    if (std::fwrite(hdr, sizeof(int32_t), 2, f) == 2 &&
        std::fwrite(matrix, sizeof(T), (size_t)rows * cols, f) == (size_t)rows * cols)
        rc = 0;
    std::fclose(f);
    return rc;
}

namespace detail {
template <class C, class R> bool read_text(std::istream &in, std::vector<C> &f, int &rows, int &cols)
{
    std::string line;
    if (!std::getline(in, line)) return false;
    {
        std::stringstream ss(line);
        std::string a, b;
        if (!std::getline(ss, a, ',') || !std::getline(ss, b, ',')) return false;
        rows = std::stoi(a);
        cols = std::stoi(b);
    }
    f.clear();
    f.reserve((size_t)rows * cols);
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        std::stringstream ss(line);
        std::string a, b;
        if (!std::getline(ss, a, ',') || !std::getline(ss, b, ',')) return false;
        C v;
        v.x = (R)std::stod(a);
        v.y = (R)std::stod(b);
        f.push_back(v);
    }
    return f.size() == (size_t)rows * cols;
}
}  // namespace detail

inline bool cufftComplexMatRead2D(std::istream &in, std::vector<cuFloatComplex> &f, int &rows, int &cols)
{
    return detail::read_text<cuFloatComplex, float>(in, f, rows, cols);
}
inline bool cufftComplexMatRead2D(std::istream &in, std::vector<cuDoubleComplex> &f, int &rows, int &cols)
{
    return detail::read_text<cuDoubleComplex, double>(in, f, rows, cols);
}

template <class C> void cufftComplexMatWrite2D(std::ostream &out, const C *f, const int rows, const int cols)
{
    out << rows << "," << cols << "\n";
    out.precision(17);
    for (size_t i = 0; i < (size_t)rows * cols; i++) out << f[i].x << "," << f[i].y << "\n";
}

}  // namespace Utils
}  // namespace WFT_FPA
