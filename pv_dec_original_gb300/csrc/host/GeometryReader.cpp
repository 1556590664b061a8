#include "GeometryReader.h"

#include <iostream>

#include "lbm_gb300.h"

std::vector<Triangle> Reader::readSTLASCII(const std::string& filename) {
    std::vector<Triangle> out;
    int64_t n = 0;
    if (lbm_read_stl_ascii(filename.c_str(), nullptr, &n) != LBM_OK) {
        std::cerr << "Error: cannot open file " << filename << std::endl;
        return out;
    }
    std::vector<double> rows(12 * (size_t)n);
    if (n > 0 && lbm_read_stl_ascii(filename.c_str(), rows.data(), &n) != LBM_OK) return out;
    out.resize((size_t)n);
    for (int64_t t = 0; t < n; ++t) {
        const double* r = rows.data() + 12 * t;
        out[t] = Triangle{r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7], r[8], r[9], r[10], r[11]};
    }
    return out;
}
