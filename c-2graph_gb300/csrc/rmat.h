// R-MAT graphs in the reference's origin/ layout (utils/convert2binary.cpp:98-129),
// built on the host (rmat.cpp) or on the device (rmat_gpu.cu) from the same draws
// (rmat_draw.h), and written by one writer.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

namespace c2g {

struct RmatGraph {
    int64_t V = 0;
    std::vector<int32_t> row, col, wgt;
    std::vector<float> fw;
};

int rmat_build(int scale, int edge_factor, uint64_t seed, int32_t wmin, int32_t wmax, double a, double b, double c,
               RmatGraph& g);
int rmat_build_gpu(int scale, int edge_factor, uint64_t seed, int32_t wmin, int32_t wmax, double a, double b,
                   double c, int device, RmatGraph& g);
int write_origin(const std::string& dir, const RmatGraph& g);

}  // namespace c2g
