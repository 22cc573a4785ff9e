// interp.h -- the natural-neighbour interpolator shared by the host queries
// (interp.cpp) and the device queries (interp_gpu.cu).
#pragma once
#include <cstdint>
#include <mutex>
#include <vector>

namespace fl {
struct InterpDevice;                   // device copy of the triangulation (interp_gpu.cu)
void interp_device_release(InterpDevice* d);
}  // namespace fl

struct fl_interpolator {
    uint32_t n = 0;
    std::vector<double> X, Y;
    std::vector<uint32_t> tri;
    std::vector<int64_t> half;
    std::vector<double> ccx, ccy;      // circumcentre of every triangle
    std::vector<int64_t> vedge;        // a half-edge starting at each vertex (-1: none)
    // point-location grid: walks start at the triangle holding the cell's centre (or,
    // for a centre beyond the hull, the hull triangle the walk to it stopped at)
    double gx0 = 0, gy0 = 0, gsx = 1, gsy = 1;
    uint32_t gw = 1, gh = 1;
    std::vector<uint32_t> gtri;
    // device queries: the triangulation uploaded on first use, one call at a time
    std::mutex device_mu;
    fl::InterpDevice* dev = nullptr;
};
