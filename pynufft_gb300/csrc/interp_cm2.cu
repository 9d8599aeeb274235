// Coil-major interpolation / gridding instantiations for 2D plans.
#include "interp_cm_launch.cuh"

namespace nufft {

int k2y_cm_dim2(int jm, const Geom& g, const float2* grid, float2* y, cudaStream_t s) {
    return k2y_cm_jm<2>(jm, g, grid, y, s);
}

int y2k_cm_dim2(int jm, bool det, const Geom& g, const float2* y, float2* grid,
                 unsigned long long* igrid, const double* dscal, cudaStream_t s) {
    return y2k_cm_jm<2>(jm, det, g, y, grid, igrid, dscal, s);
}

}  // namespace nufft
