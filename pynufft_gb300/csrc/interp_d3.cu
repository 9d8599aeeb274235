// Interpolation kernel instantiations for 3D plans.
#include "interp_launch.cuh"

namespace nufft {

void k2y_dim3(int jm, const Geom& g, const float2* grid, float2* y, cudaStream_t s) {
    k2y_jm<3>(jm, g, grid, y, s);
}

int y2k_dim3(int jm, bool det, const Geom& g, const float2* y, float2* grid,
              unsigned long long* igrid, const double* dscal, cudaStream_t s) {
    return det ? y2k_jm<3, true>(jm, g, y, grid, igrid, dscal, s)
               : y2k_jm<3, false>(jm, g, y, grid, igrid, dscal, s);
}

}  // namespace nufft
