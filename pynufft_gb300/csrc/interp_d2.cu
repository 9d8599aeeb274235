// Interpolation kernel instantiations for 2D plans.
#include "interp_launch.cuh"

namespace nufft {

void k2y_dim2(int jm, const Geom& g, const float2* grid, float2* y, cudaStream_t s) {
    k2y_jm<2>(jm, g, grid, y, s);
}

int y2k_dim2(int jm, bool det, const Geom& g, const float2* y, float2* grid,
              unsigned long long* igrid, const double* dscal, cudaStream_t s) {
    return det ? y2k_jm<2, true>(jm, g, y, grid, igrid, dscal, s)
               : y2k_jm<2, false>(jm, g, y, grid, igrid, dscal, s);
}

}  // namespace nufft
