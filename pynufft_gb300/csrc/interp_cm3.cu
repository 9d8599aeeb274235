// Coil-major gridding instantiations for 3D plans.
#include "interp_cm_launch.cuh"

namespace nufft {

int y2k_cm_dim3(int jm, bool det, const Geom& g, const float2* y, float2* grid,
                 unsigned long long* igrid, const double* dscal, cudaStream_t s) {
    return y2k_cm_jm<3>(jm, det, g, y, grid, igrid, dscal, s);
}

}  // namespace nufft
