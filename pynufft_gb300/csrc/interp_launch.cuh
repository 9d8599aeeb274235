// Launch templates for the interpolation kernels; instantiated per
// dimension in interp_d1.cu, interp_d2.cu and interp_d3.cu so the three
// translation units compile in parallel.
#pragma once
#include "interp.cuh"

#include <algorithm>
#include <string>

namespace nufft {

inline int pick_team(int B) {
    if (B >= 32) return 32;
    if (B >= 8) return 8;
    return 1;
}

template <int DIM, int JM, int G>
static void k2y_launch(const Geom& g, const float2* grid, float2* y, cudaStream_t s) {
    const int threads = 256;
    const int64_t nthr = g.M * G;
    const int64_t blocks = (nthr + threads - 1) / threads;
    k2y_kernel<DIM, JM, G><<<(unsigned)blocks, threads, 0, s>>>(g, grid, y);
}

template <int DIM, int JM>
static void k2y_team(const Geom& g, const float2* grid, float2* y, cudaStream_t s) {
    switch (pick_team(g.B)) {
        case 32: k2y_launch<DIM, JM, 32>(g, grid, y, s); break;
        case 8: k2y_launch<DIM, JM, 8>(g, grid, y, s); break;
        default: k2y_launch<DIM, JM, 1>(g, grid, y, s); break;
    }
}

template <int DIM>
static void k2y_jm(int jm, const Geom& g, const float2* grid, float2* y, cudaStream_t s) {
    switch (jm) {
        case 4: k2y_team<DIM, 4>(g, grid, y, s); break;
        case 6: k2y_team<DIM, 6>(g, grid, y, s); break;
        case 8: k2y_team<DIM, 8>(g, grid, y, s); break;
        default: k2y_team<DIM, 16>(g, grid, y, s); break;
    }
}

template <int DIM, int JM, int G, bool DET>
static int y2k_launch(const Geom& g, const float2* y, float2* grid, unsigned long long* igrid,
                      const double* dscal, cudaStream_t s) {
    int ncell = 1;
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const size_t per = DET ? 16 : 8;
    const size_t budget_small = 48 * 1024, budget_max = 200 * 1024;
    size_t cellbytes = (size_t)ncell * per;
    if (cellbytes > budget_max) {
        set_error("y2k: gridding tile does not fit in shared memory; use a smaller bin shape");
        return NUFFT_EUNSUPPORTED;
    }
    int bc = (int)std::max<size_t>(1, budget_small / cellbytes);
    bc = std::min(bc, g.B);
    size_t smem = cellbytes * bc;
    auto kern = y2k_kernel<DIM, JM, G, DET>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) {
            set_error(std::string("y2k: cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return NUFFT_ECUDA;
        }
    }
    if (g.nsub > 0) kern<<<(unsigned)g.nsub, 256, smem, s>>>(g, y, grid, igrid, bc, dscal);
    return check_launch("y2k_kernel");
}

template <int DIM, int JM, bool DET>
static int y2k_team(const Geom& g, const float2* y, float2* grid, unsigned long long* igrid,
                    const double* dscal, cudaStream_t s) {
    switch (pick_team(g.B)) {
        case 32: return y2k_launch<DIM, JM, 32, DET>(g, y, grid, igrid, dscal, s);
        case 8: return y2k_launch<DIM, JM, 8, DET>(g, y, grid, igrid, dscal, s);
        default: return y2k_launch<DIM, JM, 1, DET>(g, y, grid, igrid, dscal, s);
    }
}

template <int DIM, bool DET>
static int y2k_jm(int jm, const Geom& g, const float2* y, float2* grid, unsigned long long* igrid,
                  const double* dscal, cudaStream_t s) {
    switch (jm) {
        case 4: return y2k_team<DIM, 4, DET>(g, y, grid, igrid, dscal, s);
        case 6: return y2k_team<DIM, 6, DET>(g, y, grid, igrid, dscal, s);
        case 8: return y2k_team<DIM, 8, DET>(g, y, grid, igrid, dscal, s);
        default: return y2k_team<DIM, 16, DET>(g, y, grid, igrid, dscal, s);
    }
}

}  // namespace nufft
