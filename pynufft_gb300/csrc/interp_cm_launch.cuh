// Launch templates of the coil-major gridding kernels (interp_cm.cuh),
// instantiated per dimension in interp_cm2.cu and interp_cm3.cu.
#pragma once
#include "interp_cm.cuh"

#include <string>

namespace nufft {

// Extent along the innermost axis of a row sub-problem for which the row
// kernels are built (bins x rgroup): 16 cells (the default bins of plans
// with 8 or more coils: 16 in 2D; 4, grouped by four, in 3D).
template <int DIM>
constexpr int cm_bin_z() { return 16; }


template <int DIM, int JM, int CB, bool DET>
static int y2k_rows_launch(const Geom& g, const float2* y, float2* grid, unsigned long long* igrid,
                           const double* dscal, cudaStream_t s) {
    constexpr int TZ = cm_bin_z<DIM>() + JM - 1;
    auto kern = y2k_rows_kernel<DIM, JM, TZ, CB, DET>;
    const int threads = 256;
    const int nkey = g.bs[0] * (DIM == 3 ? g.bs[1] : 1);
    const size_t smem = rows_smem(DIM, JM, nkey, row_sub_cap(DIM), threads / 32, CB);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) {
            set_error(std::string("y2k_rows: cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return NUFFT_ECUDA;
        }
    }
    if (g.nrsub > 0) kern<<<(unsigned)g.nrsub, threads, smem, s>>>(g, y, grid, igrid, dscal);
    return check_launch("y2k_rows_kernel");
}

template <int DIM, int JM, bool DET>
static int y2k_rows_cb(const Geom& g, const float2* y, float2* grid, unsigned long long* igrid,
                       const double* dscal, cudaStream_t s) {
    if (cm_row_coils(g.B) == 32) return y2k_rows_launch<DIM, JM, 32, DET>(g, y, grid, igrid, dscal, s);
    return y2k_rows_launch<DIM, JM, 8, DET>(g, y, grid, igrid, dscal, s);
}

template <int DIM>
static int y2k_cm_jm(int jm, bool det, const Geom& g, const float2* y, float2* grid,
                     unsigned long long* igrid, const double* dscal, cudaStream_t s) {
    switch (jm) {
        case 4: return det ? y2k_rows_cb<DIM, 4, true>(g, y, grid, igrid, dscal, s)
                           : y2k_rows_cb<DIM, 4, false>(g, y, grid, igrid, dscal, s);
        case 6: return det ? y2k_rows_cb<DIM, 6, true>(g, y, grid, igrid, dscal, s)
                           : y2k_rows_cb<DIM, 6, false>(g, y, grid, igrid, dscal, s);
        default: return det ? y2k_rows_cb<DIM, 8, true>(g, y, grid, igrid, dscal, s)
                            : y2k_rows_cb<DIM, 8, false>(g, y, grid, igrid, dscal, s);
    }
}

}  // namespace nufft
