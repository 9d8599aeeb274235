// Launch templates of the coil-major interpolation / gridding kernels
// (interp_cm.cuh), instantiated per dimension in interp_cm2.cu and
// interp_cm3.cu.
#pragma once
#include "interp_cm.cuh"

#include <string>

namespace nufft {

// Extent along the innermost axis of a row sub-problem for which the row
// kernels are built (bins x rgroup): 16 cells (the default bins of plans
// with 8 or more coils: 16 in 2D; 4, grouped by four, in 3D).
template <int DIM>
constexpr int cm_bin_z() { return 16; }

// Coils per lane group of the row kernels: 32 when they divide B, else 8.
inline int cm_row_coils(int B) { return (B % 32 == 0) ? 32 : 8; }

// Coils per shared tile of the coil-major gather: the largest of 32, 16, 8,
// 4 that divides B and keeps the tile within 112 KB (two blocks per SM);
// 0 if none does.
inline int cm_tile_coils(const Geom& g, int DIM) {
    int ncell = 1;
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    for (int c : {32, 16, 8, 4})
        if (g.B % c == 0 && cmtile_smem(ncell, c) <= 112 * 1024) return c;
    return 0;
}

template <int DIM, int JM, int CB, bool DET>
static int y2k_rows_launch(const Geom& g, const float2* y, float2* grid, unsigned long long* igrid,
                           const double* dscal, cudaStream_t s) {
    constexpr int TZ = cm_bin_z<DIM>() + JM - 1;
    auto kern = y2k_rows_kernel<DIM, JM, TZ, CB, DET>;
    const int threads = 256;
    const int nkey = g.bs[0] * (DIM == 3 ? g.bs[1] : 1);
    const size_t smem = rows_smem(DIM, JM, nkey, kRowSub, threads / 32);
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

template <int DIM, int JM, int G>
static int k2y_cm_launch(const Geom& g, const float2* grid, float2* y, int cbk, cudaStream_t s) {
    auto kern = k2y_cmtile_kernel<DIM, JM, G>;
    int ncell = 1;
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const size_t smem = cmtile_smem(ncell, cbk);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) {
            set_error(std::string("k2y_cmtile: cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return NUFFT_ECUDA;
        }
    }
    if (g.ngsub > 0) kern<<<(unsigned)g.ngsub, 512, smem, s>>>(g, grid, y, cbk);
    return check_launch("k2y_cmtile_kernel");
}

template <int DIM, int JM>
static int k2y_cm_g(const Geom& g, const float2* grid, float2* y, cudaStream_t s) {
    const int cbk = cm_tile_coils(g, DIM);
    if (cbk >= 32) return k2y_cm_launch<DIM, JM, 32>(g, grid, y, cbk, s);
    if (cbk >= 8) return k2y_cm_launch<DIM, JM, 8>(g, grid, y, cbk, s);
    return k2y_cm_launch<DIM, JM, 4>(g, grid, y, cbk, s);
}

template <int DIM>
static int k2y_cm_jm(int jm, const Geom& g, const float2* grid, float2* y, cudaStream_t s) {
    switch (jm) {
        case 4: return k2y_cm_g<DIM, 4>(g, grid, y, s);
        case 6: return k2y_cm_g<DIM, 6>(g, grid, y, s);
        default: return k2y_cm_g<DIM, 8>(g, grid, y, s);
    }
}

}  // namespace nufft
