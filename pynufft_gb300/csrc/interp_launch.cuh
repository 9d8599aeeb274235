// Launch templates for the interpolation kernels; instantiated per
// dimension in interp_d1.cu, interp_d2.cu and interp_d3.cu so the three
// translation units compile in parallel.
#pragma once
#include "interp.cuh"

#include <algorithm>
#include <string>

namespace nufft {

// Threads per block of the paired kernels: two per point of an average
// sub-problem, 128 or 256.
inline int paired_threads(const Geom& g) {
    return (g.nsub > 0 && g.M > 96 * g.nsub) ? 256 : 128;
}

inline int pick_team(int B) {
    if (B >= 32) return 32;
    if (B >= 8) return 8;
    return 1;   // z-teams
}

// ---------------------------------------------------------------------------
// k2y
// ---------------------------------------------------------------------------
template <int DIM, int JM, int G>
static void k2y_launch(const Geom& g, const float2* grid, float2* y, cudaStream_t s) {
    const int threads = 256;
    if constexpr (G == 1) {
        int ncell = 1;
        for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
        const bool paired = g.kmethod == NUFFT_K2Y_TILE_POINT;
        const size_t smem = sizeof(float2) * (paired ? tile_strides(DIM, g.T).n : ncell);
        // a footprint beyond 200 KB of shared memory gathers from the grid
        const bool tiled = (g.kmethod == NUFFT_K2Y_TILE || paired);
        if (tiled && smem <= 200 * 1024) {
            void (*kern)(Geom, const float2*, float2*) = k2y_tile_kernel<DIM, JM>;
            int nt = threads;
            if (paired) {
                bool exact = true;
                for (int d = 0; d < DIM; ++d) exact = exact && (g.J[d] == JM);
                const int Kz = g.K[DIM - 1], rowlen = (g.T[DIM - 1] + 1) & ~1;
                const bool bulk = DIM > 1 && g.B == 1 && Kz % 2 == 0 && g.bs[DIM - 1] % 2 == 0 &&
                                  rowlen <= Kz && (reinterpret_cast<uintptr_t>(grid) & 15) == 0;
                if (bulk)
                    kern = exact ? k2y_spoint_kernel<DIM, JM, true, true>
                                 : k2y_spoint_kernel<DIM, JM, false, true>;
                else
                    kern = exact ? k2y_spoint_kernel<DIM, JM, true, false>
                                 : k2y_spoint_kernel<DIM, JM, false, false>;
                nt = paired_threads(g);
            }
            if (smem > 48 * 1024)
                cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (g.nsub > 0) kern<<<(unsigned)g.nsub, nt, smem, s>>>(g, grid, y);
        } else if (g.kmethod == NUFFT_K2Y_POINT || tiled) {
            const int64_t blocks = (g.M + threads - 1) / threads;
            if (g.B == 1)
                k2y_point_kernel<DIM, JM><<<(unsigned)blocks, threads, 0, s>>>(g, grid, y);
            else
                k2y_coil_kernel<DIM, JM, 1><<<(unsigned)blocks, threads, 0, s>>>(g, grid, y);
        } else {
            const int TS = g.J[DIM - 1];
            const int64_t nwarps = (g.M + (32 / TS) - 1) / (32 / TS);
            const int64_t blocks = (nwarps * 32 + threads - 1) / threads;
            k2y_zteam_kernel<DIM, JM><<<(unsigned)blocks, threads, 0, s>>>(g, grid, y);
        }
    } else {
        if constexpr (DIM > 1) {
            // coil teams on a shared tile when the tile of all coils fits two
            // blocks per SM and rows are whole 16-byte units (even B)
            int ncell = 1;
            for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
            const size_t smem = sizeof(float2) * (size_t)ncell * g.B;
            if (g.B % 2 == 0 && smem <= 112 * 1024 && g.nsub > 0 &&
                (reinterpret_cast<uintptr_t>(grid) & 15) == 0 && g.T[DIM - 1] <= g.K[DIM - 1]) {
                bool exact = true;
                for (int d = 0; d < DIM; ++d) exact = exact && (g.J[d] == JM);
                void (*kern)(Geom, const float2*, float2*) =
                    exact ? k2y_ctile_kernel<DIM, JM, G, true> : k2y_ctile_kernel<DIM, JM, G, false>;
                if (smem > 48 * 1024)
                    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
                kern<<<(unsigned)(g.gsub ? g.ngsub : g.nsub), 512, smem, s>>>(g, grid, y);
                return;
            }
        }
        const int64_t blocks = (g.M * G + threads - 1) / threads;
        k2y_coil_kernel<DIM, JM, G><<<(unsigned)blocks, threads, 0, s>>>(g, grid, y);
    }
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

// ---------------------------------------------------------------------------
// y2k
// ---------------------------------------------------------------------------
// Coils per shared-memory chunk: as many as fit in 112 KB (two blocks per
// SM), split into equal chunks, at most 64; one coil may use up to 200 KB.
inline int coil_chunk(size_t cellbytes, int B, size_t* smem) {
    const size_t target = 112 * 1024, big = 200 * 1024;
    if (cellbytes > big) return 0;
    int bmax = (int)std::min<size_t>(64, std::max<size_t>(1, target / cellbytes));
    const int n = (B + bmax - 1) / bmax;
    const int bc = (B + n - 1) / n;
    *smem = cellbytes * bc;
    return bc;
}

template <int DIM, int JM, int G, bool DET>
static int y2k_launch(const Geom& g, const float2* y, float2* grid, unsigned long long* igrid,
                      const double* dscal, cudaStream_t s) {
    if constexpr (G == 1 && !DET) {
        if (g.ymethod == NUFFT_Y2K_GLOBAL) {
            const int TS = g.J[DIM - 1];
            const int64_t nwarps = (g.M + (32 / TS) - 1) / (32 / TS);
            const int64_t blocks = (nwarps * 32 + 255) / 256;
            y2k_global_kernel<DIM, JM><<<(unsigned)blocks, 256, 0, s>>>(g, y, grid);
            return check_launch("y2k_global_kernel");
        }
    }
    int ncell = 1;
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const size_t per = DET ? 16 : 8;   // re + im accumulators per cell and coil
    size_t smem = 0;
    int bc = coil_chunk((size_t)ncell * per, (G == 1) ? std::min(g.B, 7) : g.B, &smem);
    if (bc == 0) {
        set_error("y2k: gridding tile does not fit in shared memory; use a smaller bin shape");
        return NUFFT_EUNSUPPORTED;
    }
    if constexpr (G == 1 && !DET && DIM > 1) {
        // one coil: paired threads per point on the padded tile
        const size_t psmem = 2 * sizeof(unsigned) * tile_strides(DIM, g.T).n;
        if (g.ymethod == NUFFT_Y2K_POINT && g.B == 1 && psmem <= 200 * 1024) {
            bool exact = true;
            for (int d = 0; d < DIM; ++d) exact = exact && (g.J[d] == JM);
            void (*pk)(Geom, const float2*, float2*) =
                exact ? y2k_spoint_kernel<DIM, JM, true> : y2k_spoint_kernel<DIM, JM, false>;
            if (psmem > 48 * 1024) {
                cudaError_t e = cudaFuncSetAttribute(pk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)psmem);
                if (e != cudaSuccess) {
                    set_error(std::string("y2k: cudaFuncSetAttribute: ") + cudaGetErrorString(e));
                    return NUFFT_ECUDA;
                }
            }
            if (g.nsub > 0) pk<<<(unsigned)g.nsub, paired_threads(g), psmem, s>>>(g, y, grid);
            return check_launch("y2k_spoint_kernel");
        }
    }
    void (*kern)(Geom, const float2*, float2*, unsigned long long*, int, const double*);
    int threads = 256;
    if constexpr (G == 1) {
        if (g.ymethod == NUFFT_Y2K_POINT) {
            bool exact = true;
            for (int d = 0; d < DIM; ++d) exact = exact && (g.J[d] == JM);
            kern = exact ? y2k_point_kernel<DIM, JM, true, DET> : y2k_point_kernel<DIM, JM, false, DET>;
            threads = 128;
        } else {
            kern = y2k_zteam_kernel<DIM, JM, DET>;
        }
    } else {
        bool exact = true;
        for (int d = 0; d < DIM; ++d) exact = exact && (g.J[d] == JM);
        kern = exact ? y2k_coil_kernel<DIM, JM, G, DET, true> : y2k_coil_kernel<DIM, JM, G, DET, false>;
        threads = DET ? 256 : 512;   // the 64-bit tiles of the exact mode need the registers
    }
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) {
            set_error(std::string("y2k: cudaFuncSetAttribute: ") + cudaGetErrorString(e));
            return NUFFT_ECUDA;
        }
    }
    if (g.nsub > 0) kern<<<(unsigned)g.nsub, threads, smem, s>>>(g, y, grid, igrid, bc, dscal);
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
