// Interpolation (k2y) and gridding (y2k) kernels, templated on the number of
// dimensions DIM, the per-axis neighbour bound JM (compile-time loop length;
// the runtime J[d] <= JM masks the tail) and the team width G (lanes that
// share one point and split the coils between them).
//
//   k2y  y[m,b]  = sum_{j} prod_d coef_d[m,j_d] * k[idx(m,j), b]
//                  (the CSR product sp . k of _k2y_cpu,
//                   nufft/_nufft_class_methods_cpu.py:273-288)
//   y2k  k[c,b] += sum_m conj(prod_d coef_d[m,j_d]) * y[m,b]
//                  (spH . y of _y2k_cpu, :290-314)
// coef_d holds conj(u) exactly as the reference's CSR values
// (helper.min_max returns u.T.conj(), src/_helper/helper.py:606-618).
//
// The sum over the Kronecker footprint is factorised axis by axis
// (sum_i c0_i sum_j c1_j sum_k c2_k g_ijk), so a 3D point costs
// J^3 + J^2 + J complex multiply-adds instead of 2 J^3.  The two innermost
// axes are unrolled; the outermost axis loop stays rolled and re-reads its
// coefficient through L1, which bounds code size for every JM.
#pragma once
#include "nufft_internal.cuh"

namespace nufft {

__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {  // acc += a*b
    acc.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
    acc.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
}

__device__ __forceinline__ int inst_of_sorted(const int64_t* start, int ninst, int64_t s) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= s) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Load one point's wrapped footprint indices and coefficients for axis d.
template <int JM>
__device__ __forceinline__ void load_axis(const Geom& g, int d, int64_t s, int (&idx)[JM],
                                          float2 (&c)[JM]) {
    const int K = g.K[d], J = g.J[d];
    const int p = __ldg(g.pos[d] + s);
    const float2* src = g.coef[d] + s * g.JP[d];
#pragma unroll
    for (int j = 0; j < JM; ++j) {
        if (j < J) {
            int q = p + j;
            idx[j] = (q >= K) ? q - K : q;
            c[j] = __ldg(src + j);
        } else {
            idx[j] = 0;
            c[j] = make_float2(0.f, 0.f);
        }
    }
}

template <int DIM, int JM, int G>
__global__ void __launch_bounds__(256) k2y_kernel(Geom g, const float2* __restrict__ grid,
                                                  float2* __restrict__ y) {
    const int64_t team = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
    const int lane = threadIdx.x % G;
    if (team >= g.M) return;
    const int64_t s = team;
    const int m = __ldg(g.perm + s);
    const int inst = (g.ninst > 1) ? inst_of_sorted(g.inst_start, g.ninst, s) : 0;
    const int B = g.B;
    const float2* __restrict__ base = grid + (size_t)inst * g.prodK * B;

    // innermost (fastest) axis and the one above it live in registers
    constexpr int DI = DIM - 1;                    // innermost axis
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;    // the axis above it
    int iz[JM], iy[JM];
    float2 cz[JM], cy[JM];
    load_axis<JM>(g, DI, s, iz, cz);
    if constexpr (DIM > 1) load_axis<JM>(g, DY, s, iy, cy);
    const int p0 = __ldg(g.pos[0] + s);
    const float2* c0src = g.coef[0] + s * g.JP[0];
    const int K0 = g.K[0], J0 = g.J[0];
    const int Kz = g.K[DI], Ky = g.K[DY];

    for (int b = lane; b < B; b += G) {
        float2 acc = make_float2(0.f, 0.f);
        if constexpr (DIM == 1) {
#pragma unroll
            for (int k = 0; k < JM; ++k) cfma(acc, cz[k], __ldg(base + (size_t)iz[k] * B + b));
        } else if constexpr (DIM == 2) {
#pragma unroll
            for (int j = 0; j < JM; ++j) {
                const size_t row = (size_t)iy[j] * Kz;
                float2 t = make_float2(0.f, 0.f);
#pragma unroll
                for (int k = 0; k < JM; ++k) cfma(t, cz[k], __ldg(base + (row + iz[k]) * B + b));
                cfma(acc, cy[j], t);
            }
        } else {
#pragma unroll 1
            for (int i = 0; i < J0; ++i) {
                int q = p0 + i;
                if (q >= K0) q -= K0;
                const size_t plane = (size_t)q * Ky;
                float2 ti = make_float2(0.f, 0.f);
#pragma unroll
                for (int j = 0; j < JM; ++j) {
                    const size_t row = (plane + iy[j]) * Kz;
                    float2 t = make_float2(0.f, 0.f);
#pragma unroll
                    for (int k = 0; k < JM; ++k) cfma(t, cz[k], __ldg(base + (row + iz[k]) * B + b));
                    cfma(ti, cy[j], t);
                }
                cfma(acc, __ldg(c0src + i), ti);
            }
        }
        y[(size_t)m * B + b] = acc;
    }
}

// Fixed-point conversion of one contribution for the deterministic mode.
__device__ __forceinline__ unsigned long long to_fixed(float v, float scale) {
    return (unsigned long long)__float2ll_rn(v * scale);
}

template <bool DET>
__device__ __forceinline__ void smem_add(unsigned char* smem_raw, int e, float2 w, float scale) {
    if (DET) {
        unsigned long long* sm = reinterpret_cast<unsigned long long*>(smem_raw);
        atomicAdd(sm + 2 * e, to_fixed(w.x, scale));
        atomicAdd(sm + 2 * e + 1, to_fixed(w.y, scale));
    } else {
        float* sm = reinterpret_cast<float*>(smem_raw);
        atomicAdd(sm + 2 * e, w.x);
        atomicAdd(sm + 2 * e + 1, w.y);
    }
}

// One thread block per gridding sub-problem (a bin, or a chunk of a crowded
// bin).  The block accumulates its points into a shared-memory tile covering
// the bin plus the J-1 halo, then adds the tile to the global grid with
// vector atomics.  DET selects exact 64-bit fixed-point accumulation
// (integer adds are associative, so the result does not depend on the order
// in which threads or blocks arrive).
template <int DIM, int JM, int G, bool DET>
__global__ void __launch_bounds__(256) y2k_kernel(Geom g, const float2* __restrict__ y,
                                                  float2* __restrict__ grid,
                                                  unsigned long long* __restrict__ igrid,
                                                  int bc, const double* __restrict__ dscal) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int4 sp = g.sub[blockIdx.x];
    const int inst = sp.w;
    int64_t lb = sp.x - (int64_t)inst * g.nbin_inst;
    int o[3] = {0, 0, 0};
#pragma unroll
    for (int d = DIM - 1; d >= 0; --d) {
        o[d] = (int)(lb % g.nb[d]) * g.bs[d];
        lb /= g.nb[d];
    }
    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
    const int Tz = g.T[DI];
    const int Ty = (DIM > 1) ? g.T[DY] : 1;
    int ncell = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const int B = g.B;
    const float scale = DET ? (float)dscal[1] : 1.f;
    const int team = threadIdx.x / G, lane = threadIdx.x % G, nteam = blockDim.x / G;
    const int J0 = g.J[0];

    for (int b0 = 0; b0 < B; b0 += bc) {
        const int bcur = min(bc, B - b0);
        const int nsm = ncell * bcur;
        if (DET) {
            unsigned long long* sm = reinterpret_cast<unsigned long long*>(smem_raw);
            for (int e = threadIdx.x; e < 2 * nsm; e += blockDim.x) sm[e] = 0ull;
        } else {
            float2* sm = reinterpret_cast<float2*>(smem_raw);
            for (int e = threadIdx.x; e < nsm; e += blockDim.x) sm[e] = make_float2(0.f, 0.f);
        }
        __syncthreads();

        for (int s = sp.y + team; s < sp.y + sp.z; s += nteam) {
            int iz[JM], iy[JM];
            float2 cz[JM], cy[JM];
            load_axis<JM>(g, DI, s, iz, cz);
            if constexpr (DIM > 1) load_axis<JM>(g, DY, s, iy, cy);
            // local offsets of the footprint origin inside the tile
            const int lz = __ldg(g.pos[DI] + s) - o[DI];
            const int ly = (DIM > 1) ? __ldg(g.pos[DY] + s) - o[DY] : 0;
            const int lx = (DIM > 2) ? __ldg(g.pos[0] + s) - o[0] : 0;
            const float2* c0src = g.coef[0] + (size_t)s * g.JP[0];
            const int m = __ldg(g.perm + s);
            for (int b = lane; b < bcur; b += G) {
                const float2 yv = __ldg(y + (size_t)m * B + b0 + b);
                if constexpr (DIM == 1) {
#pragma unroll
                    for (int k = 0; k < JM; ++k)
                        if (k < g.J[DI]) smem_add<DET>(smem_raw, (lz + k) * bcur + b, cmulc(yv, cz[k]), scale);
                } else {
                    const int ni = (DIM > 2) ? J0 : 1;
#pragma unroll 1
                    for (int i = 0; i < ni; ++i) {
                        const float2 wi = (DIM > 2) ? cmulc(yv, __ldg(c0src + i)) : yv;
                        const int ci = (DIM > 2) ? (lx + i) * Ty : 0;
#pragma unroll
                        for (int j = 0; j < JM; ++j) {
                            if (j >= g.J[DY]) continue;
                            const float2 wij = cmulc(wi, cy[j]);
                            const int cj = (ci + ly + j) * Tz + lz;
#pragma unroll
                            for (int k = 0; k < JM; ++k) {
                                if (k >= g.J[DI]) continue;
                                smem_add<DET>(smem_raw, (cj + k) * bcur + b, cmulc(wij, cz[k]), scale);
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();

        // flush the tile (with wrap-around) into the global grid
        const size_t ibase = (size_t)inst * g.prodK;
        for (int e = threadIdx.x; e < nsm; e += blockDim.x) {
            const int b = e % bcur;
            int cell = e / bcur;
            int t[3] = {0, 0, 0};
#pragma unroll
            for (int d = DIM - 1; d >= 0; --d) {
                t[d] = cell % g.T[d];
                cell /= g.T[d];
            }
            size_t gc = 0;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                int v = o[d] + t[d];
                while (v >= g.K[d]) v -= g.K[d];
                gc = gc * g.K[d] + v;
            }
            const size_t gi = (ibase + gc) * B + b0 + b;
            if (DET) {
                unsigned long long* sm = reinterpret_cast<unsigned long long*>(smem_raw);
                const unsigned long long vx = sm[2 * e], vy = sm[2 * e + 1];
                if (vx) atomicAdd(igrid + 2 * gi, vx);
                if (vy) atomicAdd(igrid + 2 * gi + 1, vy);
            } else {
                const float2 v = reinterpret_cast<float2*>(smem_raw)[e];
                if (v.x != 0.f || v.y != 0.f) atomicAdd(grid + gi, v);
            }
        }
        __syncthreads();
    }
}

}  // namespace nufft
