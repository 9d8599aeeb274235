// Interpolation (k2y) and gridding (y2k) kernels.
//
//   k2y  y[m,b]  = sum_{j} prod_d coef_d[m,j_d] * k[idx(m,j), b]
//                  (the CSR product sp . k of _k2y_cpu,
//                   nufft/_nufft_class_methods_cpu.py:273-288)
//   y2k  k[c,b] += sum_m conj(prod_d coef_d[m,j_d]) * y[m,b]
//                  (spH . y of _y2k_cpu, :290-314)
// coef_d holds conj(u) exactly as the reference's CSR values
// (helper.min_max returns u.T.conj(), src/_helper/helper.py:606-618).
//
// Lane mappings (the defaults; `nufft_plan_set_methods` and the autotuner
// may choose the others):
//  * paired threads (one coil, 2D/3D): a block per bin sub-problem stages the
//    bin's footprint tile in shared memory (bulk copies for k2y, a fixed-
//    point accumulator for y2k); two threads per point split the outer axis.
//  * coil teams (B >= 8): G = 8 or 32 lanes share one point and split the
//    coils, so consecutive lanes touch consecutive coils of one cell; k2y
//    gathers from a shared tile of all coils.
//  * one thread per point, z-teams (J lanes per point along the innermost
//    axis), global atomics: the remaining cases and autotuner candidates.
// All factorise the footprint sum axis by axis (outer axis rolled, middle
// axis in registers, inner axis unrolled or across lanes).
//
// Gridding accumulates in shared memory with native integer atomics: this
// GPU has no native shared-memory float add (a float atomicAdd there is a
// compare-and-swap loop).  The fast mode converts each float contribution to
// 32-bit fixed point with a scale chosen per sub-problem from a bound on any
// cell's sum (sum over the sub-problem's points of W_p (|re y| + |im y|),
// W_p = prod_d max_j |coef|), so no cell can overflow and the rounding unit
// stays near float32 resolution for sub-problems of a few hundred points; the tile is converted back to float and added to the
// grid with vector atomics.  The deterministic mode uses 64-bit fixed point
// with one global scale and flushes integers, so the whole sum is exact and
// order-independent.
#pragma once
#include "nufft_internal.cuh"

namespace nufft {

__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // a * conj(b)
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
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

__device__ __forceinline__ int wrap1(int q, int K) { return (q >= K) ? q - K : q; }
__device__ __forceinline__ int wrapn(int q, int K) {
    while (q >= K) q -= K;
    return q;
}

// Walks the cells of a DIM-dimensional tile (extents T, row-major) with a
// fixed stride, keeping the coordinates incrementally (one division chain
// per thread instead of one per cell).
template <int DIM>
struct TileWalk {
    int t[3], st[3], T[3];
    __device__ __forceinline__ void init(const int* ext, int first, int stride) {
        T[0] = ext[0]; T[1] = (DIM > 1) ? ext[1] : 1; T[2] = (DIM > 2) ? ext[2] : 1;
        // the last tile axis is the fastest: index = (t0*T1 + t1)*T2 + t2 in 3D
        t[0] = t[1] = t[2] = 0; st[0] = st[1] = st[2] = 0;
        if (DIM == 1) { t[0] = first; st[0] = stride; return; }
        const int Tl = T[DIM - 1];
        int e = first, s = stride;
        t[DIM - 1] = e % Tl; st[DIM - 1] = s % Tl;
        e /= Tl; s /= Tl;
        if (DIM == 3) { t[1] = e % T[1]; st[1] = s % T[1]; e /= T[1]; s /= T[1]; }
        t[0] = e;
        st[0] = s;
    }
    __device__ __forceinline__ void next() {
        if (DIM == 1) { t[0] += st[0]; return; }
        t[DIM - 1] += st[DIM - 1];
        int carry = 0;
        if (t[DIM - 1] >= T[DIM - 1]) { t[DIM - 1] -= T[DIM - 1]; carry = 1; }
        if (DIM == 3) {
            t[1] += st[1] + carry;
            carry = 0;
            if (t[1] >= T[1]) { t[1] -= T[1]; carry = 1; }
        }
        t[0] += st[0] + carry;
    }
    // flat grid cell (inside one instance) of tile coordinate t for origin o
    __device__ __forceinline__ size_t cell(const Geom& g, const int (&o)[3]) const {
        size_t gc = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) gc = gc * g.K[d] + wrapn(o[d] + t[d], g.K[d]);
        return gc;
    }
};

// Tile origin of a sub-problem.
template <int DIM>
__device__ __forceinline__ void tile_origin(const Geom& g, const int4& sp, int (&o)[3]) {
    int64_t lb = sp.x - (int64_t)sp.w * g.nbin_inst;
    o[0] = o[1] = o[2] = 0;
#pragma unroll
    for (int d = DIM - 1; d >= 0; --d) {
        o[d] = (int)(lb % g.nb[d]) * g.bs[d];
        lb /= g.nb[d];
    }
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
            idx[j] = wrap1(p + j, K);
            c[j] = __ldg(src + j);
        } else {
            idx[j] = 0;
            c[j] = make_float2(0.f, 0.f);
        }
    }
}

// Sum of v over the TS lanes of this lane's team (teams are TS-aligned);
// the first lane of the team receives the total.
__device__ __forceinline__ float2 team_sum(float2 v, int k, int TS) {
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) {
        const float ox = __shfl_down_sync(0xffffffffu, v.x, off);
        const float oy = __shfl_down_sync(0xffffffffu, v.y, off);
        if (off < TS && k + off < TS) {
            v.x += ox;
            v.y += oy;
        }
    }
    return v;
}

// ---------------------------------------------------------------------------
// k2y, z-teams (B < 8)
// ---------------------------------------------------------------------------
template <int DIM, int JM>
__global__ void __launch_bounds__(256) k2y_zteam_kernel(Geom g, const float2* __restrict__ grid,
                                                        float2* __restrict__ y) {
    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
    const int TS = g.J[DI];
    const int NT = 32 / TS;
    const int lane = threadIdx.x & 31;
    const int team = lane / TS, k = lane - team * TS;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t s = warp * NT + team;
    const bool active = (team < NT) && (s < g.M);
    const int64_t sl = active ? s : 0;
    const int B = g.B;
    const int inst = (g.ninst > 1) ? inst_of_sorted(g.inst_start, g.ninst, sl) : 0;
    const float2* __restrict__ base = grid + (size_t)inst * g.prodK * B;

    const int pz = __ldg(g.pos[DI] + sl);
    const int iz = wrap1(pz + k, g.K[DI]);
    const float2 cz = __ldg(g.coef[DI] + sl * g.JP[DI] + k);
    int iy[JM];
    float2 cy[JM];
    if constexpr (DIM > 1) load_axis<JM>(g, DY, sl, iy, cy);
    const int Kz = g.K[DI], Ky = g.K[DY];
    const int p0 = __ldg(g.pos[0] + sl), K0 = g.K[0], J0 = g.J[0];
    const float2* c0src = g.coef[0] + sl * g.JP[0];

    for (int b = 0; b < B; ++b) {
        float2 acc = make_float2(0.f, 0.f);
        if constexpr (DIM == 1) {
            acc = __ldg(base + (size_t)iz * B + b);
        } else if constexpr (DIM == 2) {
#pragma unroll
            for (int j = 0; j < JM; ++j)
                cfma(acc, cy[j], __ldg(base + ((size_t)iy[j] * Kz + iz) * B + b));
        } else {
#pragma unroll 1
            for (int i = 0; i < J0; ++i) {
                const size_t plane = (size_t)wrap1(p0 + i, K0) * Ky;
                float2 t = make_float2(0.f, 0.f);
#pragma unroll
                for (int j = 0; j < JM; ++j)
                    cfma(t, cy[j], __ldg(base + ((plane + iy[j]) * Kz + iz) * B + b));
                cfma(acc, __ldg(c0src + i), t);
            }
        }
        acc = cmul(acc, cz);
        acc = team_sum(acc, k, TS);
        if (active && k == 0) y[(size_t)__ldg(g.perm + s) * B + b] = acc;
    }
}

// ---------------------------------------------------------------------------
// k2y, coil-teams (B >= 8)
// ---------------------------------------------------------------------------
template <int DIM, int JM, int G>
__global__ void __launch_bounds__(256) k2y_coil_kernel(Geom g, const float2* __restrict__ grid,
                                                       float2* __restrict__ y) {
    const int64_t team = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / G;
    const int lane = threadIdx.x % G;
    if (team >= g.M) return;
    const int64_t s = team;
    const int m = __ldg(g.perm + s);
    const int inst = (g.ninst > 1) ? inst_of_sorted(g.inst_start, g.ninst, s) : 0;
    const int B = g.B;
    const float2* __restrict__ base = grid + (size_t)inst * g.prodK * B;

    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
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
                const size_t plane = (size_t)wrap1(p0 + i, K0) * Ky;
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

// ---------------------------------------------------------------------------
// k2y, one thread per point, single coil: each footprint row along the
// innermost axis is read with 16-byte loads (3 loads instead of 6 for J = 6
// on an even start), halving the L1 requests of the scattered gather.
// Rows that wrap around the grid edge, or an odd innermost extent, fall
// back to 8-byte loads.
// ---------------------------------------------------------------------------
template <int JM>
__device__ __forceinline__ float2 row_dot(const float2* __restrict__ row, int pz, int Jz, int Kz,
                                          bool vec_ok, const float2 (&cz)[JM]) {
    float2 t = make_float2(0.f, 0.f);
    const int odd = pz & 1;
    const int pa = pz - odd;
    constexpr int NV = (JM + 2) / 2;
    const int nv = (odd + Jz + 1) >> 1;
    if (vec_ok && pa + 2 * nv <= Kz) {
        const float4* r4 = reinterpret_cast<const float4*>(row + pa);
        float4 v[NV];
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q] = (q < nv) ? __ldg(r4 + q) : make_float4(0.f, 0.f, 0.f, 0.f);
        if (odd) {
#pragma unroll
            for (int k = 0; k < JM; ++k) {
                const float4 q = v[(k + 1) >> 1];
                const float2 c = ((k + 1) & 1) ? make_float2(q.z, q.w) : make_float2(q.x, q.y);
                cfma(t, cz[k], c);
            }
        } else {
#pragma unroll
            for (int k = 0; k < JM; ++k) {
                const float4 q = v[k >> 1];
                const float2 c = (k & 1) ? make_float2(q.z, q.w) : make_float2(q.x, q.y);
                cfma(t, cz[k], c);
            }
        }
    } else {
#pragma unroll
        for (int k = 0; k < JM; ++k)
            if (k < Jz) cfma(t, cz[k], __ldg(row + wrap1(pz + k, Kz)));
    }
    return t;
}

template <int DIM, int JM>
__global__ void __launch_bounds__(256) k2y_point_kernel(Geom g, const float2* __restrict__ grid,
                                                        float2* __restrict__ y) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= g.M) return;
    const int inst = (g.ninst > 1) ? inst_of_sorted(g.inst_start, g.ninst, s) : 0;
    const float2* __restrict__ base = grid + (size_t)inst * g.prodK;
    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
    const int Kz = g.K[DI], Jz = g.J[DI];
    const bool vec_ok = ((Kz & 1) == 0) && ((reinterpret_cast<uintptr_t>(base) & 15) == 0);
    const int pz = __ldg(g.pos[DI] + s);
    float2 cz[JM];
    {
        const float2* src = g.coef[DI] + s * g.JP[DI];
#pragma unroll
        for (int k = 0; k < JM; ++k) cz[k] = (k < Jz) ? __ldg(src + k) : make_float2(0.f, 0.f);
    }
    float2 acc = make_float2(0.f, 0.f);
    if constexpr (DIM == 1) {
        acc = row_dot<JM>(base, pz, Jz, Kz, vec_ok, cz);
    } else {
        int iy[JM];
        float2 cy[JM];
        load_axis<JM>(g, DY, s, iy, cy);
        const int Jy = g.J[DY];
        if constexpr (DIM == 2) {
#pragma unroll
            for (int j = 0; j < JM; ++j)
                if (j < Jy) cfma(acc, cy[j], row_dot<JM>(base + (size_t)iy[j] * Kz, pz, Jz, Kz, vec_ok, cz));
        } else {
            const int p0 = __ldg(g.pos[0] + s), K0 = g.K[0], J0 = g.J[0], Ky = g.K[DY];
            const float2* c0src = g.coef[0] + s * g.JP[0];
#pragma unroll 1
            for (int i = 0; i < J0; ++i) {
                const size_t plane = (size_t)wrap1(p0 + i, K0) * Ky;
                float2 t = make_float2(0.f, 0.f);
#pragma unroll
                for (int j = 0; j < JM; ++j)
                    if (j < Jy)
                        cfma(t, cy[j], row_dot<JM>(base + (plane + iy[j]) * Kz, pz, Jz, Kz, vec_ok, cz));
                cfma(acc, __ldg(c0src + i), t);
            }
        }
    }
    y[__ldg(g.perm + s)] = acc;
}

// ---------------------------------------------------------------------------
// y2k straight into the global grid (B < 8, fast mode only): z-teams add
// float contributions with vector atomics performed in L2; no shared tile,
// no flush, no fixed point.  Suited to sparse trajectories where a bin's
// tile would hold few contributions per cell.
// ---------------------------------------------------------------------------
template <int DIM, int JM>
__global__ void __launch_bounds__(256) y2k_global_kernel(Geom g, const float2* __restrict__ y,
                                                         float2* __restrict__ grid) {
    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
    const int TS = g.J[DI];
    const int NT = 32 / TS;
    const int lane = threadIdx.x & 31;
    const int team = lane / TS, k = lane - team * TS;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t s = warp * NT + team;
    if (team >= NT || s >= g.M) return;
    const int B = g.B;
    const int inst = (g.ninst > 1) ? inst_of_sorted(g.inst_start, g.ninst, s) : 0;
    float2* __restrict__ base = grid + (size_t)inst * g.prodK * B;
    const int iz = wrap1(__ldg(g.pos[DI] + s) + k, g.K[DI]);
    const float2 cz = __ldg(g.coef[DI] + s * g.JP[DI] + k);
    int iy[JM];
    float2 cy[JM];
    if constexpr (DIM > 1) load_axis<JM>(g, DY, s, iy, cy);
    const int Kz = g.K[DI], Ky = g.K[DY];
    const int p0 = __ldg(g.pos[0] + s), K0 = g.K[0], J0 = g.J[0];
    const float2* c0src = g.coef[0] + s * g.JP[0];
    const int m = __ldg(g.perm + s);
    for (int b = 0; b < B; ++b) {
        const float2 v = cmulc(__ldg(y + (size_t)m * B + b), cz);
        if constexpr (DIM == 1) {
            atomicAdd(base + (size_t)iz * B + b, v);
        } else {
            const int ni = (DIM > 2) ? J0 : 1;
#pragma unroll 1
            for (int i = 0; i < ni; ++i) {
                const float2 wi = (DIM > 2) ? cmulc(v, __ldg(c0src + i)) : v;
                const size_t plane = (DIM > 2) ? (size_t)wrap1(p0 + i, K0) * Ky : 0;
#pragma unroll
                for (int j = 0; j < JM; ++j) {
                    if (j >= g.J[DY]) continue;
                    atomicAdd(base + ((plane + iy[j]) * Kz + iz) * B + b, cmulc(wi, cy[j]));
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// k2y, shared-memory tile per sub-problem (B < 8): the block stages the
// bin's footprint (bin + J-1 halo) in shared memory with coalesced row loads,
// then z-teams gather from it; every point of a bin is served by one SM.
// ---------------------------------------------------------------------------
template <int DIM, int JM>
__global__ void __launch_bounds__(256) k2y_tile_kernel(Geom g, const float2* __restrict__ grid,
                                                       float2* __restrict__ y) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* tile = reinterpret_cast<float2*>(smem_raw);
    const int4 sp = g.sub[blockIdx.x];
    int o[3];
    tile_origin<DIM>(g, sp, o);
    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
    const int Tz = g.T[DI];
    const int Ty = (DIM > 1) ? g.T[DY] : 1;
    int ncell = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const int B = g.B;
    const int TS = g.J[DI], NT = 32 / TS;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int team = lane / TS, k = lane - team * TS;
    const int J0 = g.J[0];
    const size_t ibase = (size_t)sp.w * g.prodK;
    const int per_round = nwarps * NT;
    const int end = sp.y + sp.z;

    for (int b = 0; b < B; ++b) {
        TileWalk<DIM> w;
        w.init(g.T, threadIdx.x, blockDim.x);
        for (int c = threadIdx.x; c < ncell; c += blockDim.x, w.next())
            tile[c] = __ldg(grid + (ibase + w.cell(g, o)) * B + b);
        __syncthreads();
        for (int base_s = sp.y; base_s < end; base_s += per_round) {
            const int s = base_s + warp * NT + team;
            const bool active = (team < NT) && (s < end);
            const int sl = active ? s : sp.y;
            const int lz = __ldg(g.pos[DI] + sl) - o[DI] + k;
            const float2 cz = __ldg(g.coef[DI] + (size_t)sl * g.JP[DI] + k);
            float2 acc = make_float2(0.f, 0.f);
            if constexpr (DIM == 1) {
                acc = tile[lz];
            } else {
                const int ly = __ldg(g.pos[DY] + sl) - o[DY];
                float2 cy[JM];
                const float2* src = g.coef[DY] + (size_t)sl * g.JP[DY];
#pragma unroll
                for (int j = 0; j < JM; ++j)
                    cy[j] = (j < g.J[DY]) ? __ldg(src + j) : make_float2(0.f, 0.f);
                if constexpr (DIM == 2) {
#pragma unroll
                    for (int j = 0; j < JM; ++j)
                        if (j < g.J[DY]) cfma(acc, cy[j], tile[(ly + j) * Tz + lz]);
                } else {
                    const int lx = __ldg(g.pos[0] + sl) - o[0];
                    const float2* c0src = g.coef[0] + (size_t)sl * g.JP[0];
#pragma unroll 1
                    for (int i = 0; i < J0; ++i) {
                        const float2* row = tile + ((lx + i) * Ty + ly) * Tz + lz;
                        float2 t = make_float2(0.f, 0.f);
#pragma unroll
                        for (int j = 0; j < JM; ++j)
                            if (j < g.J[DY]) cfma(t, cy[j], row[j * Tz]);
                        cfma(acc, __ldg(c0src + i), t);
                    }
                }
            }
            acc = cmul(acc, cz);
            acc = team_sum(acc, k, TS);
            if (active && k == 0) y[(size_t)__ldg(g.perm + s) * B + b] = acc;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Paired-thread kernels (B == 1 gridding, B < 8 interpolation): the block
// stages the sub-problem's footprint in shared memory in the padded layout
// of tile_strides; in 2D/3D each point is served by two threads 16 lanes
// apart that take alternate taps of the outer axis (x in 3D, y in 2D).  A
// warp thus holds 16 points; the bank-aware point order gives them distinct
// padded addresses mod 16, and the padding puts a point's second thread 16
// banks from its first, so a warp's 32 accesses of one tap fall in 32
// distinct banks whenever the bin's keys allow it.
// ---------------------------------------------------------------------------
// ---- bulk-copy engine (cp.async.bulk) and mbarrier helpers -----------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
// global -> shared copy of `bytes` (multiple of 16, both addresses 16-byte
// aligned) that completes `bytes` transactions on `bar`
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
    return ok != 0;
}
// Wait for phase `parity` of `bar` with a bounded number of polls (each poll
// may suspend the thread for a hardware-chosen interval); false if it ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  int polls = 1 << 22) {
    for (int i = 0; i < polls; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Asynchronous global -> shared copies (cp.async) of 16 or 8 bytes, both
// addresses aligned to the size; cp_async_wait_all waits for the calling
// thread's copies (a barrier then makes every thread's visible).
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_addr(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;" ::: "memory");
}

template <int DIM>
__device__ __forceinline__ int tile_addr(const int (&t)[3], const TileStrides& ts) {
    if constexpr (DIM == 3) return t[0] * ts.sx + t[1] * ts.sy + t[2];
    else if constexpr (DIM == 2) return t[0] * ts.sy + t[1];
    else return t[0];
}

// k2y from the shared tile.  EX: every axis has exactly JM taps.  BULK (one
// coil, 2D/3D, even K and bin along z, tile row no longer than the grid row):
// the tile rows arrive by bulk copies (one or two per row, the second where
// the row wraps around the periodic grid) completing on one mbarrier; the
// bounded wait sets the plan's error flag and returns if the copies never
// land.  Otherwise every thread loads cells through registers.
template <int DIM, int JM, bool EX, bool BULK>
__global__ void __launch_bounds__(256) k2y_spoint_kernel(Geom g, const float2* __restrict__ grid,
                                                         float2* __restrict__ y) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* tile = reinterpret_cast<float2*>(smem_raw);
    const int4 sp = g.sub[blockIdx.x];
    int o[3];
    tile_origin<DIM>(g, sp, o);
    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
    constexpr int P = (DIM > 1) ? 2 : 1;   // threads per point
    constexpr int PW = 32 / P;             // points per warp
    const TileStrides ts = tile_strides(DIM, g.T);
    int ncell = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const int B = g.B;
    const int J0 = EX ? JM : g.J[0];
    const int Jy = EX ? JM : g.J[DY];
    const int Jz = EX ? JM : g.J[DI];
    const size_t ibase = (size_t)sp.w * g.prodK;
    const int lane = threadIdx.x & 31;
    const int q = lane / PW;
    const int pw = lane - q * PW;
    const int per_round = (int)(blockDim.x >> 5) * PW;
    const int end = sp.y + sp.z;

    for (int b = 0; b < B; ++b) {
        if constexpr (BULK) {
            __shared__ __align__(8) uint64_t s_bar;
            const int rowlen = (g.T[DI] + 1) & ~1;   // cells per row, even
            const int nrows = (DIM == 3) ? g.T[0] * g.T[1] : g.T[0];
            if (threadIdx.x == 0) {
                mbar_init(&s_bar, 1);
                mbar_arrive_expect_tx(&s_bar, (uint32_t)(nrows * rowlen) * 8u);
            }
            __syncthreads();
            const int Kz = g.K[DI], oz = o[DI];
            const int n1 = min(rowlen, Kz - oz);
            for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
                size_t rowcell;
                float2* dst;
                if constexpr (DIM == 3) {
                    const int rx = r / g.T[1], ry = r - rx * g.T[1];
                    rowcell = ((size_t)wrapn(o[0] + rx, g.K[0]) * g.K[1] + wrapn(o[1] + ry, g.K[1])) * Kz;
                    dst = tile + rx * ts.sx + ry * ts.sy;
                } else {
                    rowcell = (size_t)wrapn(o[0] + r, g.K[0]) * Kz;
                    dst = tile + r * ts.sy;
                }
                const float2* src = grid + ibase + rowcell;
                bulk_g2s(dst, src + oz, (uint32_t)n1 * 8u, &s_bar);
                if (n1 < rowlen) bulk_g2s(dst + n1, src, (uint32_t)(rowlen - n1) * 8u, &s_bar);
            }
            const bool ok = mbar_wait_bounded(&s_bar, 0);
            if (__syncthreads_or(!ok)) {
                if (threadIdx.x == 0) atomicExch(g.kerr, 1);
                mbar_wait_bounded(&s_bar, 0);   // a second bound for copies still in flight
                return;
            }
        } else {
            TileWalk<DIM> w;
            w.init(g.T, threadIdx.x, blockDim.x);
            for (int c = threadIdx.x; c < ncell; c += blockDim.x, w.next())
                tile[tile_addr<DIM>(w.t, ts)] = __ldg(grid + (ibase + w.cell(g, o)) * B + b);
            __syncthreads();
        }
        for (int base_s = sp.y; base_s < end; base_s += per_round) {
            const int s = base_s + (int)(threadIdx.x >> 5) * PW + pw;
            const bool active = s < end;
            float2 acc = make_float2(0.f, 0.f);
            if (active) {
                const int lz = __ldg(g.pos[DI] + s) - o[DI];
                float2 cz[JM];
                {
                    const float2* src = g.coef[DI] + (size_t)s * g.JP[DI];
#pragma unroll
                    for (int k = 0; k < JM; ++k)
                        cz[k] = (EX || k < Jz) ? __ldg(src + k) : make_float2(0.f, 0.f);
                }
                if constexpr (DIM == 1) {
#pragma unroll
                    for (int k = 0; k < JM; ++k)
                        if (EX || k < Jz) cfma(acc, cz[k], tile[lz + k]);
                } else if constexpr (DIM == 2) {
                    const int ly = __ldg(g.pos[DY] + s) - o[DY];
                    const float2* csrc = g.coef[DY] + (size_t)s * g.JP[DY];
#pragma unroll 1
                    for (int j = q; j < Jy; j += P) {
                        const float2* row = tile + (ly + j) * ts.sy + lz;
                        float2 r = make_float2(0.f, 0.f);
#pragma unroll
                        for (int k = 0; k < JM; ++k)
                            if (EX || k < Jz) cfma(r, cz[k], row[k]);
                        cfma(acc, __ldg(csrc + j), r);
                    }
                } else {
                    const int ly = __ldg(g.pos[DY] + s) - o[DY];
                    const int lx = __ldg(g.pos[0] + s) - o[0];
                    float2 cy[JM];
                    {
                        const float2* src = g.coef[DY] + (size_t)s * g.JP[DY];
#pragma unroll
                        for (int j = 0; j < JM; ++j)
                            cy[j] = (EX || j < Jy) ? __ldg(src + j) : make_float2(0.f, 0.f);
                    }
                    const float2* c0src = g.coef[0] + (size_t)s * g.JP[0];
#pragma unroll 1
                    for (int i = q; i < J0; i += P) {
                        const float2* pl = tile + (lx + i) * ts.sx + ly * ts.sy + lz;
                        float2 t = make_float2(0.f, 0.f);
#pragma unroll
                        for (int j = 0; j < JM; ++j) {
                            if (!EX && j >= Jy) continue;
                            float2 r = make_float2(0.f, 0.f);
#pragma unroll
                            for (int k = 0; k < JM; ++k)
                                if (EX || k < Jz) cfma(r, cz[k], pl[j * ts.sy + k]);
                            cfma(t, cy[j], r);
                        }
                        cfma(acc, __ldg(c0src + i), t);
                    }
                }
            }
            if constexpr (P == 2) {
                acc.x += __shfl_xor_sync(0xffffffffu, acc.x, 16);
                acc.y += __shfl_xor_sync(0xffffffffu, acc.y, 16);
            }
            if (active && q == 0) y[(size_t)__ldg(g.perm + s) * B + b] = acc;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// k2y, coil teams on a shared tile (2D/3D, an even number of coils): the
// block stages its sub-problem's footprint for all coils in shared memory --
// each tile row, Tz cells x B coils, is contiguous in the coil-fastest grid
// and arrives by one or two bulk copies (two where it wraps around the
// periodic grid) -- and teams of G lanes (one point each, lanes over coils)
// gather from it.  Every grid cell of a bin is read from memory once instead
// of once per point that covers it.  EX: every axis has exactly JM taps.
// ---------------------------------------------------------------------------
template <int DIM, int JM, int G, bool EX>
__global__ void __launch_bounds__(512) k2y_ctile_kernel(Geom g, const float2* __restrict__ grid,
                                                        float2* __restrict__ y) {
    static_assert(DIM > 1, "tiles of rows");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t s_bar;
    float2* tile = reinterpret_cast<float2*>(smem_raw);
    // the gather list (bins split only past kGatherSub points) when the plan has one
    const int4 sp = (g.gsub ? g.gsub : g.sub)[blockIdx.x];
    int o[3];
    tile_origin<DIM>(g, sp, o);
    constexpr int DI = DIM - 1;
    constexpr int DY = DIM - 2;
    const int B = g.B;
    const int Tz = g.T[DI], Ty = g.T[DY];
    const int rowB = Tz * B;                       // elements per tile row
    const int nrows = (DIM == 3) ? g.T[0] * g.T[1] : g.T[0];
    const size_t ibase = (size_t)sp.w * g.prodK;
    if (threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        mbar_arrive_expect_tx(&s_bar, (uint32_t)(nrows * rowB) * 8u);
    }
    __syncthreads();
    const int Kz = g.K[DI], oz = o[DI];
    const int n1 = min(Tz, Kz - oz);
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) {
        size_t rowcell;
        if constexpr (DIM == 3) {
            const int rx = r / g.T[1], ry = r - rx * g.T[1];
            rowcell = ((size_t)wrapn(o[0] + rx, g.K[0]) * g.K[1] + wrapn(o[1] + ry, g.K[1])) * Kz;
        } else {
            rowcell = (size_t)wrapn(o[0] + r, g.K[0]) * Kz;
        }
        float2* dst = tile + (size_t)r * rowB;
        const float2* src = grid + (ibase + rowcell) * B;
        bulk_g2s(dst, src + (size_t)oz * B, (uint32_t)(n1 * B) * 8u, &s_bar);
        if (n1 < Tz) bulk_g2s(dst + n1 * B, src, (uint32_t)((Tz - n1) * B) * 8u, &s_bar);
    }
    const bool ok = mbar_wait_bounded(&s_bar, 0);
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicExch(g.kerr, 1);
        mbar_wait_bounded(&s_bar, 0);   // a second bound for copies still in flight
        return;
    }
    const int J0 = EX ? JM : g.J[0];
    const int Jy = EX ? JM : g.J[DY];
    const int Jz = EX ? JM : g.J[DI];
    const int team = threadIdx.x / G, lane = threadIdx.x % G, nteam = blockDim.x / G;
    for (int s = sp.y + team; s < sp.y + sp.z; s += nteam) {
        float2 cz[JM], cy[JM];
        {
            const float2* src = g.coef[DI] + (size_t)s * g.JP[DI];
#pragma unroll
            for (int k = 0; k < JM; ++k)
                cz[k] = (EX || k < Jz) ? __ldg(src + k) : make_float2(0.f, 0.f);
            const float2* srcy = g.coef[DY] + (size_t)s * g.JP[DY];
#pragma unroll
            for (int j = 0; j < JM; ++j)
                cy[j] = (EX || j < Jy) ? __ldg(srcy + j) : make_float2(0.f, 0.f);
        }
        const int lz = __ldg(g.pos[DI] + s) - o[DI];
        const int ly = __ldg(g.pos[DY] + s) - o[DY];
        const int lx = (DIM == 3) ? __ldg(g.pos[0] + s) - o[0] : 0;
        const float2* c0src = g.coef[0] + (size_t)s * g.JP[0];
        const int m = __ldg(g.perm + s);
        for (int b = lane; b < B; b += G) {
            float2 acc = make_float2(0.f, 0.f);
            const float2* tb = tile + lz * B + b;
            if constexpr (DIM == 2) {
#pragma unroll
                for (int j = 0; j < JM; ++j) {
                    if (!EX && j >= Jy) continue;
                    const float2* row = tb + (ly + j) * rowB;
                    float2 t = make_float2(0.f, 0.f);
#pragma unroll
                    for (int k = 0; k < JM; ++k)
                        if (EX || k < Jz) cfma(t, cz[k], row[k * B]);
                    cfma(acc, cy[j], t);
                }
            } else {
#pragma unroll 1
                for (int i = 0; i < J0; ++i) {
                    const float2* pl = tb + ((lx + i) * Ty + ly) * rowB;
                    float2 ti = make_float2(0.f, 0.f);
#pragma unroll
                    for (int j = 0; j < JM; ++j) {
                        if (!EX && j >= Jy) continue;
                        const float2* row = pl + j * rowB;
                        float2 t = make_float2(0.f, 0.f);
#pragma unroll
                        for (int k = 0; k < JM; ++k)
                            if (EX || k < Jz) cfma(t, cz[k], row[k * B]);
                        cfma(ti, cy[j], t);
                    }
                    cfma(acc, __ldg(c0src + i), ti);
                }
            }
            y[(size_t)m * B + b] = acc;
        }
    }
}

// ---------------------------------------------------------------------------
// y2k shared pieces
// ---------------------------------------------------------------------------
// Fixed-point accumulator types: 32-bit with a per-sub-problem scale (fast
// mode) or 64-bit with a global scale (deterministic mode).
template <bool DET> struct Acc;
template <> struct Acc<false> {
    using T = unsigned int;
    static __device__ __forceinline__ T fix(float v, float s) { return (T)__float2int_rn(v * s); }
};
template <> struct Acc<true> {
    using T = unsigned long long;
    static __device__ __forceinline__ T fix(float v, float s) { return (T)__float2ll_rn(v * s); }
};

// Per-coil fixed-point scales of one sub-problem (fast mode), written to
// scale[0..bcur); ends with a block-wide barrier.
__device__ __forceinline__ void subproblem_scales(const Geom& g, const int4& sp, const float2* y,
                                                  int b0, int bcur, float* bound, float* scale) {
    for (int b = threadIdx.x; b < bcur; b += blockDim.x) bound[b] = 0.f;
    __syncthreads();
    const int B = g.B;
    for (int b = 0; b < bcur; ++b) {
        float acc = 0.f;
        for (int s = sp.y + threadIdx.x; s < sp.y + sp.z; s += blockDim.x) {
            const float2 v = __ldg(y + (size_t)__ldg(g.perm + s) * B + b0 + b);
            acc += __ldg(g.wpt + s) * (fabsf(v.x) + fabsf(v.y));
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
        if ((threadIdx.x & 31) == 0 && acc > 0.f) atomicAdd(bound + b, acc);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < bcur; b += blockDim.x) {
        // |sum of any cell| <= bound, so a scale of 2e9 / bound keeps every
        // partial sum below 2e9 < 2^31; the 7% left covers the rounding of the
        // contributions (half a unit each).  Clamped for vanishing bounds.
        const float bb = bound[b];
        scale[b] = (bb > 0.f && isfinite(bb)) ? fminf(2.0e9f / bb, 1.0e30f) : 1.0f;
    }
    __syncthreads();
}

// Flush one accumulated tile chunk into the global grid (float, fast mode)
// or the global fixed-point grid (deterministic mode).  Layout of the tile:
// element e = cell * bcur + b (coil fastest) when CELL_MAJOR, else
// b * ncell + cell; re plane first, im plane at offset nsm.
template <int DIM, bool DET, bool CELL_MAJOR>
__device__ __forceinline__ void flush_tile(const Geom& g, const int (&o)[3], int inst, int ncell,
                                           int b0, int bcur, const typename Acc<DET>::T* tile,
                                           const float* scale, float2* __restrict__ grid,
                                           unsigned long long* __restrict__ igrid) {
    const int nsm = ncell * bcur;
    const size_t ibase = (size_t)inst * g.prodK;
    const int B = g.B;
    auto put = [&](int e, size_t gi, float inv) {
        const typename Acc<DET>::T vx = tile[e], vy = tile[nsm + e];
        if (vx == 0 && vy == 0) return;
        if constexpr (DET) {
            if (vx) atomicAdd(igrid + 2 * gi, (unsigned long long)vx);
            if (vy) atomicAdd(igrid + 2 * gi + 1, (unsigned long long)vy);
        } else {
            atomicAdd(grid + gi, make_float2(__int2float_rn((int)vx) * inv,
                                             __int2float_rn((int)vy) * inv));
        }
    };
    // a tile that does not wrap around the periodic grid addresses its cells
    // with multiply-adds instead of wrapping each coordinate
    bool interior = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) interior = interior && (o[d] + g.T[d] <= g.K[d]);
    auto gcell = [&](const TileWalk<DIM>& w) -> size_t {
        if (!interior) return w.cell(g, o);
        size_t gc = (size_t)(o[0] + w.t[0]);
#pragma unroll
        for (int d = 1; d < DIM; ++d) gc = gc * g.K[d] + (size_t)(o[d] + w.t[d]);
        return gc;
    };
    if constexpr (CELL_MAJOR) {
        // threads split as (cell, coil), coil fastest (bcur <= blockDim): a
        // warp reads consecutive words of the tile and adds to consecutive
        // coils of the grid
        const int cpb = (int)blockDim.x / bcur;   // cells per pass
        const int b = (int)threadIdx.x % bcur, c0 = (int)threadIdx.x / bcur;
        if (c0 >= cpb) return;
        const float inv = DET ? 1.f : 1.f / scale[b];
        TileWalk<DIM> w;
        w.init(g.T, c0, cpb);
        for (int c = c0; c < ncell; c += cpb, w.next())
            put(c * bcur + b, (ibase + gcell(w)) * B + b0 + b, inv);
    } else {
        for (int b = 0; b < bcur; ++b) {
            const float inv = DET ? 1.f : 1.f / scale[b];
            TileWalk<DIM> w;
            w.init(g.T, threadIdx.x, blockDim.x);
            for (int c = threadIdx.x; c < ncell; c += blockDim.x, w.next())
                put(b * ncell + c, (ibase + gcell(w)) * B + b0 + b, inv);
        }
    }
}

// ---------------------------------------------------------------------------
// y2k, z-teams (B < 8): tile layout b-major (lanes of a team hit consecutive
// words of one plane)
// ---------------------------------------------------------------------------
template <int DIM, int JM, bool DET>
__global__ void __launch_bounds__(256) y2k_zteam_kernel(Geom g, const float2* __restrict__ y,
                                                        float2* __restrict__ grid,
                                                        unsigned long long* __restrict__ igrid,
                                                        int bc, const double* __restrict__ dscal) {
    using T = typename Acc<DET>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float s_bound[8], s_scale[8];
    const int4 sp = g.sub[blockIdx.x];
    const int inst = sp.w;
    int o[3];
    tile_origin<DIM>(g, sp, o);
    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
    const int Tz = g.T[DI];
    const int Ty = (DIM > 1) ? g.T[DY] : 1;
    int ncell = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const int B = g.B;
    const int TS = g.J[DI], NT = 32 / TS;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int team = lane / TS, k = lane - team * TS;
    const int J0 = g.J[0];
    T* tile = reinterpret_cast<T*>(smem_raw);

    for (int b0 = 0; b0 < B; b0 += bc) {
        const int bcur = min(bc, B - b0);
        const int nsm = ncell * bcur;
        for (int e = threadIdx.x; e < 2 * nsm; e += blockDim.x) tile[e] = 0;
        if constexpr (DET) {
            if (threadIdx.x < bcur) s_scale[threadIdx.x] = (float)dscal[1];
            __syncthreads();
        } else {
            subproblem_scales(g, sp, y, b0, bcur, s_bound, s_scale);
        }

        const int per_round = nwarps * NT;
        for (int base_s = sp.y; base_s < sp.y + sp.z; base_s += per_round) {
            const int s = base_s + warp * NT + team;
            if (team >= NT || s >= sp.y + sp.z) continue;
            const int lz = __ldg(g.pos[DI] + s) - o[DI] + k;
            const float2 cz = __ldg(g.coef[DI] + (size_t)s * g.JP[DI] + k);
            int ly = 0;
            float2 cy[JM];
            if constexpr (DIM > 1) {
                ly = __ldg(g.pos[DY] + s) - o[DY];
                const float2* src = g.coef[DY] + (size_t)s * g.JP[DY];
#pragma unroll
                for (int j = 0; j < JM; ++j)
                    cy[j] = (j < g.J[DY]) ? __ldg(src + j) : make_float2(0.f, 0.f);
            }
            const int lx = (DIM > 2) ? __ldg(g.pos[0] + s) - o[0] : 0;
            const float2* c0src = g.coef[0] + (size_t)s * g.JP[0];
            const int m = __ldg(g.perm + s);
            for (int b = 0; b < bcur; ++b) {
                const float sc = s_scale[b];
                float2 v = cmulc(__ldg(y + (size_t)m * B + b0 + b), cz);
                v.x *= sc;          // fixed-point scale applied once per point
                v.y *= sc;
                T* re = tile + b * ncell;
                T* im = tile + nsm + b * ncell;
                if constexpr (DIM == 1) {
                    atomicAdd(re + lz, Acc<DET>::fix(v.x, 1.f));
                    atomicAdd(im + lz, Acc<DET>::fix(v.y, 1.f));
                } else {
                    const int ni = (DIM > 2) ? J0 : 1;
#pragma unroll 1
                    for (int i = 0; i < ni; ++i) {
                        const float2 wi = (DIM > 2) ? cmulc(v, __ldg(c0src + i)) : v;
                        const int ci = (DIM > 2) ? (lx + i) * Ty : 0;
#pragma unroll
                        for (int j = 0; j < JM; ++j) {
                            if (j >= g.J[DY]) continue;
                            const float2 w = cmulc(wi, cy[j]);
                            const int cell = (ci + ly + j) * Tz + lz;
                            atomicAdd(re + cell, Acc<DET>::fix(w.x, 1.f));
                            atomicAdd(im + cell, Acc<DET>::fix(w.y, 1.f));
                        }
                    }
                }
            }
        }
        __syncthreads();
        flush_tile<DIM, DET, false>(g, o, inst, ncell, b0, bcur, tile, s_scale, grid, igrid);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// y2k, one thread per point (B < 8): tile layout cell-major, coil fastest.
// EX = every axis has exactly JM neighbours, so no loop guards are needed;
// a single coil (the common case) addresses cells directly.
// ---------------------------------------------------------------------------
template <int DIM, int JM, bool EX, bool DET>
__global__ void __launch_bounds__(128) y2k_point_kernel(Geom g, const float2* __restrict__ y,
                                                        float2* __restrict__ grid,
                                                        unsigned long long* __restrict__ igrid,
                                                        int bc, const double* __restrict__ dscal) {
    using T = typename Acc<DET>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float s_bound[8], s_scale[8];
    const int4 sp = g.sub[blockIdx.x];
    const int inst = sp.w;
    int o[3];
    tile_origin<DIM>(g, sp, o);
    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
    const int Tz = g.T[DI];
    const int Ty = (DIM > 1) ? g.T[DY] : 1;
    int ncell = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const int B = g.B;
    const int J0 = EX ? JM : g.J[0];
    const int Jy = EX ? JM : g.J[DY];
    const int Jz = EX ? JM : g.J[DI];
    T* tile = reinterpret_cast<T*>(smem_raw);

    for (int b0 = 0; b0 < B; b0 += bc) {
        const int bcur = min(bc, B - b0);
        const int nsm = ncell * bcur;
        for (int e = threadIdx.x; e < 2 * nsm; e += blockDim.x) tile[e] = 0;
        if constexpr (DET) {
            if (threadIdx.x < bcur) s_scale[threadIdx.x] = (float)dscal[1];
            __syncthreads();
        } else {
            subproblem_scales(g, sp, y, b0, bcur, s_bound, s_scale);
        }
        T* re = tile;
        T* im = tile + nsm;
        for (int s = sp.y + threadIdx.x; s < sp.y + sp.z; s += blockDim.x) {
            float2 cz[JM], cy[JM];
            {
                const float2* src = g.coef[DI] + (size_t)s * g.JP[DI];
#pragma unroll
                for (int k = 0; k < JM; ++k)
                    cz[k] = (EX || k < Jz) ? __ldg(src + k) : make_float2(0.f, 0.f);
            }
            if constexpr (DIM > 1) {
                const float2* src = g.coef[DY] + (size_t)s * g.JP[DY];
#pragma unroll
                for (int j = 0; j < JM; ++j)
                    cy[j] = (EX || j < Jy) ? __ldg(src + j) : make_float2(0.f, 0.f);
            }
            const int lz = __ldg(g.pos[DI] + s) - o[DI];
            const int ly = (DIM > 1) ? __ldg(g.pos[DY] + s) - o[DY] : 0;
            const int lx = (DIM > 2) ? __ldg(g.pos[0] + s) - o[0] : 0;
            const float2* c0src = g.coef[0] + (size_t)s * g.JP[0];
            const int m = __ldg(g.perm + s);
            for (int b = 0; b < bcur; ++b) {
                const float sc = s_scale[b];
                float2 yv = __ldg(y + (size_t)m * B + b0 + b);
                yv.x *= sc;
                yv.y *= sc;
                const int ni = (DIM > 2) ? J0 : 1;
#pragma unroll 1
                for (int i = 0; i < ni; ++i) {
                    const float2 wi = (DIM > 2) ? cmulc(yv, __ldg(c0src + i)) : yv;
                    const int ci = (DIM > 2) ? (lx + i) * Ty : 0;
#pragma unroll
                    for (int j = 0; j < ((DIM > 1) ? JM : 1); ++j) {
                        if (!EX && DIM > 1 && j >= Jy) continue;
                        const float2 wij = (DIM > 1) ? cmulc(wi, cy[j]) : wi;
                        const int cj = (DIM > 1) ? (ci + ly + j) * Tz + lz : lz;
                        if (bcur == 1) {
                            T* rr = re + cj;
                            T* ii = im + cj;
#pragma unroll
                            for (int k = 0; k < JM; ++k) {
                                if (!EX && k >= Jz) continue;
                                const float2 w = cmulc(wij, cz[k]);
                                atomicAdd(rr + k, Acc<DET>::fix(w.x, 1.f));
                                atomicAdd(ii + k, Acc<DET>::fix(w.y, 1.f));
                            }
                        } else {
#pragma unroll
                            for (int k = 0; k < JM; ++k) {
                                if (!EX && k >= Jz) continue;
                                const float2 w = cmulc(wij, cz[k]);
                                const int e = (cj + k) * bcur + b;
                                atomicAdd(re + e, Acc<DET>::fix(w.x, 1.f));
                                atomicAdd(im + e, Acc<DET>::fix(w.y, 1.f));
                            }
                        }
                    }
                }
            }
        }
        __syncthreads();
        flush_tile<DIM, DET, true>(g, o, inst, ncell, b0, bcur, tile, s_scale, grid, igrid);
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// y2k, paired threads per point (B == 1, 2D/3D, fast mode): 32-bit
// fixed-point tile in the padded layout of tile_strides (re plane, then im
// plane), flushed with float2 atomics.  EX: every axis has exactly JM taps.
// (Multiplying the innermost axis in integers, to save the float-to-integer
// conversions, measured slower than converting each tap.)
// ---------------------------------------------------------------------------
template <int JM>
__device__ __forceinline__ void add_row(unsigned* re, unsigned* im, int c, float2 u,
                                        const float2 (&cz)[JM], int Jz, bool ex) {
#pragma unroll
    for (int k = 0; k < JM; ++k) {
        if (!ex && k >= Jz) continue;
        const float2 w = cmulc(u, cz[k]);
        atomicAdd(re + c + k, Acc<false>::fix(w.x, 1.f));
        atomicAdd(im + c + k, Acc<false>::fix(w.y, 1.f));
    }
}

template <int DIM, int JM, bool EX>
__global__ void __launch_bounds__(256) y2k_spoint_kernel(Geom g, const float2* __restrict__ y,
                                                         float2* __restrict__ grid) {
    static_assert(DIM > 1, "paired gridding splits an outer axis");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float s_bound[1], s_scale[1];
    const int4 sp = g.sub[blockIdx.x];
    int o[3];
    tile_origin<DIM>(g, sp, o);
    constexpr int DI = DIM - 1;
    constexpr int DY = DIM - 2;
    const TileStrides ts = tile_strides(DIM, g.T);
    const int J0 = EX ? JM : g.J[0];
    const int Jy = EX ? JM : g.J[DY];
    const int Jz = EX ? JM : g.J[DI];
    unsigned* re = reinterpret_cast<unsigned*>(smem_raw);
    unsigned* im = re + ts.n;
    {   // zero both planes, 16 bytes per store (2 n is a multiple of 4)
        uint4* z4 = reinterpret_cast<uint4*>(smem_raw);
        for (int e = threadIdx.x; e < ts.n / 2; e += blockDim.x) z4[e] = make_uint4(0u, 0u, 0u, 0u);
    }
    subproblem_scales(g, sp, y, 0, 1, s_bound, s_scale);   // ends with a barrier
    const float sc = s_scale[0];
    const int lane = threadIdx.x & 31;
    const int q = lane >> 4, pw = lane & 15;
    const int per_round = (int)(blockDim.x >> 5) * 16;
    const int end = sp.y + sp.z;
    for (int base_s = sp.y; base_s < end; base_s += per_round) {
        const int s = base_s + (int)(threadIdx.x >> 5) * 16 + pw;
        if (s >= end) continue;
        float2 cz[JM];
        {
            const float2* src = g.coef[DI] + (size_t)s * g.JP[DI];
#pragma unroll
            for (int k = 0; k < JM; ++k)
                cz[k] = (EX || k < Jz) ? __ldg(src + k) : make_float2(0.f, 0.f);
        }
        const int lz = __ldg(g.pos[DI] + s) - o[DI];
        const int ly = __ldg(g.pos[DY] + s) - o[DY];
        float2 yv = __ldg(y + __ldg(g.perm + s));
        yv.x *= sc;
        yv.y *= sc;
        if constexpr (DIM == 2) {
            const float2* csrc = g.coef[DY] + (size_t)s * g.JP[DY];
#pragma unroll 1
            for (int j = q; j < Jy; j += 2)
                add_row<JM>(re, im, (ly + j) * ts.sy + lz, cmulc(yv, __ldg(csrc + j)), cz, Jz, EX);
        } else {
            const int lx = __ldg(g.pos[0] + s) - o[0];
            float2 cy[JM];
            {
                const float2* src = g.coef[DY] + (size_t)s * g.JP[DY];
#pragma unroll
                for (int j = 0; j < JM; ++j)
                    cy[j] = (EX || j < Jy) ? __ldg(src + j) : make_float2(0.f, 0.f);
            }
            const float2* c0src = g.coef[0] + (size_t)s * g.JP[0];
#pragma unroll 1
            for (int i = q; i < J0; i += 2) {
                const float2 wi = cmulc(yv, __ldg(c0src + i));
                const int ci = (lx + i) * ts.sx + ly * ts.sy + lz;
#pragma unroll
                for (int j = 0; j < JM; ++j) {
                    if (!EX && j >= Jy) continue;
                    add_row<JM>(re, im, ci + j * ts.sy, cmulc(wi, cy[j]), cz, Jz, EX);
                }
            }
        }
    }
    __syncthreads();
    int ncell = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const float inv = 1.f / sc;
    const size_t ibase = (size_t)sp.w * g.prodK;
    // a tile that does not wrap around the periodic grid (and a grid with
    // fewer than 2^31 cells) addresses its cells with 32-bit multiply-adds
    bool interior = g.prodK < ((int64_t)1 << 31);
#pragma unroll
    for (int d = 0; d < DIM; ++d) interior = interior && (o[d] + g.T[d] <= g.K[d]);
    TileWalk<DIM> w;
    w.init(g.T, threadIdx.x, blockDim.x);
    if (interior) {
        float2* gb = grid + ibase;
        for (int c = threadIdx.x; c < ncell; c += blockDim.x, w.next()) {
            const int a = tile_addr<DIM>(w.t, ts);
            const unsigned vx = re[a], vy = im[a];
            if (vx == 0u && vy == 0u) continue;
            int gc = o[0] + w.t[0];
#pragma unroll
            for (int d = 1; d < DIM; ++d) gc = gc * g.K[d] + o[d] + w.t[d];
            atomicAdd(gb + gc,
                      make_float2(__int2float_rn((int)vx) * inv, __int2float_rn((int)vy) * inv));
        }
    } else {
        for (int c = threadIdx.x; c < ncell; c += blockDim.x, w.next()) {
            const int a = tile_addr<DIM>(w.t, ts);
            const unsigned vx = re[a], vy = im[a];
            if (vx == 0u && vy == 0u) continue;
            atomicAdd(grid + ibase + w.cell(g, o),
                      make_float2(__int2float_rn((int)vx) * inv, __int2float_rn((int)vy) * inv));
        }
    }
}

// ---------------------------------------------------------------------------
// y2k, coil-teams (B >= 8): tile layout cell-major, coil fastest
// ---------------------------------------------------------------------------
template <int DIM, int JM, int G, bool DET, bool EX>
__global__ void __launch_bounds__(DET ? 256 : 512) y2k_coil_kernel(Geom g, const float2* __restrict__ y,
                                                       float2* __restrict__ grid,
                                                       unsigned long long* __restrict__ igrid,
                                                       int bc, const double* __restrict__ dscal) {
    using T = typename Acc<DET>::T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float s_bound[64], s_scale[64];
    const int4 sp = g.sub[blockIdx.x];
    const int inst = sp.w;
    int o[3];
    tile_origin<DIM>(g, sp, o);
    constexpr int DI = DIM - 1;
    constexpr int DY = (DIM > 1) ? DIM - 2 : 0;
    const int Tz = g.T[DI];
    const int Ty = (DIM > 1) ? g.T[DY] : 1;
    int ncell = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncell *= g.T[d];
    const int B = g.B;
    const int team = threadIdx.x / G, lane = threadIdx.x % G, nteam = blockDim.x / G;
    const int J0 = EX ? JM : g.J[0];
    const int Jy = EX ? JM : g.J[DY];
    const int Jz = EX ? JM : g.J[DI];
    T* tile = reinterpret_cast<T*>(smem_raw);

    for (int b0 = 0; b0 < B; b0 += bc) {
        const int bcur = min(bc, B - b0);
        const int nsm = ncell * bcur;
        for (int e = threadIdx.x; e < 2 * nsm; e += blockDim.x) tile[e] = 0;
        if constexpr (DET) {
            for (int b = threadIdx.x; b < bcur; b += blockDim.x) s_scale[b] = (float)dscal[1];
            __syncthreads();
        } else {
            subproblem_scales(g, sp, y, b0, bcur, s_bound, s_scale);
        }
        T* re = tile;
        T* im = tile + nsm;
        for (int s = sp.y + team; s < sp.y + sp.z; s += nteam) {
            float2 cz[JM], cy[JM];
            {
                const float2* src = g.coef[DI] + (size_t)s * g.JP[DI];
#pragma unroll
                for (int k = 0; k < JM; ++k)
                    cz[k] = (EX || k < Jz) ? __ldg(src + k) : make_float2(0.f, 0.f);
            }
            if constexpr (DIM > 1) {
                const float2* src = g.coef[DY] + (size_t)s * g.JP[DY];
#pragma unroll
                for (int j = 0; j < JM; ++j)
                    cy[j] = (EX || j < Jy) ? __ldg(src + j) : make_float2(0.f, 0.f);
            }
            const int lz = __ldg(g.pos[DI] + s) - o[DI];
            const int ly = (DIM > 1) ? __ldg(g.pos[DY] + s) - o[DY] : 0;
            const int lx = (DIM > 2) ? __ldg(g.pos[0] + s) - o[0] : 0;
            const float2* c0src = g.coef[0] + (size_t)s * g.JP[0];
            const int m = __ldg(g.perm + s);
            for (int b = lane; b < bcur; b += G) {
                const float sc = s_scale[b];
                float2 yv = __ldg(y + (size_t)m * B + b0 + b);
                yv.x *= sc;         // fixed-point scale applied once per point
                yv.y *= sc;
                const int ni = (DIM > 2) ? J0 : 1;
#pragma unroll 1
                for (int i = 0; i < ni; ++i) {
                    const float2 wi = (DIM > 2) ? cmulc(yv, __ldg(c0src + i)) : yv;
                    const int ci = (DIM > 2) ? (lx + i) * Ty : 0;
#pragma unroll
                    for (int j = 0; j < ((DIM > 1) ? JM : 1); ++j) {
                        if (!EX && DIM > 1 && j >= Jy) continue;
                        const float2 wij = (DIM > 1) ? cmulc(wi, cy[j]) : wi;
                        const int cj = (DIM > 1) ? (ci + ly + j) * Tz + lz : lz;
                        T* rr = re + cj * bcur + b;
                        T* ii = im + cj * bcur + b;
#pragma unroll
                        for (int kk = 0; kk < JM; ++kk) {
                            if (!EX && kk >= Jz) continue;
                            const float2 w = cmulc(wij, cz[kk]);
                            atomicAdd(rr + kk * bcur, Acc<DET>::fix(w.x, 1.f));
                            atomicAdd(ii + kk * bcur, Acc<DET>::fix(w.y, 1.f));
                        }
                    }
                }
            }
        }
        __syncthreads();
        flush_tile<DIM, DET, true>(g, o, inst, ncell, b0, bcur, tile, s_scale, grid, igrid);
        __syncthreads();
    }
}

}  // namespace nufft
