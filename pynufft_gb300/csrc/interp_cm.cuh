// Coil-major gridding for plans of 8 or more coils.
//
// The adjoint of a multi-coil plan grids straight into coil-major spectra --
// grid_cm[(inst * B + b) * prod(Kd) + cell] -- the layout its inverse FFTs
// read, so the gridded spectra need no transpose.  (The reference's batch
// layout, coil fastest in x / k / y, linalg/nufft_hsa.py:203-228, is kept at
// the API: images and samples stay coil-fastest.)
//
// Gridding (y2k_rows_kernel).  A block takes one row sub-problem (the points
// of one bin, or of up to four consecutive bins along the innermost axis in
// 3D) and the tile (bins + J-1 halo) it scatters to.  The tile is cut into
// "rows" along the innermost axis (TZ cells each); a warp holds the sums of
// RS rows x CB coils in registers (lane = row slot x coil, TZ complex
// accumulators per lane) and visits, in a fixed order, every point whose
// footprint crosses those rows: u = y conj(c_x c_y) for its row, then the J
// innermost taps acc[pz + k] += u conj(c_z[k]) at register indices chosen by
// a warp-uniform switch on pz.  The points' coefficients and samples (a
// coil chunk at a time) are staged in shared memory by asynchronous copies
// (cp.async) in point order, which land while the block sorts its points by
// row; the visits follow the row order through a packed (offsets, point
// index) list.  No shared-memory atomics
// and no float-to-integer conversions per tap; each lane's row is flushed
// once per row block: float2 atomics into the grid (fast mode), or 64-bit
// fixed-point integer atomics (deterministic mode: the per-row float sums
// are a fixed-order reduction, their combination across tiles is exact, so
// the result is bitwise reproducible).
#pragma once
#include "interp.cuh"

namespace nufft {

// Coils per lane group of the row kernels: 32 when they divide B, else 8.
inline int cm_row_coils(int B) { return (B % 32 == 0) ? 32 : 8; }

// Row slots of a warp: RS0 x RS1 (axis 0 x axis 1 rows) with RS0 * RS1 =
// 32 / CB; 2D rows run along axis 1 and are indexed by axis 0 only.
template <int DIM, int CB>
struct RowSlots {
    static constexpr int RS = 32 / CB;
    static constexpr int RS0 = (DIM == 2) ? RS : ((RS == 4) ? 2 : 1);
    static constexpr int RS1 = (DIM == 2) ? 1 : RS / RS0;
};

// acc[PZ + k] += u * conj(cz[k]), k < JM, at compile-time register indices.
template <int PZ, int TZ, int JM>
__device__ __forceinline__ void row_taps(float2 (&acc)[TZ], float2 u, const float2 (&cz)[JM]) {
    if constexpr (PZ + JM <= TZ) {
#pragma unroll
        for (int k = 0; k < JM; ++k) {
            acc[PZ + k].x = fmaf(u.x, cz[k].x, fmaf(u.y, cz[k].y, acc[PZ + k].x));
            acc[PZ + k].y = fmaf(u.y, cz[k].x, fmaf(-u.x, cz[k].y, acc[PZ + k].y));
        }
    }
}

template <int TZ, int JM>
__device__ __forceinline__ void row_taps_at(int pz, float2 (&acc)[TZ], float2 u,
                                            const float2 (&cz)[JM]) {
    static_assert(TZ - JM + 1 <= 32, "at most 32 tap offsets per row");
    switch (pz) {
#define NUFFT_ROW_CASE(c) \
    case c: row_taps<c, TZ, JM>(acc, u, cz); break;
        NUFFT_ROW_CASE(0) NUFFT_ROW_CASE(1) NUFFT_ROW_CASE(2) NUFFT_ROW_CASE(3)
        NUFFT_ROW_CASE(4) NUFFT_ROW_CASE(5) NUFFT_ROW_CASE(6) NUFFT_ROW_CASE(7)
        NUFFT_ROW_CASE(8) NUFFT_ROW_CASE(9) NUFFT_ROW_CASE(10) NUFFT_ROW_CASE(11)
        NUFFT_ROW_CASE(12) NUFFT_ROW_CASE(13) NUFFT_ROW_CASE(14) NUFFT_ROW_CASE(15)
        NUFFT_ROW_CASE(16) NUFFT_ROW_CASE(17) NUFFT_ROW_CASE(18) NUFFT_ROW_CASE(19)
        NUFFT_ROW_CASE(20) NUFFT_ROW_CASE(21) NUFFT_ROW_CASE(22) NUFFT_ROW_CASE(23)
        NUFFT_ROW_CASE(24) NUFFT_ROW_CASE(25) NUFFT_ROW_CASE(26) NUFFT_ROW_CASE(27)
        NUFFT_ROW_CASE(28) NUFFT_ROW_CASE(29) NUFFT_ROW_CASE(30) NUFFT_ROW_CASE(31)
#undef NUFFT_ROW_CASE
        default: break;
    }
}

// Counting sort of a sub-problem's points by row key (in-block):
// list[off[k] ..] = the local indices i, ascending, of the points whose row
// key is k.  key(i) must lie in [0, nkey).  Warp w ranks the contiguous run
// of points [w * chunk, (w + 1) * chunk) in rounds of 32 with match-any
// peer masks, so the order is fixed by the inputs alone.  Uses the per-warp
// histogram wcnt[nwarps][nkey]; ends with a block barrier.
template <typename KeyFn>
__device__ void sort_rows(int P, int nkey, KeyFn key, int* __restrict__ wcnt,
                          int* __restrict__ off, int* __restrict__ list) {
    const int nwarps = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunk = ((P + nwarps - 1) / nwarps + 31) & ~31;
    const int first = w * chunk, last = min(P, first + chunk);
    for (int e = threadIdx.x; e < nwarps * nkey; e += blockDim.x) wcnt[e] = 0;
    __syncthreads();
    int* mine = wcnt + w * nkey;
    // pass 1: points per (warp, key)
    for (int base = first; base < last; base += 32) {
        const int i = base + lane;
        const int k = (i < last) ? key(i) : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, k);
        if (k >= 0 && lane == __ffs(peers) - 1) mine[k] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per key: exclusive prefixes over warps in place, totals into off[k + 1]
    for (int k = threadIdx.x; k < nkey; k += blockDim.x) {
        int run = 0;
        for (int q = 0; q < nwarps; ++q) {
            const int c = wcnt[q * nkey + k];
            wcnt[q * nkey + k] = run;
            run += c;
        }
        off[k + 1] = run;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        off[0] = 0;
        for (int k = 0; k < nkey; ++k) off[k + 1] += off[k];
    }
    __syncthreads();
    // pass 2: place each point after its warp's earlier points of that key
    for (int base = first; base < last; base += 32) {
        const int i = base + lane;
        const int k = (i < last) ? key(i) : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, k);
        if (k >= 0) list[off[k] + mine[k] + __popc(peers & ((1u << lane) - 1u))] = i;
        __syncwarp();
        if (k >= 0 && lane == __ffs(peers) - 1) mine[k] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
}

// Shared memory of y2k_rows_kernel (bytes), for nkey row keys, at most P
// points and a block of nwarps warps: the staged per-point data
// (coefficients, tile offsets in point order and packed in row order,
// sample index) and the row sort's histogram, offsets and list.
__host__ __device__ inline size_t rows_smem(int DIM, int JM, int nkey, int P, int nwarps, int CB) {
    const size_t ints = sizeof(int) * ((size_t)3 * P + (size_t)nwarps * nkey + nkey + 1 + P);
    const size_t sy = sizeof(float2) * (size_t)P * CB + 16;
    return sizeof(float2) * (size_t)P * DIM * JM + ints + 16 + sy;
}

// Row gridding.  One block per row sub-problem: up to g.rgroup consecutive
// bins along the innermost axis (3D), at most row_sub_cap points; the tile is
// (bs0 + J - 1) x (bs1 + J - 1) rows of TZ = rgroup * bs_z + J - 1 cells.
// 3D: at most 80 registers, three blocks per SM (8-coil kooshball adjoint
// 11.0 -> 9.6 ms fast, 13.3 -> 11.9 ms deterministic); 2D: no minimum (0),
// the compiler's choice of ~80 registers ran faster than the same bound.
template <int DIM, int JM, int TZ, int CB, bool DET>
__global__ void __launch_bounds__(256, (DIM == 3) ? 3 : 0) y2k_rows_kernel(Geom g, const float2* __restrict__ y,
                                                       float2* __restrict__ grid,
                                                       unsigned long long* __restrict__ igrid,
                                                       const double* __restrict__ dscal) {
    static_assert(DIM == 2 || DIM == 3, "rows of a 2D or 3D tile");
    static_assert(JM % 2 == 0, "coefficient rows staged in 16-byte pieces");
    static_assert(TZ <= 64, "tap offset packed in 6 bits");
    using RSl = RowSlots<DIM, CB>;
    constexpr int RS0 = RSl::RS0, RS1 = RSl::RS1;
    constexpr int DI = DIM - 1;
    constexpr int PC = DIM * JM; // staged coefficients per point
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int4 sp = g.rsub[blockIdx.x];
    const int P = sp.z;
    int o[3];
    tile_origin<DIM>(g, sp, o);
    const int bs0 = g.bs[0], bs1 = (DIM == 3) ? g.bs[1] : 1;
    const int nkey = bs0 * bs1;
    const int nwarps = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    constexpr int PCAP = (DIM == 2) ? kRowSub2 : kRowSub3;   // points per sub-problem at most
    static_assert(PCAP <= 1024, "point index packed in 10 bits");
    float2* scoef = reinterpret_cast<float2*>(smem_raw);                 // PCAP x DIM x JM, point order
    int* sinfo = reinterpret_cast<int*>(scoef + (size_t)PCAP * PC);      // row order, packed
    int* sm = sinfo + PCAP;                // sample index, point order
    int* sraw = sm + PCAP;                 // point order: pz | lx << 6 | ly << 14
    int* wcnt = sraw + PCAP;
    int* off = wcnt + nwarps * nkey;
    int* list = off + nkey + 1;
    // the samples of the current coil chunk, PCAP x CB in point order,
    // 16-byte aligned
    float2* sy = reinterpret_cast<float2*>(
        (reinterpret_cast<uintptr_t>(list + PCAP) + 15) & ~static_cast<uintptr_t>(15));
    const int B = g.B;
    const bool y16 = (reinterpret_cast<uintptr_t>(y) & 15) == 0;
    // the samples of coils [b0, b0 + CB) of every point, by asynchronous copies
    auto stage_samples = [&](int b0) {
        if (y16) {
            constexpr int H = CB / 2;
            for (int e = threadIdx.x; e < P * H; e += blockDim.x) {
                const int i = e / H, c = 2 * (e - i * H);
                cp_async16(sy + i * CB + c, y + (size_t)sm[i] * B + b0 + c);
            }
        } else {
            for (int e = threadIdx.x; e < P * CB; e += blockDim.x) {
                const int i = e / CB, c = e - i * CB;
                cp_async8(sy + e, y + (size_t)sm[i] * B + b0 + c);
            }
        }
    };

    const int* __restrict__ pos0 = g.pos[0];
    const int* __restrict__ pos1 = g.pos[DIM == 3 ? 1 : 0];
    // per point (point order): tile offsets, sample index; the coefficients
    // (consecutive points' rows are contiguous) and the first coil chunk's
    // samples start copying asynchronously and land during the row sort
    for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int s = sp.y + i;
        const int lx = __ldg(pos0 + s) - o[0];
        const int ly = (DIM == 3) ? __ldg(pos1 + s) - o[1] : 0;
        const int pz = __ldg(g.pos[DI] + s) - o[DI];
        sraw[i] = pz | (lx << 6) | (ly << 14);
        sm[i] = __ldg(g.perm + s);
    }
    {
        constexpr int CQ = JM / 2;   // 16-byte pieces of one axis's coefficients
        for (int e = threadIdx.x; e < P * DIM * CQ; e += blockDim.x) {
            const int i = e / (DIM * CQ), r = e - i * (DIM * CQ), d = r / CQ, q = r - d * CQ;
            cp_async16(scoef + (size_t)i * PC + d * JM + 2 * q,
                       g.coef[d] + (size_t)(sp.y + i) * g.JP[d] + 2 * q);
        }
    }
    __syncthreads();
    stage_samples(0);
    auto key = [&](int i) {
        const int r = sraw[i];
        const int lx = (r >> 6) & 255;
        if constexpr (DIM == 3) return lx * bs1 + ((r >> 14) & 255);
        return lx;
    };
    sort_rows(P, nkey, key, wcnt, off, list);
    // row order: packed offsets and the point index
    for (int j = threadIdx.x; j < P; j += blockDim.x) {
        const int i = list[j];
        sinfo[j] = sraw[i] | (i << 22);
    }
    cp_async_wait_all();
    __syncthreads();

    const int T0 = g.T[0], T1 = (DIM == 3) ? g.T[1] : 1;
    const int nrb0 = (T0 + RS0 - 1) / RS0, nrb1 = (T1 + RS1 - 1) / RS1;
    const int nrb = nrb0 * nrb1;
    const int slot = lane / CB, b = lane % CB;
    const int gx = slot / RS1, gy = slot % RS1;
    const size_t ibase = (size_t)sp.w * B;
    const float fscale = DET ? (float)dscal[1] : 1.f;
    // a tile that does not wrap around the periodic grid addresses rows and
    // cells without wrapping
    bool interior = o[DI] + TZ <= g.K[DI];
#pragma unroll
    for (int d = 0; d < DIM - 1; ++d) interior = interior && (o[d] + g.T[d] <= g.K[d]);
    const int Kz = g.K[DI];

    // 3D: row blocks after each warp's first are handed out in the order
    // warps ask for them (their work differs: edge rows are crossed by fewer
    // points, and points are not spread evenly: the adjoint of an 8-coil,
    // 8M-point kooshball on 384^3 went 23.6 -> 21.2 ms deterministic, 18.3 ->
    // 16.4 ms fast); which warp sums a row block does not change its sums.  2D keeps the fixed assignment (J = 6: every warp
    // gets the same number of lx values, and dynamic hand-out measured no
    // faster).
    __shared__ int s_next_rb;
    auto next_rb = [&](int rb) {
        if constexpr (DIM == 2) {
            return rb + nwarps;
        } else {
            int v = 0;
            if (lane == 0) v = atomicAdd(&s_next_rb, 1);
            return __shfl_sync(0xffffffffu, v, 0);
        }
    };
    for (int b0 = 0; b0 < B; b0 += CB) {
        if (b0 > 0) {   // the next chunk's samples (the first came with the sort)
            __syncthreads();        // the previous chunk's samples are read
            stage_samples(b0);
            cp_async_wait_all();
            __syncthreads();
        }
        if (DIM == 3) {
            __syncthreads();   // every warp is done with the previous coil chunk
            if (threadIdx.x == 0) s_next_rb = nwarps;
            __syncthreads();
        }
        for (int rb = warp; rb < nrb; rb = next_rb(rb)) {
            const int R0 = (rb / nrb1) * RS0, R1 = (rb % nrb1) * RS1;
            float2 acc[TZ];
#pragma unroll
            for (int c = 0; c < TZ; ++c) acc[c] = make_float2(0.f, 0.f);
            bool touched = false;
            const int lx_lo = max(0, R0 - JM + 1), lx_hi = min(bs0 - 1, R0 + RS0 - 1);
            const int ly_lo = max(0, R1 - JM + 1), ly_hi = min(bs1 - 1, R1 + RS1 - 1);
            for (int lx = lx_lo; lx <= lx_hi; ++lx) {
                const int kb = lx * bs1;
                const int j0 = off[kb + ly_lo], j1 = off[kb + ly_hi + 1];
                if (j0 >= j1) continue;
                touched = true;
                const int ix = R0 + gx - lx;
                for (int j = j0; j < j1; ++j) {
                    const int info = sinfo[j];
                    const int pi = info >> 22;   // the point's index in the sub-problem
                    const float2 yv = sy[pi * CB + b];
                    const float2* cj = scoef + (size_t)pi * PC;
                    float2 w = make_float2(0.f, 0.f);
                    if constexpr (DIM == 3) {
                        const int iy = R1 + gy - ((info >> 14) & 255);
                        if (ix >= 0 && ix < JM && iy >= 0 && iy < JM) w = cmul(cj[ix], cj[JM + iy]);
                    } else {
                        if (ix >= 0 && ix < JM) w = cj[ix];
                    }
                    float2 cz[JM];
#pragma unroll
                    for (int k = 0; k < JM; ++k) cz[k] = cj[DI * JM + k];
                    row_taps_at<TZ, JM>(info & 63, acc, cmulc(yv, w), cz);
                }
            }
            if (!touched) continue;   // warp-uniform: no point crosses these rows
            // flush each lane's row (row slot, coil) straight from registers
            const int rx = R0 + gx, ry = R1 + gy;
            if (rx < T0 && ry < T1) {
                // the row's first cell: system-contiguous spectra, or
                // interleaved along the first axis (slab X of coil b at
                // (X B + b) times the slab size)
                const size_t X = interior ? o[0] + rx : wrapn(o[0] + rx, g.K[0]);
                size_t rbase;
                size_t cs = 1;   // element stride of consecutive cells of the row
                if constexpr (DIM == 3) {
                    const size_t Y = interior ? o[1] + ry : wrapn(o[1] + ry, g.K[1]);
                    if (g.cm_il == 2) {
                        rbase = ((size_t)sp.w * g.prodK + (X * g.K[1] + Y) * Kz) * B + b0 + b;
                        cs = B;
                    } else {
                        rbase = g.cm_il ? ((X * B + b0 + b) * g.K[1] + Y) * Kz
                                        : (ibase + b0 + b) * (size_t)g.prodK + (X * g.K[1] + Y) * Kz;
                    }
                } else {
                    if (g.cm_il == 2) {
                        rbase = ((size_t)sp.w * g.prodK + X * Kz) * B + b0 + b;
                        cs = B;
                    } else {
                        rbase = g.cm_il ? (X * B + b0 + b) * Kz
                                        : (ibase + b0 + b) * (size_t)g.prodK + X * Kz;
                    }
                }
                // a row holds TZ <= Kz cells, so it wraps at most once: cells
                // [0, cw) from o_z on, cells [cw, TZ) from 0
                const int cw = interior ? TZ : Kz - o[DI];
                const size_t e0 = rbase + (size_t)o[DI] * cs;
#pragma unroll
                for (int c = 0; c < TZ; ++c) {
                    const float2 v = acc[c];
                    if (v.x == 0.f && v.y == 0.f) continue;
                    // (wrapped past the row end: back Kz cells)
                    const size_t e =
                        (size_t)((int64_t)e0 + (int64_t)((c < cw) ? c : c - Kz) * (int64_t)cs);
                    if constexpr (DET) {
                        atomicAdd(igrid + 2 * e, (unsigned long long)__float2ll_rn(v.x * fscale));
                        atomicAdd(igrid + 2 * e + 1, (unsigned long long)__float2ll_rn(v.y * fscale));
                    } else {
                        atomicAdd(grid + e, v);
                    }
                }
            }
        }
    }
}

}  // namespace nufft
