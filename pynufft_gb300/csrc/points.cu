// Non-uniform points -> bin-sorted per-axis min-max interpolation tables.
//
// This is the GPU counterpart of the interpolator build in helper.plan
// (src/_helper/helper.py:736-786): instead of the M x prod(Jd) complex128 CSR
// (full_kron/create_csr, helper.py:449-480, 285-311) it keeps, per axis and per
// point, the J coefficients conj(u) and the first grid index of the
// footprint -- the "pELL" idea of helper.py:346-393 -- in bin-sorted order.
// The Kronecker product of the per-axis tables is formed in registers by the
// gather/scatter kernels (interp.cu).
//
// Pipeline (one stream, one host sync at the end to size the sub-problem list):
//   1. bin_points      : om -> first footprint index per axis, bin id, bank key,
//                        rank among the bin's points of that key
//   2. scan            : bin counts -> bin starts (counting sort)
//   3. deal_bins       : each (key, rank) of a bin -> its slot in the bin
//   4. build_tables    : FP64 min-max coefficients (helper.py:606-618,
//                        1086-1117, 148-162) written at the sorted slot
//   5. subproblems     : bins split into chunks of <= maxsub points
#include "nufft_internal.cuh"

#include <cub/device/device_radix_sort.cuh>

#include <cmath>
#include <algorithm>
#include <cstring>

namespace nufft {

// ---------------------------------------------------------------------------
// per-axis constants on the device
// ---------------------------------------------------------------------------
struct AxisTab {
    double cs[2 * NUFFT_MAXL + NUFFT_MAXJ + 2];  // cos(pi n N/K), n = -(L+J) .. L
    double ss[2 * NUFFT_MAXL + NUFFT_MAXJ + 2];  // sin(pi n N/K)
    double rc[NUFFT_MAXJ], rs[NUFFT_MAXJ];       // cos, sin(gam (N-1)/2 j), j = 0..J-1
};

struct PointsArgs {
    int ndim;
    AxisConst ax[3];
};

__device__ __forceinline__ int inst_of(const int64_t* start, int ninst, int64_t m) {
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= m) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Bank keys in use (the points that share a warp of the gridding /
// interpolation kernels): 32 / G for coil teams of G lanes, else bank_keys.
__host__ __device__ inline int keys_in_use(int ndim, int B) {
    return (B >= 8) ? 32 / ((B >= 32) ? 32 : 8) : bank_keys(ndim);
}

// Step 1: bins.  koff = floor(om/gam - J/2) (nufft_offset, helper.py:900-907);
// the footprint along an axis is (koff + j) mod K, j = 1..J (OMEGA_k,
// helper.py:164-210), so its first index is pos = (koff + 1) mod K.
// Within a bin, points are further keyed by the shared-memory bank of their
// footprint origin in the padded tile layout (tile_strides; address mod 16
// in 2D/3D, mod 32 in 1D); step 3 deals the keys so that the points that
// share a warp start in distinct banks wherever the bin allows it.
__global__ void bin_points_kernel(const double* __restrict__ om, int64_t M, int ndim,
                                  const AxisConst* __restrict__ axc, Geom g,
                                  int* __restrict__ bin_of, int* __restrict__ rank_of,
                                  int* __restrict__ bucket_count, int* __restrict__ err) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
         m += (int64_t)gridDim.x * blockDim.x) {
        int inst = (g.ninst > 1) ? inst_of(g.inst_start, g.ninst, m) : 0;
        int64_t bin = 0;
        int lp[3] = {0, 0, 0};
        bool ok = true;
        for (int d = 0; d < ndim; ++d) {
            double w = om[m * ndim + d];
            if (!isfinite(w)) { ok = false; break; }
            const AxisConst& a = axc[d];
            double t = w / a.gam;
            double koff = floor(t - a.J * 0.5);
            double q = koff + 1.0;
            double r = q - a.K * floor(q / a.K);
            int pos = (int)r;
            if (pos >= a.K) pos -= a.K;
            if (pos < 0) pos += a.K;
            const int b = pos / g.bs[d];
            bin = bin * g.nb[d] + b;
            lp[d] = pos - b * g.bs[d];
        }
        if (!ok) {
            atomicOr(err, 1);
            bin_of[m] = -1;
            continue;
        }
        bin += (int64_t)inst * g.nbin_inst;
        // bank key: the point's first footprint cell in the tile layout of
        // its gridding kernel, modulo the points that share a warp there
        int key;
        if (g.B >= 8) {
            // coil teams of G lanes, cell-major tile with the coils fastest:
            // 32 / G points per warp, banks set by the flat cell mod 32 / G
            int flat = lp[0];
            for (int d = 1; d < ndim; ++d) flat = flat * g.T[d] + lp[d];
            key = flat % keys_in_use(ndim, g.B);
        } else {
            const TileStrides ts = tile_strides(ndim, g.T);
            const int addr = (ndim == 3) ? lp[0] * ts.sx + lp[1] * ts.sy + lp[2]
                             : (ndim == 2) ? lp[0] * ts.sy + lp[1] : lp[0];
            key = addr & (bank_keys(ndim) - 1);
        }
        bin_of[m] = (int)(bin * 32 + key);
        rank_of[m] = atomicAdd(&bucket_count[bin * 32 + key], 1);
    }
}

// Deterministic ranks.  The counter of bin_points_kernel ranks a bucket's
// points (bin, bank key) in the order threads reach it, which changes from
// run to run; the tables would then order a bin's points differently on
// every plan, and so would the row gridding's fixed-order float sums.
// Instead: the bucket ids sorted stably (a radix sort, the point indices as
// values), and rank = position - the bucket's first position, i.e. the
// number of points of lower index in the bucket.  Invalid points (bin -1)
// take the extra bucket nb32 and no rank.
__global__ void rank_keys_kernel(const int* __restrict__ bin_of, int64_t M, unsigned nb32,
                                 unsigned* __restrict__ keys, int* __restrict__ idx) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
         m += (int64_t)gridDim.x * blockDim.x) {
        const int b = bin_of[m];
        keys[m] = (b < 0) ? nb32 : (unsigned)b;
        idx[m] = (int)m;
    }
}

__global__ void bucket_head_kernel(const unsigned* __restrict__ keys, int64_t M,
                                   int* __restrict__ head) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M;
         i += (int64_t)gridDim.x * blockDim.x)
        if (i == 0 || keys[i] != keys[i - 1]) head[keys[i]] = (int)i;
}

__global__ void sorted_rank_kernel(const unsigned* __restrict__ keys, const int* __restrict__ idx,
                                   int64_t M, unsigned nb32, const int* __restrict__ head,
                                   int* __restrict__ rank_of) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < M;
         i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned k = keys[i];
        if (k < nb32) rank_of[idx[i]] = (int)i - head[k];
    }
}

// Step 3: the order of each bin's points (one thread per bin).  The bin is
// dealt into groups of nk slots -- the points that share a warp -- group by
// group, restarting at each sub-problem boundary (multiples of maxsub).  A
// group takes at most L points of any bank key, L the least level that fills
// it, and the points of level L come from the fullest buckets, so a key whose
// bucket outlasts the others is spread over many groups instead of crowding
// the last ones.  (For 16 keys and ~244 points per bin, a round-robin deal
// costs ~1.68x the conflict-free shared-memory wavefronts, this ~1.49x; no
// order does better than max(groups, largest bucket) ~1.43x.)  Output:
// slot[bin_start + (points of lower keys) + rank] = slot within the bin.
__global__ void deal_bins_kernel(const int* __restrict__ bucket_count,
                                 const int* __restrict__ bin_start, int64_t nbins, int nk,
                                 int maxsub, int* __restrict__ slot) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbins;
         b += (int64_t)gridDim.x * blockDim.x) {
        const int* c = bucket_count + b * 32;
        int left[32], pre[32], used[32], take[32];
        int tot = 0;
        for (int k = 0; k < nk; ++k) {
            left[k] = c[k];
            pre[k] = tot;
            used[k] = 0;
            tot += c[k];
        }
        int* out = slot + bin_start[b];
        int pos = 0;
        while (pos < tot) {
            const int slots = min(min(nk, tot - pos), maxsub - pos % maxsub);
            int nonempty = 0;
            for (int k = 0; k < nk; ++k) nonempty += (left[k] > 0) ? 1 : 0;
            // least level: at least ceil(slots / nonempty); the search ends
            // where the sum reaches tot - pos >= slots
            int L = (slots + nonempty - 1) / nonempty;
            for (;; ++L) {
                int sum = 0;
                for (int k = 0; k < nk; ++k) sum += min(left[k], L);
                if (sum >= slots) break;
            }
            int filled = 0;
            for (int k = 0; k < nk; ++k) {
                take[k] = min(left[k], L - 1);
                filled += take[k];
            }
            for (; filled < slots; ++filled) {   // level L from the fullest buckets
                int best = -1;
                for (int k = 0; k < nk; ++k)
                    if (left[k] >= L && take[k] < L && (best < 0 || left[k] > left[best])) best = k;
                if (best < 0) break;
                ++take[best];
            }
            for (int k = 0; k < nk; ++k) {
                for (int t = 0; t < take[k]; ++t) out[pre[k] + used[k]++] = pos++;
                left[k] -= take[k];
            }
        }
    }
}

// Points per bin from the 32 bank buckets of each bin.
__global__ void bin_totals_kernel(const int* __restrict__ bucket_count, int64_t nbins,
                                  int* __restrict__ bin_count) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbins;
         b += (int64_t)gridDim.x * blockDim.x) {
        int t = 0;
        for (int k = 0; k < 32; ++k) t += bucket_count[b * 32 + k];
        bin_count[b] = t;
    }
}

// Exclusive scan of n ints by one block of 1024 threads; out[n] = total.
__global__ void scan_kernel(const int* __restrict__ in, int* __restrict__ out, int64_t n) {
    __shared__ long long part[1024];
    const int tid = threadIdx.x;
    const int64_t chunk = (n + blockDim.x - 1) / blockDim.x;
    const int64_t b = tid * chunk, e = min(n, b + chunk);
    long long s = 0;
    for (int64_t i = b; i < e; ++i) s += in[i];
    part[tid] = s;
    __syncthreads();
    for (int off = 1; off < blockDim.x; off <<= 1) {
        long long v = (tid >= off) ? part[tid - off] : 0;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    long long run = part[tid] - s;
    for (int64_t i = b; i < e; ++i) {
        out[i] = (int)run;
        run += in[i];
    }
    if (tid == blockDim.x - 1) out[n] = (int)part[tid];
}

// 1/x in FP64 (x normal, |x| well inside the float range) from a float32
// reciprocal refined by two Newton-Raphson steps y <- y + y (1 - x y): the
// relative error squares at each step (~2^-23 -> ~2^-46 -> below FP64
// rounding), at four FMAs instead of a full FP64 division.
__device__ __forceinline__ double rcp_newton(double x) {
    double y = (double)__frcp_rn((float)x);
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
}

__device__ __forceinline__ double sinc_direct(double x) {
    if (x == 0.0) return 1.0;
    return sinpi(x) / (M_PI * x);
}

// One axis of the min-max interpolator for one point, FP64.
//   t = om/gam, koff = floor(t - J/2), dk = t - koff, arg_j = dk - j
//   r_j = sum_l alpha_|l| sinc((arg_j + l)/(K/N))              (nufft_r)
//   c = T r                                                      (min_max)
//   u_j = exp(i gam (N-1)/2 arg_j) c_j exp(-i om N/2)            (OMEGA_u)
//   out_j = conj(u_j)                                            (.T.conj())
// The sinc argument is (dk + n) N/K with n = l - j, so only the 2L+J
// distinct reciprocals 1/(dk + n) are computed, and sin(pi (dk+n) N/K) uses
// the angle-sum identity with tabulated sin/cos(pi n N/K); the terms with
// |dk + n| < 1 are evaluated directly so the sinc keeps full relative
// accuracy near its peak.  The J phase factors come from one sincos rotated
// by the tabulated exp(-i gam (N-1)/2 j).  This GPU's FP64 rate is low, so
// transcendental calls are kept to a few per axis and the sinc denominators
// use a Newton-refined reciprocal instead of FP64 divisions.
// FP64 min-max coefficients c_j(dk), j = 0..J-1, of one axis:
//   r_j = sum_l alpha_|l| sinc((dk - j + l) N/K)   (nufft_r), c = T r (min_max).
// Each sinc value (index n = l - j in [-(L+J), L-1]) is added straight into
// the register accumulators of the J outputs it feeds (l ascending for every
// j, as a direct sum would).
template <int JM>
__device__ void minmax_c(const AxisConst& a, const AxisTab& tab, double dk, double (&c)[JM]) {
    const int J = a.J, L = a.L;
    double s0, c0;
    sincospi(dk * a.inv_ratio, &s0, &c0);
    double r[JM];
#pragma unroll
    for (int j = 0; j < JM; ++j) r[j] = 0.0;
    const double pr = M_PI * a.inv_ratio;
    for (int n = -(L + J); n <= L - 1; ++n) {
        const double xn = dk + n;
        const int q = n + L + J;
        const double sv = (fabs(xn) < 1.0) ? sinc_direct(xn * a.inv_ratio)
                                           : (s0 * tab.cs[q] + c0 * tab.ss[q]) * rcp_newton(pr * xn);
#pragma unroll
        for (int j = 0; j < JM; ++j) {
            const int l = n + j + 1;
            if (j < J && l >= -L && l <= L) r[j] += a.alpha[l < 0 ? -l : l] * sv;
        }
    }
#pragma unroll
    for (int j = 0; j < JM; ++j) {
        double acc = 0.0;
#pragma unroll
        for (int i = 0; i < JM; ++i)
            if (j < J && i < J) acc += a.T[j * J + i] * r[i];
        c[j] = acc;
    }
}

// The coefficients depend on the point only through dk = t - koff, which
// lies in [J/2, J/2 + 1).  They are smooth there, so they are tabulated once
// per axis at kCTabS samples per unit of dk (plus one guard sample at each
// end) and evaluated per point by 4-point cubic Lagrange interpolation in
// FP64: the interpolation error, O(h^4) with h = 1/kCTabS, is below 1e-10
// relative, far under the float32 rounding of the stored tables, at a small
// fraction of the FP64 work of the direct sum (this GPU's FP64 rate is low).
constexpr int kCTabS = 512;
constexpr int kCTabN = kCTabS + 3;

template <int JM>
__global__ void ctab_kernel(const AxisConst* __restrict__ axc, const AxisTab* __restrict__ tabs,
                            int ndim, double* __restrict__ ctab) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ndim * kCTabN) return;
    const int d = i / kCTabN, k = i - d * kCTabN;
    const AxisConst& a = axc[d];
    const double dk = 0.5 * a.J + (double)(k - 1) / kCTabS;
    double c[JM];
    minmax_c<JM>(a, tabs[d], dk, c);
#pragma unroll
    for (int j = 0; j < JM; ++j) ctab[(size_t)i * JM + j] = c[j];
}

// One axis of the min-max interpolator for one point.
//   t = om/gam, koff = floor(t - J/2), dk = t - koff, arg_j = dk - j
//   c_j(dk) from the table (see above)
//   u_j = exp(i gam (N-1)/2 arg_j) c_j exp(-i om N/2)            (OMEGA_u)
//   out_j = conj(u_j)                                            (.T.conj())
// The J phase factors come from one FP64 sincos rotated by the tabulated
// exp(-i gam (N-1)/2 j).
template <int JM>
__device__ float axis_coefs(const AxisConst& a, const AxisTab& tab, const double* __restrict__ ctab,
                            double w, float2* __restrict__ dst, int JP) {
    const int J = a.J;
    double t = w / a.gam;
    double koff = floor(t - J * 0.5);
    double dk = t - koff;
    double u = (dk - 0.5 * J) * kCTabS;
    int i0 = (int)floor(u);
    i0 = min(max(i0, 0), kCTabS - 1);
    const double f = fmin(fmax(u - i0, 0.0), 1.0);
    // cubic Lagrange weights for samples at -1, 0, 1, 2 (table rows i0 .. i0+3)
    const double fm1 = f - 1.0, fm2 = f - 2.0, fp1 = f + 1.0;
    const double wa = -f * fm1 * fm2 * (1.0 / 6.0);
    const double wb = fp1 * fm1 * fm2 * 0.5;
    const double wc = -fp1 * f * fm2 * 0.5;
    const double wd = fp1 * f * fm1 * (1.0 / 6.0);
    const double* row = ctab + (size_t)i0 * JM;
    // phase of j = 1: lin*(dk - 1) - om*N/2; then rotate by exp(-i lin) per step
    double sth, cth;
    sincos(a.lin * (dk - 1.0) - w * a.half_N, &sth, &cth);
    float amax = 0.f;
#pragma unroll
    for (int j = 0; j < JM; ++j) {
        if (j >= J) {
            if (j < JP) dst[j] = make_float2(0.f, 0.f);
            continue;
        }
        const double c = wa * row[j] + wb * row[JM + j] + wc * row[2 * JM + j] + wd * row[3 * JM + j];
        // exp(i th_j) with th_j = th_1 - lin*j
        const double cr = cth * tab.rc[j] + sth * tab.rs[j];
        const double ci = sth * tab.rc[j] - cth * tab.rs[j];
        const float2 v = make_float2((float)(c * cr), (float)(-c * ci));
        dst[j] = v;
        amax = fmaxf(amax, sqrtf(v.x * v.x + v.y * v.y));
    }
    return amax;
}

template <int JM>
__global__ void build_tables_kernel(const double* __restrict__ om, int64_t M, int ndim,
                                    const AxisConst* __restrict__ axc,
                                    const AxisTab* __restrict__ tabs,
                                    const double* __restrict__ ctab, Geom g,
                                    const int* __restrict__ bin_of,
                                    const int* __restrict__ rank_of,
                                    const int* __restrict__ bin_start,
                                    const int* __restrict__ bucket_count,
                                    const int* __restrict__ slot, int nkeys,
                                    int* __restrict__ perm, int* __restrict__ pos,
                                    float2* __restrict__ coef0, float2* __restrict__ coef1,
                                    float2* __restrict__ coef2, float* __restrict__ wpt,
                                    unsigned int* __restrict__ wmax) {
    for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M;
         m += (int64_t)gridDim.x * blockDim.x) {
        const int bk = bin_of[m];
        if (bk < 0) continue;
        const int bin = bk >> 5, key = bk & 31, rank = rank_of[m];
        // slot dealt by deal_bins_kernel, found from (key, rank); without a
        // deal (slot == nullptr) the keys of the bin are interleaved round
        // robin: (key, rank) follows every point of lower rank and the
        // points of equal rank and lower key
        const int* c = bucket_count + (int64_t)bin * 32;
        int pre = 0;
        if (slot) {
            for (int k = 0; k < key; ++k) pre += c[k];
            pre = slot[(int64_t)bin_start[bin] + pre + rank];
        } else {
            for (int k = 0; k < nkeys; ++k) pre += min(rank, c[k]) + ((k < key && c[k] > rank) ? 1 : 0);
        }
        const int64_t s = (int64_t)bin_start[bin] + pre;
        perm[s] = (int)m;
        float wprod = 1.f;
        for (int d = 0; d < ndim; ++d) {
            const AxisConst& a = axc[d];
            double w = om[m * ndim + d];
            double t = w / a.gam;
            double koff = floor(t - a.J * 0.5);
            double q = koff + 1.0;
            double r = q - a.K * floor(q / a.K);
            int p = (int)r;
            if (p >= a.K) p -= a.K;
            if (p < 0) p += a.K;
            pos[(int64_t)d * M + s] = p;
            float2* cd = (d == 0) ? coef0 : (d == 1) ? coef1 : coef2;
            const float amax = axis_coefs<JM>(a, tabs[d], ctab + (size_t)d * kCTabN * JM, w,
                                              cd + s * g.JP[d], g.JP[d]);
            wprod *= amax;
        }
        wpt[s] = wprod;
        atomicMax(wmax, __float_as_uint(wprod));
    }
}

__global__ void sub_count_kernel(const int* __restrict__ bin_start, int64_t nbins, int maxsub,
                                 int* __restrict__ nsub_of) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbins;
         b += (int64_t)gridDim.x * blockDim.x) {
        int c = bin_start[b + 1] - bin_start[b];
        nsub_of[b] = (c + maxsub - 1) / maxsub;
    }
}

__global__ void sub_fill_kernel(const int* __restrict__ bin_start, const int* __restrict__ sub_start,
                                int64_t nbins, int maxsub, int64_t nbin_inst,
                                int4* __restrict__ sub) {
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < nbins;
         b += (int64_t)gridDim.x * blockDim.x) {
        int c = bin_start[b + 1] - bin_start[b];
        int s0 = sub_start[b];
        for (int k = 0; k * maxsub < c; ++k) {
            int cnt = min(maxsub, c - k * maxsub);
            sub[s0 + k] = make_int4((int)b, bin_start[b] + k * maxsub, cnt, (int)(b / nbin_inst));
        }
    }
}

// Row-gridding sub-problems: along each line of bins of the innermost axis
// (one thread per line), runs of up to `group` consecutive bins holding at
// most `maxsub` points in all; a bin holding more is split into chunks of
// maxsub on its own.  count pass (out == nullptr) or fill pass.
__global__ void rowsub_kernel(const int* __restrict__ bin_start, int64_t nlines, int nbz,
                              int group, int maxsub, int64_t nbin_inst,
                              const int* __restrict__ line_start, int* __restrict__ line_count,
                              int4* __restrict__ out) {
    for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < nlines;
         l += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b0 = l * nbz;
        int n = 0;
        int w = out ? line_start[l] : 0;
        int bz = 0;
        while (bz < nbz) {
            const int64_t b = b0 + bz;
            const int c = bin_start[b + 1] - bin_start[b];
            if (c > maxsub) {   // a dense bin on its own, in chunks
                for (int k = 0; k * maxsub < c; ++k) {
                    if (out)
                        out[w + n] = make_int4((int)b, bin_start[b] + k * maxsub,
                                               min(maxsub, c - k * maxsub), (int)(b / nbin_inst));
                    ++n;
                }
                ++bz;
                continue;
            }
            int tot = c, e = bz + 1;
            while (e < nbz && e - bz < group) {
                const int ce = bin_start[b0 + e + 1] - bin_start[b0 + e];
                if (ce > maxsub || tot + ce > maxsub) break;
                tot += ce;
                ++e;
            }
            if (tot > 0) {
                if (out) out[w + n] = make_int4((int)b, bin_start[b], tot, (int)(b / nbin_inst));
                ++n;
            }
            bz = e;
        }
        if (!out) line_count[l] = n;
    }
}

void free_points(nufft_plan_s* p) {
    cudaFree(p->d_inst_start); p->d_inst_start = nullptr;
    cudaFree(p->d_perm); p->d_perm = nullptr;
    cudaFree(p->d_pos); p->d_pos = nullptr;
    cudaFree(p->d_wpt); p->d_wpt = nullptr;
    cudaFree(p->d_coef); p->d_coef = nullptr;
    cudaFree(p->d_sub); p->d_sub = nullptr;
    cudaFree(p->d_gsub); p->d_gsub = nullptr;
    p->ngsub = 0;
    cudaFree(p->d_rsub); p->d_rsub = nullptr;
    p->nrsub = 0;
    cudaFree(p->d_ybuf); p->d_ybuf = nullptr;
    p->ybuf_elems = 0;
    p->M = 0;
    p->nsub = 0;
}

static void default_bins(const nufft_plan_s* p, int bs[3], int& maxsub) {
    // cells per bin axis; the gridding tile is (bs + J - 1) per axis.  Sub-
    // problems hold at most 256 points (512 for the single-coil 3D bins, whose
    // 256-thread paired kernels take 128 points per pass), which keeps the
    // 32-bit fixed-point rounding of the fast gridding mode near float32
    // resolution (measured 5e-7 relative L2 against the exact mode).
    for (int d = 0; d < 3; ++d) bs[d] = 1;
    maxsub = 256;
    if (p->ndim == 1) { bs[0] = 1024; }
    else if (p->ndim == 2) { bs[0] = bs[1] = (p->B >= 8) ? 16 : 32; }
    else if (p->B >= 8) { bs[0] = bs[1] = 8; bs[2] = 4; }
    else { bs[0] = 8; bs[1] = bs[2] = 16; maxsub = 512; }
    for (int d = 0; d < p->ndim; ++d) {
        if (p->user_bs[d] > 0) bs[d] = p->user_bs[d];
        bs[d] = std::min(bs[d], p->Kd[d]);
    }
    if (p->user_maxsub > 0) maxsub = p->user_maxsub;
}

int set_points(nufft_plan_s* p, const int64_t* counts, const double* om, int om_on_device,
               cudaStream_t s) {
    if (!counts) { set_error("nufft_set_points: counts is NULL"); return NUFFT_EINVAL; }
    int64_t M = 0;
    for (int i = 0; i < p->ninst; ++i) {
        if (counts[i] < 0) { set_error("nufft_set_points: negative count"); return NUFFT_EINVAL; }
        M += counts[i];
    }
    if (M >= (int64_t)1 << 31) { set_error("nufft_set_points: more than 2^31-1 points"); return NUFFT_EINVAL; }
    if (M > 0 && !om) { set_error("nufft_set_points: om is NULL"); return NUFFT_EINVAL; }
    // captured CG graphs hold the old tables' pointers: drop them with the tables
    free_cg(p);
    free_points(p);
    p->counts.assign(counts, counts + p->ninst);
    default_bins(p, p->bs, p->maxsub);

    const int nd = p->ndim;
    int64_t nbin_inst = 1;
    int nb[3] = {1, 1, 1};
    for (int d = 0; d < nd; ++d) {
        nb[d] = (p->Kd[d] + p->bs[d] - 1) / p->bs[d];
        nbin_inst *= nb[d];
    }
    const int64_t nbins = nbin_inst * p->ninst;
    p->nbins_total = nbins;

    std::vector<int64_t> istart(p->ninst + 1, 0);
    for (int i = 0; i < p->ninst; ++i) istart[i + 1] = istart[i] + counts[i];
    NUFFT_CUDA_TRY(cudaMalloc(&p->d_inst_start, sizeof(int64_t) * (p->ninst + 1)));
    NUFFT_CUDA_TRY(cudaMemcpyAsync(p->d_inst_start, istart.data(), sizeof(int64_t) * (p->ninst + 1),
                                   cudaMemcpyHostToDevice, s));
    p->M = M;
    int64_t Malloc = std::max<int64_t>(M, 1);
    NUFFT_CUDA_TRY(cudaMalloc(&p->d_perm, sizeof(int) * Malloc));
    NUFFT_CUDA_TRY(cudaMalloc(&p->d_pos, sizeof(int) * Malloc * nd));
    NUFFT_CUDA_TRY(cudaMalloc(&p->d_wpt, sizeof(float) * Malloc));
    int64_t coef_elems = 0;
    int JP[3] = {0, 0, 0};
    for (int d = 0; d < nd; ++d) {
        JP[d] = (p->Jd[d] + 1) & ~1;
        coef_elems += Malloc * JP[d];
    }
    NUFFT_CUDA_TRY(cudaMalloc(&p->d_coef, sizeof(float2) * coef_elems));
    p->ybuf_elems = (size_t)Malloc * p->B;
    NUFFT_CUDA_TRY(cudaMalloc(&p->d_ybuf, sizeof(float2) * p->ybuf_elems));
    NUFFT_CUDA_TRY(cudaMemsetAsync(p->d_ybuf, 0, sizeof(float2) * p->ybuf_elems, s));

    // temporaries
    double* d_om = nullptr;
    int *d_bin_of = nullptr, *d_rank = nullptr, *d_cnt = nullptr, *d_start = nullptr;
    int *d_nsub = nullptr, *d_subst = nullptr, *d_err = nullptr, *d_bucket = nullptr;
    int *d_gnsub = nullptr, *d_gsubst = nullptr, *d_rnl = nullptr, *d_rst = nullptr;
    int* d_slot = nullptr;
    unsigned int* d_wmax = nullptr;
    unsigned *d_key = nullptr, *d_key2 = nullptr;
    int *d_idx = nullptr, *d_idx2 = nullptr, *d_head = nullptr;
    void* d_sort_tmp = nullptr;
    AxisTab* d_tab = nullptr;
    double* d_ctab = nullptr;
    auto cleanup = [&]() {
        if (!om_on_device) cudaFree(d_om);
        cudaFree(d_tab); d_tab = nullptr;
        cudaFree(d_ctab); d_ctab = nullptr;
        cudaFree(d_bin_of); cudaFree(d_rank); cudaFree(d_cnt); cudaFree(d_start);
        cudaFree(d_nsub); cudaFree(d_subst); cudaFree(d_err); cudaFree(d_wmax);
        cudaFree(d_gnsub); cudaFree(d_gsubst); cudaFree(d_rnl); cudaFree(d_rst);
        cudaFree(d_bucket); cudaFree(d_slot);
        cudaFree(d_key); cudaFree(d_key2); cudaFree(d_idx); cudaFree(d_idx2); cudaFree(d_head);
        cudaFree(d_sort_tmp);
        d_key = d_key2 = nullptr;
        d_idx = d_idx2 = d_head = nullptr;
        d_sort_tmp = nullptr;
    };
#define TRY_TMP(expr)                                                              \
    do {                                                                           \
        cudaError_t _e = (expr);                                                   \
        if (_e != cudaSuccess) {                                                   \
            set_error(std::string(#expr) + ": " + cudaGetErrorString(_e));         \
            cleanup();                                                             \
            return (_e == cudaErrorMemoryAllocation) ? NUFFT_ENOMEM : NUFFT_ECUDA; \
        }                                                                          \
    } while (0)

    if (om_on_device) {
        d_om = const_cast<double*>(om);
    } else if (M > 0) {
        TRY_TMP(cudaMalloc(&d_om, sizeof(double) * M * nd));
        TRY_TMP(cudaMemcpyAsync(d_om, om, sizeof(double) * M * nd, cudaMemcpyHostToDevice, s));
    }
    TRY_TMP(cudaMalloc(&d_bin_of, sizeof(int) * Malloc));
    TRY_TMP(cudaMalloc(&d_rank, sizeof(int) * Malloc));
    TRY_TMP(cudaMalloc(&d_slot, sizeof(int) * Malloc));
    TRY_TMP(cudaMalloc(&d_cnt, sizeof(int) * nbins));
    TRY_TMP(cudaMalloc(&d_bucket, sizeof(int) * nbins * 32));
    TRY_TMP(cudaMalloc(&d_start, sizeof(int) * (nbins + 1)));
    TRY_TMP(cudaMalloc(&d_nsub, sizeof(int) * nbins));
    TRY_TMP(cudaMalloc(&d_subst, sizeof(int) * (nbins + 1)));
    TRY_TMP(cudaMalloc(&d_err, sizeof(int)));
    TRY_TMP(cudaMalloc(&d_wmax, sizeof(unsigned int)));
    TRY_TMP(cudaMemsetAsync(d_bucket, 0, sizeof(int) * nbins * 32, s));
    TRY_TMP(cudaMemsetAsync(d_err, 0, sizeof(int), s));
    TRY_TMP(cudaMemsetAsync(d_wmax, 0, sizeof(unsigned int), s));

    // per-axis constants (angle tables for the sinc identity)
    AxisTab htab[3];
    AxisConst hax[3];
    for (int d = 0; d < nd; ++d) {
        const AxisParams& ap = p->ax[d];
        AxisConst& a = hax[d];
        a.K = ap.K; a.J = ap.J; a.L = ap.L; a.N = ap.N;
        a.gam = 2.0 * M_PI / ap.K;
        a.inv_ratio = (double)ap.N / (double)ap.K;
        a.lin = a.gam * (ap.N - 1.0) / 2.0;
        a.half_N = ap.N / 2.0;
        for (int l = 0; l <= NUFFT_MAXL; ++l) a.alpha[l] = (l <= ap.L) ? (double)ap.alpha[l] : 0.0;
        for (int i = 0; i < ap.J * ap.J; ++i) a.T[i] = ap.T[i];
        for (int n = -(ap.L + ap.J); n <= ap.L; ++n) {
            double ang = M_PI * n * a.inv_ratio;
            htab[d].cs[n + ap.L + ap.J] = std::cos(ang);
            htab[d].ss[n + ap.L + ap.J] = std::sin(ang);
        }
        for (int j = 0; j < ap.J; ++j) {
            htab[d].rc[j] = std::cos(a.lin * j);
            htab[d].rs[j] = std::sin(a.lin * j);
        }
    }
    TRY_TMP(cudaMalloc(&d_tab, sizeof(AxisTab) * 3));
    TRY_TMP(cudaMemcpyAsync(d_tab, htab, sizeof(AxisTab) * 3, cudaMemcpyHostToDevice, s));
    TRY_TMP(cudaMemcpyAsync(p->d_axc, hax, sizeof(AxisConst) * 3, cudaMemcpyHostToDevice, s));

    Geom g = p->geom();
    g.inst_start = p->d_inst_start;
    const int threads = 256;
    const int blocks = (int)std::min<int64_t>((M + threads - 1) / threads + 1, 65535 * 8);
    if (M > 0) {
        bin_points_kernel<<<blocks, threads, 0, s>>>(d_om, M, nd, p->d_axc, g, d_bin_of, d_rank,
                                                     d_bucket, d_err);
        TRY_TMP(cudaGetLastError());
        // ranks by point index (see rank_keys_kernel)
        const unsigned nb32 = (unsigned)(nbins * 32);
        int nbits = 1;
        while (nbits < 32 && (1ull << nbits) <= (unsigned long long)nb32) ++nbits;
        TRY_TMP(cudaMalloc(&d_key, sizeof(unsigned) * M));
        TRY_TMP(cudaMalloc(&d_key2, sizeof(unsigned) * M));
        TRY_TMP(cudaMalloc(&d_idx, sizeof(int) * M));
        TRY_TMP(cudaMalloc(&d_idx2, sizeof(int) * M));
        TRY_TMP(cudaMalloc(&d_head, sizeof(int) * ((size_t)nb32 + 1)));
        rank_keys_kernel<<<blocks, threads, 0, s>>>(d_bin_of, M, nb32, d_key, d_idx);
        TRY_TMP(cudaGetLastError());
        size_t tmp_bytes = 0;
        TRY_TMP(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, d_key, d_key2, d_idx, d_idx2,
                                                M, 0, nbits, s));
        TRY_TMP(cudaMalloc(&d_sort_tmp, std::max<size_t>(tmp_bytes, 16)));
        TRY_TMP(cub::DeviceRadixSort::SortPairs(d_sort_tmp, tmp_bytes, d_key, d_key2, d_idx, d_idx2,
                                                M, 0, nbits, s));
        bucket_head_kernel<<<blocks, threads, 0, s>>>(d_key2, M, d_head);
        TRY_TMP(cudaGetLastError());
        sorted_rank_kernel<<<blocks, threads, 0, s>>>(d_key2, d_idx2, M, nb32, d_head, d_rank);
        TRY_TMP(cudaGetLastError());
    }
    {
        const int tb = (int)std::min<int64_t>((nbins + threads - 1) / threads, 65535);
        bin_totals_kernel<<<tb, threads, 0, s>>>(d_bucket, nbins, d_cnt);
        TRY_TMP(cudaGetLastError());
    }
    scan_kernel<<<1, 1024, 0, s>>>(d_cnt, d_start, nbins);
    TRY_TMP(cudaGetLastError());
    float2* c0 = p->d_coef;
    float2* c1 = c0 + (nd > 1 ? Malloc * JP[0] : 0);
    float2* c2 = c1 + (nd > 2 ? Malloc * JP[1] : 0);
    const int bblocks = (int)std::min<int64_t>((nbins + threads - 1) / threads, 65535);
    // plans of 8 or more coils sort each sub-problem's points by row in the
    // gridding kernel, and their gather teams take 32 / G points per warp:
    // a round-robin interleave of the bank keys (in build_tables) replaces
    // the deal, whose per-bin loop is long for the dense bins of such plans
    const bool deal = p->B < 8;
    if (M > 0 && deal) {
        deal_bins_kernel<<<bblocks, threads, 0, s>>>(d_bucket, d_start, nbins,
                                                     keys_in_use(nd, p->B), p->maxsub, d_slot);
        TRY_TMP(cudaGetLastError());
    }
    if (M > 0) {
        int jmax = 1;
        for (int d = 0; d < nd; ++d) jmax = std::max(jmax, p->Jd[d]);
        const int jm = (jmax <= 4) ? 4 : (jmax <= 6) ? 6 : (jmax <= 8) ? 8 : 16;
        TRY_TMP(cudaMalloc(&d_ctab, sizeof(double) * nd * kCTabN * jm));
        auto ckern = (jm == 4) ? ctab_kernel<4> : (jm == 6) ? ctab_kernel<6>
                     : (jm == 8) ? ctab_kernel<8> : ctab_kernel<16>;
        ckern<<<(nd * kCTabN + 127) / 128, 128, 0, s>>>(p->d_axc, d_tab, nd, d_ctab);
        TRY_TMP(cudaGetLastError());
        auto kern = (jm == 4) ? build_tables_kernel<4> : (jm == 6) ? build_tables_kernel<6>
                    : (jm == 8) ? build_tables_kernel<8> : build_tables_kernel<16>;
        kern<<<blocks, threads, 0, s>>>(d_om, M, nd, p->d_axc, d_tab, d_ctab, g, d_bin_of, d_rank,
                                        d_start, d_bucket, deal ? d_slot : nullptr,
                                        keys_in_use(nd, p->B), p->d_perm,
                                        p->d_pos, c0, c1, c2, p->d_wpt,
                                        d_wmax);
        TRY_TMP(cudaGetLastError());
    }
    sub_count_kernel<<<bblocks, threads, 0, s>>>(d_start, nbins, p->maxsub, d_nsub);
    TRY_TMP(cudaGetLastError());
    scan_kernel<<<1, 1024, 0, s>>>(d_nsub, d_subst, nbins);
    TRY_TMP(cudaGetLastError());
    // gather list (interpolation from shared tiles of several coils): bins
    // split only past kGatherSub points, so a tile is loaded once per bin
    const bool glist = p->B >= 8;
    // row-gridding list: lines of bins along the innermost axis
    const int nbz = nb[nd - 1];
    const int64_t nlines = nbins / nbz;
    p->rgroup = (nd == 3) ? kRowGroup : 1;
    const int lblocks = (int)std::min<int64_t>((nlines + threads - 1) / threads, 65535);
    if (glist) {
        TRY_TMP(cudaMalloc(&d_gnsub, sizeof(int) * nbins));
        TRY_TMP(cudaMalloc(&d_gsubst, sizeof(int) * (nbins + 1)));
        sub_count_kernel<<<bblocks, threads, 0, s>>>(d_start, nbins, kGatherSub, d_gnsub);
        TRY_TMP(cudaGetLastError());
        scan_kernel<<<1, 1024, 0, s>>>(d_gnsub, d_gsubst, nbins);
        TRY_TMP(cudaGetLastError());
        TRY_TMP(cudaMalloc(&d_rnl, sizeof(int) * nlines));
        TRY_TMP(cudaMalloc(&d_rst, sizeof(int) * (nlines + 1)));
        rowsub_kernel<<<lblocks, threads, 0, s>>>(d_start, nlines, nbz, p->rgroup, row_sub_cap(nd),
                                                  nbin_inst, nullptr, d_rnl, nullptr);
        TRY_TMP(cudaGetLastError());
        scan_kernel<<<1, 1024, 0, s>>>(d_rnl, d_rst, nlines);
        TRY_TMP(cudaGetLastError());
    }
    int h_nsub = 0, h_gnsub = 0, h_rnsub = 0, h_err = 0;
    unsigned int h_wmax = 0;
    TRY_TMP(cudaMemcpyAsync(&h_nsub, d_subst + nbins, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (glist) {
        TRY_TMP(cudaMemcpyAsync(&h_gnsub, d_gsubst + nbins, sizeof(int), cudaMemcpyDeviceToHost, s));
        TRY_TMP(cudaMemcpyAsync(&h_rnsub, d_rst + nlines, sizeof(int), cudaMemcpyDeviceToHost, s));
    }
    TRY_TMP(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
    TRY_TMP(cudaMemcpyAsync(&h_wmax, d_wmax, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
    TRY_TMP(cudaStreamSynchronize(s));
    cudaFree(d_tab); d_tab = nullptr;
    cudaFree(d_ctab); d_ctab = nullptr;
    if (h_err) {
        cleanup();
        free_points(p);
        set_error("nufft_set_points: om holds NaN or Inf");
        return NUFFT_EOM_NONFINITE;
    }
    std::memcpy(&p->wmax, &h_wmax, sizeof(float));
    p->nsub = h_nsub;
    TRY_TMP(cudaMalloc(&p->d_sub, sizeof(int4) * std::max(h_nsub, 1)));
    if (h_nsub > 0) {
        sub_fill_kernel<<<bblocks, threads, 0, s>>>(d_start, d_subst, nbins, p->maxsub, nbin_inst,
                                                    p->d_sub);
        TRY_TMP(cudaGetLastError());
    }
    if (glist) {
        p->ngsub = h_gnsub;
        TRY_TMP(cudaMalloc(&p->d_gsub, sizeof(int4) * std::max(h_gnsub, 1)));
        if (h_gnsub > 0) {
            sub_fill_kernel<<<bblocks, threads, 0, s>>>(d_start, d_gsubst, nbins, kGatherSub,
                                                        nbin_inst, p->d_gsub);
            TRY_TMP(cudaGetLastError());
        }
        p->nrsub = h_rnsub;
        TRY_TMP(cudaMalloc(&p->d_rsub, sizeof(int4) * std::max(h_rnsub, 1)));
        if (h_rnsub > 0) {
            rowsub_kernel<<<lblocks, threads, 0, s>>>(d_start, nlines, nbz, p->rgroup, row_sub_cap(nd),
                                                      nbin_inst, d_rst, nullptr, p->d_rsub);
            TRY_TMP(cudaGetLastError());
        }
    }
    TRY_TMP(cudaStreamSynchronize(s));
    cleanup();
#undef TRY_TMP
    return NUFFT_OK;
}

}  // namespace nufft
