// solve(y, 'L1TVOLS', maxiter, rho): L1 total-variation regularised least
// squares by split Bregman (linalg/solve_cpu.py:42-163), for one coil and
// one instance.  Per outer iteration:
//
//   rhs  = mu AHyk + lmbd sum_d Dt_d(dd_d - bb_d)          tv_rhs_kernel
//   x    = k2xx((xx2k(rhs) + 1e-7) / (uker + 1e-7))        pad + FFT, tv_kdiv_kernel, IFFT + crop
//   zz_d = D_d x;  s = |zz + bb| + 1e-5                      tv_shrink_kernel
//   dd_d = (zz_d + bb_d) max(s - 1/lmbd, 0) / s;  bb_d += zz_d - dd_d
//   AHyk += AHy - selfadjoint(x)                             NUFFT pair, tv_bregman_kernel
//
// with D_d x [n] = x[n - e_d] - x[n] and Dt_d v [n] = v[n + e_d] - v[n]
// (periodic; cDiff with helper.indxmap_diff, src/_helper/helper.py:46-70),
// uker = mu |xx2k(adjoint(1))| - lmbd L, L the FFT of the periodic
// Laplacian stencil (helper.create_laplacian_kernel, helper.py:11-44), which
// is real: L[k] = sum_d 2 cos(2 pi k_d / K_d) - 2 ndim.  mu = 1, lmbd = rho.
// Every vector stays on the device; the loop has no host synchronisation.
#include "nufft_internal.cuh"

#include <cmath>

namespace nufft {
namespace {

struct ImgDims {
    int ndim;
    int n[3];       // image extents, C order (last fastest)
    int64_t st[3];  // strides
    int64_t total;
};

ImgDims img_dims(const nufft_plan_s* p) {
    ImgDims d{};
    d.ndim = p->ndim;
    int64_t s = 1;
    for (int a = p->ndim - 1; a >= 0; --a) {
        d.n[a] = p->Nd[a];
        d.st[a] = s;
        s *= p->Nd[a];
    }
    d.total = s;
    return d;
}

// flat index of n shifted by +1 (sgn = +1) or -1 along axis a, periodic
__device__ __forceinline__ int64_t shifted(const ImgDims& d, int64_t n, int a, int sgn) {
    const int c = (int)((n / d.st[a]) % d.n[a]);
    int c2 = c + sgn;
    if (c2 < 0) c2 += d.n[a];
    if (c2 >= d.n[a]) c2 -= d.n[a];
    return n + (int64_t)(c2 - c) * d.st[a];
}

__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

__global__ void fill_ones_kernel(float2* __restrict__ v, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        v[i] = make_float2(1.f, 0.f);
}

// uker[k] = mu |w[k]| - lmbd (sum_d 2 cos(2 pi k_d / K_d) - 2 ndim)
__global__ void tv_uker_kernel(const float2* __restrict__ w, float2* __restrict__ uker, int ndim,
                               int K0, int K1, int K2, int64_t n, float mu, float lmbd) {
    const int K[3] = {K0, K1, K2};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = i;
        float lap = -2.f * ndim;
        for (int a = ndim - 1; a >= 0; --a) {
            const int k = (int)(r % K[a]);
            r /= K[a];
            lap += 2.f * (float)cospi(2.0 * k / K[a]);
        }
        const float2 v = w[i];
        uker[i] = make_float2(mu * hypotf(v.x, v.y) - lmbd * lap, 0.f);
    }
}

// rhs = mu ahyk + lmbd sum_d (v_d[n + e_d] - v_d[n]),  v_d = dd_d - bb_d
__global__ void tv_rhs_kernel(ImgDims d, const float2* __restrict__ ahyk,
                              const float2* __restrict__ dd, const float2* __restrict__ bb,
                              float2* __restrict__ rhs, float mu, float lmbd) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float2 a = ahyk[i];
        float2 r = make_float2(mu * a.x, mu * a.y);
        for (int p = 0; p < d.ndim; ++p) {
            const float2* ddp = dd + p * d.total;
            const float2* bbp = bb + p * d.total;
            const int64_t j = shifted(d, i, p, +1);
            const float2 t = sub2(sub2(ddp[j], bbp[j]), sub2(ddp[i], bbp[i]));
            r.x += lmbd * t.x;
            r.y += lmbd * t.y;
        }
        rhs[i] = r;
    }
}

// k = (k + 1e-7) / (uker + 1e-7) on the oversampled grid (uker real)
__global__ void tv_kdiv_kernel(float2* __restrict__ k, const float2* __restrict__ uker, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = k[i];
        const float2 u = uker[i];
        const float ur = u.x + 1e-7f, ui = u.y;
        const float vr = v.x + 1e-7f, vi = v.y;
        const float den = ur * ur + ui * ui;
        k[i] = make_float2((vr * ur + vi * ui) / den, (vi * ur - vr * ui) / den);
    }
}

// zz_d = x[n - e_d] - x[n]; s_d = zz_d + bb_d; s = sqrt(sum_d |s_d|^2) + 1e-5;
// dd_d = s_d max(s - 1/lmbd, 0)/s; bb_d += zz_d - dd_d
__global__ void tv_shrink_kernel(ImgDims d, const float2* __restrict__ x, float2* __restrict__ dd,
                                 float2* __restrict__ bb, float thresh) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < d.total;
         i += (int64_t)gridDim.x * blockDim.x) {
        float2 zz[3], st[3];
        float s = 0.f;
        const float2 xi = x[i];
        for (int p = 0; p < d.ndim; ++p) {
            zz[p] = sub2(x[shifted(d, i, p, -1)], xi);
            const float2 b = bb[p * d.total + i];
            st[p] = make_float2(zz[p].x + b.x, zz[p].y + b.y);
            s = hypotf(hypotf(st[p].x, st[p].y), s);
        }
        s += 1e-5f;
        const float r = (s > thresh) ? (s - thresh) / s : 0.f;
        for (int p = 0; p < d.ndim; ++p) {
            const float2 nd = make_float2(st[p].x * r, st[p].y * r);
            dd[p * d.total + i] = nd;
            float2 b = bb[p * d.total + i];
            b.x += zz[p].x - nd.x;
            b.y += zz[p].y - nd.y;
            bb[p * d.total + i] = b;
        }
    }
}

// ahyk -= (aha - ahy)
__global__ void tv_bregman_kernel(float2* __restrict__ ahyk, const float2* __restrict__ ahy,
                                  const float2* __restrict__ aha, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float2 zf = sub2(aha[i], ahy[i]);
        ahyk[i] = sub2(ahyk[i], zf);
    }
}

unsigned grid_for(const nufft_plan_s* p, int64_t n) {
    const int64_t want = (n + 255) / 256;
    const int64_t cap = (int64_t)std::max(p->num_sms, 1) * 8;
    return (unsigned)std::max<int64_t>(1, std::min(want, cap));
}

}  // namespace

int solve_l1tvols(nufft_plan_s* p, const float2* y, float2* x, int maxiter, double rho,
                  cudaStream_t s) {
    if (p->B != 1 || p->ninst != 1) {
        set_error("nufft_solve_l1tvols: the L1-TV solver runs on single-coil, single-instance plans");
        return NUFFT_EUNSUPPORTED;
    }
    if (!(rho > 0) || !std::isfinite(rho)) {
        set_error("nufft_solve_l1tvols: rho must be positive and finite");
        return NUFFT_EINVAL;
    }
    const ImgDims d = img_dims(p);
    const int64_t ni = d.total, nk = p->prodK;
    const float mu = 1.f, lmbd = (float)rho;
    // workspace: ahy, ahyk, rhs, aha (image), dd and bb (ndim images each), uker (grid)
    const size_t elems = (size_t)ni * (4 + 2 * d.ndim) + (size_t)nk;
    float2* ws = nullptr;
    NUFFT_CUDA_TRY(cudaMallocAsync(&ws, sizeof(float2) * elems, s));
    float2* ahy = ws;
    float2* ahyk = ahy + ni;
    float2* rhs = ahyk + ni;
    float2* aha = rhs + ni;
    float2* dd = aha + ni;
    float2* bb = dd + (size_t)d.ndim * ni;
    float2* uker = bb + (size_t)d.ndim * ni;
    int st = NUFFT_OK;
    auto run = [&]() -> int {
        NUFFT_CUDA_TRY(cudaMemsetAsync(ahyk, 0, sizeof(float2) * ni * (3 + 2 * d.ndim), s));
        NUFFT_CUDA_TRY(cudaMemsetAsync(x, 0, sizeof(float2) * ni, s));
        // uker = mu |xx2k(adjoint(1))| - lmbd L
        fill_ones_kernel<<<grid_for(p, p->M), 256, 0, s>>>(p->d_ybuf, p->M);
        NUFFT_CUDA_TRY(cudaGetLastError());
        NUFFT_TRY(nufft_adjoint(p, p->d_ybuf, aha, s));
        NUFFT_TRY(forward_from_image(p, aha, false, p->d_grid, s));
        tv_uker_kernel<<<grid_for(p, nk), 256, 0, s>>>(p->d_grid, uker, d.ndim, p->Kd[0], p->Kd[1],
                                                       p->Kd[2], nk, mu, lmbd);
        NUFFT_CUDA_TRY(cudaGetLastError());
        NUFFT_TRY(nufft_adjoint(p, y, ahy, s));
        const unsigned gi = grid_for(p, ni), gk = grid_for(p, nk);
        for (int it = 0; it < maxiter; ++it) {
            tv_rhs_kernel<<<gi, 256, 0, s>>>(d, ahyk, dd, bb, rhs, mu, lmbd);
            NUFFT_CUDA_TRY(cudaGetLastError());
            NUFFT_TRY(forward_from_image(p, rhs, false, p->d_grid, s));
            tv_kdiv_kernel<<<gk, 256, 0, s>>>(p->d_grid, uker, nk);
            NUFFT_CUDA_TRY(cudaGetLastError());
            NUFFT_TRY(image_from_spectrum(p, p->d_grid, x, false, false, s));
            tv_shrink_kernel<<<gi, 256, 0, s>>>(d, x, dd, bb, (float)(1.0 / rho));
            NUFFT_CUDA_TRY(cudaGetLastError());
            NUFFT_TRY(nufft_selfadjoint(p, x, aha, s));
            tv_bregman_kernel<<<gi, 256, 0, s>>>(ahyk, ahy, aha, ni);
            NUFFT_CUDA_TRY(cudaGetLastError());
        }
        return NUFFT_OK;
    };
    st = run();
    cudaError_t e = cudaFreeAsync(ws, s);
    if (st == NUFFT_OK && e != cudaSuccess) {
        set_error(std::string("nufft_solve_l1tvols: cudaFreeAsync: ") + cudaGetErrorString(e));
        st = NUFFT_ECUDA;
    }
    return st;
}

}  // namespace nufft
