// Launchers for the interpolation (k2y) and gridding (y2k) kernels, and the
// fixed-point helpers of the deterministic gridding mode.  The kernel
// instantiations live in interp_d1.cu / interp_d2.cu / interp_d3.cu.
#include "nufft_internal.cuh"
#include "interp_cm.cuh"

#include <algorithm>
#include <cstring>

namespace nufft {

void k2y_dim1(int jm, const Geom& g, const float2* grid, float2* y, cudaStream_t s);
void k2y_dim2(int jm, const Geom& g, const float2* grid, float2* y, cudaStream_t s);
void k2y_dim3(int jm, const Geom& g, const float2* grid, float2* y, cudaStream_t s);
int y2k_dim1(int jm, bool det, const Geom& g, const float2* y, float2* grid,
             unsigned long long* igrid, const double* dscal, cudaStream_t s);
int y2k_dim2(int jm, bool det, const Geom& g, const float2* y, float2* grid,
             unsigned long long* igrid, const double* dscal, cudaStream_t s);
int y2k_dim3(int jm, bool det, const Geom& g, const float2* y, float2* grid,
             unsigned long long* igrid, const double* dscal, cudaStream_t s);
int y2k_cm_dim2(int jm, bool det, const Geom& g, const float2* y, float2* grid,
                unsigned long long* igrid, const double* dscal, cudaStream_t s);
int y2k_cm_dim3(int jm, bool det, const Geom& g, const float2* y, float2* grid,
                unsigned long long* igrid, const double* dscal, cudaStream_t s);

static int pick_jm(const nufft_plan_s* p) {
    int j = 1;
    for (int d = 0; d < p->ndim; ++d) j = std::max(j, p->Jd[d]);
    if (j <= 4) return 4;
    if (j <= 6) return 6;
    if (j <= 8) return 8;
    return 16;
}

// ---------------------------------------------------------------------------
// k2y
// ---------------------------------------------------------------------------
// Optional kernel timing: an event pair recorded on its own stream around
// every kperiod-th k2y / y2k kernel launch (not while the stream is being
// captured).  Sampling keeps the events' own stream work off most launches.
bool kernel_time_start(nufft_plan_s* p, int which, cudaStream_t s) {
    if (p->kperiod <= 0) return false;
    if (p->kseen[which]++ % (size_t)p->kperiod != 0) return false;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone)
        return false;
    std::vector<cudaEvent_t>& v = p->kev[which];
    while (v.size() < p->kused[which] + 2) {   // grow the pool by a pair (events are reused)
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return false;
        v.push_back(e);
    }
    cudaEventRecord(v[p->kused[which]++], s);
    return true;
}

void kernel_time_stop(nufft_plan_s* p, int which, cudaStream_t s, bool started) {
    if (started) cudaEventRecord(p->kev[which][p->kused[which]++], s);
}

void kernel_time_clear(nufft_plan_s* p) {
    for (int w = 0; w < 2; ++w) p->kused[w] = p->kseen[w] = 0;
}

void kernel_time_destroy(nufft_plan_s* p) {
    for (int w = 0; w < 2; ++w) {
        for (cudaEvent_t e : p->kev[w]) cudaEventDestroy(e);
        p->kev[w].clear();
    }
    kernel_time_clear(p);
}

int launch_k2y(nufft_plan_s* p, const float2* grid, float2* y, cudaStream_t s) {
    if (p->M == 0) return NUFFT_OK;
    Geom g = p->geom();
    const int jm = pick_jm(p);
    const bool timed = kernel_time_start(p, 0, s);
    switch (p->ndim) {
        case 1: k2y_dim1(jm, g, grid, y, s); break;
        case 2: k2y_dim2(jm, g, grid, y, s); break;
        default: k2y_dim3(jm, g, grid, y, s); break;
    }
    kernel_time_stop(p, 0, s, timed);
    return check_launch("k2y_kernel");
}

// ---------------------------------------------------------------------------
// y2k
// ---------------------------------------------------------------------------
// Sum over all samples and coils of |re| + |im|, reduced in a fixed order
// (per-block partials, then one block), so the fixed-point scale derived from
// it is itself reproducible.
__global__ void abs_sum_partial_kernel(const float2* __restrict__ y, int64_t n,
                                       double* __restrict__ part) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        float2 v = y[i];
        acc += (double)(fabsf(v.x) + fabsf(v.y));
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// dscal[1] = 2^(62 - e) with 2^e >= 1.01 * wmax * sum|y|: every partial sum of
// fixed-point contributions stays below 2^62 in magnitude.
__global__ void fixed_scale_kernel(const double* __restrict__ part, int nparts, float wmax,
                                   double* __restrict__ dscal) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += part[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double bound = 1.01 * (double)wmax * red[0];
        int e = 0;
        if (bound > 0 && isfinite(bound)) e = (int)ceil(log2(bound));
        dscal[0] = red[0];
        dscal[1] = ldexp(1.0, 62 - e);
    }
}

__global__ void fixed_to_float_kernel(const unsigned long long* __restrict__ ig, int64_t n,
                                      const double* __restrict__ dscal, float2* __restrict__ out) {
    const float inv = (float)(1.0 / dscal[1]);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const long long a = (long long)ig[2 * i], b = (long long)ig[2 * i + 1];
        out[i] = make_float2(__ll2float_rn(a) * inv, __ll2float_rn(b) * inv);
    }
}

template <bool DET>
static int y2k_dim(const nufft_plan_s* p, const Geom& g, const float2* y, float2* grid,
                   unsigned long long* igrid, const double* dscal, cudaStream_t s) {
    const int jm = pick_jm(p);
    switch (p->ndim) {
        case 1: return y2k_dim1(jm, DET, g, y, grid, igrid, dscal, s);
        case 2: return y2k_dim2(jm, DET, g, y, grid, igrid, dscal, s);
        default: return y2k_dim3(jm, DET, g, y, grid, igrid, dscal, s);
    }
}

int launch_y2k(nufft_plan_s* p, const float2* y, float2* grid, cudaStream_t s, bool pre_zeroed) {
    const size_t ncells = (size_t)p->ninst * p->prodK * p->B;
    Geom g = p->geom();
    if (!(p->flags & NUFFT_FLAG_DETERMINISTIC)) {
        if (!pre_zeroed) NUFFT_CUDA_TRY(cudaMemsetAsync(grid, 0, sizeof(float2) * ncells, s));
        if (p->M == 0) return NUFFT_OK;
        const bool timed = kernel_time_start(p, 1, s);
        const int st = y2k_dim<false>(p, g, y, grid, nullptr, nullptr, s);
        kernel_time_stop(p, 1, s, timed);
        return st;
    }
    // deterministic: exact fixed-point accumulation, then one rounding to float
    if (!p->d_igrid) {
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_igrid, sizeof(unsigned long long) * 2 * ncells));
        p->dev_bytes += sizeof(unsigned long long) * 2 * ncells;
    }
    if (!p->d_dscal) {
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_dscal, sizeof(double) * kScaleSlots));
        p->dev_bytes += sizeof(double) * kScaleSlots;
    }
    NUFFT_CUDA_TRY(cudaMemsetAsync(p->d_igrid, 0, sizeof(unsigned long long) * 2 * ncells, s));
    const int64_t ny = p->M * (int64_t)p->B;
    const int nparts = kAbsSumParts;
    double* part = p->d_dscal + 2;
    abs_sum_partial_kernel<<<nparts, 256, 0, s>>>(y, ny, part);
    NUFFT_TRY(check_launch("abs_sum_partial_kernel"));
    fixed_scale_kernel<<<1, 256, 0, s>>>(part, nparts, p->wmax, p->d_dscal);
    NUFFT_TRY(check_launch("fixed_scale_kernel"));
    if (p->M > 0) {
        const bool timed = kernel_time_start(p, 1, s);
        const int st = y2k_dim<true>(p, g, y, nullptr, p->d_igrid, p->d_dscal, s);
        kernel_time_stop(p, 1, s, timed);
        NUFFT_TRY(st);
    }
    const int blocks = (int)std::min<size_t>((ncells + 255) / 256, (size_t)p->num_sms * 16);
    fixed_to_float_kernel<<<std::max(blocks, 1), 256, 0, s>>>(p->d_igrid, (int64_t)ncells,
                                                               p->d_dscal, grid);
    return check_launch("fixed_to_float_kernel");
}

// ---------------------------------------------------------------------------
// coil-major spectra (plans of 8 or more coils)
// ---------------------------------------------------------------------------
// The row kernels are built for J in {4, 6, 8} on every axis, B a multiple
// of 8 (of 32 in 2D), and the default bins of such plans (rows of 16 cells:
// one 16-cell bin in 2D, four 4-cell bins in 3D); tiles must not wrap onto
// themselves.
bool cm_path(const nufft_plan_s* p) {
    if (p->B < 8 || p->B % 8 != 0 || (p->ndim != 2 && p->ndim != 3) || !p->d_cm || !p->d_rsub)
        return false;
    // 2D rows hold one coil per lane only with a multiple of 32 coils; with
    // four rows of 8 coils per warp the 2D tiles' few points per row block
    // leave the coil-team kernel faster (2D spiral, 8 coils: 0.05 against
    // 0.12 ms)
    if (p->ndim == 2 && p->B % 32 != 0) return false;
    const int J = p->Jd[0];
    if (J != 4 && J != 6 && J != 8) return false;
    const int DI = p->ndim - 1;
    for (int d = 0; d < p->ndim; ++d) {
        if (p->Jd[d] != J) return false;
        if (p->bs[d] + J - 1 > p->Kd[d]) return false;
    }
    // rows of 16 cells (bins x group along the innermost axis), not wrapping onto themselves
    if (p->bs[DI] * p->rgroup != 16 || 16 + J - 1 > p->Kd[DI]) return false;
    const int nkey = p->bs[0] * (p->ndim == 3 ? p->bs[1] : 1);
    // (both modes' kernels take the same shared memory)
    return nkey <= 256 && rows_smem(p->ndim, J, nkey, row_sub_cap(p->ndim), 8,
                                    cm_row_coils(p->B)) <= 200 * 1024;
}

// Deterministic row gridding into the coil-major spectra grid_cm: per-row
// float sums in a fixed order, combined across tiles exactly in 64-bit fixed
// point (igrid: 2 * ninst * prodK * B accumulators), then one rounding to
// float; dscal holds kScaleSlots doubles.  Allocates nothing.  `timer`: the
// plan whose kernel timing covers the launch, or null.  grid_cm null: the
// sums stay unrounded in igrid (for the coil-batched inverse passes).
static int y2k_cm_det(const nufft_plan_s* p, const float2* y, float2* grid_cm,
                      unsigned long long* igrid, double* dscal, nufft_plan_s* timer,
                      cudaStream_t s) {
    const size_t ncells = (size_t)p->ninst * p->prodK * p->B;
    Geom g = p->geom();
    NUFFT_CUDA_TRY(cudaMemsetAsync(igrid, 0, sizeof(unsigned long long) * 2 * ncells, s));
    const int64_t ny = p->M * (int64_t)p->B;
    abs_sum_partial_kernel<<<kAbsSumParts, 256, 0, s>>>(y, ny, dscal + 2);
    NUFFT_TRY(check_launch("abs_sum_partial_kernel"));
    fixed_scale_kernel<<<1, 256, 0, s>>>(dscal + 2, kAbsSumParts, p->wmax, dscal);
    NUFFT_TRY(check_launch("fixed_scale_kernel"));
    if (p->M > 0) {
        const int jm = pick_jm(p);
        const bool timed = timer && kernel_time_start(timer, 1, s);
        const int st = (p->ndim == 2) ? y2k_cm_dim2(jm, true, g, y, nullptr, igrid, dscal, s)
                                      : y2k_cm_dim3(jm, true, g, y, nullptr, igrid, dscal, s);
        if (timer) kernel_time_stop(timer, 1, s, timed);
        NUFFT_TRY(st);
    }
    if (!grid_cm) return NUFFT_OK;
    const int blocks = (int)std::min<size_t>((ncells + 255) / 256, (size_t)p->num_sms * 16);
    fixed_to_float_kernel<<<std::max(blocks, 1), 256, 0, s>>>(igrid, (int64_t)ncells, dscal,
                                                               grid_cm);
    return check_launch("fixed_to_float_kernel");
}

static int ensure_fixed_buffers(nufft_plan_s* p) {
    const size_t ncells = (size_t)p->ninst * p->prodK * p->B;
    if (!p->d_igrid) {
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_igrid, sizeof(unsigned long long) * 2 * ncells));
        p->dev_bytes += sizeof(unsigned long long) * 2 * ncells;
    }
    if (!p->d_dscal) {
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_dscal, sizeof(double) * kScaleSlots));
        p->dev_bytes += sizeof(double) * kScaleSlots;
    }
    return NUFFT_OK;
}

// Deterministic row gridding whose exact sums stay in p->d_igrid (scale in
// p->d_dscal), for the coil-batched inverse passes to round as they read.
int launch_y2k_cm_fixed(nufft_plan_s* p, const float2* y, cudaStream_t s) {
    NUFFT_TRY(ensure_fixed_buffers(p));
    return y2k_cm_det(p, y, nullptr, p->d_igrid, p->d_dscal, p, s);
}

int launch_y2k_cm(nufft_plan_s* p, const float2* y, float2* grid_cm, cudaStream_t s,
                  bool pre_zeroed) {
    const size_t ncells = (size_t)p->ninst * p->prodK * p->B;
    if (!(p->flags & NUFFT_FLAG_DETERMINISTIC)) {
        Geom g = p->geom();
        const int jm = pick_jm(p);
        if (!pre_zeroed) NUFFT_CUDA_TRY(cudaMemsetAsync(grid_cm, 0, sizeof(float2) * ncells, s));
        if (p->M == 0) return NUFFT_OK;
        const bool timed = kernel_time_start(p, 1, s);
        const int st = (p->ndim == 2) ? y2k_cm_dim2(jm, false, g, y, grid_cm, nullptr, nullptr, s)
                                      : y2k_cm_dim3(jm, false, g, y, grid_cm, nullptr, nullptr, s);
        kernel_time_stop(p, 1, s, timed);
        return st;
    }
    NUFFT_TRY(ensure_fixed_buffers(p));
    return y2k_cm_det(p, y, grid_cm, p->d_igrid, p->d_dscal, p, s);
}

// The y2k stage into the caller's coil-fastest spectrum k.  Deterministic
// plans with the row kernels grid coil-major and transpose once (the 8-coil,
// 8M-point kooshball: 19 ms against 111 ms for the coil-team kernel's
// per-contribution 64-bit atomics); the others run launch_y2k.
int launch_y2k_grid(nufft_plan_s* p, const float2* y, float2* k, cudaStream_t s) {
    // plans with the coil-batched passes: the row kernels grid coil-fastest
    // into k in either mode
    if (p->cfft && cm_path(p)) return launch_y2k_cm(p, y, k, s);
    if ((p->flags & NUFFT_FLAG_DETERMINISTIC) && cm_path(p)) {
        NUFFT_TRY(launch_y2k_cm(p, y, p->d_cm, s));
        return cm_to_grid(p, k, s);
    }
    return launch_y2k(p, y, k, s);
}

// Exact (fixed-point) gridding into `grid` using caller-provided scratch:
// acc holds 2 * ninst * prodK * B accumulators, scal kScaleSlots doubles.
// Allocates nothing.
int launch_y2k_exact_into(const nufft_plan_s* p, const float2* y, float2* grid,
                          unsigned long long* acc, double* scal, cudaStream_t s) {
    if (cm_path(p) && p->cfft) return y2k_cm_det(p, y, grid, acc, scal, nullptr, s);
    if (cm_path(p)) {
        // plans with the row kernels: the deterministic stage's own path
        // (launch_y2k_grid), into the plan's coil-major buffer and one transpose
        NUFFT_TRY(y2k_cm_det(p, y, p->d_cm, acc, scal, nullptr, s));
        return cm_to_grid(p, grid, s);
    }
    const size_t ncells = (size_t)p->ninst * p->prodK * p->B;
    Geom g = p->geom();
    g.ymethod = (p->B >= 8) ? NUFFT_Y2K_COIL : NUFFT_Y2K_ZTEAM;
    NUFFT_CUDA_TRY(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * 2 * ncells, s));
    const int64_t ny = p->M * (int64_t)p->B;
    const int nparts = kAbsSumParts;
    abs_sum_partial_kernel<<<nparts, 256, 0, s>>>(y, ny, scal + 2);
    NUFFT_TRY(check_launch("abs_sum_partial_kernel"));
    fixed_scale_kernel<<<1, 256, 0, s>>>(scal + 2, nparts, p->wmax, scal);
    NUFFT_TRY(check_launch("fixed_scale_kernel"));
    if (p->M > 0) NUFFT_TRY(y2k_dim<true>(p, g, y, nullptr, acc, scal, s));
    const int blocks = (int)std::min<size_t>((ncells + 255) / 256, (size_t)p->num_sms * 16);
    fixed_to_float_kernel<<<std::max(blocks, 1), 256, 0, s>>>(acc, (int64_t)ncells, scal, grid);
    return check_launch("fixed_to_float_kernel");
}

}  // namespace nufft
