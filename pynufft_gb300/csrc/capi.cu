// extern "C" entry points of libpynufft_gb300.so (declared in
// include/pynufft_gb300.h).  Each one validates its plan, then queues work on
// the caller's stream; nothing here synchronises except nufft_set_points and
// nufft_solve_cg when iteration counts are requested.
#include "nufft_internal.cuh"

#include <algorithm>
#include <cstring>

namespace nufft {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

}  // namespace nufft

using namespace nufft;

nufft::Geom nufft_plan_s::geom() const {
    Geom g{};
    g.ndim = ndim;
    g.B = B;
    for (int d = 0; d < 3; ++d) {
        g.K[d] = Kd[d];
        g.J[d] = (d < ndim) ? Jd[d] : 1;
        g.JP[d] = (d < ndim) ? ((Jd[d] + 1) & ~1) : 0;
        g.bs[d] = (d < ndim) ? bs[d] : 1;
        g.nb[d] = (d < ndim && bs[d] > 0) ? (Kd[d] + bs[d] - 1) / bs[d] : 1;
        g.T[d] = (d < ndim) ? bs[d] + Jd[d] - 1 : 1;
    }
    g.prodK = prodK;
    int64_t nbi = 1;
    for (int d = 0; d < ndim; ++d) nbi *= g.nb[d];
    g.nbin_inst = nbi;
    g.M = M;
    g.ninst = ninst;
    g.inst_start = d_inst_start;
    g.perm = d_perm;
    int64_t Ma = std::max<int64_t>(M, 1);
    const float2* c = d_coef;
    for (int d = 0; d < 3; ++d) {
        g.pos[d] = (d < ndim && d_pos) ? d_pos + (size_t)d * Ma : nullptr;
        g.coef[d] = (d < ndim) ? c : nullptr;
        if (d < ndim && c) c += (size_t)Ma * g.JP[d];
    }
    g.wpt = d_wpt;
    g.kerr = d_kerr;
    g.sub = d_sub;
    g.nsub = nsub;
    g.maxsub = maxsub;
    g.gsub = d_gsub;
    g.ngsub = ngsub;
    g.rsub = d_rsub;
    g.nrsub = nrsub;
    g.rgroup = rgroup;
    g.cm_il = cfft ? 2 : (cm_il ? 1 : 0);
    // lane mappings: coil-teams for B >= 8; otherwise the plan's choice.  The
    // defaults (fastest in measurement on 2D radial and 3D uniform
    // trajectories; the autotuner may pick others): k2y gathers from a shared
    // tile when sub-problems hold 8 or more points on average (the tile load
    // is then shared by enough points), else straight from the grid; y2k one
    // thread per point.
    const int kdef = (nsub > 0 && M >= 8 * (int64_t)nsub) ? NUFFT_K2Y_TILE_POINT : NUFFT_K2Y_POINT;
    g.kmethod = (B >= 8) ? NUFFT_K2Y_COIL : (k2y_method ? k2y_method : kdef);
    g.ymethod = (B >= 8) ? NUFFT_Y2K_COIL : (y2k_method ? y2k_method : NUFFT_Y2K_POINT);
    // the exact mode's 64-bit atomics favour the z-team mapping (fewer bank
    // conflicts); it has no global-atomic variant
    if ((flags & NUFFT_FLAG_DETERMINISTIC) && B < 8 &&
        (y2k_method == 0 || g.ymethod == NUFFT_Y2K_GLOBAL))
        g.ymethod = NUFFT_Y2K_ZTEAM;
    return g;
}

static inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

static int need_plan(nufft_plan_t p, const char* fn) {
    if (!p) {
        set_error(std::string(fn) + ": plan is NULL");
        return NUFFT_EINVAL;
    }
    return NUFFT_OK;
}

static int need_points(nufft_plan_t p, const char* fn) {
    NUFFT_TRY(need_plan(p, fn));
    if (!p->d_perm) {
        set_error(std::string(fn) + ": nufft_set_points has not been called");
        return NUFFT_ENOPOINTS;
    }
    return NUFFT_OK;
}

// Data pointers may be NULL only for arrays with no elements (an empty
// trajectory gives empty y arrays).
static int need_ptrs(const void* a, const void* b, const char* fn, const nufft_plan_s* p = nullptr) {
    const bool empty_ok = p && p->M == 0;
    if ((!a || !b) && !empty_ok) {
        set_error(std::string(fn) + ": NULL data pointer");
        return NUFFT_EINVAL;
    }
    return NUFFT_OK;
}

extern "C" {

const char* nufft_last_error(void) { return g_last_error.c_str(); }

const char* nufft_version(void) { return "pynufft_gb300 0.1.0 (sm_103a)"; }

int nufft_plan_create(int ndim, const int* Nd, const int* Kd, const int* Jd, int batch, int ninst,
                      int flags, nufft_plan_t* plan_out) {
    if (!plan_out || !Nd || !Kd || !Jd) {
        set_error("nufft_plan_create: NULL argument");
        return NUFFT_EINVAL;
    }
    *plan_out = nullptr;
    if (ndim < 1 || ndim > NUFFT_MAXDIM) {
        set_error("nufft_plan_create: ndim must be 1, 2 or 3");
        return NUFFT_EUNSUPPORTED;
    }
    if (batch < 1 || ninst < 1) {
        set_error("nufft_plan_create: batch and ninst must be >= 1");
        return NUFFT_EINVAL;
    }
    nufft_plan_s* p = new nufft_plan_s();
    p->ndim = ndim;
    p->B = batch;
    p->ninst = ninst;
    p->flags = flags;
    int64_t sumN = 0;
    for (int d = 0; d < ndim; ++d) {
        if (Nd[d] < 1 || Kd[d] < 1 || Jd[d] < 1 || Nd[d] > Kd[d] || Jd[d] > Kd[d] ||
            Jd[d] > NUFFT_MAXJ) {
            set_error("nufft_plan_create: need 1 <= Nd <= Kd, 1 <= Jd <= min(Kd, 16) on every axis");
            delete p;
            return NUFFT_EINVAL;
        }
        p->Nd[d] = Nd[d];
        p->Kd[d] = Kd[d];
        p->Jd[d] = Jd[d];
        p->prodN *= Nd[d];
        p->prodK *= Kd[d];
        sumN += Nd[d];
        int st = axis_params(Nd[d], Jd[d], Kd[d], p->ax[d]);
        if (st != NUFFT_OK) {
            set_error("nufft_plan_create: axis parameters");
            delete p;
            return st;
        }
    }
    if ((int64_t)ninst * p->prodK * batch >= ((int64_t)1 << 40)) {
        set_error("nufft_plan_create: grid too large");
        delete p;
        return NUFFT_EINVAL;
    }
    auto fail = [&](int st) {
        nufft_plan_destroy(p);
        return st;
    };
    if (cudaGetDevice(&p->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&p->num_sms, cudaDevAttrMultiProcessorCount, p->device) != cudaSuccess) {
        set_error("nufft_plan_create: no CUDA device");
        return fail(NUFFT_ECUDA);
    }
    std::vector<float> snd(sumN);
    int64_t off = 0;
    for (int d = 0; d < ndim; ++d)
        for (int n = 0; n < Nd[d]; ++n) snd[off++] = (float)p->ax[d].sn[n];
    cudaError_t e;
    e = cudaMalloc(&p->d_snd, sizeof(float) * sumN);
    if (e == cudaSuccess) e = cudaMemcpy(p->d_snd, snd.data(), sizeof(float) * sumN, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_axc, sizeof(AxisConst) * 3);
    const size_t ncell = (size_t)ninst * p->prodK * batch;
    if (e == cudaSuccess) e = cudaMalloc(&p->d_grid, sizeof(float2) * ncell);
    if (e == cudaSuccess) e = cudaMalloc(&p->d_kerr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(p->d_kerr, 0, sizeof(int));
    if (e != cudaSuccess) {
        set_error(std::string("nufft_plan_create: ") + cudaGetErrorString(e));
        return fail(e == cudaErrorMemoryAllocation ? NUFFT_ENOMEM : NUFFT_ECUDA);
    }
    p->dev_bytes = sizeof(float) * sumN + sizeof(AxisConst) * 3 + sizeof(float2) * ncell;
    // fast mode, one coil or the coil-batched FFT passes: a second grid for
    // the adjoint, zeroed on a side stream while the forward runs
    if (!(flags & NUFFT_FLAG_DETERMINISTIC) && ((batch == 1 && ninst == 1) || cfft_eligible(p))) {
        e = cudaMalloc(&p->d_grid_adj, sizeof(float2) * ncell);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->zs, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_zero, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->ev_adj, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            set_error(std::string("nufft_plan_create: ") + cudaGetErrorString(e));
            return fail(e == cudaErrorMemoryAllocation ? NUFFT_ENOMEM : NUFFT_ECUDA);
        }
        p->dev_bytes += sizeof(float2) * ncell;
    }
    int st = fft_init(p);
    if (st != NUFFT_OK) return fail(st);
    *plan_out = p;
    return NUFFT_OK;
}

int nufft_plan_destroy(nufft_plan_t p) {
    if (!p) return NUFFT_OK;
    free_points(p);
    free_cg(p);
    fft_destroy(p);
    cudaFree(p->d_snd);
    cudaFree(p->d_axc);
    cudaFree(p->d_grid);
    if (p->zs) cudaStreamSynchronize(p->zs);
    cudaFree(p->d_grid_adj);
    if (p->ev_zero) cudaEventDestroy(p->ev_zero);
    if (p->ev_adj) cudaEventDestroy(p->ev_adj);
    if (p->zs) cudaStreamDestroy(p->zs);
    cudaFree(p->d_igrid);
    cudaFree(p->d_dscal);
    cudaFree(p->d_maps);
    cudaFree(p->d_kerr);
    kernel_time_destroy(p);
    delete p;
    return NUFFT_OK;
}

int nufft_plan_set_alpha(nufft_plan_t p, int axis, const float* alpha, int L) {
    NUFFT_TRY(need_plan(p, "nufft_plan_set_alpha"));
    if (axis < 0 || axis >= p->ndim || !alpha || L < 0 || L > NUFFT_MAXL) {
        set_error("nufft_plan_set_alpha: need 0 <= axis < ndim, alpha != NULL, 0 <= L <= 14");
        return NUFFT_EINVAL;
    }
    AxisParams& ap = p->ax[axis];
    ap.L = L;
    for (int l = 0; l < NUFFT_NALPHA; ++l) ap.alpha[l] = (l <= L) ? alpha[l] : 0.f;
    NUFFT_TRY(derive_axis(ap));
    int off = 0;
    for (int d = 0; d < axis; ++d) off += p->Nd[d];
    std::vector<float> snd(p->Nd[axis]);
    for (int n = 0; n < p->Nd[axis]; ++n) snd[n] = (float)ap.sn[n];
    NUFFT_CUDA_TRY(cudaMemcpy(p->d_snd + off, snd.data(), sizeof(float) * snd.size(),
                              cudaMemcpyHostToDevice));
    // tables built from the old coefficients are stale
    free_cg(p);
    free_points(p);
    return NUFFT_OK;
}

int nufft_set_points(nufft_plan_t p, const int64_t* counts, const double* om, int om_on_device,
                     void* stream) {
    NUFFT_TRY(need_plan(p, "nufft_set_points"));
    free_cg(p);
    return set_points(p, counts, om, om_on_device, as_stream(stream));
}

int nufft_plan_set_bins(nufft_plan_t p, const int* bin_shape, int max_sub_points) {
    NUFFT_TRY(need_plan(p, "nufft_plan_set_bins"));
    if (bin_shape)
        for (int d = 0; d < p->ndim; ++d) {
            if (bin_shape[d] < 0) {
                set_error("nufft_plan_set_bins: negative bin size");
                return NUFFT_EINVAL;
            }
            p->user_bs[d] = bin_shape[d];
        }
    if (max_sub_points < 0) {
        set_error("nufft_plan_set_bins: negative max_sub_points");
        return NUFFT_EINVAL;
    }
    p->user_maxsub = max_sub_points;
    return NUFFT_OK;
}

int nufft_plan_set_methods(nufft_plan_t p, int k2y_method, int y2k_method) {
    NUFFT_TRY(need_plan(p, "nufft_plan_set_methods"));
    if (k2y_method < 0 || k2y_method > NUFFT_K2Y_TILE_POINT || y2k_method < 0 ||
        y2k_method > NUFFT_Y2K_GLOBAL) {
        set_error("nufft_plan_set_methods: unknown method");
        return NUFFT_EINVAL;
    }
    p->k2y_method = k2y_method;
    p->y2k_method = y2k_method;
    free_cg(p);   // captured graphs hold the old kernels
    return NUFFT_OK;
}

int nufft_plan_info(nufft_plan_t p, int64_t* M_total, int64_t* n_sub, int64_t* device_bytes) {
    NUFFT_TRY(need_plan(p, "nufft_plan_info"));
    if (M_total) *M_total = p->M;
    if (n_sub) *n_sub = p->nsub;
    if (device_bytes) {
        int64_t pts = 0;
        if (p->d_perm) {
            int64_t Ma = std::max<int64_t>(p->M, 1);
            pts = Ma * 4 * (1 + p->ndim);
            for (int d = 0; d < p->ndim; ++d) pts += Ma * ((p->Jd[d] + 1) & ~1) * 8;
            pts += (int64_t)p->ybuf_elems * 8 + p->nsub * 16;
        }
        *device_bytes = (int64_t)p->dev_bytes + pts;
    }
    return NUFFT_OK;
}

int nufft_plan_transform_kind(nufft_plan_t p, int* kind) {
    NUFFT_TRY(need_plan(p, "nufft_plan_transform_kind"));
    if (!kind) {
        set_error("nufft_plan_transform_kind: NULL argument");
        return NUFFT_EINVAL;
    }
    *kind = p->cfft ? NUFFT_FFT_OWN_COILS
                    : p->pfft ? NUFFT_FFT_OWN_PRUNED
                              : (p->fft_pruned ? NUFFT_FFT_CUFFT_PRUNED : NUFFT_FFT_CUFFT);
    return NUFFT_OK;
}

int nufft_plan_kernel_timing(nufft_plan_t p, int period) {
    NUFFT_TRY(need_plan(p, "nufft_plan_kernel_timing"));
    if (period < 0) {
        set_error("nufft_plan_kernel_timing: period must be >= 0");
        return NUFFT_EINVAL;
    }
    kernel_time_clear(p);
    p->kperiod = period;
    return NUFFT_OK;
}

int nufft_plan_kernel_times(nufft_plan_t p, double* k2y_ms, int* k2y_launches, double* y2k_ms,
                            int* y2k_launches) {
    NUFFT_TRY(need_plan(p, "nufft_plan_kernel_times"));
    double* ms[2] = {k2y_ms, y2k_ms};
    int* n[2] = {k2y_launches, y2k_launches};
    for (int w = 0; w < 2; ++w) {
        double tot = 0.0;
        const size_t pairs = p->kused[w] / 2;
        for (size_t i = 0; i < pairs; ++i) {
            NUFFT_CUDA_TRY(cudaEventSynchronize(p->kev[w][2 * i + 1]));
            float t = 0.f;
            NUFFT_CUDA_TRY(cudaEventElapsedTime(&t, p->kev[w][2 * i], p->kev[w][2 * i + 1]));
            tot += t;
        }
        if (ms[w]) *ms[w] = tot;
        if (n[w]) *n[w] = (int)pairs;
    }
    kernel_time_clear(p);
    return NUFFT_OK;
}

int nufft_mapped_pointer(const void* host, void** dev_out) {
    if (!host || !dev_out) {
        set_error("nufft_mapped_pointer: NULL argument");
        return NUFFT_EINVAL;
    }
    cudaPointerAttributes a{};
    cudaError_t e = cudaPointerGetAttributes(&a, host);
    if (e != cudaSuccess) {
        cudaGetLastError();   // clear the sticky-free error of an unknown pointer
        set_error(std::string("nufft_mapped_pointer: ") + cudaGetErrorString(e));
        return NUFFT_EINVAL;
    }
    if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) {
        set_error("nufft_mapped_pointer: not page-locked host memory mapped into the device");
        return NUFFT_EINVAL;
    }
    *dev_out = a.devicePointer;
    return NUFFT_OK;
}

int nufft_plan_check(nufft_plan_t p, void* stream) {
    NUFFT_TRY(need_plan(p, "nufft_plan_check"));
    int h = 0;
    cudaStream_t s = as_stream(stream);
    NUFFT_CUDA_TRY(cudaMemcpyAsync(&h, p->d_kerr, sizeof(int), cudaMemcpyDeviceToHost, s));
    NUFFT_CUDA_TRY(cudaStreamSynchronize(s));
    if (h != 0) {
        NUFFT_CUDA_TRY(cudaMemsetAsync(p->d_kerr, 0, sizeof(int), s));
        set_error("a kernel's wait for its asynchronous copies ran out (code " + std::to_string(h) +
                  "); its output is incomplete");
        return NUFFT_ETIMEOUT;
    }
    return NUFFT_OK;
}

int nufft_x2xx(nufft_plan_t p, const void* x, void* xx, void* stream) {
    NUFFT_TRY(need_plan(p, "nufft_x2xx"));
    NUFFT_TRY(need_ptrs(x, xx, "nufft_x2xx"));
    return launch_scale(p, (const float2*)x, (float2*)xx, as_stream(stream));
}

int nufft_xx2x(nufft_plan_t p, const void* xx, void* x, void* stream) {
    NUFFT_TRY(need_plan(p, "nufft_xx2x"));
    NUFFT_TRY(need_ptrs(x, xx, "nufft_xx2x"));
    return launch_scale(p, (const float2*)xx, (float2*)x, as_stream(stream));
}

int nufft_xx2k(nufft_plan_t p, const void* xx, void* k, void* stream) {
    NUFFT_TRY(need_plan(p, "nufft_xx2k"));
    NUFFT_TRY(need_ptrs(xx, k, "nufft_xx2k"));
    return forward_from_image(p, (const float2*)xx, false, (float2*)k, as_stream(stream));
}

int nufft_k2xx(nufft_plan_t p, const void* k, void* xx, void* stream) {
    NUFFT_TRY(need_plan(p, "nufft_k2xx"));
    NUFFT_TRY(need_ptrs(k, xx, "nufft_k2xx"));
    cudaStream_t s = as_stream(stream);
    if (p->B > 1) return image_from_spectrum_coils(p, (const float2*)k, (float2*)xx, false, false, s);
    if (p->pfft) return image_from_spectrum(p, (const float2*)k, (float2*)xx, false, false, s);
    const size_t n = (size_t)p->ninst * p->prodK * p->B;
    NUFFT_CUDA_TRY(cudaMemcpyAsync(p->d_grid, k, sizeof(float2) * n, cudaMemcpyDeviceToDevice, s));
    return image_from_spectrum(p, p->d_grid, (float2*)xx, false, false, s);
}

int nufft_k2y(nufft_plan_t p, const void* k, void* y, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_k2y"));
    NUFFT_TRY(need_ptrs(k, y, "nufft_k2y", p));
    return launch_k2y(p, (const float2*)k, (float2*)y, as_stream(stream));
}

int nufft_y2k(nufft_plan_t p, const void* y, void* k, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_y2k"));
    NUFFT_TRY(need_ptrs(y, k, "nufft_y2k", p));
    return launch_y2k_grid(p, (const float2*)y, (float2*)k, as_stream(stream));
}

static bool capturing(cudaStream_t s) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone;
}

int nufft_forward(nufft_plan_t p, const void* x, void* y, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_forward"));
    NUFFT_TRY(need_ptrs(x, y, "nufft_forward", p));
    cudaStream_t s = as_stream(stream);
    if (p->d_grid_adj && !p->adj_zeroed && !capturing(s)) {
        // zero the adjoint's grid on the side stream, after the last adjoint
        // has read it, while this forward runs
        if (p->adj_used) NUFFT_CUDA_TRY(cudaStreamWaitEvent(p->zs, p->ev_adj, 0));
        NUFFT_CUDA_TRY(cudaMemsetAsync(p->d_grid_adj, 0,
                                       sizeof(float2) * p->prodK * p->B * p->ninst, p->zs));
        NUFFT_CUDA_TRY(cudaEventRecord(p->ev_zero, p->zs));
        p->adj_zeroed = true;
    }
    NUFFT_TRY(forward_from_image(p, (const float2*)x, true, p->d_grid, s));
    return launch_k2y(p, p->d_grid, (float2*)y, s);
}

int nufft_adjoint(nufft_plan_t p, const void* y, void* x, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_adjoint"));
    NUFFT_TRY(need_ptrs(x, y, "nufft_adjoint", p));
    cudaStream_t s = as_stream(stream);
    if (p->d_grid_adj && !capturing(s)) {
        bool pre = false;
        if (p->adj_zeroed) {
            NUFFT_CUDA_TRY(cudaStreamWaitEvent(s, p->ev_zero, 0));
            pre = true;
        }
        p->adj_zeroed = false;   // consumed (or zeroed inline below)
        if (cm_path(p))   // several coils: the row gridding, coil-fastest
            NUFFT_TRY(launch_y2k_cm(p, (const float2*)y, p->d_grid_adj, s, pre));
        else
            NUFFT_TRY(launch_y2k(p, (const float2*)y, p->d_grid_adj, s, pre));
        const int st = image_from_spectrum(p, p->d_grid_adj, (float2*)x, true, false, s);
        NUFFT_CUDA_TRY(cudaEventRecord(p->ev_adj, s));
        p->adj_used = true;
        return st;
    }
    if (cm_path(p) && p->cfft) {   // several coils: the coil-fastest grid, own passes
        if (p->flags & NUFFT_FLAG_DETERMINISTIC) {
            // the exact sums rounded by the first inverse pass as it reads
            // them (no separate rounding pass over the grid)
            NUFFT_TRY(launch_y2k_cm_fixed(p, (const float2*)y, s));
            return cfft_inverse_fixed(p, p->d_igrid, p->d_dscal, (float2*)x, true, false, s);
        }
        NUFFT_TRY(launch_y2k_cm(p, (const float2*)y, p->d_grid, s));
        return cfft_inverse(p, p->d_grid, (float2*)x, true, false, s);
    }
    if (cm_path(p)) {   // several coils: the gridded spectra are written coil-major
        NUFFT_TRY(launch_y2k_cm(p, (const float2*)y, p->d_cm, s));
        return cm_to_image(p, (float2*)x, true, false, s);
    }
    NUFFT_TRY(launch_y2k(p, (const float2*)y, p->d_grid, s));
    if (p->B > 1) return image_from_spectrum_coils(p, p->d_grid, (float2*)x, true, false, s);
    return image_from_spectrum(p, p->d_grid, (float2*)x, true, false, s);
}

int nufft_selfadjoint(nufft_plan_t p, const void* x, void* x_out, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_selfadjoint"));
    NUFFT_TRY(need_ptrs(x, x_out, "nufft_selfadjoint"));
    NUFFT_TRY(nufft_forward(p, x, p->d_ybuf, stream));
    return nufft_adjoint(p, p->d_ybuf, x_out, stream);
}

int nufft_k2y2k(nufft_plan_t p, const void* k, void* k_out, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_k2y2k"));
    NUFFT_TRY(need_ptrs(k, k_out, "nufft_k2y2k"));
    cudaStream_t s = as_stream(stream);
    NUFFT_TRY(launch_k2y(p, (const float2*)k, p->d_ybuf, s));
    return launch_y2k_grid(p, p->d_ybuf, (float2*)k_out, s);
}

int nufft_solve_cg(nufft_plan_t p, const void* y, void* x, int maxiter, double rtol, double atol,
                   int* iters_out, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_solve_cg"));
    NUFFT_TRY(need_ptrs(y, x, "nufft_solve_cg", p));
    if (!(rtol >= 0) || !(atol >= 0)) {
        set_error("nufft_solve_cg: rtol and atol must be non-negative");
        return NUFFT_EINVAL;
    }
    return solve_cg(p, (const float2*)y, (float2*)x, maxiter, rtol, atol, iters_out,
                    as_stream(stream));
}

int nufft_solve_l1tvols(nufft_plan_t p, const void* y, void* x, int maxiter, double rho,
                        void* stream) {
    NUFFT_TRY(need_points(p, "nufft_solve_l1tvols"));
    NUFFT_TRY(need_ptrs(y, x, "nufft_solve_l1tvols", p));
    if (maxiter < 0) {
        set_error("nufft_solve_l1tvols: maxiter must be non-negative");
        return NUFFT_EINVAL;
    }
    return solve_l1tvols(p, (const float2*)y, (float2*)x, maxiter, rho, as_stream(stream));
}

int nufft_set_sense(nufft_plan_t p, const void* maps, int maps_on_device, void* stream) {
    NUFFT_TRY(need_plan(p, "nufft_set_sense"));
    if (p->ninst != 1) {
        set_error("nufft_set_sense: coil maps need a single-instance plan");
        return NUFFT_EUNSUPPORTED;
    }
    const size_t n = (size_t)p->prodN * p->B;
    if (!maps) {   // reset_sense: forget the maps
        cudaFree(p->d_maps);
        p->d_maps = nullptr;
        return NUFFT_OK;
    }
    if (!p->d_maps) {
        NUFFT_CUDA_TRY(cudaMalloc(&p->d_maps, sizeof(float2) * n));
        p->dev_bytes += sizeof(float2) * n;
    }
    NUFFT_CUDA_TRY(cudaMemcpyAsync(p->d_maps, maps, sizeof(float2) * n,
                                   maps_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                   as_stream(stream)));
    if (!maps_on_device) NUFFT_CUDA_TRY(cudaStreamSynchronize(as_stream(stream)));
    return NUFFT_OK;
}

int nufft_forward_one2many(nufft_plan_t p, const void* x, void* y, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_forward_one2many"));
    NUFFT_TRY(need_ptrs(x, y, "nufft_forward_one2many", p));
    if (!p->d_maps) {
        set_error("nufft_forward_one2many: nufft_set_sense has not been called");
        return NUFFT_EINVAL;
    }
    cudaStream_t s = as_stream(stream);
    NUFFT_TRY(launch_pad_sense(p, (const float2*)x, p->d_grid, s));
    NUFFT_TRY(fft_exec(p, p->d_grid, -1, s));
    return launch_k2y(p, p->d_grid, (float2*)y, s);
}

int nufft_adjoint_many2one(nufft_plan_t p, const void* y, void* x, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_adjoint_many2one"));
    NUFFT_TRY(need_ptrs(x, y, "nufft_adjoint_many2one", p));
    if (!p->d_maps) {
        set_error("nufft_adjoint_many2one: nufft_set_sense has not been called");
        return NUFFT_EINVAL;
    }
    cudaStream_t s = as_stream(stream);
    NUFFT_TRY(launch_y2k(p, (const float2*)y, p->d_grid, s));
    NUFFT_TRY(fft_exec(p, p->d_grid, +1, s));
    return launch_crop_sense(p, p->d_grid, (float2*)x, s);
}

int nufft_forward_dom(nufft_plan_t p, const void* x, void* dy, void* stream) {
    NUFFT_TRY(need_points(p, "nufft_forward_dom"));
    NUFFT_TRY(need_ptrs(x, dy, "nufft_forward_dom", p));
    cudaStream_t s = as_stream(stream);
    const size_t stride = (size_t)p->M * p->B;
    for (int d = 0; d < p->ndim; ++d) {
        // the forward's own path (several coils: coil-major, pruned FFTs)
        // with the image also multiplied by -i (n_d - N_d/2)
        NUFFT_TRY(forward_from_image(p, (const float2*)x, true, p->d_grid, s, d));
        NUFFT_TRY(launch_k2y(p, p->d_grid, (float2*)dy + d * stride, s));
    }
    return NUFFT_OK;
}

}  // extern "C"
